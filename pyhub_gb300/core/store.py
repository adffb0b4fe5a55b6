"""The solver.h5 tree — groups, datasets, attributes — kept in one .npz archive.

The reference writes a solve's inputs and results into solver.h5 and reads
them back lazily: the input group (core_solver.py:118-163), the solve group
(solve.f90:26-120), solve/lanczos (lanczos.f90:37-126), reduced_quantities
(static_rq.f90:16-45) and spgf (spgf_bandlanczos.f90:19-294).  h5py is not
part of this platform, so the same tree is stored as a numpy .npz archive:
dataset ``name`` of group ``G`` is the array ``"G/name"``, attribute ``name``
of group ``G`` is the array ``"G/@name"`` (attributes of the root: ``"@name"``).

A save writes a temporary file beside the target and renames it over the
target, so an interrupted save leaves the previous archive intact.
"""
from __future__ import annotations

import os

import numpy as np

ATTR = "@"


def flatten(tree: dict, prefix: str = "") -> dict:
    """Nested dict (groups) -> {"G/sub/name": array}; keys starting with '@' are attributes."""
    out = {}
    for k, v in tree.items():
        if not isinstance(k, str) or not k or "/" in k or k.startswith(ATTR + ATTR):
            raise ValueError(f"invalid group or dataset name {k!r}")
        key = prefix + k
        if isinstance(v, dict):
            if k.startswith(ATTR):
                raise ValueError(f"attribute {key!r} cannot hold a group")
            sub = flatten(v, key + "/")
            if not sub:
                sub = {key + "/" + ATTR + ATTR + "empty": np.array(True)}   # keeps empty groups
            out.update(sub)
        elif v is None:
            continue
        else:
            a = np.asarray(v)
            if a.dtype == object:
                raise TypeError(f"{key!r}: only numeric, boolean and string arrays can be stored")
            out[key] = a
    return out


def unflatten(flat) -> dict:
    """Inverse of :func:`flatten` (0-d arrays come back as numpy scalars)."""
    tree: dict = {}
    for key in sorted(flat.keys()):
        parts = key.split("/")
        node = tree
        for g in parts[:-1]:
            node = node.setdefault(g, {})
        if parts[-1] == ATTR + ATTR + "empty":
            continue
        a = np.asarray(flat[key])
        node[parts[-1]] = a[()] if a.ndim == 0 else a
    return tree


def save(path: str, tree: dict) -> str:
    """Write ``tree`` to ``path`` (".npz" is appended when missing); returns the path written."""
    if not path.endswith(".npz"):
        path = path + ".npz"
    flat = flatten(tree)
    tmp = path + ".tmp.npz"
    try:
        with open(tmp, "wb") as f:
            np.savez(f, **flat)
        os.replace(tmp, path)
    finally:
        if os.path.exists(tmp):
            os.remove(tmp)
    return path


def load(path: str) -> dict:
    """Read an archive written by :func:`save` back into a nested dict."""
    if not path.endswith(".npz") and not os.path.exists(path):
        path = path + ".npz"
    with np.load(path, allow_pickle=False) as z:
        return unflatten({k: z[k] for k in z.files})
