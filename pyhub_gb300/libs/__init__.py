"""Native library loader.

The reference keeps a ctypes loader here for a ``libsrc`` that is never built
(pyhub/libs/__init__.py:9-23).  In this package the same hook loads the CUDA
extension ``libpyhub_ed.so`` and is required: there is no CPU fallback, and
every compute entry point raises if the library is absent.
"""
from __future__ import annotations

import ctypes
import logging
import os

log = logging.getLogger(__name__)

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_libcore = None


def library_path() -> str:
    return os.path.join(_PKG, "libpyhub_ed.so")


def load_library(required: bool = True):
    """Load ``libpyhub_ed.so`` (built in-tree by ``pyhub_gb300._build``)."""
    global _libcore
    if _libcore is not None:
        return _libcore
    path = library_path()
    if not os.path.exists(path):
        msg = (f"{path} is missing: build the CUDA extension first "
               "(python -c 'import __graft_entry__ as g; g.build()' or python -m pyhub_gb300._build)")
        if required:
            raise ImportError(msg)
        log.debug(msg)
        return None
    _libcore = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    return _libcore


def libcore():
    return load_library(required=True)
