"""Single-particle Green's function by continued fractions.

The reference runs a band Lanczos over the block {c_i|psi0>} (or
{c^+_i|psi0>}) and returns Ritz values and overlap weights
(GF_BANDLANCZOS, spgf_bandlanczos.f90:309-448; or exact Lehmann sums for small
sectors, spgf_ed.f90:1-429).  Here every start vector phi = c_i|psi0>,
c^+_i|psi0> (and (c_i + c_j)|psi0> for off-diagonal elements) gets its own
three-term Lanczos on the GPU; the tridiagonal T of m steps gives
<phi|(z-H)^-1|phi> = |phi|^2 / (z - a_0 - b_1^2/(z - a_1 - ...)), i.e. poles
at the eigenvalues of T with weights |phi|^2 (first component)^2.  Poles are
placed as the reference's compute_gf places them (reduced_quantities.py:84-92):
greater at E_n - E0, lesser at E0 - E_n.  When N_up == N_down only spin up is
computed and copied to spin down, as the reference does
(spgf_bandlanczos.f90:92-97,110-115).
"""
from __future__ import annotations

import math

import numpy as np

from .. import _capi
from . import lanczos as LZ


class PoleBlock:
    """Poles of one (spin, greater|lesser) part for sites 0..n-1."""

    def __init__(self, n: int, sign: float, e0: float):
        self.n = n
        self.sign = sign          # +1: greater (E_n - E0), -1: lesser (E0 - E_n)
        self.e0 = e0
        self.diag = {}            # i -> (eigs, weights)
        self.pair = {}            # (i,j) -> (eigs, weights) of (c_i + c_j)
        self.norm2 = {}
        self.norm2_pair = {}

    def _place(self, eig):
        return (eig - self.e0) if self.sign > 0 else (self.e0 - eig)

    def pole(self, i: int, j: int):
        if i == j:
            e, w = self.diag.get(i, (np.zeros(0), np.zeros(0)))
            return self._place(e), w
        a, b = (i, j) if i < j else (j, i)
        if (a, b) not in self.pair:
            return np.zeros(0), np.zeros(0)
        ep, wp = self.pair[(a, b)]
        ei, wi = self.diag.get(a, (np.zeros(0), np.zeros(0)))
        ej, wj = self.diag.get(b, (np.zeros(0), np.zeros(0)))
        pos = np.concatenate([self._place(ep), self._place(ei), self._place(ej)])
        wts = np.concatenate([0.5 * wp, -0.5 * wi, -0.5 * wj])
        return pos, wts

    @property
    def npoles(self):
        return max((len(e) for e, _ in self.diag.values()), default=0)

    @property
    def e_lowest(self):
        """Lowest N-1 / N+1 eigenvalue reached by the start vectors."""
        vals = [e[np.argmax(w > 1e-12)] if np.any(w > 1e-12) else np.inf for e, w in self.diag.values()]
        return float(min(vals)) if vals else float("nan")

    def static(self):
        """<c^+_j c_i> (lesser) or <c_i c^+_j> (greater) from the start-vector overlaps."""
        m = np.zeros((self.n, self.n))
        for i in range(self.n):
            m[i, i] = self.norm2.get(i, 0.0)
        for (a, b), v in self.norm2_pair.items():
            m[a, b] = m[b, a] = 0.5 * (v - m[a, a] - m[b, b])
        return m


def continued_fraction_poles(sec, phi, nsteps: int):
    """Eigenvalues of the m-step Lanczos tridiagonal of phi and the pole
    weights |phi|^2 z_0k^2."""
    torch = LZ._torch()
    nrm2 = float((phi.double() * phi.double()).sum().item())
    if nrm2 <= 1e-28:
        return np.zeros(0), np.zeros(0), 0.0
    steps = int(min(nsteps, sec.dim))
    free, _ = torch.cuda.mem_get_info()
    if (steps + 2) * sec.n * phi.element_size() <= min(0.25 * free, 8e9):
        # small basis: full reorthogonalisation, exact breakdown at the Krylov dimension
        r = LZ.lanczos_full(sec, phi, steps, phi.dtype, want_vector=False)
    else:
        r = LZ.lanczos_plain(sec, phi, steps, rule=None, want_vectors=False)
    w = nrm2 * r.ritz_vectors[0, :] ** 2
    return r.ritz, w, nrm2


def particle_hole_poles(solver, psi, e0: float, ncomp: int, nsteps: int = None, offdiag: bool = True,
                        dtype=None):
    """Pole blocks {spin: {'greater': PoleBlock, 'lesser': PoleBlock}} of one state."""
    torch = LZ._torch()
    nup, ndn = solver.nup[0], solver.ndown[0]
    src = solver.sector(nup, ndn)
    out = {}
    spins = ("up",) if nup == ndn else ("up", "down")
    for spin in spins:
        res = {}
        for part, kind in (("greater", "e_" + spin), ("lesser", "h_" + spin)):
            du = (1 if part == "greater" else -1) if spin == "up" else 0
            dd = (1 if part == "greater" else -1) if spin == "down" else 0
            blk = PoleBlock(ncomp, +1.0 if part == "greater" else -1.0, e0)
            n1, d1 = nup + du, ndn + dd
            if 0 <= n1 <= solver.nb_sites and 0 <= d1 <= solver.nb_sites:
                dst = solver.sector(n1, d1)
                m = nsteps if nsteps is not None else min(max(solver.max_lcz - 10, 10), dst.dim)
                vt = dtype or psi.dtype
                starts = []
                for i in range(ncomp):
                    phi = torch.zeros(dst.n, dtype=vt, device=psi.device)
                    _capi.gf_start(src, dst, kind, i + 1, psi, phi)
                    starts.append(phi)
                    e, w, n2 = continued_fraction_poles(dst, phi, m)
                    blk.diag[i] = (e, w)
                    blk.norm2[i] = n2
                if offdiag:
                    for i in range(ncomp):
                        for j in range(i + 1, ncomp):
                            phi = starts[i] + starts[j]
                            e, w, n2 = continued_fraction_poles(dst, phi, m)
                            blk.pair[(i, j)] = (e, w)
                            blk.norm2_pair[(i, j)] = n2
                del starts
            res[part] = blk
        out[spin] = res
    if nup == ndn:
        out["down"] = out["up"]
    return out
