"""Static reduced quantities and Green's functions with the reference's API
(pyhub/core/reduced_quantities.py:6-169).

The reference reads Fortran-written datasets from solver.h5 on every
property access.  Here the same quantities are computed on the GPU
(ed_rdm: ONE_RDM, TWO_RDM's local-U branch and J_SPIN of static_rq.f90, or
J_SPIN of static_rq_heis.f90) for every Boltzmann-weighted state and kept in
memory with the reference's shapes: density matrices [NW, N, N] in the
Python view of the file (element [w][a][b] = DENS_MAT(b+1, a+1) of state w),
``ni`` [NW, N] and ``sisj`` [NW, N, N].
"""
from __future__ import annotations

import numpy as np

from ..tools.pole import Pole


def all_pairs(norb: int):
    return [(J, K) for J in range(1, norb + 1) for K in range(1, norb + 1)]


def lower_pairs(norb: int):
    """The pairs K <= J that ONE_RDM and J_SPIN evaluate before mirroring
    (static_rq.f90:161-241, 331-393)."""
    return [(J, K) for J in range(1, norb + 1) for K in range(1, J + 1)]


def scatter_pairs(raw: np.ndarray, pairs, norb: int) -> np.ndarray:
    """Raw per-pair sums of a pair list placed in the [norb*norb, nq] layout of
    all_pairs (rows of pairs that were not evaluated are zero)."""
    full = np.zeros((norb * norb, raw.shape[1]))
    idx = [(J - 1) * norb + (K - 1) for J, K in pairs]
    full[idx] = raw
    return full


def assemble_hubbard(raw: np.ndarray, norb: int, nup: int, ndn: int):
    """Reference symmetrisation of the raw ed_rdm sums in the all_pairs layout
    (only the rows K <= J are read):
    DENS_MAT(J,K) computed for K<=J and mirrored, the down matrix copied from
    the up one when N_up == N_down (static_rq.f90:161-241), NI from the local
    branch (:307-316), SMATRIX(J,K) for K<=J mirrored (:331-393).
    Returns (gamma_up, gamma_down, ni, sisj) as the reference's Python reads them."""
    q = raw.reshape(norb, norb, 6)  # q[J-1][K-1][:]
    gu = np.zeros((norb, norb))
    gd = np.zeros((norb, norb))
    sm = np.zeros((norb, norb))
    ni = np.zeros(norb)
    for J in range(norb):
        for K in range(J + 1):
            if J == K:
                nu, nd, do, zz = q[J, J, 0], q[J, J, 2], q[J, J, 3], q[J, J, 1]
                gu[J, J] = nu
                gd[J, J] = nd
                ni[J] = do
                sm[J, J] = 0.5 * (nu - do) + 0.5 * (nd - do) + zz
            else:
                gu[J, K] = gu[K, J] = q[J, K, 0]
                gd[J, K] = gd[K, J] = q[J, K, 4]
                sm[J, K] = sm[K, J] = q[J, K, 5] + q[J, K, 1]
    if nup == ndn:
        gd = gu.copy()
    return gu, gd, ni, sm


def assemble_heisenberg(raw: np.ndarray, norb: int):
    """SMATRIX(J,K) for every J,K (static_rq_heis.f90:66-114); the Python
    view of the file is its transpose."""
    q = raw.reshape(norb, norb, 2)
    smat = q[:, :, 0] + q[:, :, 1]      # [J-1][K-1] = SMATRIX(J,K)
    return smat.T.copy()


class StaticQuantities:

    def __init__(self):
        pass

    def _wnorm(self):
        return self.wgt / np.sum(self.wgt)

    @property
    def one_rdm(self):
        w = self._wnorm()
        return {"up": np.einsum("ijk,i->jk", self._rq["density_matrix_up"], w),
                "down": np.einsum("ijk,i->jk", self._rq["density_matrix_down"], w)}

    @property
    def ni(self):
        return np.einsum("ij,i->j", self._rq["ni"], self._wnorm())

    @property
    def two_rdm(self):
        """DBL_OCC(J,K,M,N) weighted over the states, as the reference's
        two_rdm returns it (reduced_quantities.py:25-27): [J-1,K-1,M-1,N-1].
        Stored only for the U_ijkl interaction (is_Uloc=3), as in the reference."""
        dbl = self._rq.get("dbl_occ") if self._rq else None
        if dbl is None:
            raise KeyError("reduced_quantities/dbl_occ is formed only for the U_ijkl interaction (is_Uloc=3)")
        return np.einsum("bijkl,b->ijkl", dbl, self._wnorm())

    @property
    def density(self):
        return {spin: np.diag(self.one_rdm[spin]) for spin in ["up", "down"]}

    @property
    def density_matrix(self):
        return self.one_rdm

    @property
    def one_rdm0(self):
        return {"up": self.Vk @ np.diag([1.0 if i < self.nup[0] else 0.0 for i in range(self.nb_sites)]) @ self.Vk.T,
                "down": self.Vk @ np.diag([1.0 if i < self.ndown[0] else 0.0 for i in range(self.nb_sites)]) @ self.Vk.T}

    @property
    def density_matrix0(self):
        return self.one_rdm0

    @property
    def wi(self):
        return self.ni

    @property
    def spin_cor_matrix(self):
        return np.einsum("ijk,i->jk", self._rq["sisj"], self._wnorm())

    @property
    def s2(self):
        return np.sum(self.spin_cor_matrix)

    @property
    def eta_k(self):
        return {"up": np.diag(self.Vk.T @ self.density_matrix["up"] @ self.Vk),
                "down": np.diag(self.Vk.T @ self.density_matrix["down"] @ self.Vk)}

    @property
    def eta_k0(self):
        return {"up": np.array([1.0 if i < self.nup[0] else 0.0 for i in range(self.nb_sites)]),
                "down": np.array([1.0 if i < self.ndown[0] else 0.0 for i in range(self.nb_sites)])}

    @property
    def e_one_body(self):
        return (np.einsum("ij,ij->", self.one_rdm["up"], self.t_matrix)
                + np.einsum("ij,ij->", self.one_rdm["down"], self.t_matrix))

    @property
    def e_two_body(self):
        """reduced_quantities.py:68-75: with the U_ijkl interaction the
        reference contracts its dbl_occ dataset ('lkjib' of the file's
        [N][M][K][J][b] = DBL_OCC(J,K,M,N)) with U[i,j,k,l]."""
        sj = np.einsum("bij,ij,b", self._rq["sisj"], self.J_matrix, self._wnorm())
        dbl = self._rq.get("dbl_occ") if self._rq else None
        if dbl is not None:
            return np.einsum("bijkl,ijkl,b", dbl, self.U_matrix, self._wnorm()) + sj
        return np.sum(self.ni * self.U_matrix) + sj


class GreenFunction:

    def __init__(self):
        pass

    def compute_gf(self):
        """G[spin][i,j] as Pole objects, with the reference's pole placement
        (reduced_quantities.py:84-92): greater poles at E_n(N+1) - E0, lesser
        poles at E0 - E_n(N-1), weights from the start-vector overlaps."""
        w = self._wnorm()
        gf = {}
        for spin in ("up", "down"):
            g = np.empty((self.nb_sites_comp, self.nb_sites_comp), dtype=object)
            for i in range(self.nb_sites_comp):
                for j in range(self.nb_sites_comp):
                    parts = []
                    for b, wb in enumerate(w):
                        if wb == 0.0:
                            continue
                        for part in ("greater", "lesser"):
                            pos, wts = self._spgf[b][spin][part].pole(i, j)
                            parts.append(Pole({"positions": pos, "weights": wts * wb}).clean(wtol=1.e-8))
                    g[i, j] = Pole.sum(parts)
            gf[spin] = g
        return gf

    @property
    def nb_poles(self):
        b0 = self._spgf[0]
        return np.array([[b0["up"]["lesser"].npoles, b0["down"]["lesser"].npoles],
                         [b0["up"]["greater"].npoles, b0["down"]["greater"].npoles]], dtype=int)

    @property
    def ip(self):
        return {spin: (self._spgf[0][spin]["lesser"].e_lowest - self.e0) for spin in ["up", "down"]}

    @property
    def ae(self):
        return {spin: (self.e0 - self._spgf[0][spin]["greater"].e_lowest) for spin in ["up", "down"]}

    @property
    def mu(self):
        return {spin: (-self.ip[spin] - self.ae[spin]) / 2 for spin in ["up", "down"]}

    @property
    def density_matrix_from_gf(self):
        return self.one_rdm_from_gf

    @property
    def one_rdm_from_gf(self):
        w = self._wnorm()
        out = {}
        for spin in ("up", "down"):
            out[spin] = sum(wb * self._spgf[b][spin]["lesser"].static() for b, wb in enumerate(w) if wb != 0.0)
        return out

    @property
    def gf0(self):
        return {"up": np.array([[Pole({"positions": self.ek, "weights": self.Vk[i, :] * self.Vk[j, :]})
                                 for i in range(self.nb_sites)] for j in range(self.nb_sites)]),
                "down": np.array([[Pole({"positions": self.ek, "weights": self.Vk[i, :] * self.Vk[j, :]})
                                   for i in range(self.nb_sites)] for j in range(self.nb_sites)])}

    def gf_matrix(self, w, eta=0.05, device=None, raw=False):
        """G_s(w)[k, i, j] = sum_p weight_p / (w_k - position_p + i eta) for all
        frequencies at once: every (i, j) pole set is padded into one [n, n, P]
        array and the sum runs as one tensor contraction (on the GPU when there
        is one).  raw=False reads the poles of self.gf (after Pole.clean, as
        compute_gf leaves them); raw=True sums the uncleaned poles of every
        computed state, as the reference's self_energy forms G from the stored
        Q and positions (reduced_quantities.py:134-161): weighted by
        wgt/sum(wgt) when N_up == N_down, unweighted otherwise.
        Returns {spin: complex128 torch tensor [nw, n, n]}."""
        import torch
        dev = device or ("cuda" if torch.cuda.is_available() else "cpu")
        wv = torch.as_tensor(np.atleast_1d(np.asarray(w, dtype=np.float64)), device=dev)
        n = self.nb_sites_comp
        out = {}
        for s in ("up", "down"):
            sets = [[None] * n for _ in range(n)]
            for i in range(n):
                for j in range(n):
                    if not raw:
                        pl = self.gf[s][i, j].pole
                        sets[i][j] = (np.asarray(pl["positions"]), np.asarray(pl["weights"]))
                        continue
                    same = self.nup[0] == self.ndown[0]
                    wn = self._wnorm() if same else np.ones(len(self.wgt))
                    ps, ws = [], []
                    for b, wb in enumerate(wn):
                        if self._spgf[b] is None:
                            continue
                        for part in ("greater", "lesser"):
                            pos, wts = self._spgf[b][s][part].pole(i, j)
                            ps.append(pos)
                            ws.append(wts * wb)
                    sets[i][j] = (np.concatenate(ps) if ps else np.zeros(0), np.concatenate(ws) if ws else np.zeros(0))
            P = max(1, max(len(sets[i][j][0]) for i in range(n) for j in range(n)))
            pos = np.zeros((n, n, P))
            wts = np.zeros((n, n, P))
            for i in range(n):
                for j in range(n):
                    k = len(sets[i][j][0])
                    pos[i, j, :k] = sets[i][j][0]
                    wts[i, j, :k] = sets[i][j][1]
            pos_t = torch.as_tensor(pos, device=dev)
            wts_t = torch.as_tensor(wts, device=dev).to(torch.complex128)
            den = wv[:, None, None, None] - pos_t[None] + 1j * eta
            out[s] = (wts_t[None] / den).sum(dim=-1)
        return out

    @property
    def galitskii_migdal(self):
        """Left unimplemented by the reference (reduced_quantities.py:164-166): None."""
        return None

    @property
    def qpw(self) -> np.ndarray:
        """Quasi-particle weight (reduced_quantities.py:168-169):
        pinv(1 - Re dSigma_up/dw) at w = mu['up'], the derivative taken as the
        reference takes it, scipy.misc.derivative(order=3, dx=1e-6): the
        three-point central difference (Sigma(mu+dx) - Sigma(mu-dx)) / (2 dx),
        of the self-energy at eta = 1e-4.  Both frequencies are evaluated in
        one batched self_energy call."""
        dx = 1.e-6
        mu = float(self.mu["up"])
        sig = self.self_energy(np.array([mu - dx, mu + dx]), eta=0.0001)["up"]   # [j][i][k]
        d = (sig[:, :, 1] - sig[:, :, 0]).T / (2.0 * dx)
        return np.linalg.pinv(np.identity(self.nb_sites) - np.real(d))

    def self_energy(self, w, eta=0.05):
        """Sigma(w) = pinv(G0(w)) - pinv(G(w)) (reduced_quantities.py:134-161):
        G0 from the hopping matrix's eigenpairs (ek, Vk), G from the uncleaned
        poles of every computed state (gf_matrix(raw=True)), as the reference
        forms it from the stored Q and positions.  For an array of frequencies
        all of them are done at once (batched pseudo-inverses) and the result
        keeps the reference's layout [j][i][k] = Sigma(w_k)[i, j]; for one
        frequency it returns {spin: [n, n]}."""
        import torch
        scalar = not isinstance(w, (list, np.ndarray))
        wv = np.atleast_1d(np.asarray(w, dtype=np.float64))
        G = self.gf_matrix(wv, eta=eta, raw=True)
        dev = G["up"].device
        n = self.nb_sites_comp
        Vk = torch.as_tensor(self.Vk, device=dev).to(torch.complex128)
        ek = torch.as_tensor(self.ek, device=dev)
        wt = torch.as_tensor(wv, device=dev)
        d0 = 1.0 / (wt[:, None] - ek[None, :] + 1j * eta)                 # [nw, nk]
        g0 = torch.einsum("ik,jk,wk->wij", Vk, Vk, d0)
        g0i = torch.linalg.pinv(g0, rtol=1e-15)[:, :n, :n]
        sig = {s: g0i - torch.linalg.pinv(G[s], rtol=1e-15) for s in ("up", "down")}
        if scalar:
            return {s: v[0].cpu().numpy() for s, v in sig.items()}
        return {s: v.permute(2, 1, 0).cpu().numpy() for s, v in sig.items()}
