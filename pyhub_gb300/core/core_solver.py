"""CoreSolver with the reference's API (pyhub/core/core_solver.py:17-291).

The reference marshals every parameter into solver.h5, runs a Fortran
executable with os.system and reads results back lazily
(core_solver.py:31-111, 118-249).  Here ``kernel`` runs in process on the
GPU through the C ABI and keeps results in memory; the property names,
signatures and return shapes are the reference's.

Solve dispatch follows SOLVE (solve.f90:1-23): a sector smaller than
``max_lcz`` is diagonalised densely (EXACT_DIAG, exact_diag.f90:2-33, its
columns built with the GPU H*v), a larger one with Lanczos under the
reference's convergence rule (lanczos.f90:44-91) at most max_lcz-5 steps.
Extra keyword arguments select the precision ("f64", "mixed" = FP32 vectors
with FP64 scalars and an FP64 refinement, "auto") and the
reorthogonalisation ("full" when the basis fits in device memory, else the
reference's three-term recurrence with the Ritz vector rebuilt by a second
pass instead of being read back from stored vectors).
"""
from __future__ import annotations

import math
import os
from copy import deepcopy as dc
from time import perf_counter as pc

import numpy as np

from .. import _capi
from ..trace import nvtx
from . import lanczos as LZ
from . import store
from .basis import Basis
from .reduced_quantities import (GreenFunction, StaticQuantities, all_pairs, assemble_heisenberg,
                                 assemble_hubbard, lower_pairs, scatter_pairs)

F32_TOL14 = float(np.float32(1e-14))
F32_TOL8 = float(np.float32(1e-8))


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pyhub_gb300 runs on a CUDA GPU; no device is visible")
    return torch


class CoreSolver(Basis, GreenFunction, StaticQuantities):

    def __init__(self, nb_sites, n_up: int, n_down: int, exec_name, T=0., order='spin'):
        Basis.__init__(self, nb_sites, hilbert=(n_up, n_down), order=order)
        self.T = T
        self.exec_name = exec_name
        self.t_matrix = np.zeros((nb_sites, nb_sites))
        self.J_matrix = np.zeros((nb_sites, nb_sites))
        self.U = 0.
        self.is_solve = False
        self.is_reduced_quantities = False
        self.is_spgf = False
        self.is_tprf = False
        self.excited_state = 0
        self._sol = None
        self._rq = None
        self._spgf = None
        self._sectors = {}

    # ----------------------------------------------------------- sectors
    @property
    def _kind(self):
        return _capi.ED_HEISENBERG if self.exec_name == 'heisenberg.x' else _capi.ED_HUBBARD

    def _u_vector(self):
        U = self.U
        if isinstance(U, (float, int, np.floating, np.integer)):
            return np.full(self.nb_sites, float(U))
        U = np.asarray(U, dtype=np.float64)
        if U.ndim == 1 and U.shape == (self.nb_sites,):
            return U
        if U.ndim == 4 and U.shape == (self.nb_sites,) * 4:
            # is_Uloc=3 (core_solver.py:141-147): the interaction replaces the on-site U
            if not np.isclose(U, np.einsum('ijkl->jilk', U)).all():
                raise ValueError('U tensor must be symmetric')
            return np.zeros(self.nb_sites)
        raise ValueError(f'U must be a float or a np.ndarray of size (nb_sites,) or '
                         f'(nb_sites,nb_sites,nb_sites,nb_sites,), not {type(self.U)}')

    @property
    def _uijkl(self):
        """The U tensor when the interaction is the general U_ijkl (is_Uloc=3), else None."""
        U = self.U
        return U if isinstance(U, np.ndarray) and U.ndim == 4 else None

    def sector(self, nup: int, ndn: int):
        key = (int(nup), int(ndn))
        if key not in self._sectors:
            if self._kind == _capi.ED_HUBBARD:
                sec = _capi.Sector(self.nb_sites, nup, ndn, _capi.ED_HUBBARD,
                                   t=np.asarray(self.t_matrix, dtype=np.float64), U=self._u_vector())
                if self._uijkl is not None:
                    sec.set_uijkl(self._uijkl)
                self._sectors[key] = sec
            else:
                self._sectors[key] = _capi.Sector(self.nb_sites, nup, ndn, _capi.ED_HEISENBERG,
                                                  J=np.asarray(self.J_matrix, dtype=np.float64))
        return self._sectors[key]

    # ----------------------------------------------------------- solve
    def kernel(self, max_lcz: int = 600, acc_lcz: float = 1.e-8, nb_comp_states=1, compute_rq=True,
               compute_spgf=False, nb_sites_comp=None, store_H=False, verbose=False, *, dtype: str = "auto",
               reorth: str = "auto", seed: int = 0, refine_steps: int = 60, store_lanczos_vectors: bool = False):
        torch = _torch()
        self.max_lcz = max_lcz
        self.acc_lcz = acc_lcz
        self.compute_rq = compute_rq
        self.nb_comp_states_ = nb_comp_states
        self.compute_spgf = compute_spgf
        self.compute_tprf = False
        self.store_H = store_H
        self.verbose = verbose
        self._store_lcz = bool(store_lanczos_vectors)
        self.nb_sites_comp = self.nb_sites if nb_sites_comp is None else nb_sites_comp
        tall = pc()
        self._sectors = {}
        self._rq = None
        self._spgf = None
        with nvtx("pyhub.sector"):
            sec = self.sector(self.nup[0], self.ndown[0])
        self.printv('start calculation')
        with nvtx("pyhub.solve"):
            if sec.dim < max_lcz:
                self._sol = self._exact_diag(sec, store_H)
            else:
                self._sol = self._lanczos(sec, max_lcz, acc_lcz, nb_comp_states, dtype, reorth, seed, refine_steps)
        self._sol["boltzmann"] = self._boltzmann(self._sol["eigenvalues"], nb_comp_states)
        self.is_solve = True
        self.wgt = dc(self.boltzmann)
        torch.cuda.synchronize()
        if compute_rq:
            self.reduced_quantities()
        if compute_spgf:
            self.spgf(nb_sites_comp=self.nb_sites_comp)
        self.time = pc() - tall
        self.printv(f'total elapsed time {np.around(self.time, 4)} s\n')

    def _exact_diag(self, sec, store_H):
        torch = _torch()
        D = sec.dim
        cols = torch.zeros((D, sec.n), dtype=torch.float64, device="cuda")
        e = torch.zeros(sec.n, dtype=torch.float64, device="cuda")
        eref = sec.to_ref(torch.arange(sec.n, device="cuda", dtype=torch.float64))
        pos = eref.long()  # internal position of reference index i
        for i in range(D):
            e.zero_()
            e[pos[i]] = 1.0
            sec.hv(e, cols[i])
        H = sec.to_ref(cols).T.contiguous().cpu().numpy()  # H[:, i] = H e_i
        val, vec = np.linalg.eigh(H)
        ndeg = 1
        for i in range(1, len(val)):
            if abs(val[i] - val[0]) < F32_TOL14:
                ndeg += 1
            else:
                break
        return {"eigenvalues": val, "eigenvectors_ref": vec, "is_lanczos": False, "deg": ndeg,
                "H": H if store_H else None, "nstates": D}

    def _lanczos(self, sec, max_lcz, acc_lcz, nb_comp_states, dtype, reorth, seed, refine_steps):
        torch = _torch()
        steps = max(max_lcz - 5, 5)
        if dtype == "auto":
            dtype = "f64" if (sec.dim <= (1 << 22) or nb_comp_states > 1 or self.T > F32_TOL8) else "mixed"
        if dtype not in ("f64", "mixed", "f32"):
            raise ValueError(f"dtype must be 'auto', 'f64', 'mixed' or 'f32', not {dtype}")
        esz = 8 if dtype == "f64" else 4
        free, _ = torch.cuda.mem_get_info()
        fits = (steps + 3) * sec.n * esz <= 0.8 * free
        if reorth == "auto":
            reorth = "full" if fits else "none"
        v0 = LZ.start_vector(sec, seed)
        rule = LZ.ReferenceRule(acc_lcz)
        lcz = None
        nvec = max(1, int(nb_comp_states))
        if reorth == "full":
            if dtype == "f64":
                r = LZ.lanczos_full(sec, v0, steps, torch.float64, rule=rule, want_vector=False, keep_basis=True)
                psis = [r.ritz_vector(k) for k in range(min(nvec, r.steps))]
                if getattr(self, "_store_lcz", False):
                    # the normalised Krylov vectors q_j = s_j u_j, reference basis order, as LANCZOS
                    # stores them in solver.h5 (lanczos.f90:42-49)
                    lcz = np.stack([sec.to_ref(r.basis[j] * float(r.scales[j])).cpu().numpy()
                                    for j in range(r.steps)], axis=1)
                ritz, alpha, beta, steps_done, conv = r.ritz, r.alpha, r.beta, r.steps, r.converged
                r.release()
            else:
                # mixed: the FP32 Ritz vector only starts the FP64 stage, so it is summed in FP32
                r = LZ.lanczos_full(sec, v0.to(torch.float32), steps, torch.float32, rule=rule,
                                    ritz_dtype=torch.float32 if dtype == "mixed" else None)
                e32 = float(r.ritz[0])
                psi = r.psi
                r.release()
                if dtype == "mixed":
                    # the FP64 stage as in lanczos.ground_state: energy checked every REFINE_CHECK steps
                    rr = LZ.EnergyRule(1e-13 * max(1.0, abs(e32)), min_steps=2 * LZ.REFINE_CHECK)
                    r2 = LZ.lanczos_full(sec, psi, refine_steps, torch.float64, rule=rr, check_every=LZ.REFINE_CHECK)
                    psi = r2.psi
                    ritz = np.concatenate([[r2.ritz[0]], r.ritz[1:]])
                    r2.release()
                else:
                    ritz = r.ritz
                psis = [psi]
                alpha, beta, steps_done, conv = r.alpha, r.beta, r.steps, r.converged
        else:
            vt = torch.float64 if dtype == "f64" else torch.float32
            # the Krylov rows are kept where they fit (one block shared by both stages),
            # else the Ritz vectors are rebuilt by a second run
            storage = LZ.kept_storage(v0.device, max((steps + 1) * sec.n * (8 if dtype == "f64" else 4),
                                                     (refine_steps + 1) * sec.n * 8 if dtype == "mixed" else 0),
                                      min_bytes=4 * sec.n * 8)
            r = LZ.lanczos_plain(sec, v0.to(vt), steps, rule=rule, nvec=nvec, storage=storage)
            psis = r.psis
            ritz, alpha, beta, steps_done, conv = r.ritz, r.alpha, r.beta, r.steps, r.converged
            if dtype == "mixed":
                # FP64 three-term refinement from the FP32 Ritz vector
                rr = LZ.EnergyRule(1e-13 * max(1.0, abs(float(ritz[0]))), min_steps=10)
                r2 = LZ.lanczos_plain(sec, psis[0], refine_steps, rule=rr, nvec=1, storage=storage)
                psis = [r2.psis[0]] + list(psis[1:])
                ritz = np.concatenate([[r2.ritz[0]], ritz[1:]])
            del storage
        out = {"eigenvalues": np.asarray(ritz), "psis": psis, "is_lanczos": True, "deg": rule.ndeg,
               "alpha": alpha, "beta": beta, "nb_lcz": steps_done, "conv": rule.conv,
               "converged": conv, "H": None, "nstates": sec.dim, "precision": dtype, "reorth": reorth}
        if lcz is not None:
            out["lcz_vectors"] = lcz
        return out

    def _boltzmann(self, val, nb_comp_states):
        """BOLTZMANN (boltzmann.f90:1-29)."""
        T = self.T
        nval = len(val)
        nw = nval + 1
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            for k in range(2, nval + 1):
                if np.exp((val[0] - val[k - 1]) / T) <= F32_TOL8:
                    nw = k
                    break
        nw = max(nw - 1, nb_comp_states)
        w = np.zeros(nw)
        if T >= F32_TOL8:
            w[:] = np.exp((val[0] - val[:nw]) / T)
        else:
            w[0] = 1.0
        return w

    def set_state(self, excited_state=-1):
        self.excited_state = excited_state
        self.wgt = dc(self.boltzmann)
        if excited_state != -1:
            self.wgt[:] = 0.
            self.wgt[excited_state] = 1.

    # ----------------------------------------------------------- states
    def _state_device(self, k: int):
        """State k (FP64, internal layout of the solve sector)."""
        torch = _torch()
        sec = self.sector(self.nup[0], self.ndown[0])
        if not self._sol["is_lanczos"]:
            v = torch.tensor(self._sol["eigenvectors_ref"][:, k], dtype=torch.float64, device="cuda")
            return sec.from_ref(v)
        psis = self._sol["psis"]
        if k >= len(psis) or psis[k] is None:
            raise IndexError(f"state {k} was not kept; raise nb_comp_states in kernel()")
        return psis[k]

    def reduced_quantities(self):
        with nvtx("pyhub.reduced_quantities"):
            self._reduced_quantities()

    def _reduced_quantities(self):
        t0 = pc()
        self.printv('start reduced quantities calculation')
        sec = self.sector(self.nup[0], self.ndown[0])
        nw = len(self.wgt)
        N = self.nb_sites
        dm_up = np.zeros((nw, N, N))
        dm_dn = np.zeros((nw, N, N))
        ni = np.zeros((nw, N))
        sisj = np.zeros((nw, N, N))
        two_body = self._uijkl is not None and self._kind == _capi.ED_HUBBARD
        dbl = np.zeros((nw, N, N, N, N)) if two_body else None
        # DBL_OCC is formed for K <= J and N <= M and copied to the three other orders (static_rq.f90:256-303)
        quads = [(J, K, M, Nn) for J in range(1, N + 1) for K in range(1, J + 1)
                 for M in range(1, N + 1) for Nn in range(1, M + 1)] if two_body else None
        for b in range(nw):
            if self.wgt[b] == 0.0 and b > 0:
                continue
            psi = self._state_device(b)
            if self._kind == _capi.ED_HUBBARD:
                flags = 2 | (1 if self.nup[0] != self.ndown[0] else 0)
                pairs = lower_pairs(N)   # K <= J, mirrored by the assembly, as the reference does
                raw, _ = sec.rdm_raw(psi, pairs=pairs, flags=flags)
                gu, gd, n_, sm = assemble_hubbard(scatter_pairs(raw, pairs, N), N, self.nup[0], self.ndown[0])
                dm_up[b], dm_dn[b], ni[b], sisj[b] = gu, gd, n_, sm
                if two_body:
                    vals, _ = sec.dbl_occ(psi, quads=quads)
                    for (J, K, M, Nn), v in zip(quads, vals):
                        for a, c in ((J, K), (K, J)):
                            dbl[b, a - 1, c - 1, M - 1, Nn - 1] = v
                            dbl[b, a - 1, c - 1, Nn - 1, M - 1] = v
                    ni[b] = [dbl[b, j, j, j, j] for j in range(N)]   # NI(J) = DBL_OCC(J,J,J,J) on this path
            else:
                raw, _ = sec.rdm_raw(psi, pairs=all_pairs(N))
                sisj[b] = assemble_heisenberg(raw, N)
        self._rq = {"density_matrix_up": dm_up, "density_matrix_down": dm_dn, "ni": ni, "sisj": sisj,
                    "dbl_occ": dbl}
        self.is_reduced_quantities = True
        self.printv(f'end calculation | elapsed time {np.around(pc() - t0, 4)} s')

    def spgf(self, nb_sites_comp=None, nsteps: int = None, offdiag: bool = True):
        with nvtx("pyhub.spgf"):
            self._spgf_run(nb_sites_comp, nsteps, offdiag)

    def _spgf_run(self, nb_sites_comp, nsteps, offdiag):
        from . import greens as GR
        self.nb_sites_comp = self.nb_sites if nb_sites_comp is None else nb_sites_comp
        if self._kind != _capi.ED_HUBBARD:
            raise NotImplementedError("Green's functions are defined for the Hubbard solver")
        if self.T > F32_TOL8 and self._sol["is_lanczos"]:
            raise ValueError('SET TEMPERATURE TO 0 FOR LANCZOS GF')
        t0 = pc()
        self.printv('start spgf calculation')
        out = []
        for b in range(len(self.wgt)):
            if self.wgt[b] == 0.0 and b > 0:
                out.append(None)
                continue
            out.append(GR.particle_hole_poles(self, self._state_device(b), float(self.e[b]), self.nb_sites_comp,
                                              nsteps=nsteps, offdiag=offdiag))
        self._spgf = out
        self.is_spgf = True
        self.printv(f'end calculation | elapsed time {np.around(pc() - t0, 4)} s')
        self.gf = self.compute_gf()

    def tprf(self):
        pass

    def printv(self, *args):
        if self.verbose:
            print(*args)

    # ----------------------------------------------------------- persistence
    @property
    def archive(self):
        """Default archive of save()/restore(): the solver.h5 tree as solver.npz."""
        return os.path.splitext(self.filename)[0] + ".npz"

    def write_in(self):
        """The input group of solver.h5 (core_solver.py:118-163): parameters and flags."""
        grp = {"@nb_sites": self.nb_sites, "@n_up": self.nup[0], "@n_down": self.ndown[0],
               "@do_solution": True, "@do_rq": bool(self.is_reduced_quantities), "@do_spgf": bool(self.is_spgf),
               "@do_tprf": False, "@store_H": bool(getattr(self, "store_H", False)),
               "@nb_sites_comp": int(getattr(self, "nb_sites_comp", self.nb_sites)), "@exec_name": self.exec_name}
        U = self._uijkl
        if U is not None:
            grp.update({"@is_Uloc": 3, "U": np.asarray(U, dtype=np.float64),
                        "Upartial": np.einsum('ijkl,ijkl->ij', U, U), "@do_rq_two_body": True})
        elif self._kind == _capi.ED_HUBBARD:
            grp.update({"@is_Uloc": 2, "U": self._u_vector(), "@do_rq_two_body": False})
        grp["t_matrix"] = np.asarray(self.t_matrix, dtype=np.float64)
        grp["J"] = np.asarray(self.J_matrix, dtype=np.float64)
        grp["@T"] = float(self.T)
        grp["@nb_comp_states"] = int(getattr(self, "nb_comp_states_", 1))
        grp["@excited_state"] = int(self.excited_state) + 1   # 0: Boltzmann average (core_solver.py:75)
        grp["lanczos"] = {"@max_lcz": int(getattr(self, "max_lcz", 600)),
                          "@acc_lcz": float(getattr(self, "acc_lcz", 1.e-8)), "@renorm": False}
        return grp

    def _solve_group(self):
        """The solve group (solve.f90:26-120, lanczos.f90:37-126).  A dense solve keeps
        eigenvectors[b] = state b; a Lanczos solve keeps its Ritz states as psi_<b>
        (reference basis order) in place of the Krylov vectors it does not store."""
        s = self._sol
        grp = {"@nstates": int(s["nstates"]), "eigenvalues": np.asarray(s["eigenvalues"], dtype=np.float64),
               "boltzmann": np.asarray(s["boltzmann"], dtype=np.float64), "@nw": len(s["boltzmann"]),
               "@deg": int(s["deg"]), "@is_lanczos": int(bool(s["is_lanczos"]))}
        if s.get("H") is not None:
            grp["H"] = np.asarray(s["H"]).T   # read back transposed, as core_solver.py:185 does
        if not s["is_lanczos"]:
            grp["eigenvectors"] = np.asarray(s["eigenvectors_ref"]).T
            return grp
        sec = self.sector(self.nup[0], self.ndown[0])
        for b, v in enumerate(s["psis"]):
            if v is not None:
                grp[f"psi_{b}"] = sec.to_ref(v).cpu().numpy()
        grp["lanczos"] = {"alpha": np.asarray(s["alpha"], dtype=np.float64),
                          "beta": np.asarray(s["beta"], dtype=np.float64),
                          "@lcz_conv": float(s["conv"]), "@nb_lcz": int(s["nb_lcz"]),
                          "@max_lcz": int(getattr(self, "max_lcz", 600)), "@converged": bool(s["converged"]),
                          "@precision": str(s.get("precision", "f64")), "@reorth": str(s.get("reorth", "full"))}
        return grp

    def _rq_group(self):
        """reduced_quantities (static_rq.f90:16-45) in the layout the reference reads
        (reduced_quantities.py:14-48): the state index last, dbl_occ as [i,j,k,l,b]."""
        rq = self._rq
        grp = {"density_matrix_up": np.transpose(rq["density_matrix_up"], (1, 2, 0)),
               "density_matrix_down": np.transpose(rq["density_matrix_down"], (1, 2, 0)),
               "ni": np.transpose(rq["ni"]), "sisj": np.transpose(rq["sisj"], (1, 2, 0))}
        if rq.get("dbl_occ") is not None:
            grp["dbl_occ"] = np.transpose(rq["dbl_occ"], (4, 3, 2, 1, 0))
        return grp

    def _spgf_group(self):
        """Pole blocks of every state: continued-fraction poles of each start vector
        c_i|psi_b> (diag_<i>) and (c_i + c_j)|psi_b> (pair_<i>_<j>) as [2, m] arrays
        (eigenvalues, weights), with the start-vector norms."""
        grp = {"@nstates": len(self._spgf), "@nb_sites_comp": int(self.nb_sites_comp)}
        for b, st in enumerate(self._spgf):
            if st is None:
                continue
            sg = {"@down_is_up": bool(st["down"] is st["up"])}
            for spin in (("up",) if st["down"] is st["up"] else ("up", "down")):
                for part, blk in st[spin].items():
                    g = {"@n": blk.n, "@sign": blk.sign, "@e0": blk.e0,
                         "norm2": np.array([blk.norm2.get(i, np.nan) for i in range(blk.n)])}
                    for i, (e, w) in blk.diag.items():
                        g[f"diag_{i}"] = np.stack([np.asarray(e, dtype=np.float64), np.asarray(w, dtype=np.float64)])
                    for (i, j), (e, w) in blk.pair.items():
                        g[f"pair_{i}_{j}"] = np.stack([np.asarray(e, dtype=np.float64), np.asarray(w, dtype=np.float64)])
                        g[f"norm2_pair_{i}_{j}"] = np.float64(blk.norm2_pair[(i, j)])
                    sg[f"{spin}_{part}"] = g
            grp[f"state_{b}"] = sg
        return grp

    def save(self, path: str = None) -> str:
        """Write the solve's inputs and results (the solver.h5 tree: input, solve,
        reduced_quantities, spgf) to one archive; returns its path."""
        if self._sol is None:
            raise RuntimeError("nothing to save: call kernel() first")
        tree = {"input": self.write_in(), "solve": self._solve_group()}
        if self._rq is not None:
            tree["reduced_quantities"] = self._rq_group()
        if self._spgf is not None:
            tree["spgf"] = self._spgf_group()
        return store.save(path or self.archive, tree)

    def restore(self, path: str = None):
        """Load an archive written by save() for the same Hamiltonian, so that the
        properties (e, e0, psi0, rq, gf ...) answer without a new solve.  Raises
        ValueError when the archive holds another model, sector or parameter set."""
        from .greens import PoleBlock
        tree = store.load(path or self.archive)
        inp, mine = tree["input"], self.write_in()
        for key in ("@nb_sites", "@n_up", "@n_down", "@exec_name", "@is_Uloc", "@T"):
            if (key in inp) != (key in mine) or (key in inp and inp[key] != mine[key]):
                raise ValueError(f"the archive holds another solve: input {key[1:]} differs")
        for key in ("t_matrix", "J", "U"):
            if (key in inp) != (key in mine) or (key in inp and not np.array_equal(inp[key], mine[key])):
                raise ValueError(f"the archive holds another solve: input {key} differs")
        lz = inp.get("lanczos", {})
        self.max_lcz, self.acc_lcz = int(lz.get("@max_lcz", 600)), float(lz.get("@acc_lcz", 1.e-8))
        self.nb_comp_states_ = int(inp["@nb_comp_states"])
        self.store_H = bool(inp["@store_H"])
        self.nb_sites_comp = int(inp["@nb_sites_comp"])
        sg = tree["solve"]
        sol = {"eigenvalues": np.asarray(sg["eigenvalues"]), "is_lanczos": bool(sg["@is_lanczos"]),
               "deg": int(sg["@deg"]), "nstates": int(sg["@nstates"]),
               "H": None if "H" not in sg else np.ascontiguousarray(np.asarray(sg["H"]).T),
               "boltzmann": np.asarray(sg["boltzmann"])}
        if sol["is_lanczos"]:
            torch = _torch()
            sec = self.sector(self.nup[0], self.ndown[0])
            nps = 1 + max([int(k[4:]) for k in sg if k.startswith("psi_")], default=-1)
            sol["psis"] = [None] * nps
            for b in range(nps):
                if f"psi_{b}" in sg:
                    sol["psis"][b] = sec.from_ref(torch.from_numpy(np.ascontiguousarray(sg[f"psi_{b}"])).cuda())
            g = sg["lanczos"]
            sol.update({"alpha": np.asarray(g["alpha"]), "beta": np.asarray(g["beta"]),
                        "conv": float(g["@lcz_conv"]), "nb_lcz": int(g["@nb_lcz"]),
                        "converged": bool(g["@converged"]), "precision": str(g["@precision"]),
                        "reorth": str(g["@reorth"])})
        else:
            sol["eigenvectors_ref"] = np.ascontiguousarray(np.asarray(sg["eigenvectors"]).T)
        self._sol = sol
        self.is_solve = True
        self.set_state(int(inp["@excited_state"]) - 1)
        self._rq, self._spgf = None, None
        self.is_reduced_quantities = self.is_spgf = False
        if "reduced_quantities" in tree:
            r = tree["reduced_quantities"]
            back = lambda a, ax: np.ascontiguousarray(np.transpose(a, ax))   # noqa: E731
            self._rq = {"density_matrix_up": back(r["density_matrix_up"], (2, 0, 1)),
                        "density_matrix_down": back(r["density_matrix_down"], (2, 0, 1)),
                        "ni": back(r["ni"], (1, 0)), "sisj": back(r["sisj"], (2, 0, 1)),
                        "dbl_occ": back(r["dbl_occ"], (4, 3, 2, 1, 0)) if "dbl_occ" in r else None}
            self.is_reduced_quantities = True
        if "spgf" in tree:
            sp = tree["spgf"]
            out = []
            for b in range(int(sp["@nstates"])):
                st = sp.get(f"state_{b}")
                if st is None:
                    out.append(None)
                    continue
                blocks = {}
                for spin in (("up",) if st["@down_is_up"] else ("up", "down")):
                    blocks[spin] = {}
                    for part in ("greater", "lesser"):
                        g = st[f"{spin}_{part}"]
                        blk = PoleBlock(int(g["@n"]), float(g["@sign"]), float(g["@e0"]))
                        for i, v in enumerate(np.asarray(g["norm2"])):
                            if not np.isnan(v):
                                blk.norm2[i] = float(v)
                        for k, v in g.items():
                            if k.startswith("diag_"):
                                blk.diag[int(k[5:])] = (v[0], v[1])
                            elif k.startswith("pair_"):
                                i, j = (int(x) for x in k[5:].split("_"))
                                blk.pair[(i, j)] = (v[0], v[1])
                                blk.norm2_pair[(i, j)] = float(g[f"norm2_pair_{i}_{j}"])
                        blocks[spin][part] = blk
                if st["@down_is_up"]:
                    blocks["down"] = blocks["up"]
                out.append(blocks)
            self._spgf = out
            self.is_spgf = True
            self.gf = self.compute_gf()
        return self

    # ----------------------------------------------------------- properties
    @property
    def filename(self):
        return 'solver.h5'

    @property
    def boltzmann(self):
        return np.array(self._sol["boltzmann"], dtype=float)

    @property
    def Z(self):
        return np.sum(self.wgt)

    @property
    def nb_deg(self):
        return self._sol["deg"]

    @property
    def H(self):
        if self._sol.get("H") is None:
            raise KeyError("H was not stored: call kernel(store_H=True) on a sector smaller than max_lcz")
        return self._sol["H"]

    @property
    def e(self):
        return np.array(self._sol["eigenvalues"])

    @property
    def etot(self):
        return self.e0

    @property
    def e0(self):
        return self.e[:self.nb_comp_states] @ self.wgt / self.Z

    @property
    def lcz_results(self):
        if not self._sol["is_lanczos"]:
            raise KeyError("the sector was diagonalised densely (no Lanczos run)")
        lcz = {'alpha': np.array(self._sol["alpha"]), 'beta': np.array(self._sol["beta"]),
               'conv': self._sol["conv"], 'step': self._sol["nb_lcz"]}
        if lcz['step'] > self.max_lcz:
            raise StopIteration('Lanczos not converged, step,', lcz['step'],
                                f' greater than the maximum wanted {self.max_lcz}')
        return lcz

    @property
    def lcz_vectors(self):
        """The normalised Lanczos vectors [D, nb_lcz] in reference order
        (core_solver.py:211-213).  They are kept only on request:
        kernel(..., dtype='f64', store_lanczos_vectors=True) on a sector that
        is solved by Lanczos (the full-reorthogonalisation run keeps them on
        the device anyway; a mixed run's are FP32 vectors of another stage)."""
        if not self._sol["is_lanczos"]:
            raise KeyError("the sector was diagonalised densely (no Lanczos vectors)")
        if "lcz_vectors" not in self._sol:
            raise KeyError("the Lanczos vectors are kept only by kernel(..., dtype='f64', "
                           "store_lanczos_vectors=True)")
        return self._sol["lcz_vectors"]

    def _exec(self):
        """The reference writes the particle numbers to basis.h5 and runs the
        Fortran solver as a process (core_solver.py:106-110); here kernel()
        solves in process, so there is nothing to launch."""
        return None

    @property
    def nb_lcz(self):
        if not self._sol["is_lanczos"]:
            raise KeyError("the sector was diagonalised densely (no Lanczos run)")
        return self._sol["nb_lcz"]

    @property
    def nb_comp_states(self):
        return len(self.boltzmann)

    @property
    def psi0(self):
        w = self.boltzmann / self.Z
        sec = self.sector(self.nup[0], self.ndown[0])
        acc = None
        # the Boltzmann-weighted sum is formed on the device; one copy to the host
        for b, wb in enumerate(w):
            if wb == 0.0:
                continue
            v = sec.to_ref(self._state_device(b)).double()
            if acc is None:
                acc = v if wb == 1.0 else v * wb
            else:
                acc = acc + wb * v
        return None if acc is None else acc.cpu().numpy()

    def psi(self, vector: int):
        sec = self.sector(self.nup[0], self.ndown[0])
        return sec.to_ref(self._state_device(vector)).double().cpu().numpy()

    def psi_as_dict(self, vector: int):
        psi = self.psi(vector)
        index = np.where(abs(psi) > 1.e-12)[0]
        return {'basis': self.basis[index], 'coeff': psi[index]}

    @property
    def is_lanczos(self):
        return bool(self._sol and self._sol["is_lanczos"])

    @property
    def U_matrix(self):
        if isinstance(self.U, np.ndarray):
            if len(self.U.shape) == 4 or len(self.U.shape) == 1:
                return self.U
            raise ValueError
        if isinstance(self.U, (float, int)):
            return np.full(self.nb_sites, self.U, dtype=float)
