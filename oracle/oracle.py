"""CPU oracle for the exact-diagonalisation hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker (or as the timed
CPU baseline).  The pyhub_gb300 package never imports it: the product path
runs on the CUDA extension alone and fails loudly without it.

What it holds:
  * ctypes bindings of ``ed_oracle.c`` -- a C restatement of PyHub's Fortran
    kernels (basis enumeration, KINOP/ANTICOM, HPROD for Hubbard and
    Heisenberg, ONE_RDM/TWO_RDM/J_SPIN, the GF start vectors);
  * numpy restatements of the loops built on them: LANCZOS
    (lanczos.f90:1-133), EXACT_DIAG (exact_diag.f90:2-33), BOLTZMANN
    (boltzmann.f90:1-29), the Lehmann Green's function of SPGF_ED
    (spgf_ed.f90:1-429) and the pole bookkeeping of
    GreenFunction.compute_gf (pyhub/core/reduced_quantities.py:84-92);
  * an independent Jordan-Wigner construction of the same Hamiltonians in
    the full Fock space (kron products of 2x2 matrices, no bit tricks), used
    to pin the sign conventions of the restatement.

Parity status: "parity unpinned" by reference execution -- the reference is
Fortran + HDF5 and cannot be built or run here (no Fortran compiler), and it
ships no tests or golden vectors for this path.  The restatement is pinned to
the Jordan-Wigner construction and to physics identities instead; the pole
evaluation semantics are pinned to golden vectors produced by the reference's
own Python (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading
from itertools import combinations

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

F32_TOL14 = float(np.float32(1e-14))   # the reference's REAL*4 literal 1.E-14
F32_TOL8 = float(np.float32(1e-8))     # 1.E-8 (boltzmann.f90:9)
F32_TOL5 = float(np.float32(1e-5))     # 1.E-5 (lanczos.f90:74)


def build() -> str:
    """Compile the C oracle with its Makefile (idempotent)."""
    src = os.path.join(_HERE, "ed_oracle.c")
    if (not os.path.exists(_LIBPATH)) or os.path.getmtime(_LIBPATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIBPATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIBPATH)
            P = ctypes.c_void_p
            i32, i64 = ctypes.c_int, ctypes.c_int64
            L.orc_binom.restype = i64
            L.orc_binom.argtypes = [i32, i32]
            L.orc_hilbert.argtypes = [i32, i32, P]
            L.orc_rank.restype = i64
            L.orc_rank.argtypes = [i32, i32, ctypes.c_uint32]
            L.orc_kinop.restype = ctypes.c_uint32
            L.orc_kinop.argtypes = [i32, ctypes.c_uint32, i32, i32]
            L.orc_anticom.restype = ctypes.c_double
            L.orc_anticom.argtypes = [i32, i32, ctypes.c_uint32]
            L.orc_hprod_hubbard_ref.argtypes = [i32, i32, i32, P, i64, P, i64, P, P, P, P]
            L.orc_hprod_hubbard_ref_pairs.argtypes = [i32, i32, i32, P, i64, P, i64, P, P, i32, P, P]
            L.orc_hprod_hubbard_ref_udiag.argtypes = [i32, P, i64, P, i64, i32, ctypes.c_double, P, P]
            L.orc_hprod_hubbard_ref_pairs_mt.argtypes = [i32, i32, i32, P, i64, P, i64, P, P, i32, P, P, i32]
            L.orc_hprod_hubbard_ref_udiag_mt.argtypes = [i32, P, i64, P, i64, i32, ctypes.c_double, P, P, i32]
            L.orc_hprod_hubbard_fast.argtypes = [i32, i32, i32, P, i64, P, i64, P, P, P, P, i32]
            L.orc_hprod_heis_ref.argtypes = [i32, P, i64, P, P, P]
            L.orc_hprod_heis_fast.argtypes = [i32, P, i64, P, P, P, i32]
            L.orc_one_rdm.argtypes = [i32, i32, i32, P, i64, P, i64, P, P, P]
            L.orc_two_rdm_ni.argtypes = [i32, P, i64, P, i64, P, P, P]
            L.orc_j_spin.argtypes = [i32, P, i64, P, i64, P, P, P]
            L.orc_j_spin_heis.argtypes = [i32, P, i64, P, P, P]
            L.orc_gf_start.argtypes = [i32, i32, i32, i32, P, i64, P, i64, P, i64, P, i64, P, P]
            L.orc_hprod_hubbard_uijkl_ref.argtypes = [i32, i32, i32, P, i64, P, i64, P, P, P, P]
            L.orc_two_rdm_dbl_occ.argtypes = [i32, P, i64, P, i64, P, P, P, P]
            L.orc_unrank.restype = ctypes.c_uint32
            L.orc_unrank.argtypes = [i32, i32, i64]
            L.orc_hashval.restype = ctypes.c_double
            L.orc_hashval.argtypes = [i64, i64, i32]
            L.orc_hprod_heis_rows.argtypes = [i32, P, i64, P, i64, i32, P, P, i32]
            L.orc_j_spin_heis_rows.argtypes = [i32, i64, P, i64, i64, i32, i32, P, P, P, i32]
            _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------- basis ---

def binom(n: int, k: int) -> int:
    return int(lib().orc_binom(n, k))


def hilbert(norb: int, ne: int) -> np.ndarray:
    """Spin strings of ne particles on norb sites in the reference's order
    (compute_basis.f90:67-96)."""
    n = binom(norb, ne)
    out = np.zeros(max(n, 0), dtype=np.uint32)
    if n > 0:
        lib().orc_hilbert(norb, ne, _p(out))
    return out


def hilbert_py(norb: int, ne: int) -> np.ndarray:
    """Same order written as subsets in lexicographic order (bit i <-> element i)."""
    return np.array([sum(1 << p for p in c) for c in combinations(range(norb), ne)], dtype=np.uint32)


def rank(norb: int, ne: int, s: int) -> int:
    return int(lib().orc_rank(norb, ne, int(s)))


class Sector:
    """(norb, nup, ndn) with its two string tables, reference layout d*nsup+u."""

    def __init__(self, norb: int, nup: int, ndn: int):
        self.norb, self.nup, self.ndn = norb, nup, ndn
        self.bup = hilbert(norb, nup)
        self.bdn = hilbert(norb, ndn)
        self.nsup, self.nsdn = len(self.bup), len(self.bdn)
        self.dim = self.nsup * self.nsdn


# ------------------------------------------------------------- H*v --------

def hprod_hubbard(sec: Sector, t, U, x, fast: bool = False, nthreads: int = 0) -> np.ndarray:
    """y = H x for the Hubbard sector (hprod_hubbard.f90:17-118).

    t: (norb, norb) hopping matrix exactly as handed to FermiHubbard;
    U: float or per-site vector (the reference's is_Uloc=2 path)."""
    t = _f64(t)
    U = _f64(np.broadcast_to(np.asarray(U, dtype=np.float64), (sec.norb,)))
    x = _f64(x)
    y = np.empty_like(x)
    if fast:
        lib().orc_hprod_hubbard_fast(sec.norb, sec.nup, sec.ndn, _p(sec.bup), sec.nsup, _p(sec.bdn),
                                     sec.nsdn, _p(t), _p(U), _p(x), _p(y), int(nthreads))
    else:
        lib().orc_hprod_hubbard_ref(sec.norb, sec.nup, sec.ndn, _p(sec.bup), sec.nsup, _p(sec.bdn),
                                    sec.nsdn, _p(t), _p(U), _p(x), _p(y))
    return y


def hprod_hubbard_uijkl(sec: Sector, t, Ul, x) -> np.ndarray:
    """y = H x with the U_ijkl interaction (IS_ULOC=3, hprod_hubbard.f90:17-118):
    Ul is the (norb,)*4 tensor as handed to FermiHubbard (C order), read by the
    reference as UL(J,K,M,N) = Ul[N-1,M-1,K-1,J-1] and gated per (J,K) by
    UPARTIAL(J,K) = sum_cd Ul[K-1,J-1,c,d]^2."""
    t = _f64(t)
    Ul = _f64(Ul)
    x = _f64(x)
    y = np.empty_like(x)
    lib().orc_hprod_hubbard_uijkl_ref(sec.norb, sec.nup, sec.ndn, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn,
                                      _p(t), _p(Ul), _p(x), _p(y))
    return y


def two_rdm_dbl_occ(sec: Sector, bra, ket=None):
    """TWO_RDM with the two-body density (static_rq.f90:247-306): returns
    (dbl, ni) with dbl[J-1,K-1,M-1,N-1] = DBL_OCC(J,K,M,N) (the array the
    reference's two_rdm property returns for one state) and NI(J) =
    DBL_OCC(J,J,J,J)."""
    ket = bra if ket is None else ket
    n = sec.norb
    dbl = np.zeros(n ** 4)
    ni = np.zeros(n)
    lib().orc_two_rdm_dbl_occ(n, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn, _p(_f64(bra)), _p(_f64(ket)),
                              _p(dbl), _p(ni))
    return dbl.reshape((n, n, n, n), order="F").copy(), ni


def hprod_hubbard_pairs(sec: Sector, t, pairs, x, y, nthreads: int = 1) -> None:
    """Reference loop restricted to the (J,K) pairs given (1-based), adds into y.
    nthreads > 1 (or 0: all cores) runs the same loop on host threads with the
    same result bit for bit."""
    t = _f64(t)
    pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    if nthreads == 1:
        lib().orc_hprod_hubbard_ref_pairs(sec.norb, sec.nup, sec.ndn, _p(sec.bup), sec.nsup, _p(sec.bdn),
                                          sec.nsdn, _p(t), _p(pr), len(pr), _p(x), _p(y))
    else:
        lib().orc_hprod_hubbard_ref_pairs_mt(sec.norb, sec.nup, sec.ndn, _p(sec.bup), sec.nsup, _p(sec.bdn),
                                             sec.nsdn, _p(t), _p(pr), len(pr), _p(x), _p(y), int(nthreads))


def hprod_hubbard_udiag(sec: Sector, J: int, uj: float, x, y, nthreads: int = 1) -> None:
    """U term of the reference loop for site J (1-based) only, adds into y."""
    if nthreads == 1:
        lib().orc_hprod_hubbard_ref_udiag(sec.norb, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn, int(J),
                                          float(uj), _p(x), _p(y))
    else:
        lib().orc_hprod_hubbard_ref_udiag_mt(sec.norb, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn, int(J),
                                             float(uj), _p(x), _p(y), int(nthreads))


def hprod_hubbard_mt(sec: Sector, t, U, x, nthreads: int = 0) -> np.ndarray:
    """The reference loop of hprod_hubbard_ref (hprod_hubbard.f90:17-118) on
    host threads: for J = 1..norb its U term, then each (J, K) pair, in the
    serial order; each piece is the threaded loop that equals the one-thread
    loop bit for bit, so y equals hprod_hubbard(fast=False) bit for bit.
    nthreads = 0: all the cores the process may use."""
    t = _f64(t)
    U = _f64(np.broadcast_to(np.asarray(U, dtype=np.float64), (sec.norb,)))
    x = _f64(x)
    y = np.zeros_like(x)
    nt = int(nthreads) if nthreads else len(os.sched_getaffinity(0))
    for J in range(1, sec.norb + 1):
        hprod_hubbard_udiag(sec, J, float(U[J - 1]), x, y, nthreads=nt)
        for K in range(1, sec.norb + 1):
            hprod_hubbard_pairs(sec, t, [(J, K)], x, y, nthreads=nt)
    return y


# ------------------------------------------- sampled rows of large sectors ---

def unrank(norb: int, ne: int, r: int) -> int:
    """String at position r of hilbert(norb, ne) (inverse of rank)."""
    return int(lib().orc_unrank(norb, ne, int(r)))


def hashvec(idx, seed: int, kind: int) -> np.ndarray:
    """orc_hashval for an array of element indices: the inputs of the
    sampled-row checks as a function of the index alone (kind 0: exact doubles
    in [-0.5, 0.5); kind 1: integers in [-3, 3])."""
    i = np.asarray(idx, dtype=np.uint64)
    h = (i * np.uint64(2654435761) + np.uint64(seed) * np.uint64(40503)) & np.uint64(0xFFFFFFFF)
    if kind == 0:
        return h.astype(np.float64) / 4294967296.0 - 0.5
    return (h % np.uint64(7)).astype(np.float64) - 3.0


def hprod_heis_rows(norb: int, J, rows, xseed: int, xkind: int, nthreads: int = 0):
    """Rows of y = H x (hprod_heis.f90:1-61) for x = hashvec(., xseed, xkind),
    summed in the reference's order (equal to hprod_heis(fast=False) at those
    rows, bit for bit).  Returns (y[rows], sum of |terms| per row)."""
    J = _f64(J)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    out = np.empty(len(rows))
    ab = np.empty(len(rows))
    lib().orc_hprod_heis_rows(norb, _p(J), len(rows), _p(rows), int(xseed), int(xkind), _p(out), _p(ab),
                              int(nthreads))
    return out, ab


def j_spin_heis_rows(norb: int, rows, bseed: int, kseed: int, kind: int, pairs, nthreads: int = 0):
    """SMATRIX(J,K) of J_SPIN (static_rq_heis.f90:58-116) for bra = hashvec(.,
    bseed, kind) restricted to rows and ket = hashvec(., kseed, kind).
    Returns (SMATRIX per pair, sum of |terms| per pair)."""
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    out = np.empty(len(pr))
    ab = np.empty(len(pr))
    lib().orc_j_spin_heis_rows(norb, len(rows), _p(rows), int(bseed), int(kseed), int(kind), len(pr), _p(pr),
                               _p(out), _p(ab), int(nthreads))
    return out, ab


def heis_sector(norb: int) -> Sector:
    """The reference's Heisenberg sector (n_up=norb//2, n_down=0), heisenberg.py:24."""
    return Sector(norb, norb // 2, 0)


def hprod_heis(norb: int, J, x, fast: bool = False, nthreads: int = 0, bup=None) -> np.ndarray:
    """y = H x for the Sz=0 Heisenberg sector (hprod_heis.f90:1-61)."""
    J = _f64(J)
    bup = hilbert(norb, norb // 2) if bup is None else bup
    x = _f64(x)
    y = np.empty_like(x)
    if fast:
        lib().orc_hprod_heis_fast(norb, _p(bup), len(bup), _p(J), _p(x), _p(y), int(nthreads))
    else:
        lib().orc_hprod_heis_ref(norb, _p(bup), len(bup), _p(J), _p(x), _p(y))
    return y


# ------------------------------------------------------------------ RDMs ---

def one_rdm(sec: Sector, bra, ket=None) -> dict:
    """ONE_RDM (static_rq.f90:153-244), returned as the reference's Python
    property one_rdm reads it (reduced_quantities.py:12-16)."""
    ket = bra if ket is None else ket
    dm = np.zeros(2 * sec.norb * sec.norb)
    lib().orc_one_rdm(sec.norb, sec.nup, sec.ndn, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn,
                      _p(_f64(bra)), _p(_f64(ket)), _p(dm))
    dm = dm.reshape(2, sec.norb, sec.norb)  # [S][K][J] in C order == Fortran (J,K,S)
    # h5py reads the Fortran dataset (NW,NORB,NORB) as [K][J][w]: element [a][b] = DENS_MAT(b,a)
    return {"up": dm[0].copy(), "down": dm[1].copy()}


def two_rdm_ni(sec: Sector, bra, ket=None) -> np.ndarray:
    ket = bra if ket is None else ket
    ni = np.zeros(sec.norb)
    lib().orc_two_rdm_ni(sec.norb, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn,
                         _p(_f64(bra)), _p(_f64(ket)), _p(ni))
    return ni


def j_spin(sec: Sector, bra, ket=None) -> np.ndarray:
    ket = bra if ket is None else ket
    sm = np.zeros(sec.norb * sec.norb)
    lib().orc_j_spin(sec.norb, _p(sec.bup), sec.nsup, _p(sec.bdn), sec.nsdn,
                     _p(_f64(bra)), _p(_f64(ket)), _p(sm))
    return sm.reshape(sec.norb, sec.norb).copy()  # symmetric


def j_spin_heis(norb: int, bra, ket=None) -> np.ndarray:
    ket = bra if ket is None else ket
    bup = hilbert(norb, norb // 2)
    sm = np.zeros(norb * norb)
    lib().orc_j_spin_heis(norb, _p(bup), len(bup), _p(_f64(bra)), _p(_f64(ket)), _p(sm))
    # Fortran SMATRIX(J,K) -> h5py [K][J]
    return sm.reshape(norb, norb).copy()


GF_KINDS = {"h_up": 0, "h_down": 1, "e_up": 2, "e_down": 3}


def gf_start(kind: str, sec0: Sector, ncomp: int, psi) -> tuple:
    """Start vectors c|psi> / c^+|psi> of the reference's band-Lanczos GF
    (spgf_bandlanczos.f90:453-560).  Returns (target sector, array [ncomp, dim])."""
    k = GF_KINDS[kind]
    dup = {0: -1, 1: 0, 2: 1, 3: 0}[k]
    ddn = {0: 0, 1: -1, 2: 0, 3: 1}[k]
    sec1 = Sector(sec0.norb, sec0.nup + dup, sec0.ndn + ddn)
    out = np.zeros(ncomp * sec1.dim)
    lib().orc_gf_start(k, sec0.norb, ncomp, sec0.ndn, _p(sec0.bup), sec0.nsup, _p(sec0.bdn), sec0.nsdn,
                       _p(sec1.bup), sec1.nsup, _p(sec1.bdn), sec1.nsdn, _p(_f64(psi)), _p(out))
    return sec1, out.reshape(ncomp, sec1.dim)


# --------------------------------------------------- dense / Lanczos loops ---

def dense_h(hv, dim: int) -> np.ndarray:
    """EXACT_DIAG's dense build, one column H e_i per call (exact_diag.f90:14-19)."""
    H = np.zeros((dim, dim))
    e = np.zeros(dim)
    for i in range(dim):
        e[i] = 1.0
        H[:, i] = hv(e)
        e[i] = 0.0
    return H


def exact_diag(H: np.ndarray):
    """DIAGMAT + degeneracy count (exact_diag.f90:20-31, diagmat.f90:34)."""
    val, vec = np.linalg.eigh(H)
    ndeg = 1
    for i in range(1, len(val)):
        if abs(val[i] - val[0]) < F32_TOL14:
            ndeg += 1
        else:
            break
    return val, vec, ndeg


def lanczos_ref(hv, v0: np.ndarray, max_lcz: int = 600, acc_lcz: float = 1e-8) -> dict:
    """Plain three-term Lanczos with the reference's convergence rule
    (lanczos.f90:1-133): blocks of NADD=5 steps, a dense eigensolve of the
    tridiagonal after each block, the norm-loss check and the
    degeneracy-aware test on Ritz value NDEG+1."""
    nadd = 5
    alpha = np.zeros(max_lcz + 2)
    beta = np.zeros(max_lcz + 2)
    nr = np.linalg.norm(v0)
    v = v0 / nr
    beta[1] = nr
    v_prev = np.zeros_like(v)
    vecs = []
    cv = False
    nb = 0
    ev = 0.0
    ndeg = 0
    val = vec = None
    norm_lost = False
    while (not cv) and nb <= max_lcz - 10:
        for _ in range(nadd):
            vecs.append(v)
            nb += 1
            w = hv(v)
            alpha[nb] = float(np.dot(v, w))
            w = w - alpha[nb] * v - beta[nb] * v_prev
            nr = float(np.linalg.norm(w))
            beta[nb + 1] = nr
            v_prev = v
            v = (1.0 / nr) * w
        T = np.diag(alpha[1:nb + 1]) + np.diag(beta[2:nb + 1], 1) + np.diag(beta[2:nb + 1], -1)
        val, vec = np.linalg.eigh(T)
        V = np.array(vecs).T
        nrm = float(np.linalg.norm(V @ vec[:, 0]))
        if abs(1 - nrm) > F32_TOL5:
            cv = True
            norm_lost = True
        elif abs(val[ndeg] - ev) < acc_lcz:
            if abs(val[ndeg] - val[0]) > acc_lcz and (ndeg + 1) > 1:
                cv = True
            else:
                ndeg += 1
        else:
            if nb <= max_lcz - 10:
                ev = val[ndeg]
    V = np.array(vecs).T
    return dict(alpha=alpha[1:nb + 1].copy(), beta=beta[1:nb + 1].copy(), nb_lcz=nb,
                eigenvalues=val, eigenvectors=vec, conv=float(val[ndeg] - ev), deg=ndeg,
                vectors=V, psi0=V @ vec[:, 0], norm_lost=norm_lost, converged=cv)


def boltzmann(val: np.ndarray, T: float, nb_comp_states: int = 1) -> np.ndarray:
    """BOLTZMANN (boltzmann.f90:1-29): number of weighted states and weights."""
    nval = len(val)
    nw = nval + 1
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for k in range(2, nval + 1):
            if np.exp((val[0] - val[k - 1]) / T) <= F32_TOL8:
                nw = k
                break
    nw = nw - 1
    nw = max(nw, nb_comp_states)
    w = np.zeros(nw)
    if T >= F32_TOL8:
        for i in range(nw):
            w[i] = np.exp((val[0] - val[i]) / T)
    else:
        w[0] = 1.0
    return w


def ground_state_dense(sec: Sector, t, U):
    H = dense_h(lambda v: hprod_hubbard(sec, t, U, v), sec.dim)
    return exact_diag(H)


# ----------------------------------------------------- Green's functions ---

def lehmann_gf_diag(sec: Sector, t, U, psi0: np.ndarray, e0: float, ncomp: int):
    """Exact G_ii poles from full ED of the N-1 / N+1 sectors, as SPGF_ED
    (spgf_ed.f90:66-290) and compute_gf (reduced_quantities.py:84-92) build them:
    greater poles at E_n - E0 with weights <n|c^+_i|psi0>^2, lesser poles at
    E0 - E_n with weights <n|c_i|psi0>^2, for spin up and down."""
    out = {}
    for spin in ("up", "down"):
        res = {}
        for part, kind in (("greater", "e_" + spin), ("lesser", "h_" + spin)):
            sec1, start = gf_start(kind, sec, ncomp, psi0)
            if sec1.dim == 0:
                res[part] = (np.zeros(0), np.zeros((ncomp, 0)))
                continue
            H1 = dense_h(lambda v: hprod_hubbard(sec1, t, U, v), sec1.dim)
            val, vec = np.linalg.eigh(H1)
            Q = start @ vec            # [ncomp, n]
            pos = (val - e0) if part == "greater" else (e0 - val)
            res[part] = (pos, Q)
        out[spin] = res
    return out


def spgf_ed(sec: Sector, t, U, psis, ncomp: int) -> dict:
    """What SPGF_ED stores (spgf_ed.f90:66-290), for the states psis (each a
    reference-layout vector of the (nup, ndn) sector): per spin and part the
    eigenvalues of the N+1 (greater) / N-1 (lesser) sector as
    'positions_{part}_{spin}' and the overlaps 'Q_{part}_{spin}'[i, n, b] =
    <n|c^+_i|psi_b> (greater) or <n|c_i|psi_b> (lesser), sites i < ncomp."""
    out = {}
    for spin in ("up", "down"):
        for part, kind in (("greater", "e_" + spin), ("lesser", "h_" + spin)):
            starts = []
            sec1 = None
            for psi in psis:
                sec1, st = gf_start(kind, sec, ncomp, psi)
                starts.append(st)
            if sec1 is None or sec1.dim == 0:
                out[f"positions_{part}_{spin}"] = np.zeros(0)
                out[f"Q_{part}_{spin}"] = np.zeros((ncomp, 0, len(psis)))
                continue
            H1 = dense_h(lambda v: hprod_hubbard(sec1, t, U, v), sec1.dim)
            val, vec = np.linalg.eigh(H1)
            out[f"positions_{part}_{spin}"] = val
            out[f"Q_{part}_{spin}"] = np.stack([st @ vec for st in starts], axis=2)
    return out


def self_energy_ref(Vk, ek, e, wgt, spgf: dict, w: float, eta: float, same_spin: bool) -> dict:
    """GreenFunction.self_energy at one frequency (reduced_quantities.py:
    139-161): pinv(sum_k Vk_ik Vk_jk / (w - ek + i eta)) minus pinv(G), with G
    summed over the states b from the stored Q and positions, greater poles at
    -e_b + position, lesser at e_b - position; weighted by wgt_b/sum(wgt) when
    N_up == N_down, unweighted (the reference's other branch) otherwise."""
    g0i = np.linalg.pinv(np.einsum("ik,jk,k->ij", Vk, Vk, 1. / (w - ek + 1j * eta)))
    out = {}
    for spin in ("up", "down"):
        src = "up" if same_spin else spin
        G = 0
        for b, bltz in enumerate(wgt):
            f = bltz / np.sum(wgt) if same_spin else 1.0
            Qg, pg = spgf[f"Q_greater_{src}"][:, :, b], spgf[f"positions_greater_{src}"]
            Ql, pl = spgf[f"Q_lesser_{src}"][:, :, b], spgf[f"positions_lesser_{src}"]
            G = G + np.einsum("ik,jk,k->ij", Qg, Qg, 1. / (w - (-e[b] + pg) + 1j * eta)) * f \
                + np.einsum("ik,jk,k->ij", Ql, Ql, 1. / (w - (e[b] - pl) + 1j * eta)) * f
        out[spin] = g0i - np.linalg.pinv(G)
    return out


def qpw_ref(Vk, ek, e, wgt, spgf: dict, mu: float, same_spin: bool, nb_sites: int) -> np.ndarray:
    """GreenFunction.qpw (reduced_quantities.py:168-169): pinv(1 - Re S'(mu))
    of the up self-energy at eta = 1e-4, S' by the published three-point
    central difference that scipy.misc.derivative(order=3) applies,
    (S(mu + dx) - S(mu - dx)) / (2 dx), dx = 1e-6."""
    dx = 1.e-6
    sp = self_energy_ref(Vk, ek, e, wgt, spgf, mu + dx, 1.e-4, same_spin)["up"]
    sm = self_energy_ref(Vk, ek, e, wgt, spgf, mu - dx, 1.e-4, same_spin)["up"]
    return np.linalg.pinv(np.identity(nb_sites) - np.real((sp - sm) / (2 * dx)))


# ---------------------------------------------------------------- operators.x
def _ops_site(norb: int, pos: int) -> int:
    return 1 << (norb - pos)                         # ISHFT(1,NORB+1-POS-1)


def _ops_anticom(norb: int, pos: int, state: int) -> float:
    """ANTICOM (funcmod.f90:29-41): -1 per occupied site among 1..POS-1."""
    a = 1.0
    for i2 in range(1, pos):
        if state & _ops_site(norb, i2):
            a = -a
    return a


def _ops_kinop(norb: int, state: int, posi: int, posf: int) -> int:
    """KINOP (funcmod.f90:18-27)."""
    A, B = _ops_site(norb, posi), _ops_site(norb, posf)
    new = 0
    if state & A and not state & B:
        new = state - A + B
    if state & A and posi == posf:
        new = state
    return new


def ops_space(norb: int, nups, ndns):
    """BUP / BDOWN of PROGRAM OPERATOR (compute_operators.f90:8-25): the
    strings of every listed particle number, concatenated in list order."""
    bup = [int(s) for n in nups for s in hilbert(norb, n)]
    bdn = [int(s) for n in ndns for s in hilbert(norb, n)]
    return bup, bdn


def ops_apply_ref(norb: int, nups, ndns, terms, psi: np.ndarray) -> np.ndarray:
    """PROGRAM OPERATOR (compute_operators.f90:28-66) with the elementary
    routines of operators.f90, loop for loop: terms = [(coeff, [(code, site1,
    spin1, site2, spin2), ...])] as _write_operator encodes them; each term
    restarts from psi, applies its factors in list order (the first one
    first) and adds COEFF * result.  The position searches are the Fortran's
    linear searches over BUP / BDOWN (a dict gives the same first match:
    the strings of a list are distinct)."""
    bup, bdn = ops_space(norb, nups, ndns)
    nsup, nsdn = len(bup), len(bdn)
    iu = {s: i for i, s in enumerate(bup)}
    idn = {s: i for i, s in enumerate(bdn)}
    out = np.zeros(nsup * nsdn)
    for coeff, ops in terms:
        if not abs(coeff) > F32_TOL14:                  # 1.E-14, a default-real literal
            continue
        v = np.array(psi, dtype=np.float64, copy=True)
        for code, si, spi, sj, spj in ops:
            if code in (0, 3):
                continue
            w = np.zeros_like(v)
            if code == 1:                       # C_DAGGER_C(J=si, K=sj, SPIN=spi)  operators.f90:1-59
                J, K = si, sj
                if spi == 1:
                    for i, b in enumerate(bup):
                        new = _ops_kinop(norb, b, K, J)
                        if new > 0 and new in iu:
                            pos = iu[new]
                            ac = _ops_anticom(norb, K, b) * _ops_anticom(norb, J, new)
                            for l1 in range(nsdn):
                                w[l1 * nsup + pos] += ac * v[l1 * nsup + i]
                else:
                    for l1, b in enumerate(bdn):
                        new = _ops_kinop(norb, b, K, J)
                        if new > 0 and new in idn:
                            pos = idn[new]
                            ac = _ops_anticom(norb, K, b) * _ops_anticom(norb, J, new)
                            for i in range(nsup):
                                w[pos * nsup + i] += ac * v[l1 * nsup + i]
            elif code in (2, 4):                # NI / NIM1  operators.f90:150-175, 194-219
                w = v.copy()
                keep_occ = code == 2
                if spi == 1:
                    for u, b in enumerate(bup):
                        if bool(b & _ops_site(norb, si)) != keep_occ:
                            w[u::nsup] = 0.0
                else:
                    for d, b in enumerate(bdn):
                        if bool(b & _ops_site(norb, si)) != keep_occ:
                            w[d * nsup:(d + 1) * nsup] = 0.0
            elif code == 5:                     # SZ_OPE  operators.f90:223-248
                for u, b in enumerate(bup):
                    if not b & _ops_site(norb, si):
                        for d in range(nsdn):
                            w[d * nsup + u] = w[d * nsup + u] + v[d * nsup + u] / 2.0
                for d, b in enumerate(bdn):
                    if not b & _ops_site(norb, si):
                        for u in range(nsup):
                            w[d * nsup + u] = w[d * nsup + u] - v[d * nsup + u] / 2.0
            elif code == 12:                    # SZ_BASIS  operators_basis.f90:134-145: VAL * SZ
                for d, bd in enumerate(bdn):
                    for u, b in enumerate(bup):
                        sz = 0.0
                        if b & _ops_site(norb, si):
                            sz = sz + 0.5
                        if bd & _ops_site(norb, si):
                            sz = sz - 0.5
                        w[d * nsup + u] = v[d * nsup + u] * sz
            elif code in (6, 7, 9):             # C_DAGGER_C_UNRES(J, K, SPINK)  operators.f90:62-144
                J = si
                K = sj if code == 9 else si
                spink = {6: 2, 7: 1}.get(code, spj)
                if spink == 1:
                    for i, b in enumerate(bup):
                        if b & _ops_site(norb, K):
                            new = b - _ops_site(norb, K)
                            if new in iu:
                                pos = iu[new]
                                ac = _ops_anticom(norb, K, new)
                                for l1, bd in enumerate(bdn):
                                    if not bd & _ops_site(norb, J):
                                        new2 = bd + _ops_site(norb, J)
                                        if new2 in idn:
                                            pos2 = idn[new2]
                                            ac2 = _ops_anticom(norb, J, new2) * _ops_anticom(norb, 0, bd)
                                            w[pos2 * nsup + pos] += ac * ac2 * v[l1 * nsup + i]
                else:
                    for i, bd in enumerate(bdn):
                        if bd & _ops_site(norb, K):
                            new = bd - _ops_site(norb, K)
                            if new in idn:
                                pos = idn[new]
                                ac = _ops_anticom(norb, K, new)
                                for l1, b in enumerate(bup):
                                    if not b & _ops_site(norb, J):
                                        new2 = b + _ops_site(norb, J)
                                        if new2 in iu:
                                            pos2 = iu[new2]
                                            ac2 = _ops_anticom(norb, 0, new) * _ops_anticom(norb, J, new2)
                                            w[pos * nsup + pos2] += ac * ac2 * v[i * nsup + l1]
            elif code in (10, 11):              # C_DAGGER / C_  operators.f90:410-523
                J = si
                create = code == 10
                if spi == 1:
                    for i, b in enumerate(bup):
                        if bool(b & _ops_site(norb, J)) != create:
                            new = b + _ops_site(norb, J) if create else b - _ops_site(norb, J)
                            if new in iu:
                                pos = iu[new]
                                ac = _ops_anticom(norb, J, b)
                                for l2, bd in enumerate(bdn):
                                    ac2 = _ops_anticom(norb, 0, bd)
                                    w[l2 * nsup + pos] += ac * ac2 * v[l2 * nsup + i]
                else:
                    for i, bd in enumerate(bdn):
                        if bool(bd & _ops_site(norb, J)) != create:
                            new = bd + _ops_site(norb, J) if create else bd - _ops_site(norb, J)
                            if new in idn:
                                pos = idn[new]
                                ac = _ops_anticom(norb, J, bd)
                                for l1 in range(nsup):
                                    w[pos * nsup + l1] += ac * v[i * nsup + l1]
            else:
                raise NotImplementedError(f"operator code {code}")
            v = w
        out = out + coeff * v
    return out


def lanczos_tridiag(hv, phi: np.ndarray, nsteps: int, reorth: bool = True):
    """Lanczos coefficients (a_n, b_n) from the normalised start phi, used for
    the continued fraction <phi|(z-H)^-1|phi>.  Full reorthogonalisation in
    FP64 (oracle quality)."""
    nrm = float(np.linalg.norm(phi))
    v = phi / nrm
    V = [v]
    a, b = [], []
    vprev = np.zeros_like(v)
    bprev = 0.0
    for k in range(nsteps):
        w = hv(v) - bprev * vprev
        ak = float(np.dot(v, w))
        w = w - ak * v
        if reorth:
            Vm = np.array(V)
            for _ in range(2):
                w = w - Vm.T @ (Vm @ w)
        bk = float(np.linalg.norm(w))
        a.append(ak)
        if bk < 1e-12 or k == nsteps - 1:
            break
        b.append(bk)
        vprev, v, bprev = v, w / bk, bk
        V.append(v)
    return np.array(a), np.array(b), nrm * nrm


def continued_fraction(a: np.ndarray, b: np.ndarray, norm2: float, z: np.ndarray, sign: float = 1.0):
    """norm2 / (z - s a0 - b1^2 / (z - s a1 - ...)) evaluated bottom-up;
    sign=-1 gives <phi|(z+H)^-1|phi>."""
    g = np.zeros_like(z, dtype=np.complex128)
    n = len(a)
    for k in range(n - 1, -1, -1):
        tail = (b[k] ** 2) * g if k < n - 1 else 0.0
        g = 1.0 / (z - sign * a[k] - tail)
    return norm2 * g


def poles_eval(positions, weights, w, eta):
    """Pole.retarded: sum_k weights_k / (w - positions_k + i eta) (pole.py:81-88)."""
    w = np.asarray(w, dtype=np.float64)
    return (np.asarray(weights)[None, :] / (w[:, None] - np.asarray(positions)[None, :] + 1j * eta)).sum(axis=1)


# ------------------------------------- independent Jordan-Wigner construction ---

def _jw_ops(nmodes: int):
    """Annihilators of nmodes fermionic modes as sparse matrices, mode 0 leftmost.
    Basis vector |n_0 ... n_{M-1}> == (c^+_0)^n_0 ... (c^+_{M-1})^n_{M-1} |vac>."""
    import scipy.sparse as sp
    I = sp.identity(2, format="csr")
    Z = sp.csr_matrix(np.diag([1.0, -1.0]))
    a = sp.csr_matrix(np.array([[0.0, 1.0], [0.0, 0.0]]))  # |1> -> |0>
    ops = []
    for m in range(nmodes):
        mats = [Z] * m + [a] + [I] * (nmodes - m - 1)
        op = mats[0]
        for q in mats[1:]:
            op = sp.kron(op, q, format="csr")
        ops.append(op)
    return ops


def _fock_index(norb: int, u: int, d: int) -> int:
    """Fock index of the sector state (u,d): modes ordered down sites 1..N then
    up sites 1..N, mode 0 the most significant bit.  Site POS (1-based) of a
    string is bit norb-POS."""
    idx = 0
    M = 2 * norb
    for pos in range(1, norb + 1):
        bit = norb - pos
        if (d >> bit) & 1:
            idx |= 1 << (M - 1 - (pos - 1))
        if (u >> bit) & 1:
            idx |= 1 << (M - 1 - (norb + pos - 1))
    return idx


def jw_hubbard_sector(sec: Sector, t, U) -> np.ndarray:
    """Dense sector matrix of H = sum_{J,K,s} T(J,K) c^+_{K s} c_{J s}
    + sum_J U_J n_{J up} n_{J down} built in the Fock space, with T(J,K) the
    reference's column-major view of t (hop J->K uses t[K][J])."""
    norb = sec.norb
    t = np.asarray(t, dtype=np.float64)
    U = np.broadcast_to(np.asarray(U, dtype=np.float64), (norb,))
    c = _jw_ops(2 * norb)
    dn = lambda pos: c[pos - 1]
    up = lambda pos: c[norb + pos - 1]
    H = None
    for J in range(1, norb + 1):
        for K in range(1, norb + 1):
            tjk = t[K - 1, J - 1]
            if abs(tjk) < F32_TOL14:
                continue
            term = tjk * (up(K).T @ up(J) + dn(K).T @ dn(J))
            H = term if H is None else H + term
        nu = up(J).T @ up(J)
        nd = dn(J).T @ dn(J)
        term = U[J - 1] * (nu @ nd)
        H = term if H is None else H + term
    idx = np.array([_fock_index(norb, int(u), int(d)) for d in sec.bdn for u in sec.bup], dtype=np.int64)
    return H[idx][:, idx].toarray()


def jw_hubbard_uijkl_sector(sec: Sector, t, Ul) -> np.ndarray:
    """Dense sector matrix of sum_{J,K,s} T(J,K) c^+_{K s} c_{J s} +
    sum UL(J,K,M,N) c^+_{K up} c_{J up} c^+_{N down} c_{M down} over
    UPARTIAL(J,K) >= 1e-14 and |UL(J,K,M,N)| >= 1e-14, in the Fock space
    (UL, UPARTIAL from Ul as the reference reads them)."""
    norb = sec.norb
    t = np.asarray(t, dtype=np.float64)
    Ul = np.asarray(Ul, dtype=np.float64)
    c = _jw_ops(2 * norb)
    dn = lambda pos: c[pos - 1]
    up = lambda pos: c[norb + pos - 1]
    H = None
    for J in range(1, norb + 1):
        for K in range(1, norb + 1):
            tjk = t[K - 1, J - 1]
            if abs(tjk) >= F32_TOL14:
                term = tjk * (up(K).T @ up(J) + dn(K).T @ dn(J))
                H = term if H is None else H + term
            if float(np.sum(Ul[K - 1, J - 1] ** 2)) < F32_TOL14:
                continue
            for M in range(1, norb + 1):
                for N in range(1, norb + 1):
                    v = Ul[N - 1, M - 1, K - 1, J - 1]
                    if abs(v) < F32_TOL14:
                        continue
                    term = v * (up(K).T @ up(J) @ dn(N).T @ dn(M))
                    H = term if H is None else H + term
    idx = np.array([_fock_index(norb, int(u), int(d)) for d in sec.bdn for u in sec.bup], dtype=np.int64)
    return H[idx][:, idx].toarray()


def jw_two_body(sec: Sector, bra, ket, J: int, K: int, M: int, N: int) -> float:
    """<ket| c^+_{K up} c_{J up} c^+_{N down} c_{M down} |bra> in the Fock space."""
    norb = sec.norb
    c = _jw_ops(2 * norb)
    op = c[norb + K - 1].T @ c[norb + J - 1] @ c[N - 1].T @ c[M - 1]
    idx = np.array([_fock_index(norb, int(u), int(d)) for d in sec.bdn for u in sec.bup], dtype=np.int64)
    return float(np.asarray(ket) @ (op[idx][:, idx] @ np.asarray(bra)))


def jw_heis_sector(norb: int, J, physical: bool = False) -> np.ndarray:
    """Dense matrix of the reference's Heisenberg operator in its Sz=0 sector,
    built in the Fock space.

    physical=False: the operator hprod_heis.f90 applies: SzSz and diagonal terms
    plus, for J != K, +J(J,K) (c^+_{K up} c_{J up})(c^+_{J down} c_{K down}).
    physical=True:  sum_{J,K} J(J,K) S_J.S_K with S+ = c^+_up c_down."""
    Jm = np.asarray(J, dtype=np.float64)
    c = _jw_ops(2 * norb)
    dn = lambda pos: c[pos - 1]
    up = lambda pos: c[norb + pos - 1]
    nu = lambda p: up(p).T @ up(p)
    nd = lambda p: dn(p).T @ dn(p)
    sz = lambda p: 0.5 * (nu(p) - nd(p))
    sp_ = lambda p: up(p).T @ dn(p)
    H = None
    for Jp in range(1, norb + 1):
        for Kp in range(1, norb + 1):
            jjk = Jm[Kp - 1, Jp - 1]
            term = jjk * (sz(Jp) @ sz(Kp))
            if physical:
                if Jp != Kp:
                    term = term + 0.5 * jjk * (sp_(Jp) @ sp_(Kp).T + sp_(Jp).T @ sp_(Kp))
                else:
                    term = term + 0.5 * jjk * (sp_(Jp) @ sp_(Jp).T + sp_(Jp).T @ sp_(Jp))
            else:
                if Jp != Kp and abs(jjk) > F32_TOL14:
                    term = term + jjk * ((up(Kp).T @ up(Jp)) @ (dn(Jp).T @ dn(Kp)))
                if Jp == Kp and abs(jjk) > F32_TOL14:
                    single = nu(Jp) + nd(Jp) - 2 * (nu(Jp) @ nd(Jp))
                    term = term + 0.5 * jjk * single
            H = term if H is None else H + term
    full = (1 << norb) - 1
    bup = hilbert(norb, norb // 2)
    idx = np.array([_fock_index(norb, int(u), full - int(u)) for u in bup], dtype=np.int64)
    return H[idx][:, idx].toarray()


# -------------------------------------------------------- lattices ---------

def ring(n: int, t: float = -1.0) -> np.ndarray:
    """Periodic ring with amplitude t on nearest-neighbour bonds
    (examples/05-fermi_hubbard.py:11-13 uses t=-1)."""
    m = np.zeros((n, n))
    for i in range(n):
        m[i, (i + 1) % n] = m[(i + 1) % n, i] = t
    return m


def square_pbc(lx: int, ly: int, t: float = -1.0) -> np.ndarray:
    """Periodic lx x ly square lattice, site s = x + lx*y."""
    n = lx * ly
    m = np.zeros((n, n))
    for y in range(ly):
        for x in range(lx):
            s = x + lx * y
            for (dx, dy) in ((1, 0), (0, 1)):
                q = (x + dx) % lx + lx * ((y + dy) % ly)
                if q != s:
                    m[s, q] = m[q, s] = t
    return m
