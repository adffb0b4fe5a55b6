"""GPU Lanczos drivers built on the sector H*v.

Replaces LANCZOS (lanczos.f90:1-133), EXACT_DIAG's role for the ground state
(exact_diag.f90:2-33) and READ_PSI_HUBBARD's Ritz-vector reconstruction
(compute_solver.f90:282-284).

Differences from the reference, by design:
  * the Krylov basis lives in HBM instead of an HDF5 file
    (lanczos.f90:42-49, 137-161);
  * full reorthogonalisation with one reduction per step: the multi-dot pass
    of step k returns both V^T H u_k and V^T u_k, so the Gram matrix
    G = V^T V is known exactly and the projection w - V G^-1 V^T w costs one
    more pass over V (delayed classical Gram-Schmidt, "DCGS2", Bielich,
    Langou, Thomas, Swirydowicz, Yamazaki, Boman, Parallel Computing 2022);
  * the scalar work of a step (Gram row, inverse-Cholesky row, projection
    coefficients, alpha, beta) runs on the device (ed_lanczos_coef), so the
    steps enqueue without host synchronisation; the host reads alpha/beta at
    convergence checks only;
  * vectors may be stored in FP32 while every scalar (dots, norms, the
    tridiagonal, its eigensolve) is FP64, followed by an FP64 refinement
    Lanczos started from the FP32 Ritz vector;
  * the three-term form (no reorthogonalisation, for bases too large for
    full reorthogonalisation) keeps its Krylov vectors in HBM where they fit,
    else rebuilds Ritz vectors by a second run;
  * the start vector is a seeded uniform[-0.5,0.5) draw (the reference's
    RAND()-0.5 is unseeded, lanczos.f90:22-25).

The convergence rule of the reference (blocks of NADD=5 steps, degeneracy
aware test on Ritz value NDEG+1, lanczos.f90:61-89) is available as
``ReferenceRule``.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

from .. import _capi

NADD = 5


def _torch():
    import torch
    return torch


class ReferenceRule:
    """lanczos.f90:44-91: check every NADD steps; the Ritz value NDEG+1 must
    move by less than acc; a converged value equal to the lowest one raises
    NDEG (a degenerate copy) and the loop goes on."""

    def __init__(self, acc: float = 1e-8):
        self.acc = float(acc)
        self.ev = 0.0
        self.ndeg = 0
        self.converged = False
        self.conv = 0.0   # VAL(NDEG+1) - EV at the last check (the lcz_conv attribute)

    def __call__(self, val: np.ndarray, step: int = 0) -> bool:
        i = min(self.ndeg, len(val) - 1)
        self.conv = float(val[i] - self.ev)
        if abs(val[i] - self.ev) < self.acc:
            if abs(val[i] - val[0]) > self.acc and (self.ndeg + 1) > 1:
                self.converged = True
            else:
                self.ndeg += 1
        else:
            self.ev = val[i]
        return self.converged


class EnergyRule:
    """Stop when the lowest Ritz value moved by less than tol over one check."""

    def __init__(self, tol: float, min_steps: int = 0):
        self.tol = float(tol)
        self.min_steps = min_steps
        self.prev = None
        self.converged = False
        self.ndeg = 1

    def __call__(self, val: np.ndarray, step: int = 1 << 30) -> bool:
        e = float(val[0])
        if self.prev is not None and abs(e - self.prev) < self.tol and step >= self.min_steps:
            self.converged = True
        self.prev = e
        return self.converged


class ResidualRule:
    """Stop when the residual norm of the lowest Ritz pair, |beta_k z_k|
    (last component of its eigenvector of T times the last beta), falls
    below tol.  Needs the eigenvectors of T, so the driver passes them."""

    wants_vectors = True

    def __init__(self, tol: float, min_steps: int = 0):
        self.tol = float(tol)
        self.min_steps = min_steps
        self.converged = False
        self.ndeg = 1
        self.residual = float("inf")

    def __call__(self, val, step: int = 1 << 30, vec=None, beta_last: float = 0.0) -> bool:
        if vec is not None:
            self.residual = abs(beta_last * vec[-1, 0])
            if self.residual < self.tol and step >= self.min_steps:
                self.converged = True
        return self.converged


@dataclass
class KrylovResult:
    alpha: np.ndarray
    beta: np.ndarray            # beta[k] couples steps k and k+1 (len == len(alpha))
    ritz: np.ndarray            # eigenvalues of the final tridiagonal
    ritz_vectors: np.ndarray    # its eigenvectors (columns)
    steps: int
    converged: bool
    breakdown: bool
    psi: object = None          # FP64 device tensor, internal layout (lowest Ritz vector)
    conv: float = 0.0
    ndeg: int = 0
    times: dict = field(default_factory=dict)
    gram_offdiag: float = 0.0   # max |G - I| of the stored basis (orthogonality check)
    basis: object = None        # kept Krylov basis (keep_basis=True)
    scales: np.ndarray = None
    _ws: object = None

    def ritz_vector(self, k: int):
        """Ritz vector k as an FP64 device tensor (needs keep_basis=True)."""
        torch = _torch()
        if self.basis is None:
            raise RuntimeError("the Krylov basis was not kept")
        z = self.ritz_vectors[:, k]
        coef = -(z * self.scales[: self.steps])
        self._ws.coef[: self.steps].copy_(torch.from_numpy(coef))
        psi = torch.zeros(self.basis.shape[1], dtype=torch.float64, device=self.basis.device)
        _capi.update(self.basis, self.steps, self._ws.coef, None, psi, norm2=self._ws.nrm, scratch=self._ws.buf)
        psi.mul_(1.0 / math.sqrt(float(self._ws.nrm[0].item())))
        return psi

    def release(self):
        self.basis = None
        self._ws = None


def start_vector(sec, seed: int = 0, dtype=None, device=None):
    """Seeded uniform[-0.5,0.5) start vector in the internal layout (padding 0).
    Drawn in the reference layout so that the draw does not depend on ld."""
    torch = _torch()
    g = torch.Generator(device=device or "cuda")
    g.manual_seed(int(seed))
    r = torch.rand(sec.dim, generator=g, dtype=torch.float64, device=device or "cuda") - 0.5
    v = sec.from_ref(r)
    return v if dtype is None else v.to(dtype)


def _tridiag_eigs(alpha, beta, k, vectors=False):
    a = np.asarray(alpha[:k], dtype=np.float64)
    b = np.asarray(beta[: k - 1], dtype=np.float64)
    if k == 1:
        return (a.copy(), np.ones((1, 1))) if vectors else a.copy()
    if vectors:
        return sla.eigh_tridiagonal(a, b)
    return sla.eigh_tridiagonal(a, b, eigvals_only=True)


class KernelTimer:
    """CUDA-event timing of the C-ABI calls of a Krylov loop, by call kind,
    on the current stream (where the calls enqueue their kernels).  Records
    algorithmic bytes and kernel launches per call; read after a
    synchronize."""

    LAUNCHES = {"hv": 3, "multidot": 2, "coef": 1, "update": 2, "ritz": 2}

    def __init__(self):
        self.ev = {}
        self.bytes = {}
        self.calls = {}

    def __call__(self, kind: str, nbytes: float):
        torch = _torch()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        self.ev.setdefault(kind, []).append((a, b))
        self.bytes[kind] = self.bytes.get(kind, 0.0) + float(nbytes)
        self.calls[kind] = self.calls.get(kind, 0) + 1
        return b

    def summary(self):
        out = {}
        for k, lst in self.ev.items():
            t = sum(a.elapsed_time(b) for a, b in lst) * 1e-3
            out[k] = {"calls": self.calls[k], "seconds": t, "bytes": self.bytes[k],
                      "launches": self.calls[k] * self.LAUNCHES.get(k, 1)}
        return out

    def launches(self):
        return sum(self.calls[k] * self.LAUNCHES.get(k, 1) for k in self.calls)


class _Scratch:
    def __init__(self, n, nvec, device):
        torch = _torch()
        nb = _capi.scratch_bytes(n, max(nvec, 2))
        self.buf = torch.empty((nb + 7) // 8, dtype=torch.float64, device=device)
        self.dots = torch.zeros(2 * max(nvec, 2) + 2, dtype=torch.float64, device=device)
        self.nrm = torch.zeros(2, dtype=torch.float64, device=device)
        self.coef = torch.zeros(max(nvec, 2), dtype=torch.float64, device=device)


def lanczos_full(sec, v0, max_steps: int, dtype=None, rule=None, check_every: int = NADD,
                 min_steps: int = 0, want_vector: bool = True, vec_index: int = 0,
                 keep_basis: bool = False, timer: KernelTimer = None, ritz_dtype=None,
                 lookahead=None) -> KrylovResult:
    """Lanczos with full reorthogonalisation (delayed CGS with the exact Gram
    matrix).  v0: start vector (device tensor, internal layout).  The basis
    of max_steps+1 vectors is stored in ``dtype`` (FP32 or FP64); scalars are
    FP64.  Stops after max_steps, on breakdown, or when ``rule`` is met at a
    check.  Returns the tridiagonal, its eigenpairs and (optionally) the Ritz
    vector ``vec_index`` as a device tensor of ``ritz_dtype`` (default FP64;
    FP32 from an FP32 basis sums in FP32, at the HBM rate, where an FP64 sum
    is bound by the FP64 pipe).

    A step is four enqueued calls with no host synchronisation: the H*v, the
    multi-dot of the basis with H u_k and u_k, the scalar work on the device
    (ed_lanczos_coef: Gram row, inverse Cholesky row, projection
    coefficients, alpha, beta) and the update, which scales H u_k by s_k on
    the device.  The host reads alpha/beta only at rule checks and at the end.
    With ``lookahead`` (default: when checks are at least 3 steps apart) a
    check's alpha/beta are copied asynchronously and the next step is enqueued
    before the host waits for them, so the GPU does not idle during the check;
    a run that converges there has done one step more than it keeps."""
    torch = _torch()
    dtype = dtype or v0.dtype
    dev = v0.device
    n = sec.n
    m = int(max_steps)
    t_start = time.perf_counter()
    # Row j of V is written (u_0 = v0, then u_{j} by the update of step j-1)
    # before any call reads it, and keeps zero padding: v0 and w have zero
    # padding, H*v leaves w's padding untouched, and the update combines them.
    V = torch.empty((m + 1, n), dtype=dtype, device=dev)
    w = torch.zeros(n, dtype=dtype, device=dev)
    ws = _Scratch(n, m + 1, dev)
    V[0].copy_(v0)
    _capi.multidot(V, 1, V[0], ws.dots, ws.buf)
    n0 = float(ws.dots[0].item())
    if not (n0 > 0.0 and math.isfinite(n0)):
        raise ValueError("start vector has zero or non-finite norm")
    state = torch.zeros(_capi.lanczos_state_doubles(m), dtype=torch.float64, device=dev)
    state[2] = 1.0 / math.sqrt(n0)
    ab = torch.zeros((2, m), dtype=torch.float64, device=dev)   # alpha, beta
    es = V.element_size()
    k_done = 0
    converged = breakdown = False

    def close(k):
        """beta[k-1], s_k and the stop test of step k-1; host copies."""
        _capi.lanczos_coef(k, m, None, ws.nrm, state, None, ab[0], ab[1])
        hs = state[:2].cpu().numpy()
        hab = ab[:, :k].cpu().numpy()
        return int(hs[0]), float(hs[1]), hab[0].copy(), hab[1].copy()

    def post(k):
        """close(k) with the copies left in flight: (k, event, host buffers)."""
        _capi.lanczos_coef(k, m, None, ws.nrm, state, None, ab[0], ab[1])
        cuda = state.is_cuda
        hs = torch.empty(2, dtype=torch.float64, pin_memory=cuda)
        hab = torch.empty((2, k), dtype=torch.float64, pin_memory=cuda)
        hs.copy_(state[:2], non_blocking=cuda)
        hab.copy_(ab[:, :k], non_blocking=cuda)
        ev = None
        if cuda:
            ev = torch.cuda.Event()
            ev.record()
        return k, ev, hs, hab

    def judge(k, stop, alpha, beta):
        """The rule at check k: True to stop there."""
        if stop != 0:
            return True
        if getattr(rule, "wants_vectors", False):
            val, vecs_t = _tridiag_eigs(alpha, beta, k, vectors=True)
            return rule(val, k, vec=vecs_t, beta_last=beta[k - 1])
        return rule(_tridiag_eigs(alpha, beta, k), k)

    if lookahead is None:
        lookahead = check_every >= 3
    pending = None
    snap = None      # (k, stop, gram, alpha, beta) of the check the run stopped at

    for k in range(m):
        e = timer("hv", 2.0 * sec.dim * es) if timer is not None else None
        sec.hv(V[k], w)
        if e is not None:
            e.record()
            e = timer("multidot", (k + 2) * sec.dim * es)
        _capi.multidot(V, k + 1, w, ws.dots, ws.buf, z=V[k])
        if e is not None:
            e.record()
            e = timer("coef", 0.0)
        _capi.lanczos_coef(k, m, ws.dots, ws.nrm, state, ws.coef, ab[0], ab[1])
        if e is not None:
            e.record()
            e = timer("update", (k + 3) * sec.dim * es)
        _capi.update(V, k + 1, ws.coef, w, V[k + 1], norm2=ws.nrm, scratch=ws.buf, wscale=state[2 + k: 3 + k])
        if e is not None:
            e.record()
        k_done = k + 1
        if pending is not None:
            # the check posted after the previous step, read while this step runs
            kc, ev, hs, hab = pending
            pending = None
            # step kc is already enqueued: its lanczos_coef part 1 rewrites beta[kc-1] and s[kc]
            # from the same norm (idempotent), so stopping at check kc leaves the Ritz scales intact
            if ev is not None:
                ev.synchronize()
            st_c, g_c = int(hs[0]), float(hs[1])
            a_c, b_c = hab[0].numpy().copy(), hab[1].numpy().copy()
            if judge(kc, st_c, a_c, b_c):
                snap = (kc, st_c, g_c, a_c, b_c)
                converged = st_c == 0
                break
        if rule is not None and k_done % check_every == 0 and k_done >= min_steps:
            if lookahead and k_done < m:
                pending = post(k_done)
                continue
            stop, gram_off, alpha, beta = close(k_done)
            if judge(k_done, stop, alpha, beta):
                snap = (k_done, stop, gram_off, alpha, beta)
                converged = stop == 0
                break
    if snap is not None:
        k_done, stop, gram_off, alpha, beta = snap
    else:
        stop, gram_off, alpha, beta = close(k_done)
    if stop < 0:
        raise FloatingPointError(f"non-finite norm at Lanczos step {-stop - 1}")
    if stop > 0:
        k_done = min(k_done, stop)
        breakdown = converged = True
        alpha, beta = alpha[:k_done], beta[:k_done]
    s = state[2: 3 + k_done].cpu().numpy()
    t_loop = time.perf_counter()
    val, vec = _tridiag_eigs(alpha, beta, k_done, vectors=True)
    res = KrylovResult(alpha=alpha[:k_done].copy(), beta=beta[:k_done].copy(), ritz=val, ritz_vectors=vec,
                       steps=k_done, converged=converged, breakdown=breakdown,
                       ndeg=getattr(rule, "ndeg", 0) if rule is not None else 0)
    res.gram_offdiag = gram_off
    if want_vector:
        z = vec[:, vec_index]
        coef = -(z * s[:k_done])
        ws.coef[:k_done].copy_(torch.from_numpy(coef))
        rdt = ritz_dtype or torch.float64
        psi = torch.empty(n, dtype=rdt, device=dev)
        e = timer("ritz", (k_done * es + psi.element_size()) * sec.dim) if timer is not None else None
        _capi.update(V, k_done, ws.coef, None, psi, norm2=ws.nrm, scratch=ws.buf)
        if e is not None:
            e.record()
        nrm = math.sqrt(float(ws.nrm[0].item()))
        psi.mul_(1.0 / nrm)
        res.psi = psi
    res.times = {"loop": t_loop - t_start, "total": time.perf_counter() - t_start}
    if rule is not None:
        res.conv = float(getattr(rule, "conv", 0.0))
    if keep_basis:
        res.basis, res.scales, res._ws = V, s, ws
    del w
    return res


@dataclass
class PlainResult:
    alpha: np.ndarray
    beta: np.ndarray
    ritz: np.ndarray
    ritz_vectors: np.ndarray
    steps: int
    converged: bool
    psis: list
    times: dict


def _zero_padding(sec, rows):
    """Zero the padding of every row of a (rows, sec.n) block: the columns
    past nsup of each down-string row (Hubbard), the tail past dim
    (Heisenberg)."""
    if sec.n == sec.dim:
        return
    if sec.kind == _capi.ED_HUBBARD:
        rows.view(rows.shape[0], sec.nsdn, sec.ld)[:, :, sec.nsup:].zero_()
    else:
        rows[:, sec.dim:].zero_()


def kept_storage(dev, need: int, frac: float = 0.85, min_bytes: int = 1 << 20):
    """One device byte block for the kept Krylov rows of lanczos_plain: need
    bytes, or ``frac`` of the free memory if less (None if not even min_bytes
    can be had).  Stages that run one after the other (FP32, then FP64
    refinement) share one block: the caching allocator would otherwise split
    the large cached block of the first stage with vectors that outlive it,
    and the second stage could not get one."""
    torch = _torch()
    # first from the driver's free memory plus what the allocator holds unused (a block a
    # previous solve left cached is reused as it is); failing that, with the cache returned
    free = torch.cuda.mem_get_info(dev)[0]
    cached = torch.cuda.memory_reserved(dev) - torch.cuda.memory_allocated(dev)
    # whole GiB when large, so that repeated solves ask for the block the previous one left cached
    gib = 1 << 30
    nbytes = min(int(need), int(frac * (free + cached)))
    nbytes = nbytes // gib * gib if nbytes >= 4 * gib else nbytes // 256 * 256
    if nbytes >= min_bytes:
        try:
            return torch.empty(nbytes, dtype=torch.uint8, device=dev)
        except torch.OutOfMemoryError:
            pass
    torch.cuda.empty_cache()
    nbytes = min(int(need), int(frac * torch.cuda.mem_get_info(dev)[0]))
    nbytes = nbytes // gib * gib if nbytes >= 4 * gib else nbytes // 256 * 256
    while nbytes >= min_bytes:
        try:
            return torch.empty(nbytes, dtype=torch.uint8, device=dev)
        except torch.OutOfMemoryError:
            nbytes = nbytes // 2 // 256 * 256
    return None


def lanczos_plain(sec, v0, max_steps: int, rule=None, check_every: int = NADD, nvec: int = 1,
                  want_vectors: bool = True, keep: bool = True, ritz_dtype=None, storage=None) -> PlainResult:
    """The reference's three-term recurrence without reorthogonalisation
    (lanczos.f90:52-58), alpha fused into the H*v pass.

    Ritz vectors: the reference stores every Krylov vector (in HDF5,
    lanczos.f90:42-49) and sums them.  Here, when the whole run fits in the
    free device memory (keep=True), the recurrence runs on rows of a kept
    basis and each Ritz vector is one update pass over it (summed in
    ``ritz_dtype``, FP64 by default).  Otherwise (or keep=False) the run uses
    three rotating vectors and the Ritz vectors are rebuilt by running the same
    deterministic recurrence a second time, accumulating sum_k z_k v_k in FP64.
    An integer ``keep`` caps the kept rows: a run longer than that moves to
    the rotating vectors when the rows run out and rebuilds by replay.
    ``storage`` (a device uint8 block, see kept_storage) holds the kept rows;
    without it a block of the free memory is taken for this call."""
    torch = _torch()
    dev = v0.device
    n = sec.n
    m = int(max_steps)
    t0 = time.perf_counter()
    ws = _Scratch(n, max(4, nvec), dev)
    R = None       # the three rotating vectors, made when a run needs them
    t_alloc = time.perf_counter()
    V = None
    if want_vectors and keep:
        es = v0.element_size()
        if storage is None:
            storage = kept_storage(dev, (m + 1) * n * es, min_bytes=4 * n * es)
        cap = 0 if storage is None else min(m + 1, storage.numel() // (n * es))
        if not isinstance(keep, bool):
            cap = min(cap, int(keep))
        if cap >= 4:
            V = storage[: cap * n * es].view(v0.dtype).view(cap, n)
            _zero_padding(sec, V)   # the H*v leaves the padding untouched
    cap = 0 if V is None else V.shape[0]
    t_alloc = time.perf_counter() - t_alloc

    def rotating():
        nonlocal R
        if R is None:
            R = torch.zeros((3, n), dtype=v0.dtype, device=dev)
        else:
            R.zero_()
        return R

    def run(steps, z=None, psis=None):
        # a replay (psis given) follows the first run's schedule of kept rows and rotating
        # vectors, so that it recomputes the same vectors bit for bit
        kept = V is not None
        R = None if kept else rotating()
        if kept:
            V[0].copy_(v0)
        else:
            R[0].copy_(v0)
        _capi.multidot(R if not kept else V, 1, v0, ws.dots, ws.buf)
        s_prev, s_cur = 0.0, 1.0 / math.sqrt(float(ws.dots[0].item()))
        alpha, beta, scales = [], [], [s_cur]
        bprev = 0.0
        done = 0
        conv = False
        for k in range(steps):
            if kept and k + 1 >= cap:
                # the kept rows are used up: continue on the rotating vectors
                R = rotating()
                R[(k + 2) % 3].copy_(V[k - 1])
                R[k % 3].copy_(V[k])
                kept = False
            if kept:
                W, cur, nxt, prv = (V[0:2], 0, 1, None) if k == 0 else (V[k - 1:k + 2], 1, 2, 0)
            else:
                W, cur, nxt, prv = R, k % 3, (k + 1) % 3, (k + 2) % 3
            if psis is not None:
                for j, p in enumerate(psis):
                    ws.coef[0] = -z[k, j] * s_cur
                    _capi.update(W[cur:cur + 1], 1, ws.coef, p, p)
            # W[nxt] = H v_k with v_k = s_cur u_k; dots[0] = <u_k, H v_k>
            sec.hv(W[cur], W[nxt], scale=s_cur, dots=ws.dots, scratch=ws.buf)
            a = s_cur * float(ws.dots[0].item())
            coef = np.zeros(W.shape[0])
            coef[cur] = a * s_cur
            if k > 0:
                coef[prv] = bprev * s_prev
            ws.coef[: W.shape[0]].copy_(torch.from_numpy(coef))
            _capi.update(W, W.shape[0], ws.coef, W[nxt], W[nxt], norm2=ws.nrm, scratch=ws.buf)
            nw2 = float(ws.nrm[0].item())
            b = math.sqrt(max(nw2, 0.0))
            alpha.append(a)
            beta.append(b)
            done = k + 1
            if not math.isfinite(nw2):
                raise FloatingPointError(f"non-finite norm at Lanczos step {k}")
            if b <= 1e-13 * max(1.0, abs(a)):
                conv = True
                break
            s_prev, s_cur, bprev = s_cur, 1.0 / math.sqrt(nw2), b
            scales.append(s_cur)
            if psis is None and rule is not None and done % check_every == 0:
                if getattr(rule, "wants_vectors", False):
                    val, vec = _tridiag_eigs(np.array(alpha), np.array(beta), done, vectors=True)
                    stop = rule(val, done, vec=vec, beta_last=b)
                else:
                    stop = rule(_tridiag_eigs(np.array(alpha), np.array(beta), done), done)
                if stop:
                    conv = True
                    break
        return np.array(alpha), np.array(beta), done, conv, (np.array(scales) if kept else None)

    t_run = time.perf_counter()
    alpha, beta, done, conv, scales = run(m)    # scales is None when the kept rows ran out
    if v0.is_cuda:
        torch.cuda.synchronize()
    t_run = time.perf_counter() - t_run
    val, vec = _tridiag_eigs(alpha, beta, done, vectors=True)
    t_ritz = time.perf_counter()
    psis = []
    if want_vectors:
        nv = min(nvec, done)
        if scales is not None:
            # u_0 .. u_{done-1} are rows of V: psi_j = sum_k z_kj s_k u_k in one pass each
            rdt = ritz_dtype or torch.float64
            for j in range(nv):
                c = torch.from_numpy(-(vec[:, j] * scales[:done])).to(dev)
                p = torch.empty(n, dtype=rdt, device=dev)
                _capi.update(V, done, c, None, p, norm2=ws.nrm, scratch=ws.buf)
                p.mul_(1.0 / math.sqrt(float(ws.nrm[0].item())))
                psis.append(p)
        else:
            psis = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(nv)]
            run(done, z=vec[:, :nv], psis=psis)
            for p in psis:
                _capi.multidot(p.view(1, -1), 1, p, ws.dots, ws.buf)
                p.mul_(1.0 / math.sqrt(float(ws.dots[0].item())))
    if v0.is_cuda:
        torch.cuda.synchronize()
    t_ritz = time.perf_counter() - t_ritz
    return PlainResult(alpha=alpha, beta=beta, ritz=val, ritz_vectors=vec, steps=done, converged=conv,
                       psis=psis, times={"total": time.perf_counter() - t0, "alloc": t_alloc, "run": t_run,
                                         "ritz": t_ritz, "kept_rows": cap,
                                         "replayed": bool(want_vectors and scales is None)})


@dataclass
class GroundState:
    e0: float
    psi: object                 # FP64 device tensor, internal layout
    ritz: np.ndarray
    alpha: np.ndarray
    beta: np.ndarray
    steps: int
    refine_steps: int
    converged: bool
    ndeg: int
    times: dict
    mode: str
    e0_unrefined: float = float("nan")
    ritz_vectors: np.ndarray = None


REFINE_CHECK = 2   # steps between energy checks of the FP64 refinement


def ground_state(sec, mode: str = "mixed", steps: int = 200, seed: int = 0, v0=None, rule=None,
                 refine_steps: int = 60, refine_tol: float = 1e-13, check_every: int = NADD,
                 timer: KernelTimer = None, reorth: str = "full", refine_rule=None) -> GroundState:
    """Ground state of the sector operator.

    mode "f64":   FP64 vectors, FP64 scalars (the plain FP64 GPU Lanczos).
    mode "f32":   FP32 vectors, FP64 scalars, no refinement.
    mode "mixed": FP32 vectors + FP64 scalars for ``steps`` steps, then an
                  FP64 Lanczos restarted from the FP32 Ritz vector until the
                  lowest Ritz value moves less than refine_tol*max(1,|E0|)
                  between checks (at most refine_steps steps).
    reorth "full" keeps every Krylov vector (lanczos_full); "none" runs the
    three-term recurrence on four vectors and rebuilds the Ritz vector by a
    second pass (lanczos_plain), for sectors whose basis would not fit;
    refine_rule replaces the energy rule of the FP64 stage."""
    torch = _torch()
    t0 = time.perf_counter()
    if v0 is None:
        v0 = start_vector(sec, seed)
    if reorth == "none":
        return _ground_state_plain(sec, mode, steps, v0, rule, refine_steps, refine_tol, check_every, t0,
                                   refine_rule=refine_rule)
    if mode == "f64":
        r = lanczos_full(sec, v0.to(torch.float64), steps, torch.float64, rule=rule, check_every=check_every,
                         timer=timer)
        torch.cuda.synchronize()
        return GroundState(e0=float(r.ritz[0]), psi=r.psi, ritz=r.ritz, alpha=r.alpha, beta=r.beta, steps=r.steps,
                           refine_steps=0, converged=r.converged, ndeg=r.ndeg,
                           times={"total": time.perf_counter() - t0, "fp64": r.times["total"]}, mode=mode,
                           e0_unrefined=float(r.ritz[0]), ritz_vectors=r.ritz_vectors)
    # in mixed mode the FP32 Ritz vector only starts the FP64 stage: its error is that of the
    # FP32 Krylov space, far above the rounding of an FP32 sum
    r32 = lanczos_full(sec, v0.to(torch.float32), steps, torch.float32, rule=rule, check_every=check_every,
                       timer=timer, ritz_dtype=torch.float32 if mode == "mixed" else None)
    t1 = time.perf_counter()
    if mode == "f32":
        return GroundState(e0=float(r32.ritz[0]), psi=r32.psi, ritz=r32.ritz, alpha=r32.alpha, beta=r32.beta,
                           steps=r32.steps, refine_steps=0, converged=r32.converged, ndeg=r32.ndeg,
                           times={"total": t1 - t0, "fp32": r32.times["total"]}, mode=mode,
                           e0_unrefined=float(r32.ritz[0]), ritz_vectors=r32.ritz_vectors)
    # the FP64 stage starts from the FP32 Ritz vector and converges in a few steps: its energy
    # is checked every REFINE_CHECK steps (two agreeing checks stop it)
    rr = refine_rule or EnergyRule(refine_tol * max(1.0, abs(float(r32.ritz[0]))), min_steps=2 * REFINE_CHECK)
    psi32 = r32.psi
    r32.release()
    r64 = lanczos_full(sec, psi32, refine_steps, torch.float64, rule=rr, check_every=REFINE_CHECK,
                       timer=timer)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return GroundState(e0=float(r64.ritz[0]), psi=r64.psi, ritz=r64.ritz, alpha=r32.alpha, beta=r32.beta,
                       steps=r32.steps, refine_steps=r64.steps, converged=r32.converged or rr.converged,
                       ndeg=r32.ndeg, times={"total": t2 - t0, "fp32": t1 - t0, "refine": t2 - t1}, mode=mode,
                       e0_unrefined=float(r32.ritz[0]), ritz_vectors=r64.ritz_vectors)


def _ground_state_plain(sec, mode, steps, v0, rule, refine_steps, refine_tol, check_every, t0,
                        refine_rule=None) -> GroundState:
    torch = _torch()
    vt = torch.float64 if mode == "f64" else torch.float32
    ts = time.perf_counter()
    storage = kept_storage(v0.device, max((steps + 1) * sec.n * (8 if mode == "f64" else 4),
                                          (refine_steps + 1) * sec.n * 8 if mode == "mixed" else 0),
                           min_bytes=4 * sec.n * 8)
    t_storage = time.perf_counter() - ts
    # mixed: the FP32 Ritz vector only starts the FP64 stage (summed in FP32 from a kept basis)
    r = lanczos_plain(sec, v0.to(vt), steps, rule=rule, check_every=check_every, nvec=1,
                      ritz_dtype=torch.float32 if mode == "mixed" else None, storage=storage)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    e0u = float(r.ritz[0])
    if mode != "mixed":
        return GroundState(e0=e0u, psi=r.psis[0], ritz=r.ritz, alpha=r.alpha, beta=r.beta, steps=r.steps,
                           refine_steps=0, converged=r.converged, ndeg=1,
                           times={"total": t1 - t0, mode: t1 - t0}, mode=mode, e0_unrefined=e0u,
                           ritz_vectors=r.ritz_vectors)
    rr = refine_rule or EnergyRule(refine_tol * max(1.0, abs(e0u)), min_steps=2 * check_every)
    psi = r.psis[0].to(torch.float64)
    r.psis = []
    r64 = lanczos_plain(sec, psi, refine_steps, rule=rr, check_every=check_every, nvec=1, storage=storage)
    del psi, storage
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return GroundState(e0=float(r64.ritz[0]), psi=r64.psis[0], ritz=r64.ritz, alpha=r.alpha, beta=r.beta,
                       steps=r.steps, refine_steps=r64.steps, converged=r.converged or rr.converged, ndeg=1,
                       times={"total": t2 - t0, "fp32": t1 - t0, "refine": t2 - t1, "storage": t_storage,
                              "fp32_alloc": r.times["alloc"], "fp32_run": r.times["run"],
                              "fp32_total": r.times["total"], "fp32_ritz": r.times["ritz"],
                              "fp32_kept_rows": r.times["kept_rows"],
                              "fp32_replayed": r.times["replayed"], "refine_alloc": r64.times["alloc"],
                              "refine_kept_rows": r64.times["kept_rows"], "refine_replayed": r64.times["replayed"]},
                       mode=mode, e0_unrefined=e0u, ritz_vectors=r64.ritz_vectors)
