"""Batched continued-fraction Green's functions.

Every particle/hole start vector of every cluster is one Lanczos instance;
all instances advance together through ed_batch_lanczos (two kernels per
step over all instances).  The whole fixed-length run enqueues with no host
synchronisation, so it is captured once in a CUDA graph and replayed.  The
per-instance alternative, one three-term Lanczos driven from the host per
start vector (``lanczos_plain``), is kept for comparison.

G^>(w) = <phi|(w + E0 - H + i eta)^-1|phi>,  phi = c^+_i psi0   (poles at E_n - E0)
G^<(w) = <phi|(w - E0 + H + i eta)^-1|phi>,  phi = c_i psi0     (poles at E0 - E_n)
as the reference places them (reduced_quantities.py:84-92); the retarded G_ii
is their sum.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .. import _capi
from ..trace import nvtx
from . import lanczos as LZ


def _torch():
    import torch
    return torch


_TUNED = {}   # (dtype, sector shapes) -> rows per CTA chosen by autotune()


def autotune(sectors, dtype, steps: int = 3, sample: int = 192, device="cuda"):
    """Rows per CTA of the batched H*v for this set of sectors: each candidate
    (4, 8, 16) runs `steps` Lanczos steps (CUDA events on the current stream,
    after one untimed run) on an evenly spaced sample of at most `sample`
    instances, which keeps the batch's mix of sector shapes; the fastest is
    kept and remembered for batches of the same set of distinct shapes and
    dtype."""
    torch = _torch()
    key = (str(dtype), tuple(sorted({(s.nsup, s.nsdn) for s in sectors})))
    if key in _TUNED:
        return _TUNED[key]
    pick = [sectors[int(j)] for j in np.linspace(0, len(sectors) - 1, min(sample, len(sectors)))]
    times = {}
    for rows in _capi.Batch.ROWS:
        b = _capi.Batch(pick, rows=rows)
        work = torch.zeros(3 * b.total, dtype=dtype, device=device)
        x0 = torch.rand(b.total, dtype=dtype, device=device)
        n = len(b.sectors)
        alpha = torch.zeros((n, steps), dtype=torch.float64, device=device)
        beta = torch.zeros((n, steps + 1), dtype=torch.float64, device=device)
        scratch = torch.empty(b.scratch_bytes() // 8 + 1, dtype=torch.float64, device=device)
        b.lanczos(work, x0, steps, alpha, beta, scratch)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.lanczos(work, x0, steps, alpha, beta, scratch)
        e1.record()
        torch.cuda.synchronize()
        times[rows] = e0.elapsed_time(e1)
        del b, work, x0, scratch
    best = min(times, key=times.get)
    _TUNED[key] = best
    return best


class BatchedLanczos:
    """Fixed-length three-term Lanczos of many instances in one enqueue.
    rows: rows of one instance per CTA of the H*v (4, 8 or 16), or "auto"
    to let autotune() pick it on this batch.  keep: keep every Krylov vector
    (Ritz vectors by one pass over them, _ritz_cycle) instead of two; "auto"
    keeps them when they fit in half of the free device memory."""

    def __init__(self, sectors, nsteps: int, dtype=None, device="cuda", rows=8, keep=False, persistent=False):
        torch = _torch()
        self.dtype = dtype or torch.float32
        self.nsteps = int(nsteps)
        if rows == "auto":
            rows = autotune(sectors, self.dtype, device=device)
        self.batch = _capi.Batch(sectors, rows=rows)
        self.rows = self.batch.rows
        self.sectors = list(sectors)
        n = len(self.sectors)
        tot = self.batch.total
        # keep=True: every Krylov vector is kept (basis slot k = u_k, written before it is read)
        # and Ritz vectors are one pass over them (ritz_sum) instead of a replay; "auto" keeps
        # them when they take at most half of the free device memory
        if keep == "auto":
            es = torch.empty(0, dtype=self.dtype).element_size()
            free = torch.cuda.mem_get_info(device)[0] + torch.cuda.memory_reserved(device) - \
                torch.cuda.memory_allocated(device)
            keep = (self.nsteps + 2) * tot * es <= 0.5 * free
        self.keep = bool(keep)
        self.basis = torch.empty((self.nsteps + 1) * tot, dtype=self.dtype, device=device) if keep else None
        # the run fills its Krylov slots itself (a copy of x0, a cleared u_{-1}) and the H*v
        # writes every element of y, row padding included
        self.work = torch.empty((1 if keep else 3) * tot, dtype=self.dtype, device=device)
        self.x0 = torch.zeros(tot, dtype=self.dtype, device=device)
        self.alpha = torch.zeros((n, self.nsteps), dtype=torch.float64, device=device)
        self.beta = torch.zeros((n, self.nsteps + 1), dtype=torch.float64, device=device)
        self.scratch = torch.empty(self.batch.scratch_bytes() // 8 + 1, dtype=torch.float64, device=device)
        self.graph = None
        # persistent: the whole run is one cooperative launch (ed_batch_lanczos_persistent)
        self.persistent = bool(persistent)

    def start(self, i: int):
        return self.batch.view(self.x0, i)

    def run(self):
        if self.persistent:
            self.batch.lanczos_persistent(self.work, self.x0, self.nsteps, self.alpha, self.beta, self.scratch,
                                          kept=self.basis if self.keep else None)
        elif self.keep:
            self.batch.lanczos_kept(self.basis, self.work, self.x0, self.nsteps, self.alpha, self.beta, self.scratch)
        else:
            self.batch.lanczos(self.work, self.x0, self.nsteps, self.alpha, self.beta, self.scratch)

    def capture(self):
        """Record run() in a CUDA graph (the batch set its kernels' attributes
        when it was created, so nothing but stream work is captured)."""
        torch = _torch()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()


@dataclass
class BatchedGroundStates:
    e0: np.ndarray          # [n] lowest Ritz values
    residual: np.ndarray    # [n] ||H psi - E0 psi|| of the returned (normalised) vectors
    psi: list               # [n] normalised FP64 ground states (views into one device vector)
    restarts: int           # FP64 cycles after the first (on the unconverged instances only)


def _lowest_ritz(a, b, tol_break: float = 1e-12, every: int = 10):
    """Lowest eigenpair of one instance's tridiagonal matrix, cut at the first
    vanishing beta (an exhausted Krylov space); returns (theta, y, estimate, m)
    with the usual estimate beta_m |y_m| of the residual.  The leading
    m x m blocks, m = every, 2*every, ... and the whole run, are compared and
    the one with the smallest estimate is kept: without reorthogonalisation
    the lost orthogonality spoils the Ritz vector once the pair has converged
    (a kept basis sums any prefix of its vectors)."""
    import scipy.linalg as sla
    scale = max(1.0, float(np.abs(a).max()) if a.size else 1.0)
    m = len(a)
    for k in range(1, len(a)):
        if b[k] <= tol_break * scale:
            m = k
            break
    if m == 1:
        return float(a[0]), np.ones(1), float(b[1]), 1
    best = None
    for mm in sorted(set(list(range(every, m, every)) + [m])):
        if mm < 2:
            continue
        w, y = sla.eigh_tridiagonal(a[:mm], b[1:mm], select="i", select_range=(0, 0))
        est = float(b[mm] * abs(y[mm - 1, 0]))
        if best is None or est < best[2]:
            best = (float(w[0]), y[:, 0], est, mm)
    return best


def _ritz_cycle(bl, out):
    """One batched Lanczos run, the lowest Ritz pair of every instance, and
    the Ritz vectors in `out` (normalised): one pass over the kept basis, or
    a replay that accumulates them."""
    torch = _torch()
    n, nsteps = len(bl.sectors), bl.nsteps
    bl.run()
    A = bl.alpha.cpu().numpy()
    B = bl.beta.cpu().numpy()
    C = np.zeros((n, nsteps))
    e0 = np.zeros(n)
    for i in range(n):
        theta, y, _, m = _lowest_ritz(A[i], B[i])
        e0[i] = theta
        C[i, :m] = y
    coef = torch.from_numpy(C).to(bl.x0.device)
    if bl.keep:
        bl.batch.ritz_sum(bl.basis, nsteps, coef, bl.beta, out)
    else:
        out.zero_()
        bl.batch.ritz(bl.work, bl.x0, nsteps, bl.alpha, bl.beta, coef, out, bl.scratch)
    for i in range(n):
        v = bl.batch.view(out, i)
        v /= torch.linalg.vector_norm(v)
    return e0


def _true_residuals(bl, out, e0):
    """||H psi_i - E0_i psi_i|| of every instance (per-sector FP64 H*v)."""
    torch = _torch()
    res = torch.empty(len(bl.sectors), dtype=torch.float64, device=out.device)
    for i, sec in enumerate(bl.sectors):
        v = bl.batch.view(out, i)
        y = torch.zeros_like(v)       # ed_hv leaves the row padding untouched
        sec.hv(v, y)
        res[i] = torch.linalg.vector_norm(y - e0[i] * v)
    return res.cpu().numpy()


def batched_ground_states(sectors, nsteps: int = 120, tol: float = 1e-10, max_restarts: int = 8, seed: int = 0,
                          mixed: bool = True, refine_steps: int = 60) -> BatchedGroundStates:
    """Ground states of many sectors at once.  Every sector is an instance of
    the batched three-term Lanczos with its Krylov vectors kept
    (ed_batch_lanczos_kept); the lowest Ritz pair of each tridiagonal matrix is
    found on the host and one pass over the kept vectors (ed_batch_ritz_sum)
    forms the Ritz vectors -- the reference's ground-state solve
    (lanczos.f90:17-86 for the coefficients and the stored vectors,
    compute_solver.f90:270-290 for V*c).

    mixed=True: a first cycle of nsteps with FP32 vectors, then FP64 cycles
    of refine_steps restarted from the previous Ritz vector; mixed=False:
    FP64 cycles of nsteps from the start.  Cycles repeat (all instances; the
    converged ones keep improving) until every true residual
    ||H psi - E0 psi|| is below tol, at most max_restarts FP64 cycles after
    the first."""
    torch = _torch()
    starts = [LZ.start_vector(sec, seed + i, dtype=torch.float64) for i, sec in enumerate(sectors)]
    if mixed:
        b32 = BatchedLanczos(sectors, nsteps, dtype=torch.float32, rows="auto", keep="auto")
        for i, v in enumerate(starts):
            b32.start(i).copy_(v)
        out32 = torch.zeros_like(b32.x0)
        _ritz_cycle(b32, out32)
        bl = BatchedLanczos(sectors, refine_steps, dtype=torch.float64, rows="auto", keep="auto")
        bl.x0.copy_(out32)
        del b32, out32
    else:
        bl = BatchedLanczos(sectors, nsteps, dtype=torch.float64, keep="auto")
        for i, v in enumerate(starts):
            bl.start(i).copy_(v)
    out = torch.zeros_like(bl.x0)
    e0 = _ritz_cycle(bl, out)
    res = _true_residuals(bl, out, e0)
    # further FP64 cycles only for the instances still above tol, each
    # restarted from its Ritz vector in a batch of their own
    it = 0
    todo = np.nonzero(res > tol)[0]
    while todo.size and it < max_restarts:
        it += 1
        sub = BatchedLanczos([bl.sectors[i] for i in todo], refine_steps, dtype=torch.float64, keep="auto")
        for j, i in enumerate(todo):
            sub.start(j).copy_(bl.batch.view(out, int(i)))
        sout = torch.zeros_like(sub.x0)
        e_sub = _ritz_cycle(sub, sout)
        r_sub = _true_residuals(sub, sout, e_sub)
        for j, i in enumerate(todo):
            if r_sub[j] < res[i]:
                bl.batch.view(out, int(i)).copy_(sub.batch.view(sout, j))
                e0[i], res[i] = e_sub[j], r_sub[j]
        del sub, sout
        todo = np.nonzero(res > tol)[0]
    psi = [bl.batch.view(out, i) for i in range(len(bl.sectors))]
    return BatchedGroundStates(e0=e0, residual=res, psi=psi, restarts=it)


def continued_fraction(alpha, beta, z, sign: float = 1.0):
    """beta_0^2 / (z - s a_0 - b_1^2 / (z - s a_1 - ...)) for every instance
    (rows of alpha [n, m], beta [n, m+1]) at every z (1-D complex tensor);
    sign=-1 evaluates <phi|(z + H)^-1|phi>.  Returns [n, len(z)] (one thread
    per instance and frequency, ed_cf_eval)."""
    torch = _torch()
    sg = torch.full((alpha.shape[0],), float(sign), dtype=torch.float64, device=alpha.device)
    return _capi.cf_eval(alpha, beta, torch.as_tensor(z, device=alpha.device), sign=sg)


def plain_coefficients(sec, phi, nsteps: int):
    """alpha, beta of one start vector by the per-instance three-term Lanczos
    (beta[0] = ||phi||, beta[k] couples steps k-1 and k)."""
    torch = _torch()
    nrm = math.sqrt(float((phi.double() ** 2).sum().item()))
    r = LZ.lanczos_plain(sec, phi, nsteps, rule=None, want_vectors=False)
    a = np.zeros(nsteps)
    b = np.zeros(nsteps + 1)
    a[: len(r.alpha)] = r.alpha
    b[0] = nrm
    b[1: len(r.beta) + 1] = r.beta
    return a, b


@dataclass
class ClusterGF:
    e0: float
    nup: int
    ndn: int
    norb: int
    # instance index ranges in the batch: [(spin, part, site) -> instance]
    index: dict


def build_start_vectors(solver_sectors, src_sector, psi0, bl: BatchedLanczos, inst_of: dict):
    """Write c|psi0> / c^+|psi0> of every (spin, part, site) into the batch
    start vectors (instance i's slot in its sector's internal layout)."""
    for (spin, part, site), i in inst_of.items():
        kind = ("e_" if part == "greater" else "h_") + spin
        # ed_gf_start converts psi0's precision to the slot's on the fly
        _capi.gf_start(src_sector, bl.sectors[i], kind, site, psi0, bl.start(i))


def c4_clusters(n: int = 256, seed: int = 0):
    """Seeded cluster set of the batched Green's-function workload: half 2x6,
    half 3x4 open-boundary square clusters, nearest-neighbour t = 1
    (t_ij = -1), next-nearest t' ~ U[-0.3, 0.3] on the plaquette diagonals,
    uniform U ~ U[0, 8], N_up = N_down in {5, 6}."""
    from ..tools import lattices as LT
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n):
        lx, ly = (6, 2) if c < n // 2 else (4, 3)
        tp = float(rng.uniform(-0.3, 0.3))
        U = float(rng.uniform(0.0, 8.0))
        N = int(rng.choice([5, 6]))
        out.append({"t": LT.square(lx, ly, -1.0, periodic=False, tp=tp), "U": U, "N": N, "shape": (lx, ly),
                    "tp": tp})
    return out


def sweep(clusters, nsteps: int = 150, chunk: int = 64, dtype=None, gs_steps: int = 120, gs_tol: float = 1e-10,
          omega=None, eta: float = 0.05, graph: bool = True, timings: dict = None, rows="auto"):
    """Ground states (batched over the clusters of a chunk), then G_ii^s(w)
    of every cluster from its 4*norb particle/hole start vectors by
    continued fractions (batched over all start vectors of the chunk).
    Returns {cluster: {'e0': E0, 'G': complex tensor [2 spins, norb, len(w)]}}."""
    torch = _torch()
    import time
    dtype = dtype or torch.float32
    timings = {} if timings is None else timings
    omega = omega if omega is not None else torch.linspace(-10.0, 10.0, 2048, dtype=torch.float64, device="cuda")
    results = {}
    t_gs = t_start = t_lz = t_cf = t_sec = 0.0
    n_inst = 0
    restarts = 0
    rows_used = []
    for c0 in range(0, len(clusters), chunk):
        cl = clusters[c0:c0 + chunk]
        secs, inst = [], []
        base = []
        t0 = time.perf_counter()
        # the five sectors of every cluster (ground state and the four N+-1 sectors), built on
        # host threads: the table construction runs in the library with the GIL released
        shapes = []
        for spec in cl:
            N = spec["N"]
            shapes.append([(N, N), (N + 1, N), (N - 1, N), (N, N + 1), (N, N - 1)])
        built = _build_sectors([(spec, key) for spec, keys in zip(cl, shapes) for key in keys])
        t_sec += time.perf_counter() - t0
        srcs = []
        for ci, spec in enumerate(cl):
            norb = spec["t"].shape[0]
            N = spec["N"]
            own = dict(zip(shapes[ci], built[5 * ci: 5 * ci + 5]))
            srcs.append(own[(N, N)])
            base.append(len(inst))
            # instance order inside a cluster: spin (up, down) x part (greater, lesser) x site
            for spin in ("up", "down"):
                for part in ("greater", "lesser"):
                    d = 1 if part == "greater" else -1
                    key = (N + d, N) if spin == "up" else (N, N + d)
                    for site in range(1, norb + 1):
                        inst.append((ci, spin, part, site))
                        secs.append(own[key])
        with nvtx("pyhub.sweep.ground_states"):
            gsb = batched_ground_states(srcs, nsteps=gs_steps, tol=gs_tol, seed=c0)
        restarts = max(restarts, gsb.restarts)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        bl = BatchedLanczos(secs, nsteps, dtype=dtype, rows=rows)
        rows_used.append(bl.rows)
        # one launch per (cluster, spin, part): its sites are consecutive instances of one sector,
        # equally spaced in the batch
        off = bl.batch.offsets
        for i, j, stride in _site_groups(inst, off):
            ci, spin, part, _ = inst[i]
            kind = ("e_" if part == "greater" else "h_") + spin
            if stride is None:
                for q in range(i, j):
                    _capi.gf_start(srcs[ci], secs[q], kind, inst[q][3], gsb.psi[ci], bl.start(q))
            else:
                _capi.gf_start_sites(srcs[ci], secs[i], kind, [inst[q][3] for q in range(i, j)], gsb.psi[ci],
                                     bl.x0[int(off[i]):], stride)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        with nvtx("pyhub.sweep.batched_lanczos"):
            if graph:
                bl.capture()
                bl.replay()
            else:
                bl.run()
            torch.cuda.synchronize()
        t3 = time.perf_counter()
        # greater: <phi|(w + E0 + i eta - H)^-1|phi>; lesser: <phi|(w - E0 + i eta + H)^-1|phi>
        sg = torch.tensor([1.0 if p == "greater" else -1.0 for (_, _, p, _) in inst], dtype=torch.float64,
                          device="cuda")
        e0s = torch.tensor([gsb.e0[ci] for (ci, _, _, _) in inst], dtype=torch.float64, device="cuda")
        with nvtx("pyhub.sweep.continued_fractions"):
            G = _capi.cf_eval(bl.alpha, bl.beta, omega.to(torch.complex128) + 1j * eta, shift=sg * e0s, sign=sg)
        for ci in range(len(cl)):
            norb = cl[ci]["t"].shape[0]
            g = G[base[ci]: base[ci] + 4 * norb].view(2, 2, norb, -1).sum(dim=1)
            results[c0 + ci] = {"e0": float(gsb.e0[ci]), "G": g}
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        t_gs += t1 - t0
        t_start += t2 - t1
        t_lz += t3 - t2
        t_cf += t4 - t3
        n_inst += len(inst)
        del bl, secs, srcs, gsb, built
        torch.cuda.empty_cache()
    timings.update({"ground_states_s": t_gs, "sectors_s": t_sec, "start_vectors_s": t_start, "lanczos_s": t_lz, "cf_eval_s": t_cf,
                    "instances": n_inst, "total_s": t_gs + t_start + t_lz + t_cf, "gs_restarts": restarts,
                    "rows_per_cta": rows_used})
    return results


def sharded_sweep(clusters, rank: int = 0, ws: int = 1, sweep_fn=None, **kw):
    """A sweep over clusters sharded across ranks: rank r sweeps clusters r,
    r+ws, ... (no collective on the data path), then rank 0 gathers every
    rank's results (reduced_quantities.py:84-92 builds G from the poles of
    each cluster; here each cluster's G_ii(w) and E0 come back as host arrays).
    Returns {cluster index: {'e0': float, 'G': complex128 ndarray [2, norb,
    nw]}} for all clusters on rank 0, None on the other ranks.  sweep_fn
    (default: sweep) maps a list of cluster specs to {local index: result}."""
    from .. import replicas as RP
    sweep_fn = sweep if sweep_fn is None else sweep_fn
    mine = RP.shard(range(len(clusters)), rank, ws)
    res = sweep_fn([clusters[i] for i in mine], **kw)
    local = {}
    for k, v in res.items():
        g = v["G"]
        local[mine[k]] = {"e0": float(v["e0"]),
                          "G": g.cpu().numpy() if hasattr(g, "cpu") else np.asarray(g)}
    parts = RP.gather_to_root(local)
    if parts is None:
        return None
    merged = {}
    for p in parts:
        merged.update(p)
    return merged


def _site_groups(inst, offsets):
    """Runs [i, j) of consecutive instances with the same (cluster, spin,
    part), and the constant distance of their slots in the batch (0 for a
    single instance), or None when the slots are not equally spaced.
    inst: [(cluster, spin, part, site)]; offsets: slot offsets by instance."""
    out = []
    i = 0
    while i < len(inst):
        j = i
        while j < len(inst) and inst[j][:3] == inst[i][:3]:
            j += 1
        stride = int(offsets[i + 1] - offsets[i]) if j - i > 1 else 0
        if j - i > 1 and any(int(offsets[q + 1] - offsets[q]) != stride for q in range(i, j - 1)):
            stride = None
        out.append((i, j, stride))
        i = j
    return out


def _build_sectors(jobs, workers: int = 8):
    """Hubbard sectors for [(cluster spec, (N_up, N_down))], built concurrently
    on host threads (each on the caller's current device)."""
    torch = _torch()
    from concurrent.futures import ThreadPoolExecutor
    dev = torch.cuda.current_device()

    def make(job):
        spec, (nu, nd) = job
        torch.cuda.set_device(dev)
        norb = spec["t"].shape[0]
        return _capi.Sector(norb, nu, nd, _capi.ED_HUBBARD, t=spec["t"], U=np.full(norb, spec["U"]))

    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(make, jobs))


