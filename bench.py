#!/usr/bin/env python3
"""Benchmark of the GB300 exact-diagonalisation engine.

Workload (one "step"): the ground state of the 4x4 periodic Hubbard cluster,
t=1, U=8, half filling (N_up = N_down = 8, sector dimension 12870^2 =
165,636,900), from a seeded uniform start vector: 200 Lanczos steps with full
reorthogonalisation on FP32 vectors with FP64 scalars, then an FP64 Lanczos
refinement from the FP32 Ritz vector until E0 moves less than 1e-13|E0|.
Inputs (hopping tables, start vector, Krylov basis) are device resident; the
vectors (0.66 GB each) are far larger than L2, so no L2 flush is needed
between solves.

Printed (rank 0, one JSON line): solves/s (``value``), the FP64 plain solve
it is compared with (|dE0| must stay < 1e-10), the roofline of the dominant
kernel of the solve and of the H*v kernel, an end-to-end number through the
public API (FermiHubbard.kernel with host inputs and psi0 copied back), the
CPU baseline (the reference's HPROD loop restated in C, on all host threads,
timed on one H*v), SM clocks sampled during the timed region.

``--impl reference`` times the reference's own algorithm on all the host cores
instead (the restated Fortran HPROD loop; the Fortran itself cannot be built
here), extrapolated from a bounded sample to the same number of H*v products.

Multi-GPU (torchrun): the sector does not shard without an all-to-all
transpose per H*v, so N GPUs run N independent replicas ("replicas only");
value aggregates all ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "4×4 Hubbard Lanczos s to |ΔE0|<1e-10 mixed vs FP64; H·v HBM GB/s; batched GF/s"
UNIT = "solve/s"
CPU_PAIRS_OURS = 64       # our line's cpu_baseline: one whole H*v (64 hop pairs + 16 U sites)
CPU_PAIRS_REF = 16        # per step of the reference arm: a quarter of one H*v


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--lanczos-steps", type=int, default=200)
    p.add_argument("--U", type=float, default=8.0)
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison solve")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-c4", action="store_true", help="skip the batched Green's-function part of the default line")
    p.add_argument("--small", action="store_true", help="3x3 cluster, for a quick functional run")
    p.add_argument("--config", default="c2", choices=["c2", "c3", "c4", "c5"],
                   help="c2: 4x4 Hubbard ground-state solve (default); c3: 4x8 Heisenberg ground state and "
                        "nearest-neighbour spin correlations; c4: batched Green's functions of 256 clusters; "
                        "c5: gradients of E0 and of a 1-RDM loss for a 14-site random-bond cluster")
    p.add_argument("--clusters", type=int, default=256)
    p.add_argument("--lattice", default="4x8", help="c3: periodic LXxLY lattice (default 4x8)")
    p.add_argument("--fd-params", type=int, default=8, help="c5: parameters checked by central differences")
    p.add_argument("--probe", action="store_true",
                   help="for profilers: c2, a few launches of each solve kernel on 4x4-sized vectors (about "
                        "4 GB); c4, two 3-step batched FP32 Lanczos runs (8 rows per CTA) over the particle/hole "
                        "instances of --clusters clusters, then one 3-step persistent run (--persistent); c5, two "
                        "all-pairs RDM passes on an FP64 vector of the 14-site sector")
    p.add_argument("--persistent", action="store_true", help="c4 --probe: add a persistent batched run")
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_table():
    """Per-kernel-class DRAM traffic from the committed ncu summary
    (profiles/ncu_traffic.txt): lines 'kind ratio note', ratio = measured
    dram__bytes_read+write / algorithmic bytes of the captured launches."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    out = {}
    try:
        for line in open(path):
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            k, b, u = line.split()[:3]
            out[k] = (float(b), u)
    except OSError:
        pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


class StreamClock:
    """Elapsed time of a region on the device: CUDA events recorded on the
    current stream (where every C-ABI call enqueues its kernels) at start()
    and stop(); stop() synchronises and returns seconds."""

    def __init__(self):
        import torch
        self.torch = torch
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def start(self):
        self.e0.record(self.torch.cuda.current_stream())
        return self

    def stop(self) -> float:
        self.e1.record(self.torch.cuda.current_stream())
        self.e1.synchronize()
        return self.e0.elapsed_time(self.e1) / 1e3


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(pairs_per_sample: int, n_udiag: int, U: float, nthreads: int = 0):
    """Time the reference's HPROD loop (restated in C: its loop order and
    linear-search rank) on a subset of its (J,K) pairs and on-site U terms, and
    extrapolate to one full H*v of the 4x4 sector.  nthreads host threads
    (0: all the process may use) split each pair's rank search and own blocks of
    output rows; the result equals the one-thread loop bit for bit."""
    nthreads = nthreads or host_threads()
    import numpy as np
    from oracle import oracle as O
    from pyhub_gb300.tools import lattices as LT
    t, _ = LT.hubbard_4x4(U)
    sec = O.Sector(16, 8, 8)
    pairs = [(J, K) for J in range(1, 17) for K in range(1, 17) if J != K and abs(t[K - 1, J - 1]) > 0]
    x = np.random.default_rng(0).uniform(-0.5, 0.5, sec.dim)
    y = np.zeros(sec.dim)
    t0 = time.perf_counter()
    O.hprod_hubbard_pairs(sec, t, pairs[:pairs_per_sample], x, y, nthreads=nthreads)
    tp = time.perf_counter() - t0
    t0 = time.perf_counter()
    for J in range(1, n_udiag + 1):
        O.hprod_hubbard_udiag(sec, J, U, x, y, nthreads=nthreads)
    tu = time.perf_counter() - t0
    hv = tp * len(pairs) / pairs_per_sample + tu * 16 / n_udiag
    return hv, tp + tu, f"{pairs_per_sample} of {len(pairs)} hop pairs + {n_udiag} of 16 U sites of one H*v", nthreads


C2_REFINE_STEPS = 4   # FP64 refinement steps of the engine's C2 solve (measured: E0 settles after 4)


def c2_config(args, dim: int, ws: int) -> dict:
    """The workload description both arms print for the 4x4 solve."""
    return {"workload": ("4x4 periodic Hubbard t=1 U=%g N_up=N_down=8 (D=%d) ground state: "
                         "%d-step full-reorth Lanczos FP32 + FP64 refinement") % (args.U, dim, args.lanczos_steps),
            "parallelism": f"replicas x{ws}", "l2": "vectors 0.66 GB >> L2; no flush needed"}


def e0_oracle_check(t, U, psi, e0: float) -> dict:
    """|dE0| of the mixed solve against the FP64 oracle: the Rayleigh quotient
    <psi|H|psi>/<psi|psi> and the residual ||H psi - E0 psi|| / ||psi|| of the
    engine's psi0 (reference layout, FP64 on the host), with H psi from the
    reference's HPROD loop restated in C (hprod_hubbard.f90:17-118) on all
    host threads."""
    import numpy as np
    from oracle import oracle as O
    t0 = time.perf_counter()
    osec = O.Sector(16, 8, 8)
    hpsi = O.hprod_hubbard_mt(osec, t, U, psi)
    nn = float(np.dot(psi, psi))
    rq = float(np.dot(psi, hpsi)) / nn
    r = hpsi - e0 * psi
    return {"rayleigh_quotient": rq, "abs_dE0_vs_oracle": abs(rq - e0),
            "residual": float(np.sqrt(np.dot(r, r) / nn)), "oracle_hv_seconds": time.perf_counter() - t0,
            "oracle": f"reference HPROD loop restated in C on {host_threads()} host threads"}


def run_reference(args):
    ws, rank, local = dist()
    if rank != 0:
        return
    # the same H*v count as one engine solve: the FP32 steps plus the FP64 refinement steps
    n_hv = args.lanczos_steps + C2_REFINE_STEPS
    times = []
    for i in range(args.warmup + args.steps):
        hv, spent, desc, nth = cpu_sample(CPU_PAIRS_REF, 4, args.U)
        if i >= args.warmup:
            times.append(hv * n_hv)
    solve_s = statistics.mean(times)
    v = 1.0 / solve_s
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": solve_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded uniform[-0.5,0.5) start vector)",
            "config": c2_config(args, 12870 * 12870, 1),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"{desc} per step; extrapolated to the {n_hv} H*v of one solve (reference "
                                       f"loop order, linear-search rank, on {nth} host threads; its HDF5 I/O is "
                                       f"not counted)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def probe(sec, torch, LZ, capi):
    """2 FP32 H*v, 2 FP64 H*v, 2 multidot and 2 update launches (4 vectors) on
    vectors of the 4x4 sector: the launches profiled under ncu."""
    x = LZ.start_vector(sec, 1, dtype=torch.float32)
    y = torch.zeros_like(x)
    for _ in range(2):
        sec.hv(x, y)
    x64, y64 = x.double(), torch.zeros(sec.n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        sec.hv(x64, y64)
    del x64, y64
    nv = 4
    V = torch.zeros((nv, sec.n), dtype=torch.float32, device="cuda")
    for j in range(nv):
        V[j].copy_(LZ.start_vector(sec, 10 + j, dtype=torch.float32))
    sc = torch.empty(capi.scratch_bytes(sec.n, nv) // 8 + 1, dtype=torch.float64, device="cuda")
    out = torch.zeros(2 * nv, dtype=torch.float64, device="cuda")
    coef = torch.full((nv,), 1e-3, dtype=torch.float64, device="cuda")
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        capi.multidot(V, nv, y, out, sc, z=V[nv - 1])
    for _ in range(2):
        capi.update(V, nv, coef, y, y, norm2=nrm, scratch=sc)
    torch.cuda.synchronize()
    print(json.dumps({"probe": "ok", "dim": sec.dim, "dots": out.cpu().tolist()[:2]}))


def probe_c4(args):
    """Two 3-step FP32 batched Lanczos runs (8 rows per CTA, fused form) over
    the 48 particle/hole instances of each of the first --clusters C4
    clusters: the launches profiled under ncu (6 H*v launches per run)."""
    import numpy as np
    import torch
    from pyhub_gb300 import _build, _capi
    from pyhub_gb300.core import greens_batched as GB
    _build.build()
    secs = []
    for spec in GB.c4_clusters(args.clusters, seed=0):
        N = spec["N"]
        for key in [(N + 1, N), (N - 1, N), (N, N + 1), (N, N - 1)]:
            s = _capi.Sector(12, key[0], key[1], _capi.ED_HUBBARD, t=spec["t"], U=np.full(12, spec["U"]))
            secs += [s] * 12
    bl = GB.BatchedLanczos(secs, 3, dtype=torch.float32, rows=8)
    bl.x0.copy_(torch.rand(bl.batch.total, dtype=torch.float32, device="cuda"))
    for _ in range(2):
        bl.run()
    if args.persistent:
        bp = GB.BatchedLanczos(secs, 3, dtype=torch.float32, rows=8, persistent=True)
        bp.x0.copy_(bl.x0)
        bp.run()
    torch.cuda.synchronize()
    print(json.dumps({"probe": "ok", "instances": len(secs), "elements": int(bl.batch.total)}))


def c4_batched(args, ws: int, rank: int, local: int, warmup: int = 1) -> dict:
    """Batched Green's functions (the metric's third part): 256 seeded 12-site
    open clusters (2x6, 3x4), ground state then 48 particle/hole start vectors
    x 150 Lanczos steps each, G_ii(w) on 2048 points of [-10, 10], eta = 0.05.
    Clusters are sharded over the ranks (every rank sweeps its share, then
    rank 0 gathers every cluster's G(w)).  Timed: the sweep (CUDA events on
    the current stream); the batched Lanczos (one CUDA-graph replay per chunk
    of 64 clusters) against per-instance runs of the same kernels on the same
    start vectors, one instance per launch sequence with its scalars on the
    device (no host synchronisation inside a run); and ed_batch_hv alone for
    the roofline of the batched H*v kernel.  Returns the rank-0 summary (None
    on other ranks)."""
    import numpy as np
    import torch
    from pyhub_gb300 import _capi
    from pyhub_gb300 import replicas as RP
    from pyhub_gb300.core import greens_batched as GB
    from pyhub_gb300.core import lanczos as LZ
    clusters = GB.c4_clusters(args.clusters, seed=0)
    mine = RP.shard(clusters, rank, ws)
    # warm-up on one cluster of each filling: the batched H*v form is tuned there
    # for every sector shape of the sweep (autotune keys on the distinct shapes)
    warm = list({spec["N"]: spec for spec in reversed(mine)}.values())
    for _ in range(max(warmup, 1)):
        GB.sweep(warm, nsteps=150, chunk=len(warm))
    RP.barrier()
    tim = {}
    clock = StreamClock().start()
    merged = GB.sharded_sweep(clusters, rank, ws, nsteps=150, chunk=64, timings=tim)
    elapsed_local = clock.stop()
    RP.barrier()
    rate, total_gf, elapsed = RP.aggregate_rate(tim["instances"], elapsed_local)
    lz_rate = RP.sum_over_ranks(tim["instances"]) / RP.max_over_ranks(tim["lanczos_s"])
    if rank != 0:
        return None
    # G(w) of every cluster is on rank 0 now
    gsum = float(sum(np.abs(v["G"]).sum() for v in merged.values()))
    # per-instance runs: the 48 start vectors of the first cluster, one batch of one instance each
    spec = clusters[0]
    norb, N = spec["t"].shape[0], spec["N"]
    U = np.full(norb, spec["U"])
    src = _capi.Sector(norb, N, N, _capi.ED_HUBBARD, t=spec["t"], U=U)
    gs = LZ.ground_state(src, mode="f64", steps=200, rule=LZ.ResidualRule(1e-10, 10))
    rows = tim["rows_per_cta"][0] if tim.get("rows_per_cta") else 8
    singles, starts, secs = [], [], []
    for spin, part in (("up", "greater"), ("up", "lesser"), ("down", "greater"), ("down", "lesser")):
        d = 1 if part == "greater" else -1
        key = (N + d, N) if spin == "up" else (N, N + d)
        dst = _capi.Sector(norb, key[0], key[1], _capi.ED_HUBBARD, t=spec["t"], U=U)
        for site in range(1, norb + 1):
            bl1 = GB.BatchedLanczos([dst], 150, dtype=torch.float32, rows=rows)
            _capi.gf_start(src, dst, ("e_" if part == "greater" else "h_") + spin, site, gs.psi, bl1.start(0))
            singles.append(bl1)
            secs.append(dst)
    for bl1 in singles[:2]:
        bl1.run()
    torch.cuda.synchronize()
    clock = StreamClock().start()
    for bl1 in singles:
        bl1.run()
    t_single = clock.stop() / len(singles)
    # the same instances batched together (equal accuracy: the same kernels and sums)
    blb = GB.BatchedLanczos(secs, 150, dtype=torch.float32, rows=rows)
    for i, bl1 in enumerate(singles):
        blb.start(i).copy_(bl1.start(0))
    blb.run()
    torch.cuda.synchronize()
    a1 = torch.stack([b1.alpha[0] for b1 in singles]).cpu().numpy()
    b1_ = torch.stack([b1.beta[0] for b1 in singles]).cpu().numpy()
    same = bool(np.array_equal(a1, blb.alpha.cpu().numpy()) and np.array_equal(b1_, blb.beta.cpu().numpy()))
    # batched H*v kernel alone on the last chunk's shape mix (one of every sector of 64 clusters)
    hb = GB.BatchedLanczos(_c4_hv_sample(clusters[:64]), 1, dtype=torch.float32, rows=rows)
    x = torch.rand(hb.batch.total, dtype=torch.float32, device="cuda")
    for i in range(len(hb.sectors)):      # zero row padding, as every engine vector has
        v = hb.batch.view(x, i).view(hb.sectors[i].nsdn, -1)
        v[:, hb.sectors[i].nsup:] = 0
    y = torch.empty_like(x)
    for _ in range(3):
        hb.batch.hv(x, y, hb.scratch)
    torch.cuda.synchronize()
    reps = 10
    clock = StreamClock().start()
    for _ in range(reps):
        hb.batch.hv(x, y, hb.scratch)
    t_hv = clock.stop() / reps
    # the whole batched run as one persistent launch against the four-launch graph, on the 64-cluster
    # chunk's particle/hole instances (3,072 instances, FP32, 40 steps), graph replays timed
    pl = {}
    res_ab = {}
    xs = None
    for pers in (False, True):
        blp = GB.BatchedLanczos(_c4_gf_instances(clusters[:64]), 40, dtype=torch.float32, rows=rows,
                                persistent=pers)
        if xs is None:
            xs = torch.rand(blp.batch.total, dtype=torch.float32, device="cuda")
            for i, sct in enumerate(blp.sectors):
                blp.batch.view(xs, i).view(sct.nsdn, -1)[:, sct.nsup:] = 0
        blp.x0.copy_(xs)
        blp.capture()
        blp.replay()
        torch.cuda.synchronize()
        clock = StreamClock().start()
        for _ in range(3):
            blp.replay()
        pl["persistent_ms_per_step" if pers else "four_launch_ms_per_step"] = clock.stop() / 3 / 40 * 1e3
        res_ab[pers] = (blp.alpha.clone(), blp.beta.clone())
        if pers:
            pl["persistent_status"] = blp.batch.persistent_status(blp.scratch)
        del blp
        torch.cuda.empty_cache()
    pl["alpha_beta_bit_identical"] = bool(torch.equal(res_ab[False][0], res_ab[True][0]) and
                                          torch.equal(res_ab[False][1], res_ab[True][1]))
    del xs, res_ab
    peak, src_kind = peaks()
    alg = sum(s.dim for s in hb.sectors) * 8.0
    n_gf = tim["instances"]
    per_step_bytes = 24.0 * sum(s.dim for s in blb.sectors) / len(blb.sectors)   # H*v 8 B + update 16 B per element
    out = {"workload": "256 clusters (128 2x6 + 128 3x4 open), t=1, t'~U[-0.3,0.3], U~U[0,8], N_up=N_down in "
                       "{5,6}; GS + 48 start vectors x 150 Lanczos steps; 2048-point w grid, eta=0.05",
           "value": rate, "unit": "GF/s", "seconds": elapsed, "gf_instances": int(total_gf),
           "clusters_gathered_on_rank0": len(merged), "G_abs_sum": gsum, "timings": tim,
           "batched_lanczos_gf_per_s": lz_rate, "per_instance_gf_per_s": 1.0 / t_single,
           "batched_over_per_instance": lz_rate * t_single,
           "per_instance_arm": ("the first cluster's 48 start vectors, each its own ed_batch_lanczos run "
                                "(4 launches per step, scalars on the device, no host synchronisation), "
                                "back to back on one stream; CUDA events"),
           "per_instance_alpha_beta_equal_batched": same,
           "batch_hv_roofline": {"kernel": "batch_hv_kernel", "bound": "hbm",
                                 "achieved": alg / t_hv / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": alg / t_hv / 1e9 / peak, "peak_kind": f"of {src_kind}",
                                 "alg_bytes_per_launch": alg, "ms": t_hv * 1e3,
                                 "instances": len(hb.sectors), "traffic": None},
           "lanczos_step_bytes_per_instance": per_step_bytes,
           "persistent_vs_four_launch": pl}
    del singles, blb, hb, x, y
    torch.cuda.empty_cache()
    return out


def _c4_hv_sample(clusters):
    """The particle/hole sectors of the given clusters (one per cluster, spin
    and part): the shape mix of one sweep chunk, for timing the batched H*v."""
    import numpy as np
    from pyhub_gb300 import _capi
    out = []
    for spec in clusters:
        norb, N = spec["t"].shape[0], spec["N"]
        U = np.full(norb, spec["U"])
        for key in [(N + 1, N), (N - 1, N), (N, N + 1), (N, N - 1)]:
            out.append(_capi.Sector(norb, key[0], key[1], _capi.ED_HUBBARD, t=spec["t"], U=U))
    return out


def _c4_gf_instances(clusters):
    """The sectors of the 48 particle/hole start vectors of each cluster (12
    instances per N+-1 sector), in the sweep's order."""
    import numpy as np
    from pyhub_gb300 import _capi
    out = []
    for spec in clusters:
        norb, N = spec["t"].shape[0], spec["N"]
        U = np.full(norb, spec["U"])
        for key in [(N + 1, N), (N - 1, N), (N, N + 1), (N, N - 1)]:
            out += [_capi.Sector(norb, key[0], key[1], _capi.ED_HUBBARD, t=spec["t"], U=U)] * norb
    return out


def run_c4(args):
    """The batched Green's-function sweep as its own JSON line."""
    import torch
    from pyhub_gb300 import _build
    from pyhub_gb300 import replicas as RP
    _build.build()
    ws, rank, local = RP.world()
    torch.cuda.set_device(local)
    RP.init("nccl")
    clocks = ClockSampler(local)
    clocks.start()
    r = c4_batched(args, ws, rank, local, warmup=args.warmup)
    clk = clocks.stop()
    if rank == 0:
        line = {"metric": METRIC, "value": r["value"], "unit": "GF/s", "n_gpus": ws, "steps": 1,
                "warmup": max(args.warmup, 1), "ms_per_step": r["seconds"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 vectors / f64 scalars",
                "data": "synthetic (seeded cluster parameters)",
                "config": {"workload": r["workload"], "clusters": args.clusters,
                           "parallelism": f"clusters sharded over {ws} ranks"},
                "batched_gf": r, "roofline": r["batch_hv_roofline"], "clocks": clk}
        print(json.dumps(line), flush=True)
    RP.finish()


def probe_c5(args):
    """Two all-pairs RDM passes (ed_rdm, every pair of the 14 sites, down hops
    and transverse term) on an FP64 start vector of the 14-site random-bond
    sector: the launches profiled under ncu."""
    import torch
    from pyhub_gb300 import _build, _capi
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.core.reduced_quantities import all_pairs
    from pyhub_gb300.tools import lattices as LT
    _build.build()
    t, U, _ = LT.random_bond_cluster(14, 7, seed=0)
    sec = _capi.Sector(14, 7, 7, _capi.ED_HUBBARD, t=t, U=U)
    psi = LZ.start_vector(sec, 0, dtype=torch.float64)
    for _ in range(2):
        raw, _ = sec.rdm_raw(psi, pairs=all_pairs(14), flags=3)
    torch.cuda.synchronize()
    print(json.dumps({"probe": "ok", "dim": sec.dim, "q0_11": float(raw[0, 0])}))


def run_c3(args):
    """4x8 periodic Heisenberg antiferromagnet (J=1 on the 64 bonds, S_z=0,
    dim C(32,16) = 601,080,390): mixed-precision ground state by the
    three-term Lanczos (FP32 vectors, FP64 scalars, 200 steps) with an FP64
    three-term refinement, then the 64 nearest-neighbour <S_i.S_j>.  The
    timed step is the whole solve; the H*v line is the structured product
    alone (FP32 and FP64, CUDA events)."""
    import numpy as np
    import torch
    from pyhub_gb300 import _build, _capi
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.tools import lattices as LT
    from pyhub_gb300 import replicas as RP
    _build.build()
    ws, rank, local = RP.world()
    torch.cuda.set_device(local)
    RP.init("nccl")
    lx, ly = (4, 4) if args.small else tuple(int(v) for v in args.lattice.lower().split("x"))
    J = LT.square(lx, ly, 1.0, periodic=True)
    norb = lx * ly
    t0 = time.perf_counter()
    sec = _capi.Sector(norb, norb // 2, 0, _capi.ED_HEISENBERG, J=J)
    t_sector = time.perf_counter() - t0
    bonds = [(i + 1, j + 1) for i in range(norb) for j in range(i + 1, norb) if J[i, j] != 0.0]
    scratch = torch.empty(_capi.scratch_bytes(sec.n, 1) // 8 + 1, dtype=torch.float64, device="cuda")
    dots = torch.zeros(2, dtype=torch.float64, device="cuda")
    hv_ms = {}
    for dt in (torch.float32, torch.float64):
        x = LZ.start_vector(sec, 0, dtype=dt)
        y = torch.zeros_like(x)
        for _ in range(2):
            sec.hv(x, y, dots=dots, scratch=scratch)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            sec.hv(x, y, dots=dots, scratch=scratch)
        e1.record()
        torch.cuda.synchronize()
        hv_ms["f32" if dt == torch.float32 else "f64"] = e0.elapsed_time(e1) / 5
        del x, y
    torch.cuda.empty_cache()
    clocks = ClockSampler(local)
    clocks.start()
    RP.barrier()
    clock = StreamClock().start()
    # FP32 stage until E0 stalls at FP32 resolution; FP64 stage until the residual estimate is below 1e-9.
    # Three-term recurrence (no reorthogonalisation) with its Krylov rows kept (55 x 2.4 GB FP32, then
    # 40 x 4.8 GB FP64 in the same block), so each Ritz vector is one pass over the rows.
    steps32, steps64, reorth = args.lanczos_steps, 150, "none"
    gs = LZ.ground_state(sec, mode="mixed", steps=steps32, reorth=reorth, refine_steps=steps64,
                         rule=LZ.EnergyRule(1e-7, min_steps=20), refine_rule=LZ.ResidualRule(1e-9, 10))
    raw, _ = sec.rdm_raw(gs.psi, pairs=bonds)
    t_solve = clock.stop()
    RP.barrier()
    clk = clocks.stop()
    rate, _, t_max = RP.aggregate_rate(1.0, t_solve)   # replicas: one solve per rank
    sij = raw[:, 0] + raw[:, 1]          # SMATRIX(J,K) as J_SPIN forms it (static_rq_heis.f90:66-114)
    # The product's flip element is -(-1)^(J+K) J (hprod_heis.f90:39-45) while J_SPIN's transverse sum
    # carries +(-1)^(J+K), so the energy is sum_{J!=K} J_JK (q1 - q0) = 2 sum_bonds (q1 - q0).
    e_bonds = 2.0 * float(np.sum(raw[:, 1] - raw[:, 0]))
    # residual ||H psi - E0 psi|| in FP64
    y = torch.zeros_like(gs.psi)
    sec.hv(gs.psi, y)
    res = float(torch.linalg.vector_norm(y - gs.e0 * gs.psi))
    peak, src = peaks()
    gbs = 2 * sec.dim * 4 / (hv_ms["f32"] * 1e-3) / 1e9
    if rank == 0:
        line = {"metric": METRIC, "value": rate, "unit": "solve/s", "n_gpus": ws, "steps": 1, "warmup": 1,
                "ms_per_step": t_max * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 vectors / f64 scalars + f64 refinement", "data": "synthetic (seeded start vector)",
                "config": {"workload": f"Heisenberg {lx}x{ly} PBC, J=1, Sz=0, dim {sec.dim}; Lanczos FP32 to E0 "
                                       f"stall (at most {steps32} steps) + FP64 refinement to residual estimate "
                                       f"1e-9 (at most {steps64}); reorthogonalisation {reorth}; nn <S.S>",
                           "parallelism": "replicas"},
                "e0": gs.e0, "e0_per_site": gs.e0 / norb, "e0_unrefined_fp32": gs.e0_unrefined,
                "residual_fp64": res, "fp32_steps": int(gs.steps), "refine_steps": int(gs.refine_steps),
                "nn_smatrix_mean": float(np.mean(sij)), "nn_sisj_energy_gauge_mean": float(np.mean(raw[:, 1] - raw[:, 0])),
                "bond_energy_identity_err": gs.e0 - e_bonds,
                "times_s": {k: (v if isinstance(v, bool) else float(v)) for k, v in gs.times.items()},
                "sector_create_s": t_sector,
                "hv_ms": hv_ms,
                "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                             "traffic": None, "kernel": "structured Heisenberg H*v (FP32), x read + y written",
                             "peak_source": src},
                "clocks": clk}
        print(json.dumps(line), flush=True)
    RP.finish()


def run_c5(args):
    """14-site random-bond Hubbard cluster (ring + 7 seeded extra bonds,
    t~U[0.5,1.5], U_i~U[2,6], eps_i~N(0,0.3^2), N_up=N_down=7, dim 3432^2 =
    11,778,624), 49 parameters.  One step: forward (mixed-precision ground
    state + spin-resolved 1-RDM) and backward (dE0/dtheta by the fused
    Hellmann-Feynman RDM pass; dL/dtheta of L = sum_s ||gamma_s - target_s||^2
    by the adjoint MINRES solve), target = the 1-RDM at a second seeded draw
    of the parameters on the same bonds.  Checked against central
    differences (h = 1e-5) of FP64 solves on a sample of parameters."""
    import numpy as np
    import torch
    from pyhub_gb300 import _build
    from pyhub_gb300.core import gradients as GR
    from pyhub_gb300.tools import lattices as LT
    from pyhub_gb300 import replicas as RP
    _build.build()
    ws, rank, local = RP.world()
    torch.cuda.set_device(local)
    RP.init("nccl")
    n = 10 if args.small else 14
    N = n // 2
    t, U, bonds = LT.random_bond_cluster(n, 7 if n == 14 else 3, seed=0)
    params = GR.HubbardParams(n, [tuple(b) for b in bonds])
    theta = params.pack(t, U)
    rng = np.random.default_rng(1)
    t2 = np.zeros_like(t)
    for (i, j) in params.bonds:
        t2[i, j] = t2[j, i] = rng.uniform(0.5, 1.5)
    t2[np.diag_indices(n)] = rng.normal(0.0, 0.3, n)
    target = GR.solve(params, params.pack(t2, rng.uniform(2.0, 6.0, n)), N, N, mode="f64").gamma

    def step():
        sol = GR.solve(params, theta, N, N, mode="mixed")
        g_e = GR.hf_gradient(params, sol)
        L, g_l, info = GR.rdm_loss_gradient(params, sol, target)
        torch.cuda.synchronize()
        return sol, g_e, L, g_l, info

    for _ in range(max(args.warmup, 1)):
        step()
    clocks = ClockSampler(local)
    clocks.start()
    RP.barrier()
    times = []
    clock_all = StreamClock().start()
    for _ in range(args.steps):
        clock = StreamClock().start()
        sol, g_e, L, g_l, info = step()
        times.append(clock.stop())
    t_all = clock_all.stop()
    RP.barrier()
    clk = clocks.stop()
    rate, _, t_max = RP.aggregate_rate(args.steps, t_all)   # replicas: args.steps evaluations per rank
    # central differences of FP64 solves on a sample of parameters (bonds, U, eps)
    nb = len(params.bonds)
    k = max(1, args.fd_params)
    pick = sorted(set([int(v) for v in np.linspace(0, nb - 1, max(1, k // 2))] +
                      [nb + int(v) for v in np.linspace(0, n - 1, max(1, k // 4))] +
                      [nb + n + int(v) for v in np.linspace(0, n - 1, max(1, k - k // 2 - k // 4))]))
    h = 1e-5
    fd_e, fd_l = [], []
    for p in pick:
        vals = []
        for sgn in (1.0, -1.0):
            th = theta.copy()
            th[p] += sgn * h
            so = GR.solve(params, th, N, N, mode="f64")
            gu, gd = so.gamma["up"], so.gamma["down"]
            vals.append((so.e0, float(np.sum((gu - target["up"]) ** 2) + np.sum((gd - target["down"]) ** 2))))
        fd_e.append((vals[0][0] - vals[1][0]) / (2 * h))
        fd_l.append((vals[0][1] - vals[1][1]) / (2 * h))
    fd_e, fd_l = np.array(fd_e), np.array(fd_l)
    err_e = float(np.max(np.abs(g_e[pick] - fd_e)) / max(1e-12, np.max(np.abs(fd_e))))
    err_l = float(np.max(np.abs(g_l[pick] - fd_l)) / max(1e-12, np.max(np.abs(fd_l))))
    ms = statistics.median(times) * 1e3
    if rank == 0:
        line = {"metric": METRIC, "value": rate, "unit": "grad-evals/s", "n_gpus": ws, "steps": args.steps,
                "warmup": max(args.warmup, 1), "ms_per_step": t_max / args.steps * 1e3, "median_ms_per_eval": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 H*v + f64 refinement (forward), f64 adjoint",
                "data": "synthetic (seeded cluster parameters)",
                "config": {"workload": f"{n}-site random-bond Hubbard (ring + extra bonds), N_up=N_down={N}, "
                                       f"dim {sol.sector.dim}, {params.nparams} parameters; forward E0 + 1-RDM, "
                                       "backward dE0/dtheta (Hellmann-Feynman) + d||gamma-target||^2/dtheta "
                                       "(adjoint MINRES)", "parallelism": "replicas"},
                "e0": sol.e0, "loss": L, "minres_iters": info["minres_iters"], "minres_relres": info["minres_relres"],
                "fd_check": {"params": [params.names()[p] for p in pick], "h": h,
                             "max_rel_err_dE0": err_e, "max_rel_err_dL": err_l},
                "clocks": clk}
        print(json.dumps(line), flush=True)
    RP.finish()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.config == "c4":
        if args.probe:
            probe_c4(args)
        else:
            run_c4(args)
        return
    if args.config == "c3":
        run_c3(args)
        return
    if args.config == "c5":
        if args.probe:
            probe_c5(args)
        else:
            run_c5(args)
        return
    import numpy as np
    import torch
    from pyhub_gb300 import _build, _capi
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.tools import lattices as LT

    from pyhub_gb300 import replicas as RP
    ws, rank, local = RP.world()
    torch.cuda.set_device(local)
    RP.init("nccl")
    _build.build()
    barrier = RP.barrier
    max_over_ranks = RP.max_over_ranks

    if args.small:
        t, U = LT.square(3, 3, -1.0), np.full(9, args.U)
        norb, nup, ndn = 9, 4, 5
    else:
        t, U = LT.hubbard_4x4(args.U)
        norb, nup, ndn = 16, 8, 8
    sec = _capi.Sector(norb, nup, ndn, _capi.ED_HUBBARD, t=t, U=U)
    hbm, hbm_kind = peaks()
    if args.probe:
        probe(sec, torch, LZ, _capi)
        return

    def solve(timer=None):
        return LZ.ground_state(sec, mode="mixed", steps=args.lanczos_steps, seed=0, timer=timer)

    # The solves keep PyTorch's cached device memory between them (the FP32 basis of 133 GB is
    # allocated once, as a long-running solver keeps its workspace); the cache is emptied only
    # before the plain FP64 solve, whose 266 GB basis needs the room.
    for _ in range(args.warmup):
        g = solve()
        del g
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    timer = LZ.KernelTimer()
    clock = StreamClock().start()
    res = []
    psi_last = None
    for i in range(args.steps):
        g = solve(timer)
        res.append((g.e0, g.steps, g.refine_steps, g.e0_unrefined))
        if i == args.steps - 1:
            psi_last = g.psi
        del g
    elapsed = clock.stop()
    # the last solve's psi0 (FP64) goes to the host for the oracle check below
    psi_host = sec.to_ref(psi_last).cpu().numpy() if (rank == 0 and not args.small) else None
    del psi_last
    barrier()
    clk = clocks.stop()
    elapsed = max_over_ranks(elapsed)
    ksum = timer.summary()
    e0_mixed = res[-1][0]
    value = ws * args.steps / elapsed

    # roofline of the dominant kernel of the solve, from the events of the timed solves
    dom = max(ksum, key=lambda k: ksum[k]["seconds"])
    tr = traffic_table()
    names = {"hv": "hub_slab_kernel+hub_row_kernel", "multidot": "multidot_kernel", "update": "update_kernel"}

    def roof(kind):
        d = ksum[kind]
        ach = d["bytes"] / d["seconds"] / 1e9
        per_launch = d["bytes"] / d["calls"]
        # DRAM bytes per launch: the ncu ratio (DRAM bytes / algorithmic bytes of the
        # captured launches) applied to this workload's algorithmic bytes per launch
        traffic = tr[kind][0] * per_launch if kind in tr else None
        return {"kernel": names.get(kind, kind), "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "peak_kind": f"of {hbm_kind}", "traffic": traffic,
                "alg_bytes_per_launch": per_launch, "launches": d["calls"], "seconds": d["seconds"],
                "share_of_solve": d["seconds"] / sum(v["seconds"] for v in ksum.values())}

    roofline = roof(dom)
    hv_roof = roof("hv")

    # H*v alone (FP32 and FP64), the kernel the metric's second part names
    x = LZ.start_vector(sec, 1, dtype=torch.float32)
    y = torch.zeros_like(x)
    for _ in range(3):
        sec.hv(x, y)
    torch.cuda.synchronize()
    ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nrep = 20
    ea.record()
    for _ in range(nrep):
        sec.hv(x, y)
    eb.record()
    torch.cuda.synchronize()
    t_hv32 = ea.elapsed_time(eb) / nrep * 1e-3
    x64, y64 = x.double(), y.double()
    del x, y
    for _ in range(2):
        sec.hv(x64, y64)
    ea.record()
    for _ in range(5):
        sec.hv(x64, y64)
    eb.record()
    torch.cuda.synchronize()
    t_hv64 = ea.elapsed_time(eb) / 5 * 1e-3
    del x64, y64
    torch.cuda.empty_cache()
    hv_alone = {"fp32_ms": t_hv32 * 1e3, "fp32_alg_GBps": 2 * sec.dim * 4 / t_hv32 / 1e9,
                "fp32_frac": 2 * sec.dim * 4 / t_hv32 / 1e9 / hbm,
                "fp64_ms": t_hv64 * 1e3, "fp64_alg_GBps": 2 * sec.dim * 8 / t_hv64 / 1e9,
                "hv_per_s_fp32": 1.0 / t_hv32}

    # plain FP64 GPU Lanczos, the comparison the metric asks for (once)
    fp64 = None
    if not args.no_fp64:
        torch.cuda.empty_cache()
        try:
            # this single FP64 solve allocates its 266 GB basis inside the timed region, which the
            # repeated mixed solves do not (their cache persists); that one-time allocation is
            # timed on its own and reported beside the speed-up
            torch.cuda.synchronize()
            ta = time.perf_counter()
            held = torch.empty(((args.lanczos_steps + 1) * sec.n,), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            t_alloc = time.perf_counter() - ta
            del held
            torch.cuda.empty_cache()
            barrier()
            clock = StreamClock().start()
            g64 = LZ.ground_state(sec, mode="f64", steps=args.lanczos_steps, seed=0)
            t64 = max_over_ranks(clock.stop())
            barrier()
            fp64 = {"seconds": t64, "e0": g64.e0, "steps": g64.steps,
                    "abs_dE0_mixed_vs_fp64": abs(e0_mixed - g64.e0),
                    "speedup_mixed_vs_fp64": t64 / (elapsed / args.steps),
                    "basis_alloc_seconds": t_alloc,
                    "speedup_excluding_alloc": (t64 - t_alloc) / (elapsed / args.steps)}
            del g64
        except Exception as ex:  # noqa: BLE001
            fp64 = {"error": f"{type(ex).__name__}: {ex}"[:300]}
        torch.cuda.empty_cache()

    # end to end through the public API: host t/U in, E0 and psi0 out
    e2e = None
    if not args.no_e2e:
        from pyhub_gb300.solver import FermiHubbard
        barrier()
        t2 = time.perf_counter()
        fh = FermiHubbard(norb, nup, ndn, t, float(args.U))
        fh.kernel(max_lcz=args.lanczos_steps + 5, acc_lcz=0.0, compute_rq=False, dtype="mixed", reorth="full")
        e_api = float(fh.e0)
        psi = fh.psi0
        barrier()
        te2e = max_over_ranks(time.perf_counter() - t2)
        h2d = t.nbytes + U.nbytes
        nu_, nd_ = sec.nnz()
        h2d += (sec.nsup + 1 + sec.nsdn + 1) * 4 + (nu_ + (nd_ if nup != ndn else 0)) * (4 + 4 + 8) \
            + (sec.nsup + sec.nsdn) * (4 + 8) + 4 * 33 * 256 * 4
        e2e = {"value": ws / te2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(psi.nbytes + 8), "seconds": te2e, "e0": e_api,
               "path": "FermiHubbard(16,8,8,t,8).kernel(max_lcz=205, acc_lcz=0, dtype='mixed') + e0 + psi0 to host"}
        del fh, psi
        torch.cuda.empty_cache()

    # the metric's third part: batched Green's functions, sharded by cluster over the ranks
    batched = None
    if not args.no_c4 and not args.small:
        torch.cuda.empty_cache()
        batched = c4_batched(args, ws, rank, local)
        torch.cuda.empty_cache()

    cpu = None
    if not args.no_cpu and rank == 0 and ws == 1 and not args.small:   # the CPU sample: rank 0 at N=1 only
        hv_cpu, spent, desc, nth = cpu_sample(CPU_PAIRS_OURS, 16, args.U)
        n_hv = sum(r[1] + r[2] for r in res) / len(res)
        cpu = {"value": 1.0 / (hv_cpu * n_hv), "unit": UNIT, "cores": nth, "kind": "port",
               "sample": f"{desc} ({spent:.1f} s); extrapolated to the {n_hv:.0f} H*v of one solve",
               "hv_seconds": hv_cpu}

    oracle_check = None
    if psi_host is not None and not args.no_cpu:
        oracle_check = e0_oracle_check(t, U, psi_host, e0_mixed)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 vectors / f64 scalars + f64 refinement",
                "data": "synthetic (seeded uniform[-0.5,0.5) start vector)",
                "config": c2_config(args, sec.dim, ws),
                "e0": e0_mixed, "e0_fp32_phase": res[-1][3], "refine_steps": res[-1][2],
                "fp64_plain": fp64, "e0_oracle_check": oracle_check, "roofline": roofline,
                "hv_roofline_in_solve": hv_roof,
                "hv_alone": hv_alone, "batched_gf": batched, "kernels": ksum, "e2e": e2e, "cpu_baseline": cpu,
                "clocks": clk,
                "gpu_launches": timer.launches()}
        print(json.dumps(line), flush=True)
    RP.finish()


if __name__ == "__main__":
    main()
