"""Batched Lanczos / continued-fraction Green's functions.

Tolerances: batched FP64 alpha/beta vs the per-instance three-term Lanczos
1e-9 relative over 30 steps; batched continued fraction vs the oracle's FP64
full-reorthogonalisation Lanczos of the same length (25 steps) 1e-8; G_ii(w)
(eta = 0.1) of a 6-site open cluster after 200 steps vs the exact Lehmann sum
1e-4 (convergence of the fraction); CUDA-graph replay bit-identical to the
eager run; FP32 vectors after 200 steps within 1e-3 of the Lehmann sum."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _setup(edlib, norb=6, nup=3, ndn=3, nsteps=30, dtype="f64"):
    import torch
    from pyhub_gb300.core import greens_batched as GB
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.tools import lattices as LT
    t = LT.square(3, 2, -1.0, periodic=False, tp=0.2)
    U = np.full(norb, 3.0)
    src = edlib.Sector(norb, nup, ndn, edlib.ED_HUBBARD, t=t, U=U)
    gs = LZ.ground_state(src, mode="f64", steps=120, rule=LZ.ResidualRule(1e-12, 10))
    secs, inst = [], {}
    cache = {}
    for spin in ("up", "down"):
        for part in ("greater", "lesser"):
            d = 1 if part == "greater" else -1
            key = (nup + d, ndn) if spin == "up" else (nup, ndn + d)
            if key not in cache:
                cache[key] = edlib.Sector(norb, key[0], key[1], edlib.ED_HUBBARD, t=t, U=U)
            for site in range(1, norb + 1):
                inst[(spin, part, site)] = len(secs)
                secs.append(cache[key])
    td = torch.float64 if dtype == "f64" else torch.float32
    bl = GB.BatchedLanczos(secs, nsteps, dtype=td)
    GB.build_start_vectors(secs, src, gs.psi, bl, inst)
    return t, U, src, gs, secs, inst, bl


def test_batched_matches_per_instance(edlib):
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, bl = _setup(edlib)
    bl.run()
    torch.cuda.synchronize()
    A, B = bl.alpha.cpu().numpy(), bl.beta.cpu().numpy()
    for key in [("up", "greater", 1), ("down", "lesser", 4), ("up", "lesser", 6)]:
        i = inst[key]
        phi = bl.start(i).clone()
        a, b = GB.plain_coefficients(secs[i], phi, bl.nsteps)
        n = np.count_nonzero(b[1:] > 1e-8)
        assert np.allclose(A[i, :n], a[:n], rtol=1e-9, atol=1e-9), key
        assert np.allclose(B[i, :n + 1], b[:n + 1], rtol=1e-9, atol=1e-9), key


def test_batched_graph_replay_is_identical(edlib):
    import torch
    t, U, src, gs, secs, inst, bl = _setup(edlib, nsteps=40)
    bl.run()
    torch.cuda.synchronize()
    a0, b0 = bl.alpha.clone(), bl.beta.clone()
    bl.capture()
    bl.alpha.zero_()
    bl.beta.zero_()
    bl.replay()
    torch.cuda.synchronize()
    assert torch.equal(bl.alpha, a0) and torch.equal(bl.beta, b0)


def test_batched_cf_matches_oracle_lanczos(edlib):
    """25 steps (before any loss of orthogonality): the batched continued
    fraction equals the oracle's FP64 full-reorthogonalisation Lanczos
    continued fraction of the same start vector, to 1e-8."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, bl = _setup(edlib, nsteps=25)
    bl.run()
    w = np.linspace(-8, 8, 201)
    z = torch.tensor(w + gs.e0 + 0.1j, device="cuda")
    g = GB.continued_fraction(bl.alpha, bl.beta, z).cpu().numpy()
    for key in [("up", "greater", 2), ("down", "greater", 5)]:
        i = inst[key]
        osec = O.Sector(6, secs[i].nup, secs[i].ndn)
        phi = secs[i].to_ref(bl.start(i)).cpu().numpy()
        a, b, n2 = O.lanczos_tridiag(lambda v: O.hprod_hubbard(osec, t, U, v, fast=True), phi, 25)
        ref = O.continued_fraction(a, b, n2, w + gs.e0 + 0.1j)
        assert np.abs(g[i] - ref).max() < 1e-8 * max(1.0, np.abs(ref).max()), key


def test_batched_gf_converges_to_lehmann(edlib):
    """200 steps: G_ii(w) at eta = 0.1 within 1e-4 of the exact Lehmann sum."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, bl = _setup(edlib, nsteps=200)
    bl.run()
    w = torch.linspace(-8, 8, 401, dtype=torch.float64, device="cuda")
    eta = 0.1
    gr = GB.continued_fraction(bl.alpha, bl.beta, w + gs.e0 + 1j * eta, sign=1.0)
    le = GB.continued_fraction(bl.alpha, bl.beta, w - gs.e0 + 1j * eta, sign=-1.0)
    osec = O.Sector(6, 3, 3)
    psi = src.to_ref(gs.psi).cpu().numpy()
    ref = O.lehmann_gf_diag(osec, t, U, psi, gs.e0, 6)
    wn = w.cpu().numpy()
    for spin in ("up", "down"):
        for site in range(1, 7):
            got = (gr[inst[(spin, "greater", site)]] + le[inst[(spin, "lesser", site)]]).cpu().numpy()
            exact = 0
            for part in ("greater", "lesser"):
                pos, Q = ref[spin][part]
                exact = exact + O.poles_eval(pos, Q[site - 1] ** 2, wn, eta)
            assert np.abs(got - exact).max() < 1e-4, (spin, site, np.abs(got - exact).max())


def test_batched_fp32_converges_to_lehmann(edlib):
    """FP32 vectors (FP64 scalars), 200 steps: G_ii(w) at eta = 0.1 within 1e-3
    of the exact Lehmann sum."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, bl = _setup(edlib, nsteps=200, dtype="f32")
    bl.run()
    w = torch.linspace(-8, 8, 401, dtype=torch.float64, device="cuda")
    eta = 0.1
    gr = GB.continued_fraction(bl.alpha, bl.beta, w + gs.e0 + 1j * eta, sign=1.0)
    le = GB.continued_fraction(bl.alpha, bl.beta, w - gs.e0 + 1j * eta, sign=-1.0)
    osec = O.Sector(6, 3, 3)
    ref = O.lehmann_gf_diag(osec, t, U, src.to_ref(gs.psi).cpu().numpy(), gs.e0, 6)
    wn = w.cpu().numpy()
    worst = 0.0
    for spin in ("up", "down"):
        for site in range(1, 7):
            got = (gr[inst[(spin, "greater", site)]] + le[inst[(spin, "lesser", site)]]).cpu().numpy()
            exact = 0
            for part in ("greater", "lesser"):
                pos, Q = ref[spin][part]
                exact = exact + O.poles_eval(pos, Q[site - 1] ** 2, wn, eta)
            worst = max(worst, np.abs(got - exact).max())
    assert worst < 1e-3, worst


def test_batched_ground_states_match_dense(edlib):
    """Batched two-pass ground states (ed_batch_lanczos, then the replay
    ed_batch_ritz that accumulates the Ritz vectors) of sectors of different
    sizes with non-uniform U and on-site energies, one of them smaller than
    the step count (exhausted Krylov space): E0 within 1e-10 of the oracle's
    dense diagonalisation, |<psi|psi_dense>| >= 1 - 1e-9."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    from pyhub_gb300.tools import lattices as LT
    cases = [(6, 3, 3, 1), (7, 3, 4, 2), (8, 4, 3, 3), (6, 2, 3, 4), (4, 1, 1, 5)]
    secs, refs = [], []
    for n, nu, nd, seed in cases:
        t, U, _ = LT.random_bond_cluster(n, 3 if n > 4 else 1, seed)
        secs.append(edlib.Sector(n, nu, nd, edlib.ED_HUBBARD, t=t, U=U))
        osec = O.Sector(n, nu, nd)
        H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, U, v), osec.dim)
        val, vec = np.linalg.eigh(H)
        assert val[1] - val[0] > 1e-6     # non-degenerate: the vector is defined
        refs.append((val[0], vec[:, 0]))
    gs = GB.batched_ground_states(secs, nsteps=60, tol=1e-11)
    torch.cuda.synchronize()
    for i, (e, v) in enumerate(refs):
        assert abs(gs.e0[i] - e) < 1e-10, (cases[i], gs.e0[i] - e)
        psi = secs[i].to_ref(gs.psi[i]).cpu().numpy()
        assert abs(float(np.dot(psi, v))) >= 1 - 1e-9, cases[i]


def test_rows_per_cta_variants_agree(edlib):
    """The three H*v work splits (4, 8, 16 rows of an instance per CTA) give
    the same alpha/beta as the per-instance three-term Lanczos (FP64, 1e-9:
    the splits group the CTA partial sums differently, and the recurrence
    amplifies the rounding difference over 30 steps), and the autotuner
    picks one of them."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, bl = _setup(edlib, nsteps=30)
    ref = None
    for rows in (4, 8, 16):
        b = GB.BatchedLanczos(secs, 30, dtype=torch.float64, rows=rows)
        assert b.rows == rows
        b.x0.copy_(bl.x0)
        b.run()
        torch.cuda.synchronize()
        A, B = b.alpha.cpu().numpy(), b.beta.cpu().numpy()
        for key in [("up", "greater", 1), ("down", "lesser", 4), ("up", "lesser", 6)]:
            i = inst[key]
            if ref is None or key not in ref:
                ref = ref or {}
                ref[key] = GB.plain_coefficients(secs[i], bl.start(i).clone(), 30)
            a, bb = ref[key]
            n = np.count_nonzero(bb[1:] > 1e-8)
            assert np.allclose(A[i, :n], a[:n], rtol=1e-9, atol=1e-9), (rows, key)
            assert np.allclose(B[i, :n + 1], bb[:n + 1], rtol=1e-9, atol=1e-9), (rows, key)
    assert GB.autotune(secs, torch.float32) in (4, 8, 16)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_kept_basis_matches_replay(edlib, dtype):
    """The batched Lanczos with every Krylov vector kept runs the same
    recurrence as the two-vector form (alpha/beta bit for bit), and the Ritz
    vectors summed over the kept vectors equal the replay's (1e-13 FP64,
    1e-6 FP32, relative)."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    dt = getattr(torch, dtype)
    t, U, src, gs, secs, inst, bl = _setup(edlib, nsteps=30)
    outs, ab = [], []
    for keep in (False, True):
        b = GB.BatchedLanczos(secs, 30, dtype=dt, keep=keep)
        b.x0.copy_(bl.x0.to(dt))
        out = torch.zeros_like(b.x0)
        GB._ritz_cycle(b, out)
        torch.cuda.synchronize()
        outs.append(out)
        ab.append((b.alpha.cpu().numpy(), b.beta.cpu().numpy()))
    assert np.array_equal(ab[0][0], ab[1][0]) and np.array_equal(ab[0][1], ab[1][1])
    tol = 1e-13 if dtype == "float64" else 1e-6
    assert float(torch.linalg.vector_norm((outs[0] - outs[1]).double())) <= tol * float(
        torch.linalg.vector_norm(outs[0].double()))


def test_cf_eval_shift_and_sign(edlib):
    """ed_cf_eval against a numpy continued fraction (complex128, bottom-up),
    per-instance shift and sign, at 1e-12 relative."""
    import torch
    from pyhub_gb300 import _capi
    rng = np.random.default_rng(3)
    n, m = 7, 40
    alpha = rng.uniform(-4, 4, (n, m))
    beta = np.abs(rng.normal(1.0, 0.5, (n, m + 1)))
    beta[3, 17:] = 0.0       # an exhausted Krylov space: the fraction ends there
    z = np.linspace(-9, 9, 301) + 0.05j
    shift = rng.uniform(-5, 5, n)
    sign = np.where(rng.random(n) < 0.5, 1.0, -1.0)
    dev = "cuda"
    got = _capi.cf_eval(torch.tensor(alpha, device=dev), torch.tensor(beta, device=dev),
                        torch.tensor(z, device=dev), shift=torch.tensor(shift, device=dev),
                        sign=torch.tensor(sign, device=dev)).cpu().numpy()
    for i in range(n):
        zz = z + shift[i]
        g = np.zeros_like(zz)
        for k in range(m - 1, -1, -1):
            tail = beta[i, k + 1] ** 2 * g if k < m - 1 else 0.0
            g = 1.0 / (zz - sign[i] * alpha[i, k] - tail)
        ref = beta[i, 0] ** 2 * g
        assert np.abs(got[i] - ref).max() <= 1e-12 * np.abs(ref).max(), i


@pytest.mark.parametrize("rows", [4, 8, 16])
def test_batch_hv_matches_oracle(edlib, rows):
    """ed_batch_hv over sectors of several shapes (N_up != N_down, per-site U,
    t' bonds): each instance's product equals the oracle's HPROD to 1e-14
    (FP64, norm), and bit for bit for integer t, U and x (FP64 and FP32);
    the row padding of y stays zero."""
    import torch
    from pyhub_gb300 import _capi
    rng = np.random.default_rng(rows)
    specs = [(6, 3, 3), (7, 3, 2), (8, 4, 4), (6, 2, 3)]
    for integer in (False, True):
        secs, osecs, pars = [], [], []
        for norb, nu, nd in specs:
            if integer:
                t = rng.integers(-2, 3, (norb, norb)).astype(np.float64)
                U = rng.integers(0, 6, norb).astype(np.float64)
            else:
                t = rng.standard_normal((norb, norb))
                U = rng.uniform(0, 6, norb)
            t = np.triu(t) + np.triu(t, 1).T
            secs.append(edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U))
            osecs.append(O.Sector(norb, nu, nd))
            pars.append((t, U))
        b = _capi.Batch(secs, rows=rows)
        sc = torch.empty(b.scratch_bytes() // 8 + 1, dtype=torch.float64, device="cuda")
        xs = [rng.integers(-3, 4, o.dim).astype(np.float64) if integer else rng.standard_normal(o.dim) for o in osecs]
        for dt in ((torch.float64, torch.float32) if integer else (torch.float64,)):
            x = torch.zeros(b.total, dtype=dt, device="cuda")
            for i, s in enumerate(secs):
                b.view(x, i).copy_(s.from_ref(torch.tensor(xs[i], dtype=dt, device="cuda")))
            y = torch.full_like(x, float("nan"))
            b.hv(x, y, sc)
            torch.cuda.synchronize()
            for i, s in enumerate(secs):
                yi = b.view(y, i)
                pad = yi.view(s.nsdn, s.ld)[:, s.nsup:]
                assert torch.count_nonzero(pad) == 0
                got = s.to_ref(yi).double().cpu().numpy()
                ref = O.hprod_hubbard(osecs[i], pars[i][0], pars[i][1], xs[i])
                if integer:
                    assert np.array_equal(got, ref), (i, dt)
                else:
                    assert np.linalg.norm(got - ref) <= 1e-14 * np.linalg.norm(ref), i


@pytest.mark.parametrize("dtype,keep,rows", [("f64", False, 8), ("f32", False, 8), ("f32", True, 4),
                                              ("f64", True, 16), ("f32", False, 16)])
def test_persistent_run_is_bit_identical(edlib, dtype, keep, rows):
    """The one-launch persistent run gives the four-launch run's alpha/beta
    bit for bit (same partials, same summation order), keeps the same Krylov
    vectors, reports status 0, and replays identically from a CUDA graph."""
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, _ = _setup(edlib, nsteps=25, dtype=dtype)
    td = torch.float64 if dtype == "f64" else torch.float32
    ref = GB.BatchedLanczos(secs, 25, dtype=td, rows=rows, keep=keep)
    per = GB.BatchedLanczos(secs, 25, dtype=td, rows=rows, keep=keep, persistent=True)
    x0 = torch.rand(ref.batch.total, dtype=td, device="cuda")
    for i, s in enumerate(secs):      # zero row padding, as every engine vector has
        ref.batch.view(x0, i).view(s.nsdn, -1)[:, s.nsup:] = 0
    ref.x0.copy_(x0)
    per.x0.copy_(x0)
    ref.run()
    per.run()
    torch.cuda.synchronize()
    assert per.batch.persistent_status(per.scratch) == 0
    assert torch.equal(ref.alpha, per.alpha) and torch.equal(ref.beta, per.beta)
    if keep:
        assert torch.equal(ref.basis, per.basis)
    a0, b0 = per.alpha.clone(), per.beta.clone()
    per.alpha.zero_()
    per.beta.zero_()
    per.capture()
    per.replay()
    torch.cuda.synchronize()
    assert per.batch.persistent_status(per.scratch) == 0
    assert torch.equal(per.alpha, a0) and torch.equal(per.beta, b0)


def test_persistent_wait_limit_sets_status(edlib):
    """An instance whose first H*v phase never completes: the CTAs waiting on
    it give up after the wait limit, the run stops with status 1 well within
    the call, and the next run on the same context completes with the
    four-launch alpha/beta."""
    import time

    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U, src, gs, secs, inst, _ = _setup(edlib, nsteps=25, dtype="f32")
    ref = GB.BatchedLanczos(secs, 25, dtype=torch.float32, rows=8)
    per = GB.BatchedLanczos(secs, 25, dtype=torch.float32, rows=8, persistent=True)
    x0 = torch.rand(ref.batch.total, dtype=torch.float32, device="cuda")
    for i, s in enumerate(secs):
        ref.batch.view(x0, i).view(s.nsdn, -1)[:, s.nsup:] = 0
    ref.x0.copy_(x0)
    per.x0.copy_(x0)
    ref.run()
    torch.cuda.synchronize()
    per.batch.persistent_watchdog(0.25, stall_instance=len(secs) // 2)
    t0 = time.perf_counter()
    per.run()
    torch.cuda.synchronize()
    took = time.perf_counter() - t0
    assert per.batch.persistent_status(per.scratch) == 1
    assert took < 5.0
    per.batch.persistent_watchdog(10.0, -1)
    per.run()
    torch.cuda.synchronize()
    assert per.batch.persistent_status(per.scratch) == 0
    assert torch.equal(ref.alpha, per.alpha) and torch.equal(ref.beta, per.beta)
    with pytest.raises(RuntimeError):
        per.batch.persistent_watchdog(0.0)
    with pytest.raises(RuntimeError):
        per.batch.persistent_watchdog(1.0, stall_instance=len(secs))


def test_persistent_run_full_size_clusters(edlib):
    """Two C4 clusters' particle/hole instances (sectors of 392,040 to
    853,776 elements, mixed shapes): persistent and four-launch runs agree
    bit for bit over 40 FP32 steps."""
    import torch
    from pyhub_gb300 import _capi
    from pyhub_gb300.core import greens_batched as GB
    secs = []
    for spec in GB.c4_clusters(2, seed=3):
        N = spec["N"]
        for key in [(N + 1, N), (N - 1, N), (N, N + 1), (N, N - 1)]:
            s = _capi.Sector(12, key[0], key[1], _capi.ED_HUBBARD, t=spec["t"], U=np.full(12, spec["U"]))
            secs += [s] * 3
    ref = GB.BatchedLanczos(secs, 40, dtype=torch.float32, rows=8)
    per = GB.BatchedLanczos(secs, 40, dtype=torch.float32, rows=8, persistent=True)
    x0 = torch.rand(ref.batch.total, dtype=torch.float32, device="cuda")
    for i, s in enumerate(secs):
        ref.batch.view(x0, i).view(s.nsdn, -1)[:, s.nsup:] = 0
    ref.x0.copy_(x0)
    per.x0.copy_(x0)
    ref.run()
    per.run()
    torch.cuda.synchronize()
    assert per.batch.persistent_status(per.scratch) == 0
    assert torch.equal(ref.alpha, per.alpha) and torch.equal(ref.beta, per.beta)
