"""CPU tests of host-side logic of the engine that needs no GPU: the choice
of Ritz pairs for the batched ground states and the padding of kept Krylov
rows."""
import numpy as np


def test_lowest_ritz_takes_the_best_prefix():
    """greens_batched._lowest_ritz compares the leading blocks of a
    tridiagonal matrix and keeps the lowest Ritz pair with the smallest
    residual estimate beta_m |y_m|; a vanishing beta cuts the matrix."""
    import scipy.linalg as sla
    from pyhub_gb300.core import greens_batched as GB
    rng = np.random.default_rng(7)
    a = rng.uniform(-2, 2, 60)
    b = np.concatenate([[1.0], rng.uniform(0.1, 1.0, 60)])
    theta, y, est, m = GB._lowest_ritz(a, b, every=10)
    cands = []
    for mm in list(range(10, 60, 10)) + [60]:
        w, v = sla.eigh_tridiagonal(a[:mm], b[1:mm], select="i", select_range=(0, 0))
        cands.append((float(b[mm] * abs(v[mm - 1, 0])), mm, float(w[0])))
    e_best, m_best, w_best = min(cands)
    assert m == m_best and abs(est - e_best) < 1e-15 and abs(theta - w_best) < 1e-12
    assert abs(np.linalg.norm(y) - 1.0) < 1e-12 and len(y) == m
    b2 = b.copy()
    b2[25] = 0.0                       # Krylov space exhausted after 25 steps
    theta2, y2, est2, m2 = GB._lowest_ritz(a, b2, every=10)
    assert m2 <= 25


def test_zero_padding_of_kept_rows():
    """lanczos._zero_padding clears exactly the padding of each kept row: the
    columns past nsup of every down-string row (Hubbard layout) or the tail
    past dim (Heisenberg), and leaves every element of the vector alone."""
    import torch
    from types import SimpleNamespace
    from pyhub_gb300 import _capi
    from pyhub_gb300.core import lanczos as LZ
    hub = SimpleNamespace(kind=_capi.ED_HUBBARD, nsup=5, nsdn=3, ld=8, n=24, dim=15)
    rows = torch.full((4, hub.n), 7.0)
    LZ._zero_padding(hub, rows)
    v = rows.view(4, hub.nsdn, hub.ld)
    assert bool((v[:, :, hub.nsup:] == 0).all()) and bool((v[:, :, :hub.nsup] == 7).all())
    heis = SimpleNamespace(kind=_capi.ED_HEISENBERG, nsup=70, nsdn=1, ld=70, n=96, dim=70)
    rows = torch.full((3, heis.n), 7.0)
    LZ._zero_padding(heis, rows)
    assert bool((rows[:, heis.dim:] == 0).all()) and bool((rows[:, :heis.dim] == 7).all())
    flat = SimpleNamespace(kind=_capi.ED_HEISENBERG, nsup=64, nsdn=1, ld=64, n=64, dim=64)
    rows = torch.full((2, 64), 7.0)
    LZ._zero_padding(flat, rows)
    assert bool((rows == 7).all())


def test_site_groups_of_the_sweep():
    """greens_batched._site_groups: runs of one (cluster, spin, part) and the
    distance of their slots; irregular slots fall back to per-site launches."""
    from pyhub_gb300.core import greens_batched as GB
    inst = [(0, "up", "greater", s) for s in (1, 2, 3)] + [(0, "up", "lesser", 1)] + \
        [(1, "down", "greater", s) for s in (1, 2)]
    offsets = [0, 64, 128, 192, 224, 288]
    assert GB._site_groups(inst, offsets) == [(0, 3, 64), (3, 4, 0), (4, 6, 64)]
    irregular = [0, 64, 160, 192, 224, 288]
    assert GB._site_groups(inst, irregular)[0] == (0, 3, None)
