"""CPU tests of host-side logic of the engine that needs no GPU: the choice
of Ritz pairs for the batched ground states."""
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
