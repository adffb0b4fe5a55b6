"""CPU tests of the host control flow of the Lanczos drivers
(core.lanczos): for lanczos_full, rule checks with and without the one-step
lookahead, the device stop codes, truncation at a breakdown; for
lanczos_plain, the kept rows, the move to rotating vectors and the replay.  The C-ABI calls
are replaced by torch stand-ins on CPU tensors; the stand-in of
ed_lanczos_coef restates the kernel's arithmetic (csrc/ed_lanczos.cu) so the
device state follows the same protocol."""
import math

import numpy as np
import pytest
import torch


class FakeSector:
    """A dense symmetric matrix behind the sector's H*v interface."""

    def __init__(self, H):
        self.H = H
        self.n = self.dim = H.shape[0]

    def hv(self, x, y, scale=1.0, dots=None, scratch=None, ld=None, stream=None):
        y.copy_((scale * (self.H @ x.double())).to(y.dtype))
        if dots is not None:
            dots[0] = float(x.double() @ y.double())
            dots[1] = float(y.double() @ y.double())


def fake_multidot(V, nvec, w, out, scratch, z=None, n=None, stream=None):
    Vd = V[:nvec].double()
    out[:nvec] = Vd @ w.double()
    if z is not None:
        out[nvec:2 * nvec] = Vd @ z.double()


def fake_update(V, nvec, coef, w, out, norm2=None, scratch=None, n=None, stream=None, wscale=None):
    ws = float(wscale[0]) if wscale is not None else 1.0
    r = ws * w.double() if w is not None else torch.zeros(out.numel(), dtype=torch.float64)
    if nvec > 0:
        r = r - coef[:nvec].double() @ V[:nvec].double()
    out.copy_(r.to(out.dtype))
    if norm2 is not None:
        norm2[0] = float((out.double() ** 2).sum())


def fake_coef(k, mmax, dots, nrm, state, coef, alpha, beta, stream=None):
    """ed_lanczos_coef's arithmetic on CPU tensors (same state layout)."""
    s = state[2:3 + mmax]
    ldl = mmax + 1
    off = 3 + mmax
    Linv = state[off: off + ldl * ldl].view(ldl, ldl)
    if k >= 1 and state[0] == 0:
        nb = float(nrm[0])
        bk = math.sqrt(max(nb, 0.0))
        if not math.isfinite(nb):
            state[0], s[k] = -k, 0.0
        else:
            beta[k - 1] = bk
            if bk <= 1e-13 * max(1.0, abs(float(alpha[k - 1]))):
                state[0], s[k] = k, 0.0
            else:
                s[k] = 1.0 / bk
    if dots is None:
        return
    if state[0] != 0:
        coef[:k + 1] = 0.0
        return
    sv = s[:k + 1].clone()
    sk = float(s[k])
    g = sv * sk * dots[k + 1:2 * k + 2]
    c = sv * sk * dots[:k + 1]
    l = Linv[:k, :k] @ g[:k]
    ll = float(l @ l)
    if k >= 1 and not (float(g[k]) - ll >= 0.5 * float(g[k])):
        coef[:k + 1] = 0.0
        state[0] = k
        return
    lam = math.sqrt(max(float(g[k]) - ll, 1e-300))
    Linv[k, :k] = -(l @ Linv[:k, :k]) / lam
    Linv[k, k] = 1.0 / lam
    off_g = max(float(g[:k].abs().max()) if k else 0.0, abs(float(g[k]) - 1.0))
    state[1] = max(float(state[1]), off_g)
    z = Linv[:k + 1, :k + 1] @ c
    y = Linv[:k + 1, :k + 1].T @ z
    coef[:k + 1] = y * sv
    alpha[k] = c[k]


@pytest.fixture
def stand_ins(edlib, monkeypatch):
    from pyhub_gb300 import _capi
    monkeypatch.setattr(_capi, "multidot", fake_multidot)
    monkeypatch.setattr(_capi, "update", fake_update)
    monkeypatch.setattr(_capi, "lanczos_coef", fake_coef)
    from pyhub_gb300.core import lanczos as LZ
    return LZ


def _matrix(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    return torch.tensor(0.5 * (a + a.T))


def test_full_lanczos_control_flow_ground_state(stand_ins):
    LZ = stand_ins
    H = _matrix(80, 1)
    sec = FakeSector(H)
    v0 = torch.tensor(np.random.default_rng(2).uniform(-0.5, 0.5, 80))
    r = LZ.lanczos_full(sec, v0, 60, torch.float64)
    e = np.linalg.eigvalsh(H.numpy())[0]
    assert r.steps == 60 and not r.breakdown
    assert abs(r.ritz[0] - e) < 1e-8
    res = float(torch.linalg.vector_norm(H @ r.psi - r.ritz[0] * r.psi))
    assert res < 1e-4 and abs(float(torch.linalg.vector_norm(r.psi)) - 1) < 1e-12
    assert r.gram_offdiag < 1e-12


@pytest.mark.parametrize("acc", [1e-6, 1e-12])
def test_lookahead_checks_stop_where_synchronous_checks_stop(stand_ins, acc):
    """The rule sees the same alpha/beta at the same checks with and without
    the lookahead, so both runs keep the same steps and coefficients."""
    LZ = stand_ins
    H = _matrix(120, 3)
    sec = FakeSector(H)
    v0 = torch.tensor(np.random.default_rng(4).uniform(-0.5, 0.5, 120))
    runs = [LZ.lanczos_full(sec, v0, 100, torch.float64, rule=LZ.ReferenceRule(acc), lookahead=la)
            for la in (False, True)]
    assert runs[0].steps == runs[1].steps and runs[0].steps % LZ.NADD == 0
    assert runs[0].converged == runs[1].converged
    assert np.array_equal(runs[0].alpha, runs[1].alpha) and np.array_equal(runs[0].beta, runs[1].beta)
    assert float(torch.linalg.vector_norm(runs[0].psi - runs[1].psi)) < 1e-14


def test_exhausted_krylov_space_stops_the_run(stand_ins):
    """A 12-dimensional space run for 30 steps: the stop code truncates the
    run at <= 12 steps (with and without rule checks), E0 is exact."""
    LZ = stand_ins
    H = _matrix(12, 5)
    sec = FakeSector(H)
    v0 = torch.tensor(np.random.default_rng(6).uniform(-0.5, 0.5, 12))
    e = np.linalg.eigvalsh(H.numpy())[0]
    for rule in (None, LZ.ReferenceRule(1e-14)):
        r = LZ.lanczos_full(sec, v0, 30, torch.float64, rule=rule)
        assert r.breakdown and r.converged and r.steps <= 12
        assert abs(r.ritz[0] - e) < 1e-10
        assert bool(torch.isfinite(r.psi).all())


def test_three_term_schedules_agree(stand_ins):
    """lanczos_plain with all rows kept, with 12 rows (the run moves to the
    rotating vectors, then replays on the same schedule) and with none
    (replay): the same coefficients to rounding and the same Ritz vectors."""
    LZ = stand_ins
    H = _matrix(90, 7)
    sec = FakeSector(H)
    v0 = torch.tensor(np.random.default_rng(8).uniform(-0.5, 0.5, 90))
    storage = torch.empty(41 * 90 * 8, dtype=torch.uint8)
    runs = [LZ.lanczos_plain(sec, v0, 40, nvec=2, keep=k, storage=storage) for k in (True, 12, False)]
    assert [r.times["replayed"] for r in runs] == [False, True, True]
    assert runs[0].times["kept_rows"] == 41 and runs[1].times["kept_rows"] == 12
    for r in runs[1:]:
        assert r.steps == runs[0].steps == 40
        assert np.allclose(r.alpha, runs[0].alpha, rtol=1e-12, atol=0)
        assert np.allclose(r.beta, runs[0].beta, rtol=1e-12, atol=0)
        for p, q in zip(r.psis, runs[0].psis):
            assert float(torch.linalg.vector_norm(p - q)) < 1e-10
    e = np.linalg.eigvalsh(H.numpy())[0]
    assert abs(runs[0].ritz[0] - e) < 1e-6
