"""Pole evaluation semantics against golden vectors produced by the
reference's own pyhub/tools/pole.py (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from pyhub_gb300.tools.pole import Pole

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "pole_golden.npz"))


@pytest.mark.parametrize("case", range(4))
def test_pole_evaluation_matches_reference(case):
    pos, wts, w, eta = G[f"pos{case}"], G[f"wts{case}"], G[f"w{case}"], float(G[f"eta{case}"])
    P = Pole({"positions": pos, "weights": wts})
    np.testing.assert_allclose(P.retarded(w, eta=eta), G[f"ret{case}"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(P.advanced(w, eta=eta), G[f"adv{case}"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(P.spectral_density(w, eta=eta), G[f"spec{case}"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(P.retarded(0.37, eta=eta), G[f"ret_scalar{case}"], rtol=1e-12)
    Q = Pole({"positions": pos, "weights": wts}).clean(wtol=1.e-8)
    np.testing.assert_array_equal(Q.pole["positions"], G[f"clean_pos{case}"])
    np.testing.assert_allclose(Q.pole["weights"], G[f"clean_wts{case}"], rtol=1e-13, atol=1e-15)
    S = Pole.sum([P, P.shift(0.5) * 2.0, P / 3.0])
    np.testing.assert_array_equal(S.pole["positions"], G[f"sum_pos{case}"])
    np.testing.assert_allclose(S.pole["weights"], G[f"sum_wts{case}"], rtol=1e-15)


def test_pole_key_order_rule():
    with pytest.raises(ValueError):
        Pole({"weights": [1.0], "positions": [0.0]})
