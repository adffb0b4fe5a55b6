"""Generate golden vectors from the reference's own Python modules.

Run where the reference is checked out: its path is the first argument, or
the environment variable PYHUB_REFERENCE.  Only
pyhub/tools/pole.py and pyhub/solver/bethe_anzatz.py are imported, by file
path: the package __init__ needs h5py and the Fortran executables, which are
not available.  Output: pole_golden.npz beside this script.
"""
import importlib.util
import os
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYHUB_REFERENCE", "")
HERE = os.path.dirname(os.path.abspath(__file__))


def load(rel, name):
    spec = importlib.util.spec_from_file_location(name, os.path.join(REF, rel))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    if not REF or not os.path.isfile(os.path.join(REF, "pyhub", "tools", "pole.py")):
        sys.exit("usage: make_golden.py <reference checkout> (or set PYHUB_REFERENCE)")
    pole = load("pyhub/tools/pole.py", "ref_pole")
    ba = load("pyhub/solver/bethe_anzatz.py", "ref_bethe")
    rng = np.random.default_rng(2024)
    out = {}
    for case in range(4):
        n = [7, 20, 64, 150][case]
        pos = rng.uniform(-6, 6, n)
        if case == 2:
            pos[10:20] = pos[0] + rng.uniform(-2e-6, 2e-6, 10)   # near-degenerate poles for clean()
        wts = rng.uniform(0, 1, n) * (rng.uniform(0, 1, n) > 0.1)
        if case == 3:
            wts[::7] = 1e-9                                        # below the clean() weight cut
        w = np.linspace(-8, 8, 257)
        eta = [0.05, 0.1, 0.01, 0.05][case]
        P = pole.Pole({"positions": pos, "weights": wts})
        out[f"pos{case}"] = pos
        out[f"wts{case}"] = wts
        out[f"w{case}"] = w
        out[f"eta{case}"] = np.array(eta)
        out[f"ret{case}"] = P.retarded(w, eta=eta)
        out[f"adv{case}"] = P.advanced(w, eta=eta)
        out[f"spec{case}"] = P.spectral_density(w, eta=eta)
        out[f"ret_scalar{case}"] = np.array(P.retarded(0.37, eta=eta))
        Q = pole.Pole({"positions": pos, "weights": wts}).clean(wtol=1.e-8)
        out[f"clean_pos{case}"] = Q.pole["positions"]
        out[f"clean_wts{case}"] = Q.pole["weights"]
        S = pole.Pole.sum([P, P.shift(0.5) * 2.0, P / 3.0])
        out[f"sum_pos{case}"] = S.pole["positions"]
        out[f"sum_wts{case}"] = S.pole["weights"]
    out["e_bessel_U4"] = np.array(ba.E_bessel(4.0))
    np.savez(os.path.join(HERE, "pole_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "pole_golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
