"""KI heating/cooling balance n*Lambda(T)/Gamma = 1 against the reference's
equilibrium curve KIcool/KIcoolbr.dat (KIcool/nibun.f90, cmetal = 1).

The curve is re-derived with the same bisection but with exp evaluated by
detmath.h (the deterministic exp the CPU restatement and the GPU share),
which pins the Lambda/Gamma formula and the exp implementation at once."""
import os

import numpy as np

from oracle.pyoracle import lib  # noqa: F401  (builds the oracle, exercising detmath)


def _detmath_exp():
    import ctypes
    import subprocess
    import tempfile
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(os.path.dirname(here), "code_tohoku_gb300", "csrc", "detmath.h")
    d = tempfile.mkdtemp()
    c = os.path.join(d, "dm.cpp")
    with open(c, "w") as f:
        f.write('#include "%s"\nextern "C" double dm_exp(double x){return detmath::exp(x);}\n'
                'extern "C" double dm_log10(double x){return detmath::log10(x);}\n'
                'extern "C" double dm_exp10(double x){return detmath::exp10(x);}\n' % src)
    so = os.path.join(d, "dm.so")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", c, "-o", so], check=True)
    L = ctypes.CDLL(so)
    for n in ("dm_exp", "dm_log10", "dm_exp10"):
        getattr(L, n).restype = ctypes.c_double
        getattr(L, n).argtypes = [ctypes.c_double]
    return L


def test_equilibrium_curve(golden_dir):
    g = np.load(os.path.join(golden_dir, "ki_equilibrium.npz"))
    L = _detmath_exp()
    ex = L.dm_exp
    pos = 1e-10
    for n, pref in zip(g["n"], g["p"]):
        p1, p2 = 1.0, 1e7
        for _ in range(50):
            pmid = (p1 + p2) * 0.5
            def kai(pp):
                T = pp / (n + pos)
                return 1 - (1.0e7 * ex(-118400.0 / (T + 1000.0)) + 1.4e-2 * np.sqrt(T) * ex(-92.0 / T)) * n
            if abs(p1 - p2) < 1e-6:
                break
            k1, k2, k3 = kai(p1), kai(p2), kai(pmid)
            if k1 * k3 < 0:
                p2 = pmid
            elif k2 * k3 < 0:
                p1 = pmid
        assert abs(pmid - pref) <= 2e-6 + 1e-12 * pref, (n, pmid, pref)


def test_detmath_accuracy():
    L = _detmath_exp()
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-700, 700, 4000), rng.uniform(-1, 1, 4000), [0.0, 1e-300, -1e-300]])
    for x in xs:
        a, b = L.dm_exp(x), np.exp(x)
        if b == 0 or not np.isfinite(b):
            continue
        assert abs(a - b) <= 2 * np.spacing(b), (x, a, b)
    ys = np.exp(rng.uniform(-700, 700, 4000))
    for y in ys:
        a, b = L.dm_log10(y), np.log10(y)
        assert abs(a - b) <= 2 * np.spacing(abs(b)) + 1e-300, (y, a, b)
    for y in rng.uniform(-30, 30, 4000):
        a, b = L.dm_exp10(y), 10.0 ** y
        assert abs(a - b) <= 3 * np.spacing(b), (y, a, b)
