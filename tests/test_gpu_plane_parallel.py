"""The GPU step on the plane-parallel cases where the 3D scheme and the
golden-pinned 1D restatement do the same arithmetic (see
test_oracle_3d_vs_1d.py): the plain FP64 kernels reproduce the 1D code to
round-off after 200 steps through a shocked, cooling layer; the chosen form
stays within its FP32 rounding of it."""
import numpy as np
import pytest

from code_tohoku_gb300 import native
from oracle.pyoracle import Oracle1D
from test_oracle_3d_vs_1d import _cold_deck, _slab_from_1d

pytestmark = pytest.mark.gpu


def _run(precision, ifthrm, steps=200):
    o1 = Oracle1D(_cold_deck(2.0, 1.57734, ifthrm))
    o1.set_riemann_iterations(4)   # the 3D RIEMAN's count
    st = _slab_from_1d(o1.state())
    st.params = st.params.replace(ifthrm=ifthrm, pmin=1e-20, rmin=1e-20)
    g = native.Mhd3D(st.params, precision=precision)
    g.upload(st)
    for _ in range(steps):
        dt, _ = g.step()
        o1.step_dt(dt)
    U, sp, _ = g.download()
    s1 = o1.state()
    c = (slice(2, -2),) * 3
    out = {}
    for name, a, col in (("rho", U[0], 1), ("vx", U[1], 2), ("p", U[4], 5), ("H", sp[0], 9)):
        d = np.abs(a[c] - s1[:, col])
        out[name] = (float(d.max() / np.abs(s1[:, col]).max()), float(d.mean() / np.abs(s1[:, col]).mean()))
    return out


@pytest.mark.parametrize("ifthrm", [0, 2])
def test_fp64_gpu_equals_1d_to_round_off(ifthrm):
    errs = _run(native.PREC_FP64, ifthrm)
    assert max(e[0] for e in errs.values()) < 1e-12, errs


@pytest.mark.parametrize("ifthrm", [0, 2])
def test_chosen_form_follows_1d(ifthrm):
    errs = _run(native.PREC_FP32, ifthrm)
    assert max(e[1] for e in errs.values()) < 1e-4, errs
