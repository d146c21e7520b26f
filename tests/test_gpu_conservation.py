"""Periodic conservation on the GPU, read through mhd_diagnostics.

The Mach-2 decaying turbulence with its uniform Bx (plasma beta 1), DISSIP
off: every stage is in conservation form and the limiter switch of MOC
agrees between each ghost and its periodic image (the energy-based T stays
below 3), so the plain FP64 form holds mass and momentum to FP64 round-off
(it is the oracle bit for bit, tests/test_oracle_conservation.py shows the
oracle does).  The chosen form differences its FP32 mass fluxes in FP64, so
mass holds to FP64 round-off too; its momentum increments are FP32 per cell
(v_new = v + (double) dv), so momentum holds to FP32 rounding of the
increments, far below the change the step makes."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems

pytestmark = pytest.mark.gpu


def _run(precision, steps=12):
    st = problems.turbulence(24, mach=2.0, kmax=4)
    assert st.params.dissip == 0 and all(b == 3 for b in st.params.bc)
    g = native.Mhd3D(st.params, precision=precision)
    g.upload(st)
    d0 = g.diagnostics()
    U, _, _ = g.download(with_bcc=False)
    c = (slice(2, -2),) * 3
    dV = float(st.dx[2] * st.dy[2] * st.dz[2])   # uniform cells
    scale = sum(float((U[0][c] * np.abs(U[q][c])).sum()) for q in (1, 2, 3)) * dV
    for _ in range(steps):
        g.step()
    d1 = g.diagnostics()
    return d0, d1, scale


@pytest.mark.parametrize("precision,mom_tol", [(native.PREC_FP64, 1e-14), (native.PREC_FP32, 1e-6)])
def test_periodic_mass_and_momentum(precision, mom_tol):
    d0, d1, scale = _run(precision)
    assert abs(d1["mass"] - d0["mass"]) <= 1e-13 * d0["mass"]
    dp = np.abs(np.array(d1["momentum"]) - np.array(d0["momentum"]))
    assert np.all(dp <= mom_tol * scale), (dp / scale).tolist()
    assert d1["divb_max"] <= 1e-11
