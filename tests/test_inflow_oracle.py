"""BC=4 inflow (BC_MPI :814-890, BC_MPI_OT :948-1080) in the oracle, and
its argument checks at the C ABI.  CPU only.

The reference's default run (3DMHD-CfCA/INPUT3D.DAT) drives WNM into the
box through both x faces at +-9.778 km/s from the DTF reservoir.  Mass
then enters at 2 rho_in v_in A per unit time while the flows meet in the
middle: checked (without cooling) over the first steps, before anything
reaches the boundaries.  Ghost cells on the inflow sides carry the inflow values
(species = BBRV_cm rho of the reservoir)."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from oracle.pyoracle import Oracle3D


def _run(n=16, steps=12, reservoir=None, ifthrm=2):
    st = problems.wnm_shock_tube(n, dissip=0, ifthrm=ifthrm)
    inflow, dinit = problems.shock_tube_inflow()
    o = Oracle3D(st.params)
    o.upload(st)
    o.set_inflow(inflow.vector(), reservoir, dinit)
    U0, _, _ = o.download()
    for _ in range(steps):
        o.step()
    return st, inflow, dinit, o, U0


def test_mass_enters_through_both_inflow_faces():
    # without cooling (with it, the interior WNM cools below the fixed inflow
    # pressure and the boundary cells accelerate, adding ~6 % more inflow)
    st, inflow, dinit, o, U0 = _run(ifthrm=0)
    U, sp, _ = o.download()
    c = (slice(2, -2),) * 3
    vol = st.dx[2] * st.dy[2] * st.dz[2]
    dm = (U[0][c].sum() - U0[0][c].sum()) * vol
    area = st.params.ny * st.dy[2] * st.params.nz * st.dz[2]
    expect = 2.0 * dinit * inflow.v[0][0] * area * o.time
    assert abs(dm / expect - 1.0) < 0.01, dm / expect
    # the solution stays symmetric about the collision plane
    rho = U[0][4, 4, 2:-2]
    assert np.allclose(rho, rho[::-1], rtol=1e-10)


def test_inflow_ghosts_hold_reservoir_values():
    _, inflow, dinit, o, _ = _run(steps=3)
    U, sp, _ = o.download()
    for g in (0, 1, -2, -1):   # the two ghost layers on each x side
        assert np.allclose(U[0][2:-2, 2:-2, g], dinit)
        assert np.allclose(sp[0][2:-2, 2:-2, g], inflow.species[0] * dinit)
    assert np.allclose(U[1][2:-2, 2:-2, 0], inflow.v[0][0])
    assert np.allclose(U[1][2:-2, 2:-2, -1], inflow.v[1][0])


def test_reservoir_pattern_enters_the_box():
    n = 16
    st = problems.wnm_shock_tube(n, dissip=0)
    inflow, dinit = problems.shock_tube_inflow()
    res = np.full(st.U[0].shape, dinit, dtype=np.float32)
    res[:, :, : n // 2 + 2] *= 1.5     # denser gas in the left half of the reservoir
    _, _, _, o, _ = _run(n, steps=12, reservoir=res)
    U, _, _ = o.download()
    # the left inflow ghosts read the reservoir upstream of x = 0 (its wrapped
    # right half at early times), the right ones the left half
    assert U[0][4, 4, 1] == pytest.approx(dinit)
    assert U[0][4, 4, -1] == pytest.approx(1.5 * dinit, rel=1e-6)


def test_inflow_only_on_x_sides():
    p = problems.MhdParams(16, 16, 16, bc=(3, 3, 4, 4, 3, 3))
    with pytest.raises(native.MhdError) as e:
        native.Mhd3D(p)
    assert e.value.code == 1   # MHD_ERR_ARG
