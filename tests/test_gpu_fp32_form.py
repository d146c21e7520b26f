"""Properties of the chosen form (FP32 reconstruction/flux, FP64 state).

The FP32 path is not bit-exact against the oracle by design; what it keeps:
the mass of a periodic box to FP64 round-off (the remap differences its
FP32 fluxes in FP64), div B of constrained transport to FP64 round-off (the
face update differences its FP32 EMFs in FP64), and the oracle's solution
to FP32-level accuracy on any grid shape, including the padded pencil
groups of the y and z sweeps when nx is not a multiple of 4."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from oracle.pyoracle import Oracle3D

pytestmark = pytest.mark.gpu


def _random_box(shape, seed=7):
    nx, ny, nz = shape
    st = problems.turbulence(1, kmax=2)   # physics values of the periodic setup
    p = st.params.replace(nx=nx, ny=ny, nz=nz)
    base = problems._empty_state(p, 1.0, 0.8, 1.2)
    rng = np.random.default_rng(seed)
    base.U[0][...] = 1.0 + 0.2 * rng.random(base.U[0].shape)
    for c in (1, 2, 3):
        base.U[c][...] = rng.normal(0, 1.0, base.U[c].shape)
    base.U[4][...] = 0.6 + 0.1 * rng.random(base.U[4].shape)
    base.U[5][...] = 0.7
    base.U[6][...] = 0.3
    base.U[7][...] = -0.2
    base.species[0][...] = 1.0
    problems._fill_ghosts_periodic(base.U)
    return base


def test_fp32_mass_conserved_and_divb():
    st = problems.turbulence(16, kmax=4)
    g = native.Mhd3D(st.params, precision=native.PREC_FP32)
    g.upload(st)
    d0 = g.diagnostics()
    for _ in range(6):
        g.step()
    d1 = g.diagnostics()
    assert abs(d1["mass"] - d0["mass"]) <= 1e-13 * d0["mass"]
    assert d1["divb_max"] <= 1e-11


# (260, 8, 8), (8, 300, 8) and (8, 8, 300): pencils longer than 256 cells
# take the sweep kernels of the 512^3 grid (a second compile-time stride).  An even
# nx stages the y sweep's inputs with TMA boxes of 132 positions (one box
# per pencil group; two for (10, 150, 6), whose second box ends beyond the
# grid); an odd nx keeps the per-thread loads.
@pytest.mark.parametrize("shape", [(12, 10, 8), (9, 7, 11), (18, 13, 6), (20, 12, 16), (10, 150, 6), (260, 8, 8),
                                   (8, 300, 8), (8, 8, 300)])
def test_fp32_close_to_oracle_on_any_grid(shape):
    st = _random_box(shape)
    g = native.Mhd3D(st.params, precision=native.PREC_FP32)
    g.upload(st)
    o = Oracle3D(st.params)
    o.upload(st)
    for _ in range(3):
        dt, _ = o.timestep()
        o.advance(dt)
        g.advance(dt)
    Ug, sg, bg = g.download()
    Uo, so, bo = o.download()
    c = (slice(2, -2),) * 3
    for f in range(5):
        a, b = Ug[f][c], Uo[f][c]
        l1 = np.abs(a - b).mean() / np.abs(b).mean()
        assert l1 < 1e-4, (f, l1)
        assert np.abs(a - b).max() < 1e-2 * np.abs(b).max(), f
    l1b = np.abs(bg[(slice(None),) + c] - bo[(slice(None),) + c]).mean() / np.abs(bo).mean()
    assert l1b < 1e-4
    # the ghost x-columns the y and z sweeps compute along are never stored:
    # nothing non-finite reaches the padded arrays
    assert np.isfinite(Ug).all() and np.isfinite(sg).all()


def _states_for_dt():
    from test_chem_oracle import chem_state, shield_state
    from test_gpu_inflow import shock_tube
    stiff = problems.colliding_flows(24)
    stiff.U[0] *= 30.0
    stiff.species *= 30.0
    cs = chem_state(12, seed=9)
    cs.params = cs.params.replace(ifthrm=2)
    ss = shield_state(12, seed=10)
    ss.params = ss.params.replace(ifthrm=2)
    tube = shock_tube(16, 8, 8)   # two uniform halves: many cells tie for the minimum
    tube.params = tube.params.replace(bc=(1, 1, 3, 3, 3, 3))
    return {"colliding_flows": problems.colliding_flows(32), "turbulence": problems.turbulence(24, kmax=4),
            "stiff_floored": stiff, "chemistry": cs, "chemistry_shield": ss, "uniform_shock_tube": tube}


@pytest.mark.parametrize("name", ["colliding_flows", "turbulence", "stiff_floored", "chemistry",
                                  "chemistry_shield", "uniform_shock_tube"])
def test_chosen_form_time_step_is_the_fp64_one(name):
    """The CFL minimum stays FP64: the chosen form's FP32 screen plus the
    FP64 recomputation of its candidates gives dt_kernel's result bit for
    bit -- on the uploaded state, and (without the chemistry, whose FP32
    network keeps nde and ndtot the upload would rebuild) after steps of
    the chosen form, compared with an FP64 handle holding that state."""
    st = _states_for_dt()[name]
    g32 = native.Mhd3D(st.params, precision=native.PREC_FP32)
    g32.upload(st)
    g64 = native.Mhd3D(st.params)
    g64.upload(st)
    assert g32.timestep() == g64.timestep()
    if getattr(st.params, "ifchem", 0) == 2:
        return
    for _ in range(3):
        g32.step()
    U, sp, _ = g32.download(with_bcc=False)
    s2 = st.copy()
    s2.U[...] = U
    s2.species[...] = sp
    g64b = native.Mhd3D(st.params)
    g64b.upload(s2)
    assert g32.timestep() == g64b.timestep()
