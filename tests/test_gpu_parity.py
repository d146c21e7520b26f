"""The CUDA FP64 path against the oracle, bit for bit.

Both sides run the same seeded state; the GPU through the C ABI
(include/mhd_gb300.h via code_tohoku_gb300.native), the oracle through its
CPU restatement of MCF3DSGincfca3.f90 with the KI cooling splice.  The
plain form is compiled without contraction and shares detmath.h, so every
interior cell, species and magnetic-field value must agree exactly."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from parity_util import compare, pair

pytestmark = pytest.mark.gpu


def small_turbulence(n=16, **kw):
    return problems.turbulence(n, kmax=4, **kw)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_single_sweep_bit_exact(d):
    g, o = pair(small_turbulence())
    dt, _ = o.timestep()
    g.sweep(d, dt)
    o.sweep(d, dt)
    compare(g, o)


def test_ct_bit_exact():
    g, o = pair(small_turbulence())
    dt, _ = o.timestep()
    for d in (0, 1, 2):
        g.sweep(d, dt)
        o.sweep(d, dt)
    g.ct(dt)
    o.ct(dt)
    compare(g, o)


def test_timestep_bit_exact():
    st = problems.colliding_flows(16)
    g, o = pair(st)
    assert g.timestep() == o.timestep()


def test_source_bit_exact():
    st = problems.colliding_flows(16)
    g, o = pair(st)
    dt, _ = o.timestep()
    g.source(0.5 * dt)
    o.source(0.5 * dt)
    compare(g, o)


def test_turbulence_steps_bit_exact():
    g, o = pair(small_turbulence())
    for _ in range(6):   # all six sweep orders
        assert g.step() == o.step()
    compare(g, o)


def test_colliding_flows_steps_bit_exact():
    st = problems.colliding_flows(16)
    g, o = pair(st)
    for _ in range(6):
        assert g.step() == o.step()
    compare(g, o)


@pytest.mark.parametrize("shape", [(12, 10, 8), (9, 7, 11), (264, 8, 4)])
def test_non_cubic_grids_bit_exact(shape):
    nx, ny, nz = shape
    st = problems.turbulence(1, kmax=2)   # placeholder for the physics values
    p = st.params.replace(nx=nx, ny=ny, nz=nz)
    base = problems._empty_state(p, 1.0, 0.8, 1.2)
    rng = np.random.default_rng(7)
    base.U[0][...] = 1.0 + 0.2 * rng.random(base.U[0].shape)
    for c in (1, 2, 3):
        base.U[c][...] = rng.normal(0, 1.0, base.U[c].shape)
    base.U[4][...] = 0.6 + 0.1 * rng.random(base.U[4].shape)
    base.U[5][...] = 0.7
    base.U[6][...] = 0.3
    base.U[7][...] = -0.2
    base.species[0][...] = 1.0
    problems._fill_ghosts_periodic(base.U)
    g, o = pair(base)
    for _ in range(3):
        assert g.step() == o.step()
    compare(g, o)


def test_periodic_mass_conserved_and_divb():
    g, o = pair(small_turbulence())
    d0 = g.diagnostics()
    for _ in range(4):
        g.step()
    d1 = g.diagnostics()
    assert abs(d1["mass"] - d0["mass"]) <= 1e-13 * d0["mass"]
    assert d1["divb_max"] <= 1e-11
    assert d1["steps"] == 4


def test_nonfinite_state_is_reported():
    st = small_turbulence(8)
    st.U[4][5, 5, 5] = np.nan
    g = native.Mhd3D(st.params)
    g.upload(st)
    with pytest.raises(native.MhdError) as e:
        g.step()
        g.synchronize()
    assert e.value.code in (3, 4)


def test_fp32_form_close_to_fp64():
    st = problems.colliding_flows(16)
    g64 = native.Mhd3D(st.params, precision=native.PREC_FP64)
    g32 = native.Mhd3D(st.params, precision=native.PREC_FP32)
    g64.upload(st)
    g32.upload(st)
    for _ in range(10):
        dt, _ = g64.timestep()
        g64.advance(dt)
        g32.advance(dt)
    U64, _, b64 = g64.download()
    U32, _, b32 = g32.download()
    c = (slice(2, -2),) * 3
    for f in (0, 4):
        l1 = np.abs(U32[f][c] - U64[f][c]).mean() / np.abs(U64[f][c]).mean()
        assert l1 < 1e-4, (f, l1)
    l1b = np.abs(b32[:, 2:-2, 2:-2, 2:-2] - b64[:, 2:-2, 2:-2, 2:-2]).mean() / np.abs(b64).mean()
    assert l1b < 1e-4


@pytest.mark.parametrize("bc", [(1, 1, 1, 1, 1, 1), (3, 3, 1, 1, 3, 3), (1, 1, 3, 3, 1, 1)])
def test_free_boundaries_bit_exact(bc):
    """Free (code 1) sides on y and z as well as x: every ghost exchange,
    the in-pencil fills of the sweeps and CT with outflow on each axis."""
    st = problems.colliding_flows(16)
    st.params = st.params.replace(bc=bc)
    g, o = pair(st)
    for _ in range(4):
        assert g.step() == o.step()
    compare(g, o)
