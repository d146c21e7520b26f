"""The chemistry network and species cooling (ifchem = 2, the shipped
deck's setting: 3DMHD-CfCA/MCF3DSGincfca3.f90 SOURCE :2576-2776, Fcool
:2825-2880, RATES :3037-3131) on the GPU against the oracle.  The plain
FP64 path must match bit for bit, for a source step over a spread of
densities and temperatures and for full steps of the inflow shock tube; the
chosen form (FP32 rates and network, FP64 state) stays close."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from oracle.pyoracle import Oracle3D
from parity_util import compare, pair
from test_chem_oracle import chem_state, nuclei
from test_gpu_inflow import shock_tube

pytestmark = pytest.mark.gpu
C = (slice(2, -2),) * 3


def chem_inflow_pair(shape=(16, 16, 16), precision=native.PREC_FP64):
    st = shock_tube(*shape)
    st.params = st.params.replace(ifchem=2)
    inflow, dinit = problems.shock_tube_inflow()
    g = native.Mhd3D(st.params, precision=precision)
    g.set_inflow(inflow, None, dinit)
    g.upload(st)
    o = Oracle3D(st.params)
    o.set_inflow(inflow.vector(), None, dinit)
    o.upload(st)
    return g, o


def test_chem_source_bit_exact():
    st = chem_state()
    g, o = pair(st)
    g.source(0.05)
    o.source(0.05)
    compare(g, o)
    # a second source step reads the nde / ndtot the first one left
    g.source(0.05)
    o.source(0.05)
    compare(g, o)


def test_chem_timestep_bit_exact():
    st = chem_state(seed=7)
    g, o = pair(st)
    assert g.timestep() == o.timestep()


def test_chem_inflow_steps_bit_exact():
    g, o = chem_inflow_pair()
    for _ in range(6):
        assert g.step() == o.step()
    compare(g, o)


def test_chem_periodic_steps_bit_exact():
    st = problems.wnm_shock_tube(16, bc=(3, 3, 3, 3, 3, 3))
    st.params = st.params.replace(ifchem=2)
    g, o = pair(st)
    for _ in range(5):
        assert g.step() == o.step()
    compare(g, o)


def test_chem_fp32_close_to_oracle():
    st = chem_state()
    g, o = pair(st, precision=native.PREC_FP32)
    g.source(0.05)
    o.source(0.05)
    Ug, sg, _ = g.download()
    Uo, so, _ = o.download()
    # densities and pressure: FP32 rates and network in a cell of FP64 state
    np.testing.assert_allclose(Ug[0][C], Uo[0][C], rtol=2e-4)
    np.testing.assert_allclose(Ug[4][C], Uo[4][C], rtol=2e-3)
    for s in range(5):
        np.testing.assert_allclose(sg[s][C], so[s][C], rtol=2e-3, atol=1e-12 * so[s][C].max())
    # the network's nuclei bookkeeping holds in the chosen form too
    for a, b in zip(nuclei(sg), nuclei(so)):
        np.testing.assert_allclose(a[C], b[C], rtol=1e-4)


def test_chem_fp32_steps_close():
    g, o = chem_inflow_pair(precision=native.PREC_FP32)
    for _ in range(6):
        dt, _ = o.timestep()
        o.advance(dt)
        g.advance(dt)
    Ug, sg, _ = g.download()
    Uo, so, _ = o.download()
    np.testing.assert_allclose(Ug[0][C], Uo[0][C], rtol=1e-4)
    np.testing.assert_allclose(Ug[4][C], Uo[4][C], rtol=2e-3)
    np.testing.assert_allclose(sg[1][C], so[1][C], rtol=5e-3)
