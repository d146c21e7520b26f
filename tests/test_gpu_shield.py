"""SHIELD (ifrad = 2: column densities from both x sides, :2924-3036) on
the GPU against the oracle: the columns after INITIA's 20 iterations, and
the chemistry and species cooling they shield over full steps, bit for bit
in the plain FP64 form; the chosen form stays close."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from oracle.pyoracle import Oracle3D
from parity_util import compare, pair
from test_chem_oracle import shield_state
from test_gpu_inflow import shock_tube

pytestmark = pytest.mark.gpu
C = (slice(2, -2),) * 3


def exact(a, b, what):
    bad = np.argwhere(a.view(np.int64) != b.view(np.int64))
    assert not len(bad), f"{what}: {len(bad)} values differ, first {tuple(bad[0])}: {a[tuple(bad[0])]!r} {b[tuple(bad[0])]!r}"


def test_shield_columns_after_upload_bit_exact():
    st = shield_state()
    g, o = pair(st)
    exact(g.columns()[(slice(None),) + C], o.columns()[(slice(None),) + C], "columns")


def test_shield_source_bit_exact():
    st = shield_state(seed=6)
    g, o = pair(st)
    for _ in range(2):
        g.source(0.05)
        o.source(0.05)
    compare(g, o)
    exact(g.columns()[(slice(None),) + C], o.columns()[(slice(None),) + C], "columns")


def test_shield_inflow_steps_bit_exact():
    st = shock_tube(16, 16, 16)
    st.params = st.params.replace(ifchem=2, ifrad=2)
    inflow, dinit = problems.shock_tube_inflow()
    g = native.Mhd3D(st.params)
    g.set_inflow(inflow, None, dinit)
    g.upload(st)
    o = Oracle3D(st.params)
    o.set_inflow(inflow.vector(), None, dinit)
    o.upload(st)
    for _ in range(5):
        assert g.step() == o.step()
    compare(g, o)
    exact(g.columns()[(slice(None),) + C], o.columns()[(slice(None),) + C], "columns")


def test_shield_fp32_close():
    st = shield_state(seed=7)
    g, o = pair(st, precision=native.PREC_FP32)
    g.source(0.05)
    o.source(0.05)
    cg, co = g.columns(), o.columns()
    for q in range(8):   # Ntot, NH2, NnC, NCO: FP64 sums of FP64 densities
        np.testing.assert_allclose(cg[q][C], co[q][C], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(cg[8:][(slice(None),) + C], co[8:][(slice(None),) + C], rtol=2e-3,
                               atol=1e-4 * np.abs(co[8:]).max())
    Ug, sg, _ = g.download()
    Uo, so, _ = o.download()
    np.testing.assert_allclose(Ug[4][C], Uo[4][C], rtol=2e-3)
    np.testing.assert_allclose(sg[1][C], so[1][C], rtol=2e-3, atol=1e-12 * so[1][C].max())


def test_columns_need_ifrad():
    st = problems.colliding_flows(16)
    g = native.Mhd3D(st.params)
    g.upload(st)
    with pytest.raises(native.MhdError):
        g.columns()
