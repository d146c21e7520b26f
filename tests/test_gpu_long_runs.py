"""Long runs of the plain FP64 path against the oracle, bit for bit: the
required agreement is 1e-12 relative per cell after 100 steps; these hold every
interior value identical after 100 steps of the decaying turbulence and of
the KI colliding flows (and of the turbulence at 64^3), and after 50 steps of the shipped deck's setup
(inflow boundaries, chemistry network and species cooling), at sizes the
oracle runs in seconds."""
import pytest

from code_tohoku_gb300 import native, problems
from oracle.pyoracle import Oracle3D
from parity_util import compare, pair
from test_gpu_inflow import shock_tube

pytestmark = pytest.mark.gpu


def run(g, o, steps):
    for s in range(steps):
        a, b = g.step(), o.step()
        assert a == b, (s, a, b)


def test_turbulence_100_steps_bit_exact():
    g, o = pair(problems.turbulence(24, kmax=6))
    run(g, o, 100)
    compare(g, o)


def test_config2_turbulence_64_cubed_100_steps_bit_exact():
    """The decaying Mach-5 MHD turbulence workload (k^-4 on |k| = 1..8, ran0
    seed 1, beta 1, CFL 0.4) at 64^3: steps 1..100 bit for bit, the time
    step of every step included."""
    g, o = pair(problems.turbulence(64))
    run(g, o, 100)
    compare(g, o)


def test_colliding_flows_100_steps_bit_exact():
    g, o = pair(problems.colliding_flows(32))
    run(g, o, 100)
    compare(g, o)


def test_deck_setup_50_steps_bit_exact():
    st = shock_tube(16, 16, 16)
    st.params = st.params.replace(ifchem=2)
    inflow, dinit = problems.shock_tube_inflow()
    g = native.Mhd3D(st.params)
    g.set_inflow(inflow, None, dinit)
    g.upload(st)
    o = Oracle3D(st.params)
    o.set_inflow(inflow.vector(), None, dinit)
    o.upload(st)
    run(g, o, 50)
    compare(g, o)
