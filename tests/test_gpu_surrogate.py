"""The learned part: the KI-cooling surrogate and the FP32 source.

* labels from the GPU's plain integrator equal the oracle's IMC bit for bit
* the training kernels' gradients agree with the NumPy restatement
  (oracle/surrogate_ref.py, same BF16 rounding points)
* training on the GPU lowers the loss
* the tensor-core (tcgen05) forward matches the NumPy forward
* inside SOURCE the network's guesses are accepted for the stiff cells and
  land closer to the FP64 integrator than the same solver's without it
"""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from oracle import pyoracle
from oracle import surrogate_ref as S

pytestmark = pytest.mark.gpu

BOX_LO = np.array([-2.0, -2.0, -3.0])
BOX_HI = np.array([5.0, np.log10(20.0), 3.0])


def sample(n, seed):
    return np.random.default_rng(seed).uniform(BOX_LO, BOX_HI, (n, 3)).astype(np.float32)


@pytest.fixture(scope="module")
def trained():
    p0 = S.init_params(0)
    p, hist = native.surrogate_train(p0, n_data=1 << 20, batch=8192, steps=3000, lr=1e-3, seed=3)
    return p, hist


@pytest.mark.parametrize("kb", [8.63359, 6.0])
def test_labels_bit_exact_vs_oracle(kb):
    x = sample(3000, 1)
    gpu = native.surrogate_label(x, kb=kb)
    cpu = pyoracle.ki_labels(x, kb=kb).astype(np.float32)
    assert np.array_equal(gpu, cpu)


def test_training_gradients_match_numpy():
    p = S.init_params(5)
    x = sample(1024, 2)
    y = pyoracle.ki_labels(x).astype(np.float32)
    g_gpu, loss_gpu = native.surrogate_grad(p, x, y)
    g_cpu, loss_cpu = S.grad(p, x, y)
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * abs(loss_cpu) + 1e-7
    rel = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    cos = float(g_gpu @ g_cpu / (np.linalg.norm(g_gpu) * np.linalg.norm(g_cpu)))
    assert rel < 2e-2 and cos > 0.9998, (rel, cos)
    # every parameter block, not only the large ones
    for lo, hi in ((0, 192), (192, 256), (256, 4352), (4352, 4416), (4416, 4544), (4544, 4546)):
        a, b = g_gpu[lo:hi], g_cpu[lo:hi]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-9, (lo, hi)


def test_training_lowers_loss(trained):
    p, hist = trained
    assert np.all(np.isfinite(hist))
    assert hist[-50:].mean() < 0.05 * hist[:10].mean()
    x = sample(20000, 9)
    y = native.surrogate_label(x)
    out = native.surrogate_eval(p, x)
    err = np.abs(out[:, 0] - y)
    assert np.median(err) < 0.05, np.median(err)


def stiff_state(n=32):
    """Colliding-flow state, dense enough that most cells cool faster than
    the forced step below (stiff)."""
    st = problems.colliding_flows(n)
    st.U[0] *= 30.0
    st.species *= 30.0
    return st


def test_fp32_source_matches_fp64():
    st = problems.colliding_flows(32)
    g64 = native.Mhd3D(st.params, precision=native.PREC_FP64)
    g32 = native.Mhd3D(st.params, precision=native.PREC_FP32)
    g64.upload(st)
    g32.upload(st)
    dt, _ = g64.timestep()
    g64.source(dt)
    g32.source(dt)
    p64 = g64.download()[0][4][2:-2, 2:-2, 2:-2]
    p32 = g32.download()[0][4][2:-2, 2:-2, 2:-2]
    assert np.abs(p32 - p64).mean() / np.abs(p64).mean() < 1e-5


def test_tensor_core_inference_matches_numpy(trained):
    """The tcgen05 forward (128-row tiles, BF16 operands in shared memory,
    FP32 accumulators in tensor memory) against the NumPy forward with the
    same BF16 rounding points; the GPU's SiLU is the tanh form on BF16
    pairs, so agreement is to BF16 activation rounding.  5001 samples: a
    partial last tile too."""
    p, _ = trained
    x = sample(5001, 21)
    out = native.surrogate_eval(p, x)
    ref = S.forward(p, x)["y"]
    d = np.abs(out - ref)
    # measured: max 0.06, mean 0.008 (the tanh-form SiLU on BF16 pairs); a
    # wrong operand layout or descriptor gives errors of order 1
    assert d.max() < 0.15 and d.mean() < 0.02, (d.max(0), d.mean(0))


def test_network_gain_over_the_same_solver_without_it(trained):
    """What the trained network gains.  Stiff cells start their implicit
    solve from a guess, take two Newton steps and are accepted when the
    implicit residual is <= 1e-3, else they take the bisection.  With the
    network the guess is its answer; without it (MHD_COOL_NEWTON) the
    frozen-rate implicit update P / (1 + c Lambda / P).  Both accept every
    stiff cell of this state; the network's answers are far closer to the
    FP64 integrator's (measured 1.7e-7 against 1.0e-5 in L1 of p): its
    guess needs fewer Newton steps for the same accuracy.  It costs time:
    bench.py reports the network path slower than both the frozen-rate
    start and the FP32 bisection on this GPU."""
    p, _ = trained
    st = stiff_state()
    dt = 0.05
    runs = {}
    for name, prec, cool in (("fp64", native.PREC_FP64, native.COOL_EXACT),
                             ("exact", native.PREC_FP32, native.COOL_EXACT),
                             ("surrogate", native.PREC_FP32, native.COOL_SURROGATE),
                             ("newton", native.PREC_FP32, native.COOL_NEWTON)):
        g = native.Mhd3D(st.params, precision=prec, cooling=cool)
        if cool == native.COOL_SURROGATE:
            g.surrogate_load(p, 1e-3)
        g.upload(st)
        g.source(dt)
        d = g.diagnostics()
        runs[name] = (g.download()[0][4][2:-2, 2:-2, 2:-2], d)
    p64 = runs["fp64"][0]
    n_stiff = runs["exact"][1]["imc_cells"]
    assert n_stiff > 0.5 * 2 * 32 ** 3            # both passes, most cells stiff
    l1 = {k: float(np.abs(runs[k][0] - p64).mean() / np.abs(p64).mean()) for k in ("exact", "surrogate", "newton")}
    for name in ("surrogate", "newton"):
        d = runs[name][1]
        # every stiff cell is either an accepted guess or a bisection
        assert d["surrogate_cells"] + d["imc_cells"] == n_stiff, (name, d)
        assert d["surrogate_cells"] >= 0.9 * n_stiff, (name, d)
    assert max(l1.values()) < 1e-3, l1
    assert 10.0 * l1["surrogate"] < l1["newton"], l1

