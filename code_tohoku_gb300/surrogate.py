"""Host helpers for the KI-cooling surrogate (the network itself, its
training and its inference are CUDA kernels in csrc/mhd_surrogate*).

Parameter vector (FP32, the layout the C ABI expects): W1[64][3], b1[64],
W2[64][64], b2[64], W3[2][64], b3[2].
"""
import numpy as np

from . import native

NPARAM = 64 * 3 + 64 + 64 * 64 + 64 + 2 * 64 + 2


def init_params(seed=0):
    """He-normal hidden layers, small output layer, zero biases."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / 3), (64, 3))
    W2 = rng.normal(0, np.sqrt(2.0 / 64), (64, 64))
    W3 = rng.normal(0, np.sqrt(1.0 / 64), (2, 64)) * 0.1
    parts = [W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3.ravel(), np.zeros(2)]
    return np.concatenate(parts).astype(np.float32)


def train(n_data=1 << 24, batch=65536, steps=2000, lr=1e-3, seed=1, init_seed=0, device=0):
    """Generate n_data labelled states with the plain integrator and train
    with Adam on the GPU; returns (params, per-step batch MSE)."""
    return native.surrogate_train(init_params(init_seed), n_data=n_data, batch=batch, steps=steps, lr=lr,
                                  seed=seed, device=device)


def save(path, params, history=None):
    np.savez_compressed(path, params=np.asarray(params, np.float32),
                        history=np.asarray(history if history is not None else [], np.float32))


def load(path):
    return np.load(path)["params"].astype(np.float32)
