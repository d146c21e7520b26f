"""NumPy restatement of the KI-cooling surrogate network (test
infrastructure only): forward pass and gradients with the same BF16
rounding points as the GPU kernels, used to check the GPU training
kernels' gradients.

Rounding points (mirroring code_tohoku_gb300/csrc/mhd_surrogate_net.cuh and
mhd_surrogate.cu): inputs normalised in FP32; W1 rounded to BF16, first
layer in FP32; hidden activations h1 = bf16(SiLU(z1)), h2 = bf16(SiLU(z2));
W2, W3 rounded to BF16; every gradient product runs on the tensor cores with
BF16 operands: dz2 where it enters dW2 = dz2^T h1, gb2 = sum dz2 and
dh1 = dz2 W2; the output gradients d where they enter gW3 = d^T h2 and
gb3 = sum d; dz1 and the normalised inputs where they enter gW1 = dz1^T x
and gb1 = sum dz1.
"""
import numpy as np

H = 64
NPARAM = 64 * 3 + 64 + 64 * 64 + 64 + 2 * 64 + 2
CENTRE = np.array([1.5, -0.3494850, 0.0], dtype=np.float32)
SCALE = np.array([3.5, 1.6505150, 3.0], dtype=np.float32)
CONF_WEIGHT = 0.1


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, dtype=np.float32)
    o = 0
    W1 = p[o:o + 192].reshape(64, 3); o += 192
    b1 = p[o:o + 64]; o += 64
    W2 = p[o:o + 4096].reshape(64, 64); o += 4096
    b2 = p[o:o + 64]; o += 64
    W3 = p[o:o + 128].reshape(2, 64); o += 128
    b3 = p[o:o + 2]
    return W1, b1, W2, b2, W3, b3


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / 3), (64, 3))
    W2 = rng.normal(0, np.sqrt(2.0 / 64), (64, 64))
    W3 = rng.normal(0, np.sqrt(1.0 / 64), (2, 64)) * 0.1
    parts = [W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3.ravel(), np.zeros(2)]
    return np.concatenate(parts).astype(np.float32)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * _sig(z)


def dsilu(z):
    s = _sig(z)
    return s * (1.0 + z * (1.0 - s))


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = ((np.asarray(X, np.float32) - CENTRE) / SCALE).astype(np.float64)
    z1 = b1 + n @ bf16(W1).astype(np.float64).T
    h1 = bf16(silu(z1).astype(np.float32)).astype(np.float64)
    z2 = b2 + h1 @ bf16(W2).astype(np.float64).T
    h2 = bf16(silu(z2).astype(np.float32)).astype(np.float64)
    y = b3 + h2 @ bf16(W3).astype(np.float64).T
    return dict(n=n, z1=z1, h1=h1, z2=z2, h2=h2, y=y)


def grad(p, X, Y):
    """Gradient of mean[(y0 - Y)^2 + w (y1 - log10(|y0 - Y| + 1e-4))^2]
    (error in the second term held constant) and the mean squared error."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    f = forward(p, X)
    B = len(Y)
    e = f["y"][:, 0] - np.asarray(Y, np.float64)
    tc = np.log10(np.abs(e) + 1e-4)
    d = np.stack([2 * e / B, CONF_WEIGHT * 2 * (f["y"][:, 1] - tc) / B], axis=1)
    db = bf16(d.astype(np.float32)).astype(np.float64)
    gW3 = db.T @ f["h2"]
    gb3 = db.sum(0)
    dh2 = d @ bf16(W3).astype(np.float64)
    dz2 = dh2 * dsilu(f["z2"])
    dz2b = bf16(dz2.astype(np.float32)).astype(np.float64)
    gb2 = dz2b.sum(0)
    gW2 = dz2b.T @ f["h1"]
    dh1 = dz2b @ bf16(W2).astype(np.float64)
    dz1 = dh1 * dsilu(f["z1"])
    dz1b = bf16(dz1.astype(np.float32)).astype(np.float64)
    gb1 = dz1b.sum(0)
    gW1 = dz1b.T @ bf16(f["n"].astype(np.float32)).astype(np.float64)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return g, float(np.mean(e * e))
