"""CPU oracle of the warm-start MLP (test infrastructure only).

An FP64 numpy restatement of the device MLP of
idea.deploy_gb300/csrc/mlp.cu: 5 -> 64 -> 64 -> 64 -> 1 with SiLU, the mean
squared error, its gradient by back-propagation, and Adam.  The device
computes with the parameters rounded to BF16, rounds the hidden activations
h1, h2 and the back-propagated dZ2, dZ3 to BF16 where they enter a
tensor-core GEMM, and accumulates in FP32; the oracle applies the same BF16
roundings (round to nearest even) and accumulates in FP64, so the two differ
only by FP32 accumulation and the odd BF16 rounding flip.  The reference
project has no counterpart (it starts every droplet from a tanh profile).

Only tests/ may import this module.
"""
import numpy as np

H, IN = 64, 5
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + H
NP = OFF_B4 + 1


def bf16(a):
    """Round to bfloat16 (nearest, ties to even) via FP32, returned as float64."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return dict(W1=p[OFF_W1:OFF_B1].reshape(H, IN), b1=p[OFF_B1:OFF_W2], W2=p[OFF_W2:OFF_B2].reshape(H, H),
                b2=p[OFF_B2:OFF_W3], W3=p[OFF_W3:OFF_B3].reshape(H, H), b3=p[OFF_B3:OFF_W4], W4=p[OFF_W4:OFF_B4],
                b4=p[OFF_B4])


def sigm(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigm(z)


def dsilu(z):
    s = sigm(z)
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, exact=False):
    """Outputs and the intermediates of the device forward pass (exact=True:
    no BF16 rounding anywhere, for finite-difference checks)."""
    r = (lambda a: np.asarray(a, np.float64)) if exact else bf16
    w = unpack(r(p))
    x = np.asarray(x, np.float64).reshape(-1, IN)
    z1 = x @ w['W1'].T + w['b1']
    h1 = r(silu(z1))
    z2 = h1 @ w['W2'].T + w['b2']
    h2 = r(silu(z2))
    z3 = h2 @ w['W3'].T + w['b3']
    h3 = silu(z3)
    y = h3 @ w['W4'] + w['b4']
    return y, dict(w=w, x=x, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3)


def gradient(p, x, t, exact=False):
    """(grad[NP], loss) of mean((y - t)^2) over the given samples."""
    r = (lambda a: np.asarray(a, np.float64)) if exact else bf16
    y, c = forward(p, x, exact)
    t = np.asarray(t, np.float64).ravel()
    n = y.size
    d = y - t
    loss = float((d * d).sum() / n)
    w = c['w']
    dy = 2.0 * d / n
    g = np.zeros(NP)
    g[OFF_W4:OFF_B4] = c['h3'].T @ dy
    g[OFF_B4] = dy.sum()
    dz3 = dy[:, None] * w['W4'][None, :] * dsilu(c['z3'])
    g[OFF_B3:OFF_W4] = dz3.sum(0)
    dz3b = r(dz3)
    g[OFF_W3:OFF_B3] = (dz3b.T @ c['h2']).ravel()
    dz2 = (dz3b @ w['W3']) * dsilu(c['z2'])
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz2b = r(dz2)
    g[OFF_W2:OFF_B2] = (dz2b.T @ c['h1']).ravel()
    dz1 = (dz2b @ w['W2']) * dsilu(c['z1'])
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W1:OFF_B1] = (dz1.T @ c['x']).ravel()
    return g, loss


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


_M64 = (1 << 64) - 1


def _mix64(z):
    z = int(z) & _M64
    z = ((z ^ (z >> 30)) * 0xbf58476d1ce4e5b9) & _M64
    z = ((z ^ (z >> 27)) * 0x94d049bb133111eb) & _M64
    return z ^ (z >> 31)


def sample_indices(seed, step, batch, n):
    """The training samples the device draws at a step (counter-based hash)."""
    return np.array([_mix64(int(seed) ^ _mix64((step * 0x9E3779B97F4A7C15 + j) & _M64)) % n for j in range(batch)],
                    np.int64)
