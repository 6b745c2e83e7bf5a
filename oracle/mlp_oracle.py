"""Output-size predictor oracle -- TEST INFRASTRUCTURE ONLY.

Numpy restatement of the block statistics and of the network (34 -> 64 -> 64
-> 1, ReLU) that the library's predictor kernels compute, used by the tests to
check them: the statistics bit for bit (float32, the kernels' operation
order), the forward pass and the gradient of the mean squared error in
float64.  The product never imports this module.

Parameter layout (flat): W1 [34][64], b1 [64], W2 [64][64], b2 [64], W3 [64], b3.
"""
import numpy as np

N_IN, N_HID, BLOCK = 34, 64, 16
SIZES = [N_IN * N_HID, N_HID, N_HID * N_HID, N_HID, N_HID, 1]
N_PARAMS = sum(SIZES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, at = [], 0
    for s in SIZES:
        out.append(p[at:at + s])
        at += s
    w1, b1, w2, b2, w3, b3 = out
    return w1.reshape(N_IN, N_HID), b1, w2.reshape(N_HID, N_HID), b2, w3, b3[0]


def block_stats(vol, block=BLOCK):
    """Per block of block^3 cells (its (block+1)^3 points, clipped at the far
    faces): min, max and the 32-bin histogram over [min, max] as fractions,
    bin = min(31, max(0, int((v - min) * (32 / (max - min))))) in float32."""
    vol = np.asarray(vol, dtype=np.float32)
    nz, ny, nx = vol.shape
    nb = [(n - 2) // block + 1 if n >= 2 else 0 for n in (nx, ny, nz)]
    out = np.zeros((nb[0] * nb[1] * nb[2], N_IN), dtype=np.float32)
    for bz in range(nb[2]):
        for by in range(nb[1]):
            for bx in range(nb[0]):
                v = vol[bz * block: min(bz * block + block, nz - 1) + 1,
                        by * block: min(by * block + block, ny - 1) + 1,
                        bx * block: min(bx * block + block, nx - 1) + 1].reshape(-1)
                lo, hi = v.min(), v.max()
                rng = np.float32(hi - lo)
                scale = np.float32(32.0) / rng if rng > 0 else np.float32(0.0)
                bins = np.clip(((v - lo) * scale).astype(np.float32).astype(np.int64), 0, 31)
                b = (bz * nb[1] + by) * nb[0] + bx
                out[b, 0], out[b, 1] = lo, hi
                out[b, 2:] = np.bincount(bins, minlength=32).astype(np.float32) / np.float32(v.size)
    return out


def inputs(stats, iso):
    """The network's inputs: (min - iso) / (max - min), (max - iso) / (max - min), the 32 fractions
    (float32, as the kernels form them; 0 for a constant block)."""
    stats = np.asarray(stats, dtype=np.float32)
    iso = np.broadcast_to(np.asarray(iso, dtype=np.float32), (stats.shape[0],))
    x = stats.copy()
    rng = (stats[:, 1] - stats[:, 0]).astype(np.float32)
    ok = rng > 0
    for c in (0, 1):
        x[:, c] = np.where(ok, (stats[:, c] - iso) / np.where(ok, rng, 1), 0).astype(np.float32)
    return x


def forward(p, x):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ w1 + b1, 0.0)
    h2 = np.maximum(h1 @ w2 + b2, 0.0)
    return h2 @ w3 + b3, (x, h1, h2)


def loss_and_gradient(p, x, target):
    """(1/n) sum (y - target)^2 and its gradient (flat, the parameter layout)."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    y, (x, h1, h2) = forward(p, x)
    n = x.shape[0]
    e = y - np.asarray(target, dtype=np.float64)
    dy = 2.0 * e / n
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    d2 = np.outer(dy, w3) * (h2 > 0)
    gw2 = h1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ w2.T) * (h1 > 0)
    gw1 = x.T @ d1
    gb1 = d1.sum(0)
    g = np.concatenate([gw1.ravel(), gb1, gw2.ravel(), gb2, gw3, [gb3]])
    return float((e * e).mean()), g
