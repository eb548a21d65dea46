"""CPU restatement of the pair-energy surrogate -- TEST INFRASTRUCTURE ONLY.

Only tests/ (and the bench's CPU leg) import this module, as the CPU statement that the GPU
surrogate (sc_gb300/csrc/surrogate.cuh, surrogate.cu) is compared with.  The surrogate has no
counterpart in the reference (robertvacha/SC evaluates every pair exactly), so there is
nothing of the reference to pin it to; what it pins is the GPU code itself:

  * pair_features / wca32: the same FP32 operation sequence as the device functions
    (numpy float32 arithmetic is IEEE round-to-nearest like CUDA's without fast-math and
    without FMA contraction), so the features compare bit for bit;
  * forward / backward: the network in FP64 with the kernel's BF16 rounding points
    emulated (inputs, weights, hidden activations and back-propagated errors are rounded
    to BF16 where the tensor-core kernels round them); the kernels accumulate in FP32,
    so the comparison carries a tolerance;
  * forward / backward with emulate=False: the plain FP64 network, whose gradient the
    tests check against finite differences.
"""
import numpy as np

F32 = np.float32
N_FEAT, N_HID = 16, 64
OFF_W1 = 0
OFF_W2 = OFF_W1 + N_FEAT * N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID * N_HID
OFF_W4 = OFF_B3 + N_HID
OFF_B4 = OFF_W4 + N_HID
N_PARAMS = OFF_B4 + 1


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


# ---- features (FP32, device operation order) -------------------------------------------

def frac32(x):
    """Wrapped FP32 box fraction of an FP64 box fraction (frac32 of surrogate.cuh)."""
    x = np.asarray(x, dtype=np.float64)
    v = (x - np.floor(x)).astype(np.float32)
    return np.where(v >= F32(1.0), F32(0.0), v).astype(np.float32)


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def pair_vec(c1, c2, box):
    """FP32 minimum image c1 - c2 of wrapped fractions, times the FP32 box."""
    d = (c1 - c2).astype(np.float32)
    d = (d - np.rint(d)).astype(np.float32)
    return (d * box.astype(np.float32)).astype(np.float32)


def seg_closest(r, u, v, h1, h2):
    b = _dot(u, v)
    d = _dot(u, r)
    e = _dot(v, r)
    den = F32(1.0) - b * b
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(den > F32(1e-6), (b * e - d) / den, F32(0.0)).astype(np.float32)
    s = np.minimum(np.maximum(s, -h1), h1)
    t = np.minimum(np.maximum(b * s + e, -h2), h2)
    s = np.minimum(np.maximum(b * t - d, -h1), h1)
    t = np.minimum(np.maximum(b * s + e, -h2), h2)
    w = np.stack([(r[..., k] + s * u[..., k]) - t * v[..., k] for k in range(3)], -1).astype(np.float32)
    return _dot(w, w), s, t, w


def pair_features(r, a1, p1, h1, tc1, a2, p2, h2, tc2):
    """The 16 surrogate inputs of ordered pairs (arrays of shape (n, 3) / (n,), float32).
    Returns (inputs (n, 16), segment distance^2)."""
    args = [np.asarray(x, dtype=np.float32) for x in (r, a1, p1, h1, tc1, a2, p2, h2, tc2)]
    r, a1, p1, h1, tc1, a2, p2, h2, tc2 = args
    d2, s, t, w = seg_closest(r, a1, a2, h1, h2)
    d = np.sqrt(d2)
    rr = np.sqrt(_dot(r, r))
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(rr > F32(1e-12), F32(1.0) / rr, F32(0.0)).astype(np.float32)
    ar1 = _dot(a1, r) * inv
    ar2 = _dot(a2, r) * inv
    sg = np.where(ar1 < 0, F32(-1.0), F32(1.0)) * np.where(ar2 < 0, F32(-1.0), F32(1.0))
    wa1 = _dot(w, a1)
    wa2 = _dot(w, a2)
    n1 = np.stack([-w[:, k] + wa1 * a1[:, k] for k in range(3)], -1).astype(np.float32)
    n2 = np.stack([w[:, k] - wa2 * a2[:, k] for k in range(3)], -1).astype(np.float32)
    l1 = np.sqrt(_dot(n1, n1))
    l2 = np.sqrt(_dot(n2, n2))
    n = len(r)
    f = np.zeros((n, N_FEAT), dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        f[:, 0] = d
        f[:, 1] = rr * F32(0.25)
        f[:, 2] = np.abs(ar1)
        f[:, 3] = np.abs(ar2)
        f[:, 4] = _dot(a1, a2) * sg
        f[:, 5] = np.where(l1 > F32(1e-6), _dot(p1, n1) / l1, F32(0.0))
        f[:, 6] = np.where(l2 > F32(1e-6), _dot(p2, n2) / l2, F32(0.0))
        f[:, 7] = np.where(h1 > 0, np.abs(s) / h1, F32(0.0))
        f[:, 8] = np.where(h2 > 0, np.abs(t) / h2, F32(0.0))
    f[:, 9] = _dot(p1, p2)
    f[:, 10] = tc1
    f[:, 11] = tc2
    f[:, 12] = 1.0
    return f, d2


def wca32(d2, sigma, epsilon, rcutwca_sq):
    d2 = np.asarray(d2, dtype=np.float32)
    sigma, epsilon, rc = F32(sigma), F32(epsilon), F32(rcutwca_sq)
    with np.errstate(over="ignore", invalid="ignore"):
        x = (sigma * sigma) / np.maximum(d2, F32(1e-12))
        x3 = (x * x) * x
        e = (F32(4.0) * epsilon) * (x3 * x3 - x3) + epsilon
    e = np.minimum(e, F32(1e30))
    return np.where(d2 < rc, e, F32(0.0)).astype(np.float32)


# ---- network ------------------------------------------------------------------------------

def unpack(theta):
    t = np.asarray(theta, dtype=np.float64)
    return dict(W1=t[OFF_W1:OFF_W2].reshape(N_FEAT, N_HID), W2=t[OFF_W2:OFF_B2].reshape(N_HID, N_HID),
                b2=t[OFF_B2:OFF_W3], W3=t[OFF_W3:OFF_B3].reshape(N_HID, N_HID), b3=t[OFF_B3:OFF_W4],
                W4=t[OFF_W4:OFF_B4], b4=t[OFF_B4])


def pack(p):
    out = np.zeros(N_PARAMS)
    out[OFF_W1:OFF_W2] = p["W1"].ravel()
    out[OFF_W2:OFF_B2] = p["W2"].ravel()
    out[OFF_B2:OFF_W3] = p["b2"]
    out[OFF_W3:OFF_B3] = p["W3"].ravel()
    out[OFF_B3:OFF_W4] = p["b3"]
    out[OFF_W4:OFF_B4] = p["W4"]
    out[OFF_B4] = p["b4"]
    return out


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * _sig(z)


def silu_grad(z):
    s = _sig(z)
    return s * (1.0 + z * (1.0 - s))


def forward(theta, X, emulate=True):
    """Outputs y (n,) and the cache for backward.  emulate: BF16 rounding where the
    tensor-core kernels round (FP32 values rounded to BF16)."""
    p = unpack(theta)
    r = (lambda a: bf16(np.asarray(a, dtype=np.float32)).astype(np.float64)) if emulate else (lambda a: np.asarray(a, np.float64))
    W1, W2, W3, W4 = r(p["W1"]), r(p["W2"]), r(p["W3"]), r(p["W4"])
    X = np.asarray(X, dtype=np.float64)
    if emulate:
        W1[13:] = 0.0
    x0 = r(X)
    z1 = x0 @ W1
    h1 = r(silu(z1))
    z2 = h1 @ W2 + p["b2"]
    h2 = r(silu(z2))
    z3 = h2 @ W3 + p["b3"]
    h3 = r(silu(z3))
    y = h3 @ W4 + p["b4"]
    cache = dict(x0=x0, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, W2=W2, W3=W3, W4=W4, r=r)
    return y, cache


def backward(theta, X, target, emulate=True):
    """Gradient of mean((y - target)^2) with respect to theta, and that loss."""
    y, c = forward(theta, X, emulate)
    r = c["r"]
    n = len(y)
    e = y - np.asarray(target, dtype=np.float64)
    loss = float(np.mean(e * e))
    dy = 2.0 * e / n
    if emulate:
        dy = dy.astype(np.float32).astype(np.float64)
    dz3 = r(np.outer(dy, c["W4"]) * silu_grad(c["z3"]))
    dz2 = r((dz3 @ c["W3"].T) * silu_grad(c["z2"]))
    dz1 = r((dz2 @ c["W2"].T) * silu_grad(c["z1"]))
    g = dict(W1=c["x0"].T @ dz1, W2=c["h1"].T @ dz2, b2=dz2.sum(0), W3=c["h2"].T @ dz3, b3=dz3.sum(0),
             W4=c["h3"].T @ dy, b4=dy.sum())
    return pack(g), loss
