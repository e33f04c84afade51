"""CPU statement (numpy, float64) of the learned cut quadrature's network, its
training objective and gradient, and of the training data generators.

THIS IS TEST INFRASTRUCTURE: tests/ and bench.py (to generate seeded inputs
and to check the GPU kernels) use it; the product never does.

Network: x (10) -> SiLU(x W1 + b1) (256) -> SiLU(. W2 + b2) (256) -> . W3 + b3 (24),
with W1, W2, W3 rounded to BF16 (round to nearest even) in every product and
FP32 biases, as the GPU kernels use them.  Objective of a batch:
mean_i sum_a ((U y_i / 256 - t_i)_a / s_i)^2, V = U R the thin QR (positive diag R) of
V[a][j] = p_j^a over the 24 fixed points and the 35 monomials of degree <= 4
(graded order); the weights at the points are R^-1 y."""
import itertools

import numpy as np

N_IN, N_HID, N_OUT, N_MOM = 10, 256, 24, 35
SHAPES = [("W1", (N_IN, N_HID)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_OUT)), ("b3", (N_OUT,))]


def bf16(a):
    """float32 -> bfloat16 (round to nearest even) -> float64."""
    f = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((f >> 16) & 1) + 0x7FFF
    f = ((f + r) & 0xFFFF0000).astype(np.uint32)
    return f.view(np.float32).astype(np.float64)


def unpack(params):
    out, k = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(params[k:k + n], dtype=np.float64).reshape(shp)
        k += n
    return out


def point_set():
    """The 24 fixed points: orbits s31(0.075), s31(0.16), s211(0.025, 0.36),
    s31(0.32) of barycentric coordinates, each orbit's distinct permutations in
    lexicographic order; point = (lambda_0, lambda_1, lambda_2)."""
    pts = []
    for b in ([1 - 3 * 0.075, 0.075, 0.075, 0.075], [1 - 3 * 0.16, 0.16, 0.16, 0.16],
              [0.025, 0.025, 0.36, 1 - 2 * 0.025 - 0.36], [1 - 3 * 0.32, 0.32, 0.32, 0.32]):
        pts += sorted(set(itertools.permutations(sorted(b))))
    return np.array([p[:3] for p in pts])


def exponents():
    return [(a, b, t - a - b) for t in range(5) for a in range(t, -1, -1) for b in range(t - a, -1, -1)]


def vandermonde():
    P = point_set()
    return np.array([[x ** a * y ** b * z ** c for (x, y, z) in P] for (a, b, c) in exponents()])


def basis():
    """U of the thin QR V = U R with positive diag(R): the network output y gives
    the weights R^-1 y at the points and the moment correction U y."""
    Q, R = np.linalg.qr(vandermonde())
    return Q * np.sign(np.diag(R))[None, :]


OUT_SCALE = 1.0 / 256.0
EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def features(v):
    """u = v / max|v|; the 4 vertex values of u, then the 6 edge-midpoint
    deviations u_e - (u_a + u_b) / 2."""
    v = np.asarray(v, dtype=np.float64)
    u = v / np.abs(v).max(1)[:, None]
    d = np.stack([u[:, 4 + k] - 0.5 * (u[:, a] + u[:, b]) for k, (a, b) in enumerate(EDGES)], 1)
    return np.concatenate([u[:, :4], d], 1)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x):
    p = unpack(params)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ bf16(p["W1"]) + p["b1"]
    h1 = silu(z1)
    z2 = h1 @ bf16(p["W2"]) + p["b2"]
    h2 = silu(z2)
    y = h2 @ bf16(p["W3"]) + p["b3"]
    return y, (x, z1, h1, z2, h2)


def forward_bf16_activations(params, x):
    """The network as the tensor-core inference kernel runs it: the input
    features and both hidden activations also rounded to BF16 before each
    product (FP32 biases, exact products, FP64 sums here)."""
    p = unpack(params)
    x = bf16(np.asarray(x, dtype=np.float32))
    h1 = bf16(silu(x @ bf16(p["W1"]) + p["b1"]).astype(np.float32))
    h2 = bf16(silu(h1 @ bf16(p["W2"]) + p["b2"]).astype(np.float32))
    return h2 @ bf16(p["W3"]) + p["b3"]


def loss_grad(params, x, t, s):
    """(loss, flat gradient) of the batch objective."""
    p = unpack(params)
    V = basis()
    y, (x, z1, h1, z2, h2) = forward(params, x)
    B = x.shape[0]
    r = (OUT_SCALE * (y @ V.T) - t) / s[:, None]
    loss = float(np.mean((r ** 2).sum(1)))
    dy = (2.0 / B) * OUT_SCALE * (r / s[:, None]) @ V
    g = {"W3": h2.T @ dy, "b3": dy.sum(0)}
    dz2 = (dy @ bf16(p["W3"]).T) * dsilu(z2)
    g["W2"], g["b2"] = h1.T @ dz2, dz2.sum(0)
    dz1 = (dz2 @ bf16(p["W2"]).T) * dsilu(z1)
    g["W1"], g["b1"] = x.T @ dz1, dz1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SHAPES])


# ---- training data -----------------------------------------------------------
def spec_values(n, rng):
    """10 nodal values ~ N(0,1), shifted by a uniform draw between their min and
    max (so the ten values have a zero crossing), scaled to max |v| = 1."""
    v = rng.standard_normal((n, 10))
    s = rng.uniform(v.min(1), v.max(1))
    v = v - s[:, None]
    return v / np.abs(v).max(1)[:, None]


def resolved_values(n, rng, curvature=0.15):
    """Mildly curved elements (a level set resolved by the mesh): linear vertex
    values with a zero crossing among them, edge midpoints = the linear mean plus
    a quadratic perturbation of relative size U(0, curvature); scaled to max |v| = 1."""
    v = rng.standard_normal((n, 4))
    s = rng.uniform(v.min(1), v.max(1))
    v = v - s[:, None]
    E = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    scale = np.abs(v).max(1)
    amp = rng.uniform(0, curvature, n) * scale
    mids = np.stack([0.5 * (v[:, a] + v[:, b]) for a, b in E], 1) + amp[:, None] * rng.standard_normal((n, 6))
    out = np.concatenate([v, mids], 1)
    return out / np.abs(out).max(1)[:, None]
