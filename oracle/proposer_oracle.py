"""CPU restatement of the learned hit proposer's network (numpy).

TEST INFRASTRUCTURE ONLY: the GPU kernels' encoding, forward pass, loss and
gradients are checked against these functions; nothing in the product calls
them.  The reference has no learned component, so there is nothing of it to
restate here; the network is this library's own (hash-grid encoding after
Mueller et al. 2022, "Instant neural graphics primitives", spatial hash of
Teschner et al. 2003, 32-64-64-64-4096 MLP, softmax cross-entropy).

The encoding is computed in float32 with the same operation order as the GPU
(no fused multiply-adds), so its BF16 features are bit-identical.  The MLP runs
in float64 with BF16 rounding at the same points as the GPU kernels: encoded
features, hidden activations after bias + ReLU, the softmax gradient and the
back-propagated hidden gradients.  `rounding=False` keeps everything float64
(for finite-difference checks of the analytic gradients).
"""
import numpy as np

LEVELS = 16
ORIGIN_LEVELS = 8
LOG2_TABLE = 18
TABLE = 1 << LOG2_TABLE
FEAT = 2
IN = LEVELS * FEAT
HIDDEN = 64
TREELETS = 4096

OFF_W1 = LEVELS * TABLE * FEAT
OFF_B1 = OFF_W1 + HIDDEN * IN
OFF_W2 = OFF_B1 + HIDDEN
OFF_B2 = OFF_W2 + HIDDEN * HIDDEN
OFF_W3 = OFF_B2 + HIDDEN
OFF_B3 = OFF_W3 + HIDDEN * HIDDEN
OFF_W4 = OFF_B3 + HIDDEN
OFF_B4 = OFF_W4 + TREELETS * HIDDEN
NUM_PARAMS = OFF_B4 + TREELETS


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def level_resolution(l):
    return 16 << l if l < ORIGIN_LEVELS else 4 << (l - ORIGIN_LEVELS)


def grid_index(R, x, y, z):
    n = np.uint64(R + 1)
    if int(n) ** 3 <= TABLE:
        return (x.astype(np.uint64) + n * (y.astype(np.uint64) + n * z.astype(np.uint64))).astype(np.uint32)
    x, y, z = (v.astype(np.uint32) for v in (x, y, z))
    with np.errstate(over="ignore"):
        h = x ^ (y * np.uint32(2654435761)) ^ (z * np.uint32(805459861))
    return h & np.uint32(TABLE - 1)


def level_points(rays, grid_lo, grid_scale, l):
    """(N, 3) float32 points of level l in [0, 1]^3 (gb_learned.cu level_point)."""
    f32 = np.float32
    if l < ORIGIN_LEVELS:
        o = np.stack([rays["org_x"], rays["org_y"], rays["org_z"]], -1).astype(f32)
        q = (o - np.asarray(grid_lo, f32)) * np.asarray(grid_scale, f32)
    else:
        d = np.stack([rays["dir_x"], rays["dir_y"], rays["dir_z"]], -1).astype(f32)
        n2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        with np.errstate(divide="ignore"):
            inv = np.where(n2 > 0, f32(1.0) / np.sqrt(n2), f32(0.0)).astype(f32)
        q = (d * inv[:, None] + f32(1.0)) * f32(0.5)
    return np.fmin(np.fmax(q.astype(f32), f32(0.0)), f32(1.0))


def corners(rays, grid_lo, grid_scale, l):
    """Table entries (N, 8) and float32 weights (N, 8) of level l."""
    f32 = np.float32
    R = level_resolution(l)
    q = level_points(rays, grid_lo, grid_scale, l)
    p = (q * f32(R)).astype(f32)
    i = np.minimum(np.floor(p).astype(np.int64), R - 1).astype(np.int64)
    fr = (p - i.astype(f32)).astype(f32)
    ents, ws = [], []
    for k in range(8):
        bx, by, bz = k & 1, (k >> 1) & 1, (k >> 2) & 1
        wx = fr[:, 0] if bx else f32(1.0) - fr[:, 0]
        wy = fr[:, 1] if by else f32(1.0) - fr[:, 1]
        wz = fr[:, 2] if bz else f32(1.0) - fr[:, 2]
        ws.append(((wx * wy).astype(f32) * wz).astype(f32))
        ents.append(grid_index(R, i[:, 0] + bx, i[:, 1] + by, i[:, 2] + bz))
    return np.stack(ents, 1), np.stack(ws, 1)


def encode(params, rays, grid_lo, grid_scale):
    """BF16 features (N, 32) as float32, plus the corner data of each level."""
    f32 = np.float32
    table = bf16(params[:OFF_W1]).reshape(LEVELS, TABLE, FEAT)
    n = rays.shape[0]
    X = np.zeros((n, IN), f32)
    cdata = []
    for l in range(LEVELS):
        e, w = corners(rays, grid_lo, grid_scale, l)
        s0 = np.zeros(n, f32)
        s1 = np.zeros(n, f32)
        for k in range(8):
            s0 = (s0 + (w[:, k] * table[l, e[:, k], 0]).astype(f32)).astype(f32)
            s1 = (s1 + (w[:, k] * table[l, e[:, k], 1]).astype(f32)).astype(f32)
        X[:, 2 * l] = s0
        X[:, 2 * l + 1] = s1
        cdata.append((e, w))
    return bf16(X), cdata


def _unpack(params, rounding):
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1 = r(params[OFF_W1:OFF_B1]).astype(np.float64).reshape(HIDDEN, IN)
    W2 = r(params[OFF_W2:OFF_B2]).astype(np.float64).reshape(HIDDEN, HIDDEN)
    W3 = r(params[OFF_W3:OFF_B3]).astype(np.float64).reshape(HIDDEN, HIDDEN)
    W4 = r(params[OFF_W4:OFF_B4]).astype(np.float64).reshape(TREELETS, HIDDEN)
    b = [np.asarray(params[o:o + n], np.float64) for o, n in
         ((OFF_B1, HIDDEN), (OFF_B2, HIDDEN), (OFF_B3, HIDDEN), (OFF_B4, TREELETS))]
    return (W1, W2, W3, W4), b


def logits(params, rays, grid_lo, grid_scale, rounding=True):
    """(N, 4096) float64 logits."""
    X, _ = encode(params, rays, grid_lo, grid_scale) if rounding else _encode_exact(params, rays, grid_lo,
                                                                                       grid_scale)
    (W1, W2, W3, W4), (b1, b2, b3, b4) = _unpack(params, rounding)
    rd = (lambda a: bf16(a).astype(np.float64)) if rounding else (lambda a: a)
    h = X.astype(np.float64)
    for W, b in ((W1, b1), (W2, b2), (W3, b3)):
        h = rd(np.maximum(h @ W.T + b, 0.0))
    return h @ W4.T + b4


def _encode_exact(params, rays, grid_lo, grid_scale):
    """float64 trilinear features without BF16 rounding (finite-difference checks)."""
    table = np.asarray(params[:OFF_W1], np.float64).reshape(LEVELS, TABLE, FEAT)
    n = rays.shape[0]
    X = np.zeros((n, IN))
    cdata = []
    for l in range(LEVELS):
        e, w = corners(rays, grid_lo, grid_scale, l)
        X[:, 2 * l] = (w.astype(np.float64) * table[l, e, 0]).sum(1)
        X[:, 2 * l + 1] = (w.astype(np.float64) * table[l, e, 1]).sum(1)
        cdata.append((e, w))
    return X, cdata


def loss_and_grad(params, rays, labels, grid_lo, grid_scale, rounding=True, want_grad=True):
    """Mean softmax cross-entropy over the batch (rows with label < 0 count as
    zero) and its gradient in the flat parameter layout (float64; None when
    want_grad is False)."""
    labels = np.asarray(labels, np.int64)
    B = rays.shape[0]
    if rounding:
        X, cdata = encode(params, rays, grid_lo, grid_scale)
        X = X.astype(np.float64)
    else:
        X, cdata = _encode_exact(params, rays, grid_lo, grid_scale)
    (W1, W2, W3, W4), (b1, b2, b3, b4) = _unpack(params, rounding)
    rd = (lambda a: bf16(a).astype(np.float64)) if rounding else (lambda a: a)
    H1 = rd(np.maximum(X @ W1.T + b1, 0.0))
    H2 = rd(np.maximum(H1 @ W2.T + b2, 0.0))
    H3 = rd(np.maximum(H2 @ W3.T + b3, 0.0))
    Z = H3 @ W4.T + b4
    mx = Z.max(1, keepdims=True)
    lse = mx[:, 0] + np.log(np.exp(Z - mx).sum(1))
    P = np.exp(Z - lse[:, None])
    lab = labels >= 0
    onehot = np.zeros_like(Z)
    onehot[np.nonzero(lab)[0], labels[lab]] = 1.0
    loss = float((lse[lab] - Z[np.nonzero(lab)[0], labels[lab]]).sum() / B)
    if not want_grad:
        return loss, None
    dZ4 = rd((P - onehot) / B)
    dZ4[~lab] = 0.0
    g = np.zeros(NUM_PARAMS)
    g[OFF_B4:OFF_B4 + TREELETS] = dZ4.sum(0)
    g[OFF_W4:OFF_B4] = (dZ4.T @ H3).ravel()
    dH = dZ4 @ W4
    for H, Xin, W, offW, offB in ((H3, H2, W3, OFF_W3, OFF_B3), (H2, H1, W2, OFF_W2, OFF_B2),
                                  (H1, X, W1, OFF_W1, OFF_B1)):
        dZ = rd(dH * (H > 0))
        g[offB:offB + HIDDEN] = dZ.sum(0)
        g[offW:offW + W.size] = (dZ.T @ Xin).ravel()
        dH = dZ @ W
    # hash table: scatter of the feature gradients to the 8 corners of each level
    gt = np.zeros((LEVELS, TABLE, FEAT))
    for l, (e, w) in enumerate(cdata):
        for f in range(FEAT):
            np.add.at(gt[l, :, f], e.ravel(), (w.astype(np.float64) * dH[:, 2 * l + f][:, None]).ravel())
    g[:OFF_W1] = gt.ravel()
    return loss, g


def segments():
    """(name, start, end) of every parameter tensor."""
    return [("table", 0, OFF_W1), ("W1", OFF_W1, OFF_B1), ("b1", OFF_B1, OFF_W2), ("W2", OFF_W2, OFF_B2),
            ("b2", OFF_B2, OFF_W3), ("W3", OFF_W3, OFF_B3), ("b3", OFF_B3, OFF_W4), ("W4", OFF_W4, OFF_B4),
            ("b4", OFF_B4, NUM_PARAMS)]


def random_params(seed=0, table_scale=0.5):
    """A parameter vector with non-trivial features (table entries +-table_scale)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NUM_PARAMS, np.float32)
    p[:OFF_W1] = rng.uniform(-table_scale, table_scale, OFF_W1)
    for name, a, b in segments()[1:]:
        fan_in = IN if name == "W1" else HIDDEN
        if name.startswith("W"):
            p[a:b] = rng.uniform(-1, 1, b - a) * np.sqrt(6.0 / fan_in)
        else:
            p[a:b] = rng.uniform(-0.1, 0.1, b - a)
    return p
