"""The proposer network's CPU restatement (oracle/proposer_oracle.py), pinned
without a GPU: its analytic gradients against central finite differences in
float64, its BF16 rounding against torch's, and its hash-grid indexing."""
import numpy as np
import pytest

import proposer_oracle as PO
from rtcgb import rays as R


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return R.make_rays(rng.uniform(0.05, 0.95, (n, 3)), d)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(size=10000).astype(np.float32) * 10.0 ** rng.integers(-8, 8, 10000),
                        # exact halfway cases round to even
                        (np.arange(1, 200, dtype=np.uint32) << 16 | 0x8000).view(np.float32)])
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert (PO.bf16(x).view(np.uint32) == ref.view(np.uint32)).all()


def test_grid_indexing():
    # dense while (R+1)^3 fits the table, hashed afterwards
    R = PO.level_resolution(1)  # 32: 33^3 = 35937 entries
    idx = PO.grid_index(R, np.array([1, 32]), np.array([2, 0]), np.array([3, 32]))
    assert list(idx) == [1 + 33 * (2 + 33 * 3), 32 + 33 * (0 + 33 * 32)]
    R = PO.level_resolution(5)  # 512: hashed
    x, y, z = np.array([7], np.uint32), np.array([9], np.uint32), np.array([11], np.uint32)
    want = (7 ^ ((9 * 2654435761) & 0xFFFFFFFF) ^ ((11 * 805459861) & 0xFFFFFFFF)) & (PO.TABLE - 1)
    assert int(PO.grid_index(R, x, y, z)[0]) == want
    # corner weights of a level sum to one
    rays = _rays(50, 1)
    for l in (0, 7, 8, 15):
        e, w = PO.corners(rays, np.zeros(3, np.float32), np.ones(3, np.float32), l)
        assert np.allclose(w.astype(np.float64).sum(1), 1.0, atol=1e-6)
        assert e.max() < PO.TABLE


def test_analytic_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    params = PO.random_params(seed=3).astype(np.float64)
    rays = _rays(6, 4)
    labels = np.array([5, 17, -1, 4095, 17, 300])
    lo, sc = np.zeros(3, np.float32), np.ones(3, np.float32)
    loss, g = PO.loss_and_grad(params, rays, labels, lo, sc, rounding=False)
    # parameters to probe: table entries the batch touches, and weights/biases of every layer
    _, cdata = PO._encode_exact(params, rays, lo, sc)
    probes = []
    for l in (0, 5, 9, 15):
        e = cdata[l][0][rng.integers(0, 6), rng.integers(0, 8)]
        probes.append(int(l * PO.TABLE * 2 + 2 * e + rng.integers(0, 2)))
    for name, a, b in PO.segments()[1:]:
        probes += [int(v) for v in rng.integers(a, b, 3)]
    probes += [PO.OFF_B4 + 17, PO.OFF_W4 + 17 * PO.HIDDEN + 3]  # the labelled class
    for k in probes:
        eps = 1e-6 * max(1.0, abs(params[k]))
        p1, p2 = params.copy(), params.copy()
        p1[k] += eps
        p2[k] -= eps
        l1, _ = PO.loss_and_grad(p1, rays, labels, lo, sc, rounding=False, want_grad=False)
        l2, _ = PO.loss_and_grad(p2, rays, labels, lo, sc, rounding=False, want_grad=False)
        fd = (l1 - l2) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(g[k]), (k, fd, g[k])


def test_rounded_gradients_close_to_exact():
    """BF16 rounding points perturb the gradient (the 4096-wide softmax gradient
    is stored in BF16, so the back-propagated gradients carry ~10% noise) but
    keep its direction: cosine similarity above 0.99 for every tensor."""
    params = PO.random_params(seed=8)
    rays = _rays(64, 9)
    labels = np.random.default_rng(10).integers(-1, 4096, 64)
    lo, sc = np.zeros(3, np.float32), np.ones(3, np.float32)
    l0, g0 = PO.loss_and_grad(params.astype(np.float64), rays, labels, lo, sc, rounding=False)
    l1, g1 = PO.loss_and_grad(params, rays, labels, lo, sc, rounding=True)
    assert abs(l0 - l1) < 2e-2 * abs(l0)
    for name, a, b in PO.segments():
        x, y = g0[a:b], g1[a:b]
        assert x @ y >= 0.99 * np.linalg.norm(x) * np.linalg.norm(y), name
