"""The CPU oracle pinned against the reference's own known-answer tests.

Each test restates one of the reference's verify tests for the triangle path
(tutorials/verify/verify.cpp) and runs it on the oracle; together they are
the oracle's pin (the reference ships no golden data files for this path).
"""
import numpy as np
import pytest

from rtcgb import rays as R
from rtcgb import workloads as W

ULP = np.float32(np.finfo(np.float32).eps)  # embree's `ulp` constant


def _single_triangle_rays(n=256, seed=0):
    """Rays of TriangleHitTest (verify.cpp:2339-2426): from (0,0,-1) towards a
    random interior point of triangle (0,0,0),(1,0,0),(0,1,0)."""
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    rng = np.random.default_rng(seed)
    u = rng.random(n, dtype=np.float32)
    v = rng.random(n, dtype=np.float32)
    su = np.sqrt(u)
    v = v * su
    u = np.float32(1.0) - su
    edge = (u < 0.001) | (v < 0.001) | (u + v > 0.999)
    u[edge] = np.float32(0.333)
    v[edge] = np.float32(0.333)
    a, b, c = verts[1], verts[2], verts[0]
    to = c + u[:, None] * (a - c) + v[:, None] * (b - c)
    frm = np.array([0, 0, -1], np.float32)
    rays = R.make_rayhits(np.broadcast_to(frm, (n, 3)), to - frm)
    return verts, np.array([[0, 1, 2]], np.uint32), rays, u, v


def check_triangle_hit(rays, u, v, verts):
    """TriangleHitTest's assertions (verify.cpp:2397-2419)."""
    tol = 16 * ULP
    assert np.all(rays["geomID"] == 0) and np.all(rays["primID"] == 0)
    assert np.abs(rays["u"] - u).max() <= tol
    assert np.abs(rays["v"] - v).max() <= tol
    assert np.abs(rays["tfar"] - 1.0).max() <= tol
    org = np.stack([rays["org_x"], rays["org_y"], rays["org_z"]], -1)
    d = np.stack([rays["dir_x"], rays["dir_y"], rays["dir_z"]], -1)
    ht = org + rays["tfar"][:, None] * d
    huv = verts[0] + rays["u"][:, None] * (verts[1] - verts[0]) + rays["v"][:, None] * (verts[2] - verts[0])
    assert np.abs(ht - huv).max() <= tol
    Ng = np.stack([rays["Ng_x"], rays["Ng_y"], rays["Ng_z"]], -1)
    assert np.abs(Ng - np.array([0, 0, 1], np.float32)).max() <= tol


def test_triangle_hit_known_answer(oracle):
    verts, idx, rays, u, v = _single_triangle_rays()
    sc = oracle.OracleScene([(0, verts, idx)])
    sc.intersect(rays, nthreads=1)
    check_triangle_hit(rays, u, v, verts)


def test_triangle_hit_occluded_known_answer(oracle):
    verts, idx, rays, _, _ = _single_triangle_rays()
    sc = oracle.OracleScene([(0, verts, idx)])
    r = np.ascontiguousarray(rays)
    sc.occluded(r, nthreads=1)
    assert np.all(r["tfar"] == -np.inf)


def test_moeller_single_matches_formulas(oracle):
    """Hand-checked values of the restated leaf test: a unit right triangle
    hit head-on at its centroid."""
    ok, uvtd, tuv, ng = oracle.moeller1((0, 0, 0), (1, 0, 0), (0, 1, 0), (1 / 3, 1 / 3, -1), (0, 0, 1))
    assert ok
    # Ng = cross(e2, e1) with e1 = v0-v1 = (-1,0,0), e2 = v2-v0 = (0,1,0) -> (0,0,1)
    assert ng == (0.0, 0.0, 1.0)
    assert uvtd[3] == 1.0 and tuv[0] == 1.0
    assert abs(tuv[1] - 1 / 3) < 1e-7 and abs(tuv[2] - 1 / 3) < 1e-7
    # parallel ray: den == 0 -> no hit; hit behind tnear / beyond tfar -> no hit
    assert not oracle.moeller1((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.2, 0.2, -1), (1, 0, 0))[0]
    assert not oracle.moeller1((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.2, 0.2, -1), (0, 0, 1), 0.0, 0.5)[0]
    assert not oracle.moeller1((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.2, 0.2, -1), (0, 0, 1), 1.5, np.inf)[0]
    # tfar is inclusive, tnear exclusive (triangle_intersector_moeller.h:92)
    assert oracle.moeller1((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.2, 0.2, -1), (0, 0, 1), 0.0, 1.0)[0]
    assert not oracle.moeller1((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.2, 0.2, -1), (0, 0, 1), 1.0, 2.0)[0]


@pytest.mark.parametrize("model", ["sphere", "plane"])
def test_watertight(oracle, model):
    """WatertightTest (verify.cpp:2898-2979): rays from inside a closed sphere
    (or towards a plane) must not slip through edges; miss rate <= 2e-5."""
    rng = np.random.default_rng(7)
    pos = np.zeros(3, np.float32)
    n = 20000
    if model == "sphere":
        verts, idx = W.triangle_sphere(pos, 2.0, 50)
        org = pos + (2 * rng.random((n, 3), dtype=np.float32) - 1)
        d = 2 * rng.random((n, 3), dtype=np.float32) - 1
    else:
        verts, idx = W.triangle_plane((pos[0], -6, -6), (0, 0, 12), (0, 12, 0), 50, 50)
        org = np.broadcast_to(np.array([pos[0] - 3, 0, 0], np.float32), (n, 3))
        d = 2 * rng.random((n, 3), dtype=np.float32) - 1
        d[:, 0] = 1.0
    sc = oracle.OracleScene([(0, verts, idx)])
    rays = R.make_rayhits(org, d)
    sc.intersect(rays)
    miss = np.mean(rays["geomID"] == 0xFFFFFFFF)
    assert miss <= 2e-5, miss


def test_inactive_rays_untouched(oracle):
    """InactiveRaysTest (verify.cpp:2838-2896): rays with tnear=+inf, tfar=0
    come back bit-identical, for both queries."""
    verts, idx = W.triangle_sphere((0, 0, 0), 2.0, 50)
    sc = oracle.OracleScene([(0, verts, idx)])
    rng = np.random.default_rng(3)
    n = 1000
    rays = R.make_rayhits(2 * rng.random((n, 3)) - 1, 2 * rng.random((n, 3)) - 1)
    inactive = rng.random(n) < 0.5
    rays["tnear"][inactive] = np.inf
    rays["tfar"][inactive] = 0.0
    before = rays.copy()
    sc.intersect(rays)
    assert R.hits_equal_bits(rays[inactive], before[inactive]).all()
    assert np.all(rays["geomID"][~inactive] == 0)
    r2 = before.copy()
    sc.occluded(r2)
    assert (r2[inactive].view(np.uint8) == before[inactive].view(np.uint8)).all()
    assert np.all(r2["tfar"][~inactive] == -np.inf)


def test_empty_scene(oracle):
    """EmptySceneTest (verify.cpp:1061): queries on an empty scene leave rays untouched."""
    sc = oracle.OracleScene([])
    rays = W.sphere_rays(100)
    before = rays.copy()
    sc.intersect(rays)
    assert (rays.view(np.uint8) == before.view(np.uint8)).all()


def test_invalid_triangles_are_skipped(oracle):
    """scene_triangle_mesh.h:127-147: out-of-range indices and vertices beyond
    FLT_LARGE (or NaN) drop the triangle from the build."""
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2e18, 0, 0], [np.nan, 0, 0]], np.float32)
    idx = np.array([[0, 1, 2], [0, 1, 7], [0, 1, 3], [0, 4, 2], [2, 1, 0]], np.uint32)
    sc = oracle.OracleScene([(5, verts, idx)])
    assert sc.num_prims == 2
    rays = R.make_rayhits([[0.2, 0.2, -1]] * 2, [[0, 0, 1]] * 2)
    sc.intersect(rays)
    assert set(rays["primID"]) <= {0, 4} and np.all(rays["geomID"] == 5)


def test_bvh_matches_brute_force(oracle):
    """The oracle's BVH traversal agrees with a brute-force loop over all
    triangles (identical bits) on a heightfield and a soup."""
    for verts, idx, rays in [
        (*W.heightfield(24), W.camera_rays(48, 48)),
        (*W.gaussian_soup(3000, seed=5), W.sphere_rays(3000, seed=6)),
    ]:
        sc = oracle.OracleScene([(0, verts, idx)])
        a, b = rays.copy(), rays.copy()
        sc.intersect(a)
        sc.brute_intersect(b)
        same = R.hits_equal_bits(a, b)
        # exact ties may legitimately resolve differently; none expected here
        assert same.mean() > 0.999
        for i in np.nonzero(~same)[0]:
            code = sc.adjudicate(rays[i], (a["geomID"][i], a["primID"][i], a["tfar"][i]),
                                 (b["geomID"][i], b["primID"][i], b["tfar"][i]))
            assert code in (1, 2), code
        sa, sb = np.ascontiguousarray(rays.copy()), np.ascontiguousarray(rays.copy())
        sc.occluded(sa)
        sc.brute_occluded(sb)
        assert np.array_equal(sa["tfar"] == -np.inf, sb["tfar"] == -np.inf)


def test_overlapping_geometry_builds(oracle):
    """OverlappingGeometryTest (verify.cpp:1216-1260): a two-triangle plane
    with thousands of copies of its last triangle builds and traces."""
    verts, idx = W.triangle_plane((0, 0, 0), (1, 0, 0), (0, 1, 0), 1, 1)
    idx = np.concatenate([idx, np.repeat(idx[-1:], 2000, 0)])
    sc = oracle.OracleScene([(0, verts, idx)])
    st = sc.stats()
    assert sc.num_prims == idx.shape[0]
    assert st.depth <= 41
    rays = R.make_rayhits([[0.25, 0.25, -1], [0.75, 0.75, -1]], [[0, 0, 1], [0, 0, 1]])
    sc.intersect(rays)
    assert np.all(rays["geomID"] == 0)


def test_sah_statistic_semantics(oracle):
    """bvh_statistics.cpp: SAH = (sum inner areas + sum leaf area*blocks) / root
    area; a single Triangle4 leaf costs exactly 1."""
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    sc = oracle.OracleScene([(0, verts, np.array([[0, 1, 2]], np.uint32))])
    st = sc.stats()
    assert st.num_nodes == 0 and st.num_leaves == 1 and st.sah == pytest.approx(1.0)
    verts, idx = W.heightfield(64)
    st = oracle.OracleScene([(0, verts, idx)]).stats()
    assert st.num_prims == idx.shape[0]
    assert st.sah == pytest.approx((st.node_sah + st.leaf_sah) / ((st.bounds[3] - st.bounds[0]) * (
        (st.bounds[4] - st.bounds[1]) + (st.bounds[5] - st.bounds[2])) + (st.bounds[4] - st.bounds[1]) * (
        st.bounds[5] - st.bounds[2])), rel=1e-5)
    assert 3.0 < st.sah < 20.0


def test_adjudicator_codes(oracle):
    """FP64 adjudication: identical-distance hits are near ties; a clearly
    closer triangle wins."""
    verts = np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1], [0, 0, 2], [1, 0, 2], [0, 1, 2],
                      [0, 0, 1], [1, 0, 1], [0, 1, 1]], np.float32)
    idx = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8]], np.uint32)
    sc = oracle.OracleScene([(0, verts, idx)])
    ray = R.make_rayhits([[0.2, 0.2, 0]], [[0, 0, 1]])[0]
    assert sc.adjudicate(ray, (0, 0, 1.0), (0, 2, 1.0)) == 1   # duplicate triangle: tie
    assert sc.adjudicate(ray, (0, 0, 1.0), (0, 1, 2.0)) == 3   # A closer
    assert sc.adjudicate(ray, (0, 1, 2.0), (0, 0, 1.0)) == 4   # B closer
    assert sc.adjudicate(ray, (0xFFFFFFFF, 0, 0), (0, 0, 1.0)) == 4  # A missed a robust hit


WATERTIGHT_FAR = np.array([148376.0, 1234.0, -223423.0], np.float32)  # verify.cpp:5498


def watertight_rays(model, pos, n, seed):
    """Rays of WatertightTest (verify.cpp:2898-2979)."""
    rng = np.random.default_rng(seed)
    if model == "sphere":
        verts, idx = W.triangle_sphere(pos, 2.0, 500)
        org = pos + (2 * rng.random((n, 3), dtype=np.float32) - 1)
        d = 2 * rng.random((n, 3), dtype=np.float32) - 1
    else:
        verts, idx = W.triangle_plane((pos[0], -6, -6), (0, 0, 12), (0, 12, 0), 500, 500)
        org = np.broadcast_to(np.array([pos[0] - 3, 0, 0], np.float32), (n, 3))
        d = 2 * rng.random((n, 3), dtype=np.float32) - 1
        d[:, 0] = 1.0
    return verts, idx, R.make_rayhits(org, d)


@pytest.mark.parametrize("model", ["sphere", "plane"])
def test_watertight_robust_far_from_origin(oracle, model):
    """The verify suite runs WatertightTest on robust scenes far from the
    origin (verify.cpp:5496-5504): the Pluecker path must stay watertight
    there (miss rate <= 2e-5)."""
    verts, idx, rays = watertight_rays(model, WATERTIGHT_FAR, 50000, 17)
    sc = oracle.OracleScene([(0, verts, idx)], robust=True)
    sc.intersect(rays)
    assert np.mean(rays["geomID"] == 0xFFFFFFFF) <= 2e-5


def test_triangle_hit_known_answer_robust(oracle):
    """TriangleHitTest on a robust scene (Triangle4v + Pluecker)."""
    verts, idx, rays, u, v = _single_triangle_rays()
    sc = oracle.OracleScene([(0, verts, idx)], robust=True)
    sc.intersect(rays, nthreads=1)
    check_triangle_hit(rays, u, v, verts)


def test_robust_bvh_matches_brute_force(oracle):
    verts, idx = W.gaussian_soup(3000, seed=5)
    rays = W.sphere_rays(3000, seed=6)
    sc = oracle.OracleScene([(0, verts, idx)], robust=True)
    a, b = rays.copy(), rays.copy()
    sc.intersect(a)
    sc.brute_intersect(b)
    assert R.hits_equal_bits(a, b).mean() > 0.999
    ok, tuv, ng = oracle.pluecker1((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.25, 0.25, -1), (0, 0, 1))
    assert ok and tuv == (1.0, 0.25, 0.25) and ng == (0.0, 0.0, 1.0)


def test_fp32_hit_and_order_tie(oracle):
    """orc_fp32_hit is the single-triangle test the traversal uses: for every
    closest hit of the oracle's own traversal it accepts the reported triangle
    with the reported t, bit for bit; order_tie holds for a triangle with
    itself and fails against a triangle the ray misses."""
    v, i = W.heightfield(24, seed=2)
    orc = oracle.OracleScene([(0, v, i)])
    rays = W.camera_rays(96, 96)
    ref = rays.copy()
    orc.intersect(ref)
    hits = np.nonzero(ref["geomID"] == 0)[0]
    assert hits.size > 1000
    for k in hits[::7]:
        ok, t = orc.fp32_hit(rays[k], 0, ref["primID"][k])
        assert ok and np.float32(t).view(np.uint32) == ref["tfar"][k].view(np.uint32)
    k = hits[0]
    p = int(ref["primID"][k])
    assert orc.order_tie(rays[k], (0, p), (0, p))
    far = (p + i.shape[0] // 2) % i.shape[0]
    assert not orc.fp32_hit(rays[k], 0, far)[0]
    assert not orc.order_tie(rays[k], (0, p), (0, far))
    assert not orc.order_tie(rays[k], (0, p), (0xFFFFFFFF, 0))
    orc.close()
