"""The GPU BVH builder: structural invariants of the 8-wide quantised BVH,
determinism, and SAH quality against the oracle's restatement of the
reference's binned-SAH builder (bvh_statistics.cpp semantics on both)."""
import numpy as np
import pytest

from rtcgb import workloads as W

pytestmark = pytest.mark.gpu


def decode(nodes):
    """80-byte node records -> dict of arrays (layout of csrc/gb_common.h)."""
    n = nodes.shape[0]
    f = nodes[:, 0:12].copy().view(np.float32).reshape(n, 3)
    e = nodes[:, 12:15].astype(np.uint32)
    imask = nodes[:, 15]
    child_base = nodes[:, 16:20].copy().view(np.uint32).reshape(n)
    tri_base = nodes[:, 20:24].copy().view(np.uint32).reshape(n)
    meta = nodes[:, 24:32]
    q = nodes[:, 32:80].reshape(n, 6, 8).astype(np.float64)
    scale = np.ldexp(1.0, e.astype(np.int64) - 127)
    lo = f[:, None, :].astype(np.float64) + q[:, 0:3, :].transpose(0, 2, 1) * scale[:, None, :]
    hi = f[:, None, :].astype(np.float64) + q[:, 3:6, :].transpose(0, 2, 1) * scale[:, None, :]
    return dict(imask=imask, child_base=child_base, tri_base=tri_base, meta=meta, lo=lo, hi=hi)


def check_structure(nodes, tris, verts, idx):
    d = decode(nodes)
    n = nodes.shape[0]
    seen = np.zeros(tris.shape[0], np.int32)
    reached = np.zeros(n, np.int32)
    reached[0] = 1
    prim = tris[:, 3].view(np.uint32)
    for k in range(n):
        internal_rank = 0
        for s in range(8):
            m = int(d["meta"][k, s])
            if m == 0:
                # empty slot: an inverted box, which the traversal's slab test misses
                q = nodes[k, 32:80].reshape(6, 8)[:, s]
                assert np.all(q[0:3] == 255) and np.all(q[3:6] == 0), (k, s, q)
                continue
            lo, hi = d["lo"][k, s], d["hi"][k, s]
            if d["imask"][k] >> s & 1:
                c = d["child_base"][k] + internal_rank
                internal_rank += 1
                assert c < n
                reached[c] += 1
            else:
                assert m & 0x80
                cnt = ((m >> 5) & 3) + 1
                first = d["tri_base"][k] + (m & 31)
                for t in range(first, first + cnt):
                    seen[t] += 1
                    pv = verts[idx[prim[t]]]  # 3x3 vertices of the triangle
                    assert np.all(pv >= lo - 1e-30) and np.all(pv <= hi + 1e-30), (k, s)
    assert np.all(seen == 1)      # every valid triangle exactly once
    assert np.all(reached == 1)   # every node has exactly one parent (root: itself)


def test_structure_and_determinism(rtc, device):
    for verts, idx in (W.heightfield(48), W.gaussian_soup(20000, seed=3), W.triangle_sphere((0, 0, 0), 1.0, 30)):
        sc = rtc.Scene(device)
        sc.add_mesh(verts, idx)
        sc.commit()
        nodes, tris = sc.bvh()
        assert tris.shape[0] == idx.shape[0]
        check_structure(nodes, tris, verts, idx)
        # e1 = v0 - v1, e2 = v2 - v0 exactly as Triangle4 (triangle.h:40-41)
        p = tris[:, 3].view(np.uint32)
        v = verts[idx[p]]
        assert np.array_equal(tris[:, 0:3], v[:, 0])
        assert np.array_equal(tris[:, 4:7], v[:, 0] - v[:, 1])
        assert np.array_equal(tris[:, 8:11], v[:, 2] - v[:, 0])
        sc.commit()
        nodes2, tris2 = sc.bvh()
        assert np.array_equal(nodes, nodes2) and np.array_equal(tris, tris2)


@pytest.mark.parametrize("name,config,limit,leaf", [("heightfield", b"", 1.15, 2), ("heightfield", b"gpu.leaf_max=4", 1.15, 4),
                                                    ("soup", b"", 1.15, 1), ("soup", b"gpu.leaf_max=2", 1.15, 2)])
def test_sah_against_reference_builder(rtc, oracle, name, config, limit, leaf):
    """SAH of the GPU BVH vs the oracle's binned-SAH builder: within the 1.15x
    target at the default settings (radius-1 PLOC, SAH-optimal collapse, leaf
    size by scene shape: 2 for the flat heightfield, 1 for the soup) and with
    other leaf sizes."""
    device = rtc.Device(config)
    if name == "heightfield":
        verts, idx = W.heightfield(256)
    else:
        verts, idx = W.gaussian_soup(500_000, seed=11)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    gpu = sc.build_stats()
    ref = oracle.OracleScene([(0, verts, idx)]).stats()
    ratio = gpu["sah"] / ref.sah
    print(name, "gpu SAH", gpu["sah"], "reference-builder SAH", ref.sah, "ratio", ratio)
    assert gpu["num_prims"] == ref.num_prims
    assert gpu["leaf_max"] == leaf
    assert ratio <= limit
    sc.release()
    device.release()


@pytest.mark.parametrize("config", [b"gpu.collapse=greedy", b"gpu.ploc_radius=2", b"gpu.ploc_radius=4",
                                    b"gpu.ploc_radius=8", b"gpu.ploc_radius=16", b"gpu.morton=axis",
                                    b"gpu.morton=cube", b"gpu.leaf_max=1", b"gpu.leaf_max=3", b"gpu.leaf_max=4",
                                    b"gpu.morton_bits=63", b"gpu.morton_bits=63,gpu.morton=axis"])
def test_builder_options_valid_and_exact(rtc, oracle, config):
    """Every build option (collapse rule, PLOC radius, Morton scaling and key width,
    leaf size) yields a well-formed BVH over every triangle, and closest hits equal
    the oracle's on a heightfield + soup scene."""
    from parity import assert_clean, compare_closest
    device = rtc.Device(config)
    hv, hi = W.heightfield(64, seed=5)
    sv, si = W.gaussian_soup(30_000, seed=6)
    verts = np.concatenate([hv, sv])
    idx = np.concatenate([hi, si + hv.shape[0]]).astype(np.uint32)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    nodes, tris = sc.bvh()
    check_structure(nodes, tris, verts, idx)
    rays = W.sphere_rays(100_000, seed=7)
    g = rays.copy()
    sc.intersect(g)
    r = rays.copy()
    orc = oracle.OracleScene([(0, verts, idx)])
    orc.intersect(r)
    assert_clean(compare_closest(orc, rays, g, r))
    sc.release()
    device.release()


def test_refit_after_displacement(rtc, device, oracle):
    """RTC_BUILD_QUALITY_REFIT geometry whose vertices move (the animated-soup
    displacement) is refitted in place; the refitted BVH contains every
    triangle and its hits equal the oracle's on the displaced mesh."""
    from parity import assert_clean, compare_closest
    verts, idx = W.gaussian_soup(60_000, seed=61)
    rays = W.sphere_rays(200_000, seed=62)
    sc = rtc.Scene(device)
    gid = sc.add_mesh(verts, idx, quality=rtc.RTC_BUILD_QUALITY_REFIT)
    sc.commit()
    assert sc.build_stats()["refit"] == 0
    assert sc.build_stats()["leaf_max"] == 2  # a tree built to be refitted takes 2-triangle leaves
    nodes0, _ = sc.bvh()
    for frame in (1, 7):
        moved = W.displace_soup(verts, frame)
        sc.update_vertices(gid, moved)
        sc.commit()
        st = sc.build_stats()
        assert st["refit"] == 1
        nodes, tris = sc.bvh()
        assert nodes.shape == nodes0.shape
        check_structure(nodes, tris, moved, idx)
        g = rays.copy()
        sc.intersect(g)
        so = oracle.OracleScene([(gid, moved, idx)])
        r = rays.copy()
        so.intersect(r)
        assert_clean(compare_closest(so, rays, g, r))
    # a topology change forces a full build
    sc.update_indices(gid, idx[::-1].copy())
    sc.commit()
    assert sc.build_stats()["refit"] == 0
    # a vertex that becomes invalid cannot be refitted: the commit rebuilds and drops it
    bad = W.displace_soup(verts, 3)
    bad[0] = np.nan
    sc.update_vertices(gid, bad)
    sc.commit()
    st = sc.build_stats()
    assert st["refit"] == 0 and st["num_prims"] == idx.shape[0] - 1
    sc.release()


def _committed(rtc, config, meshes, batched=False):
    device = rtc.Device(config)
    sc = rtc.Scene(device)
    if batched:
        sc.set_batched()
    for v, i in meshes:
        sc.add_mesh(v, i)
    return device, sc


@pytest.mark.parametrize("batched", [False, True], ids=["plain", "batched"])
def test_replayed_rebuild_equals_host_driven_build(rtc, batched):
    """From its second commit with an unchanged layout a scene's rebuilds are replayed
    from a captured build graph (no host reads between the build's phases): the BVH is
    byte-identical to the host-driven build of a device with gpu.graph_rebuild=0, and so
    are the hits; a vertex update between commits is picked up."""
    meshes = ([W.heightfield(40, seed=2), W.gaussian_soup(20_000, seed=4), W.heightfield(24, seed=6)] if batched
              else [W.gaussian_soup(60_000, seed=8)])
    dref, ref = _committed(rtc, b"gpu.graph_rebuild=0", meshes, batched)
    dgr, gr = _committed(rtc, b"", meshes, batched)
    rays = W.sphere_rays(50_000, seed=9)
    start = np.array([0, 20_000, 35_000, 50_000], np.uint32)
    for step in range(4):
        if step == 3:  # move the vertices of geometry 0 (same layout)
            v0 = meshes[0][0] * np.float32(0.97) + np.float32(0.01)
            ref.update_vertices(0, v0)
            gr.update_vertices(0, v0)
        ref.commit()
        gr.commit()
        n1, t1 = ref.bvh()
        n2, t2 = gr.bvh()
        assert np.array_equal(n1, n2) and np.array_equal(t1.view(np.uint32), t2.view(np.uint32)), step
        a, b = rays.copy(), rays.copy()
        if batched:
            ref.intersect_batched(a, start)
            gr.intersect_batched(b, start)
        else:
            ref.intersect(a)
            gr.intersect(b)
        assert (a.view(np.uint8) == b.view(np.uint8)).all()
        sa, sb = ref.build_stats(), gr.build_stats()
        assert sa["num_nodes"] == sb["num_nodes"] and abs(sa["sah"] - sb["sah"]) <= 1e-9 * sa["sah"]
    for s, d in ((ref, dref), (gr, dgr)):
        s.release()
        d.release()


def test_replayed_rebuild_falls_back_when_valid_count_changes(rtc, oracle):
    """A replay whose number of valid triangles differs from the captured plan (here:
    triangles made degenerate by NaN vertices) is detected on the device; the commit
    then builds the host-driven way and the hits still match the oracle."""
    from parity import assert_clean, compare_closest
    v, i = W.gaussian_soup(30_000, seed=12)
    device, sc = _committed(rtc, b"", [(v, i)])
    for _ in range(3):
        sc.commit()
    bad = v.copy()
    bad[: 3 * 500] = np.nan   # the first 500 triangles become invalid
    sc.update_vertices(0, bad)
    sc.commit()
    assert sc.build_stats()["num_prims"] == 30_000 - 500
    rays = W.sphere_rays(40_000, seed=13)
    g = rays.copy()
    sc.intersect(g)
    orc = oracle.OracleScene([(0, bad, i)])
    r = rays.copy()
    orc.intersect(r)
    assert_clean(compare_closest(orc, rays, g, r))
    sc.release()
    device.release()


def test_build_phase_timestamps(rtc):
    """gpu.build_phases=1: a replayed rebuild reports the device time of its eight
    phases (rtcgbGetSceneBuildPhases), which add up to about the build's own time,
    and the tree is the one built without the timestamps."""
    meshes = [W.gaussian_soup(80_000, seed=14)]
    dp, sp = _committed(rtc, b"gpu.build_phases=1", meshes, False)
    dq, sq = _committed(rtc, b"", meshes, False)
    sp.commit()
    sq.commit()
    assert sp.build_phases() == {}  # the first commit is host-driven
    for _ in range(3):
        sp.commit()
        sq.commit()
    ph = sp.build_phases()
    assert list(ph) == list(rtc.Scene.BUILD_PHASES)
    assert all(v >= 0.0 for v in ph.values()) and ph["ploc_rounds"] > 0 and ph["collapse_levels"] > 0
    total_ms = sum(ph.values()) * 1e-3
    assert total_ms <= sp.build_stats()["build_ms"] * 1.05 + 0.05
    n1, t1 = sp.bvh()
    n2, t2 = sq.bvh()
    assert np.array_equal(n1, n2) and np.array_equal(t1.view(np.uint32), t2.view(np.uint32))
    for s, d in ((sp, dp), (sq, dq)):
        s.release()
        d.release()


@pytest.mark.parametrize("config", [b"", b"gpu.morton_bits=63", b"gpu.graph_rebuild=0"])
def test_invalid_triangles_sort_after_the_corner_triangle(rtc, config):
    """Invalid triangles (NaN vertices) get a sort key above every valid one: the
    triangle whose centroid is the largest on all three axes -- the all-ones Morton
    code -- stays in the tree even when invalid triangles precede it."""
    from rtcgb import rays as R
    rng = np.random.default_rng(5)
    base = (rng.random((600, 3, 3)) * 0.8 + 0.05).astype(np.float32)
    bad = np.zeros((10, 3, 3), np.float32)
    bad[:, 0, 0] = np.nan
    corner = np.array([[[0.99, 0.99, 1.0], [1.0, 0.99, 0.99], [0.99, 1.0, 0.99]]], np.float32)
    tris = np.concatenate([bad, base, corner])
    verts = tris.reshape(-1, 3)
    idx = np.arange(verts.shape[0], dtype=np.uint32).reshape(-1, 3)
    device = rtc.Device(config)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    for _ in range(3):  # host-driven, then replayed rebuilds
        sc.commit()
        ray = np.zeros(1, R.RAYHIT_DTYPE)
        ray["org_x"], ray["org_y"], ray["org_z"] = 2.0, 2.0, 2.0
        ray["dir_x"] = ray["dir_y"] = ray["dir_z"] = -1.0
        ray["tnear"], ray["tfar"] = 0.0, np.inf
        ray["mask"] = 0xFFFFFFFF
        ray["geomID"], ray["primID"] = 0xFFFFFFFF, 0xFFFFFFFF
        sc.intersect(ray)
        assert ray["geomID"][0] == 0 and ray["primID"][0] == idx.shape[0] - 1, ray
        assert sc.build_stats()["num_prims"] == idx.shape[0] - 10
    sc.release()
    device.release()
