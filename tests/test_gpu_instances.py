"""Two-level scenes: RTC_GEOMETRY_TYPE_INSTANCE geometries (rtcSetGeometryInstancedScene,
rtcSetGeometryTransform) next to ordinary triangle meshes, against the oracle's
instance restatement.  The ray transform and the world-to-local map are the same
operations on both sides, so hits agree bit for bit."""
import numpy as np
import pytest

from rtcgb import rays as R
from rtcgb import workloads as W

pytestmark = pytest.mark.gpu


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _instances(rng, n):
    """n local-to-world maps (rotation x anisotropic scale + translation), column-major 3x4."""
    out = []
    for _ in range(n):
        m = _rotation(rng) @ np.diag(rng.uniform(0.2, 0.6, 3))
        t = rng.uniform(0.0, 1.0, 3)
        out.append(np.concatenate([m[:, 0], m[:, 1], m[:, 2], t]).astype(np.float32))
    return out


@pytest.fixture(scope="module")
def two_level(rtc, device, oracle):
    rng = np.random.default_rng(17)
    meshes = [W.heightfield(24, seed=3), W.triangle_sphere((0.0, 0.0, 0.0), 0.5, 16), W.gaussian_soup(5000, seed=4)]
    children, ochildren = [], []
    for v, i in meshes:
        c = rtc.Scene(device)
        c.add_mesh(v, i)
        c.commit()
        children.append(c)
        ochildren.append(oracle.OracleScene([(0, v, i)]))
    top = rtc.Scene(device)
    plane = W.triangle_plane((0.0, 0.0, -0.05), (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), 8, 8)
    top.add_mesh(*plane)  # geomID 0: a triangle mesh of the top scene itself
    xfms = _instances(rng, 12)
    insts = []
    for k, x in enumerate(xfms):
        gid = top.add_instance(children[k % 3], x)
        insts.append((ochildren[k % 3], x, gid))
    top.commit()
    otop = oracle.OracleScene([(0, *plane)])
    return top, otop, insts, children


def test_instances_closest_hits_match_oracle(rtc, oracle, two_level):
    top, otop, insts, _ = two_level
    rays = W.sphere_rays(60000, seed=21)
    g, r = rays.copy(), rays.copy()
    top.intersect(g)
    oracle.instanced(otop, insts, r)
    hit = r["geomID"] != 0xFFFFFFFF
    inst_hits = hit & (r["instID"] != 0xFFFFFFFF)
    assert inst_hits.sum() > 1000 and (hit & ~inst_hits).sum() > 100
    ids_same = (g["geomID"] == r["geomID"]) & (g["primID"] == r["primID"]) & (g["instID"] == r["instID"])
    # different triangles at exactly the same distance are ties of the visiting order
    tie = ~ids_same & (g["tfar"].view(np.uint32) == r["tfar"].view(np.uint32))
    assert (ids_same | tie).all(), int((~(ids_same | tie)).sum())
    assert tie.sum() <= 10
    same = ids_same & hit
    for f in ("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z"):
        assert (g[f][same].view(np.uint32) == r[f][same].view(np.uint32)).all(), f
    # world origins and directions are restored after every instance
    for f in ("org_x", "org_y", "org_z", "dir_x", "dir_y", "dir_z", "tnear"):
        assert (g[f].view(np.uint32) == rays[f].view(np.uint32)).all(), f


def test_instances_occlusion_matches_oracle(rtc, oracle, two_level):
    top, otop, insts, _ = two_level
    rays = W.sphere_rays(60000, seed=22, tfar=0.3)
    sh = np.zeros(rays.shape[0], R.RAY_DTYPE)
    for f in R.RAY_DTYPE.names:
        sh[f] = rays[f]
    g, r = sh.copy(), sh.copy()
    top.occluded(g)
    oracle.instanced(otop, insts, r, anyhit=True)
    assert (r["tfar"] < 0).sum() > 1000
    assert ((g["tfar"] < 0) == (r["tfar"] < 0)).all()


def test_transform_formats_round_trip(rtc, device):
    L = rtc.load()
    child = rtc.Scene(device)
    child.add_mesh(*W.heightfield(4))
    child.commit()
    g = L.rtcNewGeometry(device.h, rtc.RTC_GEOMETRY_TYPE_INSTANCE)
    L.rtcSetGeometryInstancedScene(g, child.h)
    cm = np.arange(12, dtype=np.float32) + 1  # columns vx, vy, vz, p
    L.rtcSetGeometryTransform(g, 0, rtc.RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR, cm.ctypes.data)
    rm = np.zeros(12, np.float32)
    L.rtcGetGeometryTransform(g, 0.0, rtc.RTC_FORMAT_FLOAT3X4_ROW_MAJOR, rm.ctypes.data)
    assert (rm.reshape(3, 4) == cm.reshape(4, 3).T).all()
    m4 = np.zeros(16, np.float32)
    L.rtcGetGeometryTransform(g, 0.0, rtc.RTC_FORMAT_FLOAT4X4_COLUMN_MAJOR, m4.ctypes.data)
    assert (m4.reshape(4, 4)[:, :3].ravel() == cm).all() and (m4.reshape(4, 4)[:, 3] == [0, 0, 0, 1]).all()
    L.rtcSetGeometryTransform(g, 0, rtc.RTC_FORMAT_FLOAT3X4_ROW_MAJOR, rm.ctypes.data)
    back = np.zeros(12, np.float32)
    L.rtcGetGeometryTransform(g, 0.0, rtc.RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR, back.ctypes.data)
    assert (back == cm).all()
    assert device.error() == 0
    L.rtcSetGeometryTransform(g, 0, 0x9003, cm.ctypes.data)  # RTC_FORMAT_FLOAT3: not a matrix
    assert device.error() == 3
    L.rtcSetGeometryTransform(g, 1, rtc.RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR, cm.ctypes.data)  # no time step 1
    assert device.error() == 3
    tri = L.rtcNewGeometry(device.h, 0)
    L.rtcSetGeometryTransform(tri, 0, rtc.RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR, cm.ctypes.data)
    assert device.error() == 3
    L.rtcReleaseGeometry(tri)
    L.rtcReleaseGeometry(g)


def test_instanced_scene_changes_need_a_new_commit(rtc, device):
    child = rtc.Scene(device)
    v, i = W.heightfield(16)
    child.add_mesh(v, i)
    child.commit()
    top = rtc.Scene(device)
    top.add_instance(child, [1, 0, 0, 0, 1, 0, 0, 0, 1, 0.0, 0.0, 0.5])
    # an instance with a singular map is never hit; an uncommitted child fails the commit
    top.add_instance(child, [0, 0, 0, 0, 1, 0, 0, 0, 1, 0.0, 0.0, 0.0])
    top.commit()
    rays = W.camera_rays(32, 32)
    out = rays.copy()
    top.intersect(out)
    hit = out["geomID"] != 0xFFFFFFFF
    assert hit.sum() > 30 and (out["instID"][hit] == 0).all()
    child.commit()  # the child's BVH was rebuilt: the top scene must be committed again
    with pytest.raises(rtc.RTCError):
        top.intersect(rays.copy())
    top.commit()
    out2 = rays.copy()
    top.intersect(out2)
    assert (out2.view(np.uint8) == out.view(np.uint8)).all()
    lone = rtc.Scene(device)
    lone.add_mesh(v, i)  # never committed
    bad = rtc.Scene(device)
    bad.add_instance(lone, [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0])
    with pytest.raises(rtc.RTCError):
        bad.commit()
