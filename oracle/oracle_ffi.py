"""ctypes bridge to the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by `__graft_entry__.smoke()` and
by the CPU-baseline leg of bench.py, always as the checker / the CPU
reference arm, never as part of the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


def build(force=False):
    """Compiles liboracle.so with the committed Makefile."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "liboracle.so"], check=True)
    return LIB_PATH


class OrcStats(ctypes.Structure):
    _fields_ = [("sah", ctypes.c_double), ("node_sah", ctypes.c_double), ("leaf_sah", ctypes.c_double),
                ("num_nodes", ctypes.c_uint64), ("num_leaves", ctypes.c_uint64),
                ("num_blocks", ctypes.c_uint64), ("num_prims", ctypes.c_uint64),
                ("depth", ctypes.c_uint32), ("bounds", ctypes.c_float * 6)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, sz, u, i, f = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint, ctypes.c_int, ctypes.c_float
        L.orc_scene_new.restype = vp
        L.orc_scene_free.argtypes = [vp]
        L.orc_scene_add_mesh.argtypes = [vp, u, vp, sz, u, vp, sz, u]
        L.orc_scene_commit.argtypes = [vp]
        L.orc_scene_commit.restype = ctypes.c_long
        L.orc_scene_stats.argtypes = [vp, ctypes.POINTER(OrcStats)]
        for fn in (L.orc_intersect1M, L.orc_occluded1M):
            fn.argtypes = [vp, vp, u, sz, i]
        for fn in (L.orc_brute_intersect1M, L.orc_brute_occluded1M):
            fn.argtypes = [vp, vp, u, sz]
        L.orc_counters.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
        L.orc_adjudicate.argtypes = [vp, vp, u, u, f, u, u, f, i]
        L.orc_adjudicate.restype = i
        L.orc_fp64_hit.argtypes = [vp, vp, u, u, ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.orc_fp64_hit.restype = i
        L.orc_fp32_hit.argtypes = [vp, vp, u, u, ctypes.POINTER(f)]
        L.orc_fp32_hit.restype = i
        L.orc_moeller1.argtypes = [ctypes.POINTER(f)] * 5 + [f, f] + [ctypes.POINTER(f)] * 3
        L.orc_moeller1.restype = i
        L.orc_scene_set_robust.argtypes = [vp, i]
        L.orc_scene_set_filters.argtypes = [vp, FILTER_FN, FILTER_FN, vp]
        L.orc_pluecker1.argtypes = [ctypes.POINTER(f)] * 5 + [f, f] + [ctypes.POINTER(f)] * 2
        L.orc_pluecker1.restype = i
        L.orc_intersect_instanced.argtypes = [vp, u, vp, vp, vp, vp, u, sz]
        L.orc_occluded_instanced.argtypes = [vp, u, vp, vp, vp, u, sz]
        _lib = L
    return _lib


# int filter(void* user, unsigned geomID, unsigned primID, float u, float v, float t)
FILTER_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_float,
                             ctypes.c_float, ctypes.c_float)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class OracleScene:
    """A committed oracle scene built from (geomID, verts, idx) meshes."""

    def __init__(self, meshes, robust=False):
        L = lib()
        self._h = ctypes.c_void_p(L.orc_scene_new())
        L.orc_scene_set_robust(self._h, 1 if robust else 0)
        self._keep = []
        for gid, verts, idx in meshes:
            verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
            idx = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
            self._keep.append((verts, idx))
            L.orc_scene_add_mesh(self._h, gid, _ptr(verts), 12, verts.shape[0], _ptr(idx), 12, idx.shape[0])
        self.num_prims = L.orc_scene_commit(self._h)

    def set_filters(self, intersect=None, occluded=None):
        """Python callables f(geomID, primID, u, v, t) -> bool (True accepts the
        hit) offered every candidate hit, as the reference's filter callbacks
        are; None removes one."""
        def wrap(fn):
            if fn is None:
                return FILTER_FN()
            return FILTER_FN(lambda _user, g, p, u, v, t: 1 if fn(g, p, u, v, t) else 0)
        self._filters = (wrap(intersect), wrap(occluded))   # kept alive with the scene
        lib().orc_scene_set_filters(self._h, self._filters[0], self._filters[1], None)

    def close(self):
        if self._h:
            lib().orc_scene_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        st = OrcStats()
        lib().orc_scene_stats(self._h, ctypes.byref(st))
        return st

    def intersect(self, rayhits, nthreads=0):
        """In-place closest hit on an RTCRayHit record array."""
        assert rayhits.dtype.itemsize == 80 and rayhits.flags.c_contiguous
        lib().orc_intersect1M(self._h, _ptr(rayhits), rayhits.shape[0], 80, nthreads)
        return rayhits

    def occluded(self, rays, nthreads=0):
        stride = rays.dtype.itemsize
        assert rays.flags.c_contiguous
        lib().orc_occluded1M(self._h, _ptr(rays), rays.shape[0], stride, nthreads)
        return rays

    def brute_intersect(self, rayhits):
        lib().orc_brute_intersect1M(self._h, _ptr(rayhits), rayhits.shape[0], 80)
        return rayhits

    def brute_occluded(self, rays):
        lib().orc_brute_occluded1M(self._h, _ptr(rays), rays.shape[0], rays.dtype.itemsize)
        return rays

    def counters(self):
        c = (ctypes.c_uint64 * 3)()
        lib().orc_counters(c)
        return dict(nodes=c[0], leaves=c[1], tris=c[2])

    def adjudicate(self, ray_in, hitA, hitB, tie_ulps=4):
        """ray_in: one RTCRayHit record as originally submitted.
        hitA/hitB: (geomID, primID, t)."""
        rec = np.ascontiguousarray(np.asarray(ray_in).reshape(1))
        return lib().orc_adjudicate(self._h, _ptr(rec), int(hitA[0]), int(hitA[1]), float(hitA[2]),
                                    int(hitB[0]), int(hitB[1]), float(hitB[2]), int(tie_ulps))

    def fp32_hit(self, ray_in, geomID, primID):
        """(accepted, t) of the reference's single-triangle FP32 test."""
        rec = np.ascontiguousarray(np.asarray(ray_in).reshape(1))
        t = ctypes.c_float()
        ok = lib().orc_fp32_hit(self._h, _ptr(rec), int(geomID), int(primID), ctypes.byref(t))
        return bool(ok), t.value

    def order_tie(self, ray_in, hitA, hitB, max_ulps=2):
        """True when both reported triangles pass the reference's FP32 test for
        the ray with distances at most max_ulps apart (the visiting order
        decides which one a traversal reports)."""
        if int(hitA[0]) == 0xFFFFFFFF or int(hitB[0]) == 0xFFFFFFFF:
            return False
        oa, ta = self.fp32_hit(ray_in, hitA[0], hitA[1])
        ob, tb = self.fp32_hit(ray_in, hitB[0], hitB[1])
        if not (oa and ob):
            return False
        ia = int(np.float32(ta).view(np.int32))
        ib = int(np.float32(tb).view(np.int32))
        return abs(ia - ib) <= max_ulps

    def classify(self, ray_in, hitA, hitB, tie_ulps=4):
        """Class of a ray whose two implementations report different triangles
        (hits are (geomID, primID, t)): 'near_tie' (both hit in FP64, distances within
        tie_ulps FP32 ulps), 'grazing' (within 1e-6 of an edge or of tnear/tfar),
        'fp32_tie' (both pass the reference's FP32 test, distances within 2 ulps: the
        test order decides), else ('fail', adjudicator code)."""
        code = self.adjudicate(ray_in, hitA, hitB, tie_ulps)
        if code == 1:
            return "near_tie"
        if code == 2:
            return "grazing"
        if self.order_tie(ray_in, hitA[:2], hitB[:2]):
            return "fp32_tie"
        return ("fail", int(code))

    def fp64_hit(self, ray_in, geomID, primID):
        rec = np.ascontiguousarray(np.asarray(ray_in).reshape(1))
        t, u, v = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        ok = lib().orc_fp64_hit(self._h, _ptr(rec), geomID, primID, ctypes.byref(t), ctypes.byref(u), ctypes.byref(v))
        return bool(ok), t.value, u.value, v.value


def pluecker1(v0, v1, v2, org, d, tnear=0.0, tfar=float("inf")):
    f3 = ctypes.c_float * 3
    tuv, ng = f3(), f3()
    ok = lib().orc_pluecker1(f3(*v0), f3(*v1), f3(*v2), f3(*org), f3(*d), tnear, tfar, tuv, ng)
    return bool(ok), tuple(tuv), tuple(ng)


def moeller1(v0, v1, v2, org, d, tnear=0.0, tfar=float("inf")):
    f3 = ctypes.c_float * 3
    out4, tuv, ng = (ctypes.c_float * 4)(), f3(), f3()
    ok = lib().orc_moeller1(f3(*v0), f3(*v1), f3(*v2), f3(*org), f3(*d), tnear, tfar, out4, tuv, ng)
    return bool(ok), tuple(out4), tuple(tuv), tuple(ng)


def instanced(top, instances, rays, anyhit=False):
    """Rays (in place) against `top` (an OracleScene or None) and instances
    [(OracleScene, l2w 12 floats column-major, instance geomID)]."""
    n = len(instances)
    scenes = (ctypes.c_void_p * max(n, 1))(*[inst[0]._h.value for inst in instances])
    l2w = np.ascontiguousarray(np.array([inst[1] for inst in instances], np.float32).reshape(-1))
    gids = np.ascontiguousarray(np.array([inst[2] for inst in instances], np.uint32))
    th = top._h if top is not None else None
    stride = rays.dtype.itemsize
    if anyhit:
        lib().orc_occluded_instanced(th, n, scenes, _ptr(l2w), _ptr(rays), rays.shape[0], stride)
    else:
        lib().orc_intersect_instanced(th, n, scenes, _ptr(l2w), _ptr(gids), _ptr(rays), rays.shape[0], stride)
    return rays
