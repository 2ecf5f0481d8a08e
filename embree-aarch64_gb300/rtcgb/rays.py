"""Ray/hit record layouts shared by the tests, the bench and the ctypes binding.

The layouts are the reference's `RTCRay` (48 B), `RTCHit` (32 B) and
`RTCRayHit` (80 B) from include/embree3/rtcore_ray.h:11-49 (one instance level).
"""
import numpy as np

RTC_INVALID_GEOMETRY_ID = 0xFFFFFFFF

RAYHIT_DTYPE = np.dtype([
    ("org_x", "<f4"), ("org_y", "<f4"), ("org_z", "<f4"), ("tnear", "<f4"),
    ("dir_x", "<f4"), ("dir_y", "<f4"), ("dir_z", "<f4"), ("time", "<f4"),
    ("tfar", "<f4"), ("mask", "<u4"), ("id", "<u4"), ("flags", "<u4"),
    ("Ng_x", "<f4"), ("Ng_y", "<f4"), ("Ng_z", "<f4"), ("u", "<f4"), ("v", "<f4"),
    ("primID", "<u4"), ("geomID", "<u4"), ("instID", "<u4"),
], align=False)
assert RAYHIT_DTYPE.itemsize == 80

RAY_DTYPE = np.dtype([
    ("org_x", "<f4"), ("org_y", "<f4"), ("org_z", "<f4"), ("tnear", "<f4"),
    ("dir_x", "<f4"), ("dir_y", "<f4"), ("dir_z", "<f4"), ("time", "<f4"),
    ("tfar", "<f4"), ("mask", "<u4"), ("id", "<u4"), ("flags", "<u4"),
])
assert RAY_DTYPE.itemsize == 48


def make_rayhits(org, dirs, tnear=0.0, tfar=np.inf):
    """Builds an RTCRayHit array the way the reference's tutorials do
    (mask -1, geomID/primID/instID invalid, hit fields zero)."""
    org = np.asarray(org, np.float32).reshape(-1, 3)
    dirs = np.asarray(dirs, np.float32).reshape(-1, 3)
    n = org.shape[0]
    r = np.zeros(n, RAYHIT_DTYPE)
    r["org_x"], r["org_y"], r["org_z"] = org[:, 0], org[:, 1], org[:, 2]
    r["dir_x"], r["dir_y"], r["dir_z"] = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    r["tnear"] = tnear
    r["tfar"] = tfar
    r["mask"] = 0xFFFFFFFF
    r["geomID"] = RTC_INVALID_GEOMETRY_ID
    r["primID"] = RTC_INVALID_GEOMETRY_ID
    r["instID"] = RTC_INVALID_GEOMETRY_ID
    return r


def make_rays(org, dirs, tnear=0.0, tfar=np.inf):
    """RTCRay array (occlusion queries)."""
    rh = make_rayhits(org, dirs, tnear, tfar)
    r = np.zeros(rh.shape[0], RAY_DTYPE)
    for name in RAY_DTYPE.names:
        r[name] = rh[name]
    return r


def hits_equal_bits(a, b, fields=("tfar", "Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID")):
    """Per-ray boolean: all listed fields bit-identical."""
    ok = np.ones(a.shape[0], bool)
    for f in fields:
        ok &= a[f].view(np.uint32) == b[f].view(np.uint32)
    return ok
