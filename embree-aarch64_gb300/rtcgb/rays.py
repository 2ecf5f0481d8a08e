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


def to_soa(records, K, stride_words=None):
    """Packs AOS records (RAYHIT_DTYPE or RAY_DTYPE) into packets of K lanes in the SOA
    layout of RTCRayHit4/8/16 and RTCRayHitN (include/embree3/rtcore_ray.h:222-248):
    field f of lane i of packet p is the uint32 at p * stride_words + f * K + i.
    Lanes past the end of `records` are zero.  Returns a (packets, stride_words) uint32 array."""
    nf = records.dtype.itemsize // 4
    n = records.shape[0]
    P = (n + K - 1) // K
    stride_words = stride_words or nf * K
    words = np.zeros((P * K, nf), np.uint32)
    words[:n] = np.ascontiguousarray(records).view(np.uint32).reshape(n, nf)
    out = np.zeros((P, stride_words), np.uint32)
    out[:, :nf * K] = words.reshape(P, K, nf).transpose(0, 2, 1).reshape(P, nf * K)
    return out


def from_soa(packets, K, n, dtype):
    """Inverse of to_soa for the first n lanes."""
    nf = dtype.itemsize // 4
    P = packets.shape[0]
    words = packets[:, :nf * K].reshape(P, nf, K).transpose(0, 2, 1).reshape(P * K, nf)[:n]
    return np.ascontiguousarray(words).view(dtype).reshape(n)
