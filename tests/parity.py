"""Ray-by-ray comparison of the GPU library with the CPU oracle.

Rules (the parity bar of this path):
  * geomID/primID identical, except rays the FP64 adjudicator classifies as a
    near tie (both triangles hit at the same distance within `tie_ulps` FP32
    ulps), a grazing hit (within 1e-6 of an edge or an interval end), a case
    where the GPU's triangle is genuinely closer, or an FP32 order tie (both
    triangles pass the reference's FP32 test with distances <= 2 ulps apart:
    the test accepts T <= absDen * tfar before dividing, so the visiting
    order decides);
  * where both report the same triangle, t/u/v/Ng are bit-identical (the
    arithmetic is the same); the documented tolerance is 1e-6 relative;
  * rays that miss come back bit-identical to their input;
  * occlusion flags identical, disagreements only at grazing hits.
"""
import numpy as np

from rtcgb import rays as R

INVALID = 0xFFFFFFFF
TIE_ULPS = 16
REL_TOL = 1e-6


def compare_closest(orc_scene, rays_in, gpu, ref, tie_ulps=TIE_ULPS):
    """Returns a report dict; report['failures'] lists unexplained rays."""
    same_id = (gpu["geomID"] == ref["geomID"]) & (gpu["primID"] == ref["primID"])
    rep = dict(n=int(rays_in.shape[0]), hits=int((ref["geomID"] != INVALID).sum()),
               id_mismatch=int((~same_id).sum()), near_tie=0, grazing=0, gpu_closer=0, order_tie=0, failures=[])
    for i in np.nonzero(~same_id)[0]:
        code = orc_scene.adjudicate(rays_in[i], (gpu["geomID"][i], gpu["primID"][i], gpu["tfar"][i]),
                                    (ref["geomID"][i], ref["primID"][i], ref["tfar"][i]), tie_ulps)
        if code == 1:
            rep["near_tie"] += 1
        elif code == 2:
            rep["grazing"] += 1
        elif code == 3:
            rep["gpu_closer"] += 1
        elif orc_scene.order_tie(rays_in[i], (gpu["geomID"][i], gpu["primID"][i]), (ref["geomID"][i], ref["primID"][i])):
            rep["order_tie"] += 1
        else:
            rep["failures"].append((int(i), code))
    both = same_id & (ref["geomID"] != INVALID)
    fields = ("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "instID")
    bits_equal = R.hits_equal_bits(gpu[both], ref[both], fields)
    rep["same_hit_bit_identical"] = int(bits_equal.sum())
    rep["same_hit_bit_differs"] = int((~bits_equal).sum())
    if rep["same_hit_bit_differs"]:
        g, r = gpu[both][~bits_equal], ref[both][~bits_equal]
        rel = max(float(np.max(np.abs(g[f] - r[f]) / np.maximum(np.abs(r[f]), 1e-30))) for f in ("tfar", "u", "v"))
        rep["max_rel_tuv"] = rel
        if rel > REL_TOL:
            rep["failures"].append(("tuv", rel))
    miss = (gpu["geomID"] == INVALID) & (ref["geomID"] == INVALID)
    untouched = (gpu[miss].view(np.uint8).reshape(-1, 80) == rays_in[miss].view(np.uint8).reshape(-1, 80)).all(1)
    if not untouched.all():
        rep["failures"].append(("miss_modified", int((~untouched).sum())))
    return rep


def compare_occluded(orc_scene, rays_in, gpu, ref, gpu_scene=None):
    """Occlusion flags: identical except grazing cases (checked in FP64 with
    the closest hit of the disagreeing implementation)."""
    og, orr = gpu["tfar"] == -np.inf, ref["tfar"] == -np.inf
    bad = np.nonzero(og != orr)[0]
    rep = dict(n=int(rays_in.shape[0]), occluded=int(orr.sum()), flag_mismatch=int(bad.size), grazing=0,
               failures=[])
    if bad.size:
        # closest hit within the shadow interval identifies the contested triangle
        rh = np.zeros(bad.size, R.RAYHIT_DTYPE)
        for name in R.RAY_DTYPE.names:
            rh[name] = rays_in[name][bad]
        rh["geomID"] = INVALID
        rh["primID"] = INVALID
        a = rh.copy()
        orc_scene.intersect(a)
        b = rh.copy()
        if gpu_scene is not None:
            gpu_scene.intersect(b)
        for k, i in enumerate(bad):
            code = orc_scene.adjudicate(rh[k], (b["geomID"][k], b["primID"][k], b["tfar"][k]),
                                        (a["geomID"][k], a["primID"][k], a["tfar"][k]), TIE_ULPS)
            if code in (1, 2):
                rep["grazing"] += 1
            else:
                rep["failures"].append((int(i), code))
    untouched = ~og
    same = gpu[untouched].view(np.uint8) == rays_in[untouched].view(np.uint8)
    if not np.all(same):
        rep["failures"].append(("unoccluded_modified", 1))
    return rep


def assert_clean(rep):
    assert not rep["failures"], rep
