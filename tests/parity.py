"""Ray-by-ray comparison of two implementations of rtcIntersect1M / rtcOccluded1M
(the GPU library against the reference's own outputs, or against the oracle).

Rules (the parity bar of this path):
  * geomID/primID identical, except rays whose two reported triangles form a tie,
    counted by class; the classes and the unexplained failures add up to the
    number of differing rays:
      near_tie  both triangles are hit in FP64 and their FP64 distances agree
                within TIE_ULPS (4) FP32 ulps;
      fp32_tie  both triangles pass the reference's own single-triangle FP32 test
                for the ray (triangle_intersector_moeller.h:62-104 / the Pluecker
                test in robust scenes) with distances at most 2 ulps apart: the
                test accepts T <= absDen * tfar before dividing, so the order in
                which a traversal tests them decides;
      grazing   the contested hit lies within 1e-6 (barycentric) of a triangle
                edge, or within 1e-6 relative of the ray's tnear / tfar.
    A ray where one side is simply closer in FP64 is NOT accepted: it is a failure.
  * where both report the same triangle, t/u/v agree within REL_TOL = 1e-6
    relative (against the oracle they are bit-identical: same arithmetic; the
    reference's rcp is a hardware estimate + Newton step, so against the
    reference they differ by an ulp or two); Ng is compared the same way;
  * rays that miss come back bit-identical to their input;
  * occlusion flags identical, except where the contested triangle is a near tie
    or grazing case.
"""
import numpy as np

from rtcgb import rays as R

INVALID = 0xFFFFFFFF
TIE_ULPS = 4
REL_TOL = 1e-6
CLASSES = ("near_tie", "fp32_tie", "grazing")


def classify(orc_scene, ray_in, hit_a, hit_b, tie_ulps=TIE_ULPS):
    """Class of one ray whose two reported hits (geomID, primID, t) differ:
    'near_tie', 'fp32_tie', 'grazing', or ('fail', adjudicator code)."""
    return orc_scene.classify(ray_in, hit_a, hit_b, tie_ulps)


def compare_closest(orc_scene, rays_in, got, ref, tie_ulps=TIE_ULPS, rel_tol=REL_TOL):
    """Compares closest-hit records `got` (the implementation under test) with `ref`
    (the reference's outputs, or the oracle's) for the input records `rays_in`.
    Returns a report; report['failures'] lists the unexplained rays."""
    same_id = (got["geomID"] == ref["geomID"]) & (got["primID"] == ref["primID"])
    rep = dict(n=int(rays_in.shape[0]), hits=int((ref["geomID"] != INVALID).sum()),
               id_mismatch=int((~same_id).sum()), failures=[])
    for c in CLASSES:
        rep[c] = 0
    for i in np.nonzero(~same_id)[0]:
        c = classify(orc_scene, rays_in[i], (got["geomID"][i], got["primID"][i], got["tfar"][i]),
                     (ref["geomID"][i], ref["primID"][i], ref["tfar"][i]), tie_ulps)
        if isinstance(c, tuple):
            rep["failures"].append((int(i), c[1]))
        else:
            rep[c] += 1
    assert sum(rep[c] for c in CLASSES) + len(rep["failures"]) == rep["id_mismatch"]
    both = same_id & (ref["geomID"] != INVALID)
    fields = ("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "instID")
    bits_equal = R.hits_equal_bits(got[both], ref[both], fields)
    rep["same_hit_bit_identical"] = int(bits_equal.sum())
    rep["same_hit_bit_differs"] = int((~bits_equal).sum())
    rep["max_rel_tuv"] = 0.0
    if rep["same_hit_bit_differs"]:
        g, r = got[both][~bits_equal], ref[both][~bits_equal]
        rel = max(float(np.max(np.abs(g[f].astype(np.float64) - r[f]) / np.maximum(np.abs(r[f]), 1e-30)))
                  for f in ("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z"))
        rep["max_rel_tuv"] = rel
        if rel > rel_tol:
            rep["failures"].append(("tuv", rel))
        if not np.array_equal(g["instID"], r["instID"]):
            rep["failures"].append(("instID", int((g["instID"] != r["instID"]).sum())))
    miss = (got["geomID"] == INVALID) & (ref["geomID"] == INVALID)
    untouched = (got[miss].view(np.uint8).reshape(-1, 80) == rays_in[miss].view(np.uint8).reshape(-1, 80)).all(1)
    if not untouched.all():
        rep["failures"].append(("miss_modified", int((~untouched).sum())))
    return rep


def compare_occluded(orc_scene, rays_in, got, ref, gpu_scene=None, tie_ulps=TIE_ULPS):
    """Occlusion flags of `got` against `ref`: identical except where the contested
    triangle (the closest hit inside the shadow interval, found by the oracle and by
    `gpu_scene`) is a near tie or grazing case."""
    og, orr = got["tfar"] == -np.inf, ref["tfar"] == -np.inf
    bad = np.nonzero(og != orr)[0]
    rep = dict(n=int(rays_in.shape[0]), occluded=int(orr.sum()), flag_mismatch=int(bad.size), near_tie=0,
               grazing=0, failures=[])
    if bad.size:
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
                                        (a["geomID"][k], a["primID"][k], a["tfar"][k]), tie_ulps)
            if code == 1:
                rep["near_tie"] += 1
            elif code == 2:
                rep["grazing"] += 1
            else:
                rep["failures"].append((int(i), code))
    untouched = ~og
    same = got[untouched].view(np.uint8) == rays_in[untouched].view(np.uint8)
    if not np.all(same):
        rep["failures"].append(("unoccluded_modified", 1))
    return rep


def assert_clean(rep):
    assert not rep["failures"], rep
