"""Parity against the reference itself, through the fixtures of tests/golden/ (written
by tests/golden/make_golden.py from the reference library compiled from its own
sources): the two small scenes, config 0 (every ray of the 1024^2 view of the 256^2
heightfield), config 0 in robust mode (every 16th ray), and a 100k-ray sample of
config 1 (4M soup, 16M uniform-sphere rays), plus the reference builder's SAH.

CPU tests pin the oracle restatement (oracle/oracle.c) to the reference: the same
parity rule as the GPU (tests/parity.py: ids identical except classified ties, t/u/v
within 1e-6 relative, occlusion flags identical). GPU tests hold the library to the
same rule against the same fixtures. Where the reference library is built here
(oracle/_ref), a further test re-runs it and requires the fixtures bit for bit.
"""
import os
import sys

import numpy as np
import pytest

import refgold
from parity import CLASSES, assert_clean, compare_closest, compare_occluded
from rtcgb import workloads as W

SMALL = refgold.SMALL
# differing ids allowed per fixture, every one of them a classified tie (parity.py)
MAX_TIES = {"small": 5, "heightfield256": 8, "robust": 4, "soup4M": 4}


def _oracle_scene(oracle, case):
    return oracle.OracleScene([(g, v, i) for g, (v, i) in enumerate(case["meshes"])], robust=case["robust"])


def _check_oracle(oracle, case, max_ties):
    orc = _oracle_scene(oracle, case)
    got = case["rays"].copy()
    orc.intersect(got)
    rep = compare_closest(orc, case["rays"], got, case["expected"])
    assert_clean(rep)
    assert rep["id_mismatch"] <= max_ties, rep
    sh = case["shadow"].copy()
    orc.occluded(sh)
    occ = compare_occluded(orc, case["shadow"], sh, _occ_records(case))
    assert_clean(occ)
    assert occ["flag_mismatch"] <= max_ties, occ
    orc.close()
    return rep, occ


def _occ_records(case):
    """The reference's occlusion result as records: tfar = -inf where occluded."""
    r = case["shadow"].copy()
    r["tfar"][case["occluded"]] = -np.inf
    return r


def test_fixtures_present():
    names = sorted(os.listdir(refgold.GOLDEN))
    for n in SMALL + ("ref_heightfield256.npz", "ref_robust_heightfield256.npz", "ref_soup4M_sample.npz",
                      "ref_build_stats.json", "make_golden.py"):
        assert n in names


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference_small(oracle, name):
    case = refgold.small(name)
    rep, occ = _check_oracle(oracle, case, MAX_TIES["small"])
    assert rep["hits"] > 1000 and occ["occluded"] > 900


def test_oracle_matches_reference_heightfield256(oracle):
    case = refgold.heightfield256()
    rep, occ = _check_oracle(oracle, case, MAX_TIES["heightfield256"])
    assert rep["n"] == 1024 * 1024 and rep["hits"] == 376469
    assert occ["occluded"] > 100_000
    # same triangles: Ng bit-identical, t/u/v within the rcp's ulp or two
    assert rep["max_rel_tuv"] <= 1e-6


def test_oracle_matches_reference_robust(oracle):
    case = refgold.heightfield256(robust=True)
    rep, occ = _check_oracle(oracle, case, MAX_TIES["robust"])
    assert rep["hits"] > 20_000 and occ["occluded"] > 5_000


def test_oracle_matches_reference_soup4M_sample(oracle):
    case = refgold.soup4M_sample()
    rep, occ = _check_oracle(oracle, case, MAX_TIES["soup4M"])
    assert rep["hits"] > 40_000 and occ["occluded"] > 40_000


@pytest.mark.parametrize("scene", ["heightfield256", "heightfield724", "soup1M", "ao_scene"])
def test_oracle_builder_sah_equals_reference_builder(oracle, scene):
    """The oracle's binned-SAH builder restatement gives the reference builder's own SAH
    (BENCHMARK_BUILD, kernels/bvh/bvh.cpp:173-179; printed to 6 digits)."""
    meshes = {"heightfield256": lambda: [W.heightfield(256)], "heightfield724": lambda: [W.heightfield(724)],
              "soup1M": lambda: [W.gaussian_soup(1_000_000)], "ao_scene": W.ao_scene}[scene]()
    ref = refgold.build_stats()["scenes"][scene]["sah"]
    orc = oracle.OracleScene([(g, v, i) for g, (v, i) in enumerate(meshes)])
    assert abs(orc.stats().sah - ref) <= 5e-6 * ref, (orc.stats().sah, ref)
    orc.close()


def _ref_ffi():
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(here, "oracle"))
    import ref_ffi
    return ref_ffi


def test_reference_reproduces_fixtures():
    """Re-runs the reference library (where oracle/_ref is built) on the small scenes and
    config 0: the fixtures come back bit for bit."""
    ref_ffi = _ref_ffi()
    if not ref_ffi.available():
        pytest.skip("reference library not built here (oracle/ref.mk needs the reference source tree)")
    for case in [refgold.small(n) for n in SMALL] + [refgold.heightfield256()]:
        sc = ref_ffi.RefScene(case["meshes"], threads=2)
        got = case["rays"].copy()
        sc.intersect(got, nthreads=2)
        assert (got.view(np.uint8) == case["expected"].view(np.uint8)).all()
        sh = case["shadow"].copy()
        sc.occluded(sh, nthreads=2)
        assert np.array_equal(sh["tfar"] == -np.inf, case["occluded"])
        sc.close()


# ---------------------------------------------------------------------------
# the GPU library against the reference
# ---------------------------------------------------------------------------

def _check_gpu(rtc, device, oracle, case, max_ties, soup=None):
    sc = rtc.Scene(device, flags=rtc.RTC_SCENE_FLAG_ROBUST if case["robust"] else 0)
    for v, i in case["meshes"]:
        sc.add_mesh(v, i)
    sc.commit()
    got = case["rays"].copy()
    sc.intersect(got)
    orc = _oracle_scene(oracle, case)
    rep = compare_closest(orc, case["rays"], got, case["expected"])
    assert_clean(rep)
    assert rep["id_mismatch"] <= max_ties, rep
    sh = case["shadow"].copy()
    sc.occluded(sh)
    occ = compare_occluded(orc, case["shadow"], sh, _occ_records(case), gpu_scene=sc)
    assert_clean(occ)
    assert occ["flag_mismatch"] <= max_ties, occ
    print({k: rep[k] for k in ("n", "hits", "id_mismatch", *CLASSES, "max_rel_tuv")},
          {k: occ[k] for k in ("occluded", "flag_mismatch", "near_tie", "grazing")})
    orc.close()
    sc.release()
    return rep, occ


@pytest.mark.gpu
@pytest.mark.parametrize("name", SMALL)
def test_gpu_matches_reference_small(rtc, device, oracle, name):
    _check_gpu(rtc, device, oracle, refgold.small(name), MAX_TIES["small"])


@pytest.mark.gpu
def test_gpu_matches_reference_heightfield256(rtc, device, oracle):
    rep, _ = _check_gpu(rtc, device, oracle, refgold.heightfield256(), MAX_TIES["heightfield256"])
    assert rep["hits"] == 376469


@pytest.mark.gpu
def test_gpu_matches_reference_robust(rtc, device, oracle):
    _check_gpu(rtc, device, oracle, refgold.heightfield256(robust=True), MAX_TIES["robust"])


@pytest.mark.gpu
def test_gpu_matches_reference_soup4M_sample(rtc, device, oracle):
    rep, _ = _check_gpu(rtc, device, oracle, refgold.soup4M_sample(), MAX_TIES["soup4M"])
    assert rep["hits"] > 40_000


@pytest.mark.gpu
@pytest.mark.parametrize("scene", ["heightfield256", "soup4M"])
def test_gpu_builder_sah_within_target_of_reference_builder(rtc, device, scene):
    """SAH of the GPU builder's tree over the reference builder's own SAH on the same
    scene (target: at most 1.15x)."""
    v, i = W.heightfield(256) if scene == "heightfield256" else W.gaussian_soup(4_000_000)
    sc = rtc.Scene(device)
    sc.add_mesh(v, i)
    sc.commit()
    ratio = sc.build_stats()["sah"] / refgold.build_stats()["scenes"][scene]["sah"]
    sc.release()
    print(scene, "SAH ratio", ratio)
    assert ratio <= 1.15
