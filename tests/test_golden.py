"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py
from the oracle): scene buffers, input rays, expected closest-hit records and
occlusion flags for two small seeded scenes.  The oracle must reproduce them
bit for bit (CPU), and the GPU library must match them under the parity rules
(GPU)."""
import glob
import os

import numpy as np
import pytest

from rtcgb import rays as R

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(HERE, "*.npz")))
HIT_FIELDS = ("tfar", "Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID")


def load(path):
    d = np.load(path)
    rays = d["rays"].view(R.RAYHIT_DTYPE).copy()
    shadow = d["shadow_rays"].view(R.RAY_DTYPE).copy()
    expected = rays.copy()
    for f in HIT_FIELDS:
        expected[f] = d["hit_" + f]
    return d["verts"].copy(), d["idx"].copy(), rays, shadow, expected, d["occluded"].copy()


def test_fixtures_present():
    names = [os.path.basename(p) for p in FIXTURES]
    assert names == ["soup_camera40_sphere.npz", "terrain_camera48.npz"]


@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_oracle_reproduces_golden(oracle, path):
    verts, idx, rays, shadow, expected, occluded = load(path)
    orc = oracle.OracleScene([(0, verts, idx)])
    got = rays.copy()
    orc.intersect(got)
    assert (got.view(np.uint8) == expected.view(np.uint8)).all()
    sh = shadow.copy()
    orc.occluded(sh)
    assert np.array_equal(sh["tfar"] == -np.inf, occluded)
    assert (expected["geomID"] != 0xFFFFFFFF).sum() > 1000 and occluded.sum() > 900
    orc.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_gpu_matches_golden(rtc, device, oracle, path):
    from parity import assert_clean, compare_closest
    verts, idx, rays, shadow, expected, occluded = load(path)
    sc = rtc.Scene(device)
    sc.add_mesh(verts, idx)
    sc.commit()
    got = rays.copy()
    sc.intersect(got)
    orc = oracle.OracleScene([(0, verts, idx)])
    rep = compare_closest(orc, rays, got, expected)
    assert_clean(rep)
    assert rep["id_mismatch"] <= 5
    sh = shadow.copy()
    sc.occluded(sh)
    assert np.array_equal(sh["tfar"] == -np.inf, occluded)
    orc.close()
    sc.release()
