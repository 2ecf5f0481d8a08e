"""The C ABI without a GPU: the library builds, loads, exports every entry
point that include/*.h declares, and the record layouts match the reference's
(include/embree3/rtcore_ray.h:11-49, rtcore_common.h:88-224)."""
import os
import re
import subprocess
import textwrap

import numpy as np
import pytest

from rtcgb import build
from rtcgb import rays as R

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(REPO, "include")


def declared_symbols():
    names = set()
    for f in os.listdir(INC):
        if f.endswith(".h"):
            txt = open(os.path.join(INC, f)).read()
            names.update(re.findall(r"^RTC_API\s+[^;(]*?\b(rtc\w+)\s*\(", txt, re.M))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    declared = declared_symbols()
    assert len(declared) >= 55
    missing = declared - exported
    assert not missing, missing
    # nothing but the API leaks out of the library
    extra = {s for s in exported if s.startswith("rtc")} - declared
    assert not extra, extra


def test_library_loads_without_gpu():
    import ctypes
    lib = ctypes.CDLL(build.build())
    for name in declared_symbols():
        assert hasattr(lib, name)


def test_ctypes_binding_covers_all_symbols():
    from rtcgb import api
    assert set(api.EXPORTS) == declared_symbols()


LAYOUT_C = textwrap.dedent(r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "rtcore_gb300.h"
    #include "rtcore_gb300_ext.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n",
             sizeof(struct RTCRay), sizeof(struct RTCHit), sizeof(struct RTCRayHit),
             offsetof(struct RTCRayHit, hit), offsetof(struct RTCRay, tfar),
             offsetof(struct RTCHit, primID), offsetof(struct RTCHit, geomID),
             offsetof(struct RTCHit, instID), sizeof(struct RTCIntersectContext),
             sizeof(struct RTCBounds), _Alignof(struct RTCRay));
      return 0;
    }
""")


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_layout(tmp_path, lang):
    src = tmp_path / ("layout.c" if lang == "c" else "layout.cpp")
    src.write_text(LAYOUT_C.replace("_Alignof", "alignof") if lang == "c++" else LAYOUT_C)
    exe = tmp_path / "layout"
    cc = "gcc" if lang == "c" else "g++"
    subprocess.run([cc, "-Wall", "-Werror", "-I", INC, str(src), "-o", str(exe)], check=True)
    vals = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    assert vals == [48, 32, 80, 48, 32, 20, 24, 28, 24, 32, 16]
    assert R.RAYHIT_DTYPE.fields["tfar"][1] == 32
    assert R.RAYHIT_DTYPE.fields["primID"][1] == 48 + 20
    assert R.RAYHIT_DTYPE.fields["geomID"][1] == 48 + 24


def test_drop_in_include_path(tmp_path):
    """A program written against <embree3/rtcore.h> compiles unchanged."""
    src = tmp_path / "prog.cpp"
    src.write_text(textwrap.dedent("""
        #include <embree3/rtcore.h>
        int main() {
          RTCDevice d = rtcNewDevice(nullptr);
          RTCScene s = rtcNewScene(d);
          RTCGeometry g = rtcNewGeometry(d, RTC_GEOMETRY_TYPE_TRIANGLE);
          rtcAttachGeometry(s, g); rtcReleaseGeometry(g); rtcCommitScene(s);
          RTCIntersectContext ctx; rtcInitIntersectContext(&ctx);
          RTCRayHit rh; rtcIntersect1M(s, &ctx, &rh, 1, sizeof(rh));
          rtcReleaseScene(s); rtcReleaseDevice(d); return 0;
        }
    """))
    subprocess.run(["g++", "-c", "-Wall", "-I", INC, str(src), "-o", str(tmp_path / "prog.o")], check=True)


PACKET_C = textwrap.dedent("""
    #include <stdio.h>
    #include <stddef.h>
    #include "rtcore_gb300.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",
             sizeof(struct RTCRayHit4), sizeof(struct RTCRayHit8), sizeof(struct RTCRayHit16),
             sizeof(struct RTCRay4), sizeof(struct RTCRay8), sizeof(struct RTCRay16),
             offsetof(struct RTCRayHit8, hit), offsetof(struct RTCRay16, tfar),
             offsetof(struct RTCHit8, geomID), _Alignof(struct RTCRay4), _Alignof(struct RTCRay8),
             _Alignof(struct RTCRay16));
      printf("%zu %zu %zu\\n", sizeof(struct RTCRayNp), sizeof(struct RTCHitNp), offsetof(struct RTCRayHitNp, hit));
      return 0;
    }
""")


def test_packet_layouts(tmp_path):
    """RTCRayHit4/8/16 and the pointer-SOA structs have the reference's SOA layout
    (include/embree3/rtcore_ray.h:51-213): 20 fields of K lanes, 12 for rays."""
    src = tmp_path / "packets.c"
    src.write_text(PACKET_C)
    exe = tmp_path / "packets"
    subprocess.run(["gcc", "-Wall", "-Werror", "-I", INC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert list(map(int, out[0].split())) == [320, 640, 1280, 192, 384, 768, 384, 512, 192, 16, 32, 64]
    assert list(map(int, out[1].split())) == [96, 64, 96]
    # the numpy SOA packing used by the tests follows the same layout
    rh = R.make_rayhits(np.arange(15, dtype=np.float32).reshape(5, 3), np.ones((5, 3), np.float32))
    soa = R.to_soa(rh, 4)
    assert soa.shape == (2, 20 * 4)
    assert soa.view(np.float32)[0, 2 * 4 + 1] == rh["org_z"][1]
    back = R.from_soa(soa, 4, 5, R.RAYHIT_DTYPE)
    assert (back.view(np.uint8) == rh.view(np.uint8)).all()


SOA_HELPERS_CPP = textwrap.dedent("""
    #include <embree3/rtcore.h>
    #include <cstdio>
    // the way filter callbacks read their arguments
    static void cutout(const RTCFilterFunctionNArguments* args) {
      for (unsigned i = 0; i < args->N; i++)
        if (RTCHitN_u(args->hit, args->N, i) < 0.5f) args->valid[i] = 0;
    }
    int main() {
      RTCRayHitNt<4> p{};
      for (int i = 0; i < 4; i++) {
        p.ray.tfar[i] = 1.0f + i; p.ray.id[i] = 30 + i;
        p.hit.u[i] = 0.25f * i; p.hit.primID[i] = 10 + i; p.hit.instID[0][i] = 20 + i;
      }
      RTCRayHitN* rh = (RTCRayHitN*)&p;
      RTCRayN* r = RTCRayHitN_RayN(rh, 4);
      RTCHitN* h = RTCRayHitN_HitN(rh, 4);
      RTCRayHit one = rtcGetRayHitFromRayHitN(rh, 4, 2);
      RTCHit last = rtcGetHitFromHitN(h, 4, 3);
      last.primID = 99;
      rtcCopyHitToHitN(h, &last, 4, 0);
      int valid[4] = {-1, -1, -1, -1};
      RTCFilterFunctionNArguments args = {valid, nullptr, nullptr, r, h, 4};
      cutout(&args);
      std::printf("%g %u %u %u %g %u %u %d %d %d %d\\n", RTCRayN_tfar(r, 4, 1), RTCHitN_primID(h, 4, 2),
                  one.hit.instID[0], one.ray.id, one.ray.tfar, p.hit.primID[0], RTCHitN_instID(h, 4, 0, 0),
                  valid[0], valid[1], valid[2], valid[3]);
      return 0;
    }
""")


def test_soa_helpers_for_filter_callbacks(tmp_path):
    """The C++ RTCRayN / RTCHitN accessors and packet templates of the reference's
    include/embree3/rtcore_ray.h:219-375 compile against the drop-in header and
    address the SOA layout (field f of lane i at f * N + i)."""
    src = tmp_path / "soa.cpp"
    src.write_text(SOA_HELPERS_CPP)
    exe = tmp_path / "soa"
    subprocess.run(["g++", "-Wall", "-Werror", "-I", INC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    # lane 0 now holds lane 3's hit (u = 0.75, kept); lane 1 has u = 0.25 (rejected)
    assert out == ["2", "12", "22", "32", "3", "99", "23", "-1", "0", "-1", "-1"]


def test_autotune_config_strings():
    """Autotuner candidates become rtcNewDevice configuration strings."""
    from rtcgb import autotune
    s = autotune.config_string({"gpu.leaf_max": 2, "gpu.morton": "cube", "gpu.ploc_radius": 4}, "gpu.device=0")
    assert s == "gpu.device=0,gpu.leaf_max=2,gpu.morton=cube,gpu.ploc_radius=4"
    assert all(set(c) == {"gpu.leaf_max", "gpu.morton", "gpu.ploc_radius", "gpu.morton_bits"} for c in autotune.CANDIDATES)
    assert {c["gpu.morton_bits"] for c in autotune.CANDIDATES} == {63, 30}
