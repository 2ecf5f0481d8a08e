"""A C++ host program written against <embree3/rtcore.h> links the library as
libembree3 and runs unchanged: the call sequence of the reference's minimal
tutorial (a device, a scene with one triangle, rtcIntersect1 / rtcOccluded1,
rtcIntersect1M over a small stream, error handling)."""
import os
import subprocess
import textwrap

import pytest

from rtcgb import build

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(REPO, "include")
PKG = os.path.join(REPO, "embree-aarch64_gb300")

PROGRAM = textwrap.dedent(r"""
    #include <embree3/rtcore.h>
    #include <cmath>
    #include <cstdio>
    #include <limits>
    #include <vector>

    static void on_error(void*, RTCError code, const char* msg) { std::printf("error %d %s\n", (int)code, msg); }

    // filter callbacks as Embree programs write them (RTCRayN / RTCHitN accessors)
    static int filter_calls = 0;
    static void reject_odd_ids(const RTCFilterFunctionNArguments* args) {
      filter_calls++;
      for (unsigned i = 0; i < args->N; i++)
        if (RTCRayN_id(args->ray, args->N, i) & 1u) args->valid[i] = 0;
    }
    static void reject_all(const RTCFilterFunctionNArguments* args) {
      filter_calls++;
      for (unsigned i = 0; i < args->N; i++) args->valid[i] = 0;
    }
    static RTCGeometry triangle_at(RTCDevice device, float z) {
      RTCGeometry g = rtcNewGeometry(device, RTC_GEOMETRY_TYPE_TRIANGLE);
      float* v = (float*)rtcSetNewGeometryBuffer(g, RTC_BUFFER_TYPE_VERTEX, 0, RTC_FORMAT_FLOAT3, 3 * sizeof(float), 3);
      unsigned* ix = (unsigned*)rtcSetNewGeometryBuffer(g, RTC_BUFFER_TYPE_INDEX, 0, RTC_FORMAT_UINT3, 3 * sizeof(unsigned), 1);
      v[0] = 0.f; v[1] = 0.f; v[2] = z;  v[3] = 1.f; v[4] = 0.f; v[5] = z;  v[6] = 0.f; v[7] = 1.f; v[8] = z;
      ix[0] = 0; ix[1] = 1; ix[2] = 2;
      rtcCommitGeometry(g);
      return g;
    }

    int main() {
      RTCDevice device = rtcNewDevice(nullptr);
      rtcSetDeviceErrorFunction(device, on_error, nullptr);
      RTCScene scene = rtcNewScene(device);
      RTCGeometry geom = rtcNewGeometry(device, RTC_GEOMETRY_TYPE_TRIANGLE);
      float* v = (float*)rtcSetNewGeometryBuffer(geom, RTC_BUFFER_TYPE_VERTEX, 0, RTC_FORMAT_FLOAT3, 3 * sizeof(float), 3);
      unsigned* ix = (unsigned*)rtcSetNewGeometryBuffer(geom, RTC_BUFFER_TYPE_INDEX, 0, RTC_FORMAT_UINT3, 3 * sizeof(unsigned), 1);
      v[0] = 0.f; v[1] = 0.f; v[2] = 0.f;  v[3] = 1.f; v[4] = 0.f; v[5] = 0.f;  v[6] = 0.f; v[7] = 1.f; v[8] = 0.f;
      ix[0] = 0; ix[1] = 1; ix[2] = 2;
      rtcCommitGeometry(geom);
      unsigned id = rtcAttachGeometry(scene, geom);
      rtcReleaseGeometry(geom);
      rtcCommitScene(scene);
      RTCIntersectContext ctx;
      rtcInitIntersectContext(&ctx);
      RTCRayHit rh;
      rh.ray.org_x = 0.33f; rh.ray.org_y = 0.33f; rh.ray.org_z = -1.f;
      rh.ray.dir_x = 0.f; rh.ray.dir_y = 0.f; rh.ray.dir_z = 1.f;
      rh.ray.tnear = 0.f; rh.ray.tfar = std::numeric_limits<float>::infinity();
      rh.ray.mask = -1; rh.ray.flags = 0; rh.ray.time = 0.f;
      rh.hit.geomID = RTC_INVALID_GEOMETRY_ID; rh.hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
      rtcIntersect1(scene, &ctx, &rh);
      std::printf("hit geom %u prim %u t %.6f u %.4f v %.4f\n", rh.hit.geomID, rh.hit.primID, rh.ray.tfar, rh.hit.u, rh.hit.v);
      RTCRay sh = rh.ray;
      sh.tfar = 2.f;
      rtcOccluded1(scene, &ctx, &sh);
      std::printf("occluded %d\n", sh.tfar == -std::numeric_limits<float>::infinity() ? 1 : 0);
      std::vector<RTCRayHit> stream(1000, rh);
      int hits = 0;
      for (int i = 0; i < 1000; i++) {
        stream[i].ray.org_x = (i % 40) / 40.f;
        stream[i].ray.org_y = (i / 40) / 25.f;
        stream[i].ray.tfar = std::numeric_limits<float>::infinity();
        stream[i].hit.geomID = RTC_INVALID_GEOMETRY_ID;
      }
      rtcIntersect1M(scene, &ctx, stream.data(), 1000, sizeof(RTCRayHit));
      for (const RTCRayHit& r : stream) hits += r.hit.geomID == id;
      std::printf("stream hits %d\n", hits);
      rtcIntersect1M(scene, &ctx, nullptr, 5, sizeof(RTCRayHit));  // invalid argument
      std::printf("last error %d\n", (int)rtcGetDeviceError(device));
      // two stacked triangles; the near one (z = 0) has filter callbacks
      RTCScene layered = rtcNewScene(device);
      RTCGeometry near_g = triangle_at(device, 0.f), far_g = triangle_at(device, 1.f);
      rtcSetGeometryIntersectFilterFunction(near_g, reject_odd_ids);
      rtcSetGeometryOccludedFilterFunction(near_g, reject_all);
      rtcAttachGeometry(layered, near_g);
      rtcAttachGeometry(layered, far_g);
      rtcReleaseGeometry(near_g);
      rtcReleaseGeometry(far_g);
      rtcCommitScene(layered);
      std::vector<RTCRayHit> four(4, rh);
      for (int i = 0; i < 4; i++) {
        four[i].ray.id = i;
        four[i].ray.tfar = std::numeric_limits<float>::infinity();
        four[i].hit.geomID = RTC_INVALID_GEOMETRY_ID;
      }
      rtcIntersect1M(layered, &ctx, four.data(), 4, sizeof(RTCRayHit));
      std::printf("filtered");
      for (const RTCRayHit& r : four) std::printf(" %u:%.3f", r.hit.geomID, r.ray.tfar);
      std::printf("\n");
      RTCRay shadows[2] = {rh.ray, rh.ray};
      shadows[0].tfar = 1.5f;  // reaches only the near triangle, whose occlusion callback rejects
      shadows[1].tfar = 2.5f;  // reaches the far one too
      rtcOccluded1M(layered, &ctx, shadows, 2, sizeof(RTCRay));
      std::printf("filtered occluded %d %d calls %d error %d\n", shadows[0].tfar < 0.f ? 1 : 0,
                  shadows[1].tfar < 0.f ? 1 : 0, filter_calls, (int)rtcGetDeviceError(device));
      rtcReleaseScene(layered);
      rtcReleaseScene(scene);
      rtcReleaseDevice(device);
      return 0;
    }
""")


def test_cpp_host_program_links_and_runs(tmp_path):
    build.build()
    src = tmp_path / "minimal.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "minimal"
    subprocess.run(["g++", "-O1", "-I", INC, str(src), "-o", str(exe), "-L", PKG, "-lembree3",
                    "-Wl,-rpath," + PKG], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True, timeout=300).stdout
    assert out.startswith("hit geom 0 prim 0 t 1.000000 u 0.3300 v 0.3300"), out
    assert "occluded 1" in out
    # rays of the 40 x 25 grid through the triangle x, y >= 0, x + y <= 1; grid
    # points on the triangle's edges may go either way
    inside = edge = 0
    for i in range(1000):
        k, j = i % 40, i // 40
        on_edge = k == 0 or j == 0 or 5 * k + 8 * j == 200
        edge += on_edge
        inside += (not on_edge) and 5 * k + 8 * j < 200
    hits = int(out.split("stream hits ")[1].split()[0])
    assert inside <= hits <= inside + edge, (hits, inside, edge)
    # the callback saw the invalid argument, which also stays set for rtcGetDeviceError
    assert "error 2" in out and "last error 2" in out
    # filter callbacks: odd ray IDs pass through the near triangle to the far one
    assert "filtered 0:1.000 1:2.000 0:1.000 1:2.000" in out, out
    # 4 intersect calls (one per ray's near hit) + 2 occlusion calls (each shadow ray's near hit)
    assert "filtered occluded 0 1 calls 6 error 0" in out, out
