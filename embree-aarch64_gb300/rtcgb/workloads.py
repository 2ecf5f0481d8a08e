"""Seeded synthetic scenes and ray sets for the triangle ray-query path.

No public dataset is named for this path, so every input is generated here
from fixed seeds:

  heightfield   256x256-cell grid in [0,1]^2 x z, two triangles per cell with a
                fixed diagonal, z = 4-octave value noise (integer-hash lattice,
                smoothstep interpolation), amplitude 0.1, seed 1.
  camera        pinhole at (0.5,-0.5,0.6) looking at (0.5,0.5,0), up +z,
                60 deg vertical FOV, pixel centres, tnear 0, tfar inf.
  soup          triangle soup whose centroids come from a mixture of 64
                isotropic Gaussians (means U[0,1]^3, sigma log-uniform
                [0.01,0.1]); each vertex = centroid + an edge vector of
                log-uniform length [1e-4,1e-2] and uniform direction.
  sphere rays   origins U[0,1]^3, directions uniform on the sphere.
  shadow rays   from each closest hit toward one point light U[0,1]^3,
                tnear 1e-4, tfar 0.999 * distance; misses become inactive
                rays (tnear = +inf, tfar = 0), which the query leaves untouched.

Small scenes restated from the reference's verify tests (sphere and plane
tessellations of tutorials/common/scenegraph/geometry_creation.cpp:8-35,121-180)
are generated by `triangle_sphere` / `triangle_plane`.
"""
import math

import numpy as np

from .rays import RAYHIT_DTYPE, make_rayhits, make_rays


# --------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------

def _hash_u32(x):
    """Integer hash (lowbias32 style) on uint32 arrays."""
    x = np.asarray(x, np.uint32).copy()
    x ^= x >> np.uint32(16)
    x *= np.uint32(0x7FEB352D)
    x ^= x >> np.uint32(15)
    x *= np.uint32(0x846CA68B)
    x ^= x >> np.uint32(16)
    return x


def _lattice(ix, iy, seed, octave):
    h = _hash_u32(ix.astype(np.uint32) * np.uint32(0x9E3779B1)
                  ^ _hash_u32(iy.astype(np.uint32) + np.uint32((0x632BE5AB * (octave + 1)) & 0xFFFFFFFF))
                  ^ np.uint32(seed * 0x85EBCA77 & 0xFFFFFFFF))
    return h.astype(np.float64) / 4294967295.0


def value_noise(x, y, seed=1, octaves=4):
    """4-octave value noise in [0,1) on float64 coordinates."""
    total = np.zeros_like(x, dtype=np.float64)
    amp, freq, norm = 1.0, 4.0, 0.0
    for o in range(octaves):
        fx, fy = x * freq, y * freq
        ix, iy = np.floor(fx).astype(np.int64), np.floor(fy).astype(np.int64)
        tx, ty = fx - ix, fy - iy
        sx, sy = tx * tx * (3 - 2 * tx), ty * ty * (3 - 2 * ty)
        ixm, iym = ix & 0xFFFFFFFF, iy & 0xFFFFFFFF
        v00 = _lattice(ixm, iym, seed, o)
        v10 = _lattice(ixm + 1, iym, seed, o)
        v01 = _lattice(ixm, iym + 1, seed, o)
        v11 = _lattice(ixm + 1, iym + 1, seed, o)
        a = v00 + (v10 - v00) * sx
        b = v01 + (v11 - v01) * sx
        total += amp * (a + (b - a) * sy)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def heightfield(cells=256, seed=1, amplitude=0.1):
    """(vertices float32 [(cells+1)^2,3], indices uint32 [2*cells^2,3])."""
    n = cells + 1
    g = np.arange(n, dtype=np.float64) / cells
    X, Y = np.meshgrid(g, g, indexing="xy")
    Z = amplitude * value_noise(X, Y, seed=seed)
    verts = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    y, x = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    p00 = (y * n + x).ravel()
    p01 = p00 + 1
    p10 = p00 + n
    p11 = p10 + 1
    tri = np.empty((2 * cells * cells, 3), np.uint32)
    tri[0::2] = np.stack([p00, p01, p10], -1)
    tri[1::2] = np.stack([p11, p10, p01], -1)
    return verts, tri


def _unit_vectors(rng, n):
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], -1)


def gaussian_soup(ntris=4_000_000, seed=11, nclusters=64):
    """Triangle soup: (vertices float32 [3n,3], indices uint32 [n,3])."""
    rng = np.random.default_rng(seed)
    means = rng.uniform(0.0, 1.0, (nclusters, 3))
    sigma = np.exp(rng.uniform(math.log(0.01), math.log(0.1), nclusters))
    which = rng.integers(0, nclusters, ntris)
    cent = means[which] + rng.standard_normal((ntris, 3)) * sigma[which, None]
    verts = np.empty((ntris, 3, 3), np.float64)
    for k in range(3):
        length = np.exp(rng.uniform(math.log(1e-4), math.log(1e-2), ntris))
        verts[:, k, :] = cent + _unit_vectors(rng, ntris) * length[:, None]
    verts = verts.reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * ntris, dtype=np.uint32).reshape(-1, 3)
    return verts, idx


def displace_soup(verts, frame, seed=14, amplitude=0.002):
    """Per-frame displacement of a triangle soup: every triangle moves by
    amplitude * sin(2 pi (frame/60 + x)) along its own random unit normal
    (x = the triangle centroid's x coordinate).  Returns new float32 vertices."""
    v = np.asarray(verts, np.float64).reshape(-1, 3, 3)
    rng = np.random.default_rng(seed)
    nrm = _unit_vectors(rng, v.shape[0])
    x = v[:, :, 0].mean(1)
    off = amplitude * np.sin(2 * math.pi * (frame / 60.0 + x))
    return (v + (off[:, None] * nrm)[:, None, :]).reshape(-1, 3).astype(np.float32)


def triangle_sphere(center=(0.0, 0.0, 0.0), radius=2.0, N=50):
    """UV-sphere tessellation with numPhi=N, numTheta=2N (pole fans)."""
    numPhi, numTheta = N, 2 * N
    cx, cy, cz = center
    verts = np.zeros((numTheta * (numPhi + 1), 3), np.float32)
    rT, rP = np.float32(1.0) / np.float32(numTheta), np.float32(1.0) / np.float32(numPhi)
    for phi in range(numPhi + 1):
        phif = np.float32(phi) * np.float32(math.pi) * rP
        theta = np.arange(numTheta, dtype=np.float32)
        thetaf = theta * np.float32(2.0) * np.float32(math.pi) * rT
        base = phi * numTheta
        verts[base:base + numTheta, 0] = cx + radius * np.sin(phif) * np.sin(thetaf)
        verts[base:base + numTheta, 1] = cy + radius * np.cos(phif)
        verts[base:base + numTheta, 2] = cz + radius * np.sin(phif) * np.cos(thetaf)
    tris = []
    for phi in range(1, numPhi + 1):
        for theta in range(1, numTheta + 1):
            if phi == 1:
                p00 = numTheta - 1
                p10 = phi * numTheta + theta - 1
                p11 = phi * numTheta + theta % numTheta
                tris.append((p10, p00, p11))
            elif phi == numPhi:
                p00 = (phi - 1) * numTheta + theta - 1
                p01 = (phi - 1) * numTheta + theta % numTheta
                p10 = numPhi * numTheta
                tris.append((p10, p00, p01))
            else:
                p00 = (phi - 1) * numTheta + theta - 1
                p01 = (phi - 1) * numTheta + theta % numTheta
                p10 = phi * numTheta + theta - 1
                p11 = phi * numTheta + theta % numTheta
                tris.append((p10, p00, p11))
                tris.append((p01, p11, p00))
    return verts, np.asarray(tris, np.uint32)


def triangle_plane(p0, dx, dy, width, height):
    """Grid of 2*width*height triangles spanning p0 + [0,1]dx + [0,1]dy."""
    p0, dx, dy = (np.asarray(a, np.float32) for a in (p0, dx, dy))
    ys, xs = np.meshgrid(np.arange(height + 1), np.arange(width + 1), indexing="ij")
    fx = (xs.astype(np.float32) / np.float32(width))[..., None]
    fy = (ys.astype(np.float32) / np.float32(height))[..., None]
    verts = (p0 + fx * dx + fy * dy).reshape(-1, 3).astype(np.float32)
    tris = np.empty((2 * width * height, 3), np.uint32)
    k = 0
    for y in range(height):
        for x in range(width):
            p00 = y * (width + 1) + x
            p01 = p00 + 1
            p10 = (y + 1) * (width + 1) + x
            p11 = p10 + 1
            tris[k] = (p00, p01, p10)
            tris[k + 1] = (p11, p10, p01)
            k += 2
    return verts, tris


# --------------------------------------------------------------------------
# rays
# --------------------------------------------------------------------------

def camera_rays(width=1024, height=1024, eye=(0.5, -0.5, 0.6), look=(0.5, 0.5, 0.0),
                up=(0.0, 0.0, 1.0), fov_deg=60.0, tnear=0.0, tfar=np.inf):
    """Pinhole primary rays through pixel centres (row-major, y down)."""
    eye, look, up = (np.asarray(v, np.float64) for v in (eye, look, up))
    w = look - eye
    w /= np.linalg.norm(w)
    u = np.cross(w, up)
    u /= np.linalg.norm(u)
    v = np.cross(u, w)
    th = math.tan(math.radians(fov_deg) * 0.5)
    aspect = width / height
    px = (np.arange(width) + 0.5) / width * 2.0 - 1.0
    py = 1.0 - (np.arange(height) + 0.5) / height * 2.0
    PX, PY = np.meshgrid(px * th * aspect, py * th, indexing="xy")
    d = w[None, None, :] + PX[..., None] * u[None, None, :] + PY[..., None] * v[None, None, :]
    d = d.reshape(-1, 3)
    org = np.broadcast_to(eye, d.shape)
    return make_rayhits(org, d, tnear, tfar)


def sphere_rays(n, seed=12, tnear=0.0, tfar=np.inf):
    """Origins uniform in the unit cube, directions uniform on the sphere."""
    rng = np.random.default_rng(seed)
    org = rng.uniform(0.0, 1.0, (n, 3))
    d = _unit_vectors(rng, n)
    return make_rayhits(org, d, tnear, tfar)


def shadow_rays(hits, seed=13, eps=1e-4):
    """Shadow rays from the closest hits of `hits` (RTCRayHit array) toward a
    point light; misses become inactive rays (tnear=+inf, tfar=0)."""
    rng = np.random.default_rng(seed)
    light = rng.uniform(0.0, 1.0, 3)
    n = hits.shape[0]
    hit = hits["geomID"] != 0xFFFFFFFF
    o = np.stack([hits["org_x"], hits["org_y"], hits["org_z"]], -1).astype(np.float64)
    d = np.stack([hits["dir_x"], hits["dir_y"], hits["dir_z"]], -1).astype(np.float64)
    t = np.where(hit, hits["tfar"], 0.0).astype(np.float64)
    p = o + d * t[:, None]
    to = light[None, :] - p
    dist = np.linalg.norm(to, axis=1)
    dist = np.where(dist > 0, dist, 1.0)
    rays = make_rays(p, to / dist[:, None], eps, 0.999 * dist)
    rays["tnear"] = np.where(hit, np.float32(eps), np.float32(np.inf))
    rays["tfar"] = np.where(hit, (0.999 * dist).astype(np.float32), np.float32(0.0))
    return rays, light


def ao_scene(cells=724, soup_tris=300_000, seed=3):
    """Heightfield (value noise seed 1, amplitude 0.1) plus a Gaussian-mixture
    soup: [(verts, idx) of the heightfield, (verts, idx) of the soup]."""
    return [heightfield(cells), gaussian_soup(soup_tris, seed=seed)]


def hemisphere_rays(hits, per_hit=8, seed=21, tnear=1e-4, tfar=np.inf, record=RAYHIT_DTYPE):
    """Cosine-weighted rays about the geometric normal (facing the incoming
    ray) of every hit of `hits` (RTCRayHit after a closest-hit query):
    `per_hit` rays per hit, in hit order.  Ambient-occlusion rays use a short
    tfar, diffuse bounce rays tfar = inf.  Returns (rays, index of the hit of
    each ray)."""
    rng = np.random.default_rng(seed)
    hit = np.nonzero(hits["geomID"] != 0xFFFFFFFF)[0]
    h = hits[hit]
    o = np.stack([h["org_x"], h["org_y"], h["org_z"]], -1).astype(np.float64)
    d = np.stack([h["dir_x"], h["dir_y"], h["dir_z"]], -1).astype(np.float64)
    p = o + d * h["tfar"].astype(np.float64)[:, None]
    nrm = np.stack([h["Ng_x"], h["Ng_y"], h["Ng_z"]], -1).astype(np.float64)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    nrm *= np.where((nrm * d).sum(1) > 0, -1.0, 1.0)[:, None]
    # orthonormal basis (Duff et al. 2017, "Building an orthonormal basis, revisited")
    sgn = np.where(nrm[:, 2] >= 0, 1.0, -1.0)
    a = -1.0 / (sgn + nrm[:, 2])
    b = nrm[:, 0] * nrm[:, 1] * a
    t1 = np.stack([1.0 + sgn * nrm[:, 0] ** 2 * a, sgn * b, -sgn * nrm[:, 0]], -1)
    t2 = np.stack([b, sgn + nrm[:, 1] ** 2 * a, -nrm[:, 1]], -1)
    n = hit.shape[0] * per_hit
    src = np.repeat(np.arange(hit.shape[0]), per_hit)
    u1, u2 = rng.random(n), rng.random(n)
    r, phi = np.sqrt(u1), 2.0 * np.pi * u2
    lx, ly, lz = r * np.cos(phi), r * np.sin(phi), np.sqrt(np.maximum(0.0, 1.0 - u1))
    dirs = t1[src] * lx[:, None] + t2[src] * ly[:, None] + nrm[src] * lz[:, None]
    rays = make_rayhits(p[src], dirs, tnear, tfar)
    if record is not RAYHIT_DTYPE:
        out = np.zeros(n, record)
        for name in record.names:
            out[name] = rays[name]
        rays = out
    return rays, hit[src]


def config_workload(name, scale=1.0):
    """Named workloads.  Returns dict(verts, idx, rays, label)."""
    if name == "heightfield":
        cells = max(4, int(round(256 * math.sqrt(scale))))
        v, i = heightfield(cells)
        res = max(8, int(round(1024 * math.sqrt(scale))))
        r = camera_rays(res, res)
        return dict(verts=v, idx=i, rays=r,
                    label=f"heightfield {cells}x{cells} ({i.shape[0]} tris), {res}x{res} primary rays")
    if name == "soup":
        ntris = max(16, int(4_000_000 * scale))
        nrays = max(64, int(16_000_000 * scale))
        v, i = gaussian_soup(ntris)
        r = sphere_rays(nrays)
        return dict(verts=v, idx=i, rays=r,
                    label=f"gaussian soup {ntris} tris, {nrays} uniform-sphere rays")
    raise ValueError(name)
