"""Seeded synthetic geometry and the solver configurations the benchmarks run.

Meshes are generated in code as the reference's tests do
(aeros/tests/voxel_headless.cpp:56-108): icosphere (subdivided icosahedron),
UV sphere, box, torus. Random streams use splitmix64 so a seed names the same
geometry on every machine.
"""
from __future__ import annotations

import functools
import math

import numpy as np

from . import capi

MASK64 = (1 << 64) - 1


def splitmix64(seed: int):
    """Infinite splitmix64 stream (Steele, Lea & Flood 2014) of uint64."""
    x = seed & MASK64
    while True:
        x = (x + 0x9E3779B97F4A7C15) & MASK64
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        yield z ^ (z >> 31)


def uniform(gen, lo: float, hi: float) -> float:
    return lo + (hi - lo) * ((next(gen) >> 11) * (1.0 / (1 << 53)))


def uniform_array(seed: int, n: int, lo: float, hi: float, skip: int = 0) -> np.ndarray:
    """Draws skip .. skip+n-1 of the splitmix64(seed) stream as uniform(lo, hi),
    vectorized: the same float64 values as `uniform` on that stream."""
    with np.errstate(over="ignore"):
        k = np.arange(skip + 1, skip + n + 1, dtype=np.uint64)
        z = np.uint64(seed & MASK64) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return lo + (hi - lo) * ((z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53)))


# ---- meshes --------------------------------------------------------------
def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Subdivided icosahedron: 20 * 4**level triangles, vertices on the sphere.
    Returns float32 [ntri, 9]."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, np.int64)
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}
        vl = list(v)

        def mid(a, b):
            k = (a, b) if a < b else (b, a)
            if k not in cache:
                m = vl[a] + vl[b]
                vl.append(m / np.linalg.norm(m))
                cache[k] = len(vl) - 1
            return cache[k]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        v = np.array(vl)
        f = np.array(nf, np.int64)
    v = v * radius + np.asarray(center, np.float64)
    return v[f].reshape(-1, 9).astype(np.float32)


_ICO_FACES = ((0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
              (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
              (6, 2, 10), (8, 6, 7), (9, 8, 1))


@functools.lru_cache(maxsize=4)
def geodesic_unit(n: int):
    """Class-I geodesic sphere of frequency n: every icosahedron face cut
    into n^2 triangles, the points projected radially onto the unit sphere
    (20 n^2 triangles; any count 20 n^2, where subdivision levels give
    20 * 4^level). Returns (vertices [nv, 3] float64, corners [20 n^2, 3]
    int64). A point on an edge is computed once from the edge's lower
    vertex index, so faces share their edge vertices exactly: the mesh is
    closed, as the voxelizer's inside test needs."""
    n = int(n)
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V0 = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
                   (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    V0 /= np.linalg.norm(V0, axis=1, keepdims=True)
    pts = [V0]
    nid = 12
    k = np.arange(1, n, dtype=np.float64)[:, None] / n
    edge_base = {}
    for a, b, c in _ICO_FACES:
        for u, v in ((a, b), (b, c), (a, c)):
            e = (min(u, v), max(u, v))
            if e not in edge_base and n > 1:
                p = V0[e[0]] + (V0[e[1]] - V0[e[0]]) * k
                pts.append(p / np.linalg.norm(p, axis=1, keepdims=True))
                edge_base[e] = nid
                nid += n - 1

    def edge_ids(u, v, steps):
        """Ids of the points u + (v - u) * steps / n (0 < steps < n)."""
        base = edge_base[(min(u, v), max(u, v))]
        return base + (steps - 1 if u < v else n - steps - 1)

    tris = []
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    for a, b, c in _ICO_FACES:
        G = np.full((n + 1, n + 1), -1, np.int64)   # G[i, j]: the point A + (B-A) i/n + (C-A) j/n
        G[0, 0], G[n, 0], G[0, n] = a, b, c
        if n > 1:
            s = np.arange(1, n)
            G[s, 0] = edge_ids(a, b, s)
            G[0, s] = edge_ids(a, c, s)
            G[n - s, s] = edge_ids(b, c, s)
        inner = (i >= 1) & (j >= 1) & (i + j <= n - 1)
        m = int(inner.sum())
        if m:
            ii, jj = i[inner].astype(np.float64)[:, None], j[inner].astype(np.float64)[:, None]
            p = V0[a] + (V0[b] - V0[a]) * ii / n + (V0[c] - V0[a]) * jj / n
            pts.append(p / np.linalg.norm(p, axis=1, keepdims=True))
            G[inner] = np.arange(nid, nid + m)
            nid += m
        up = i + j <= n - 1
        ui, uj = i[up], j[up]
        tris.append(np.stack([G[ui, uj], G[ui + 1, uj], G[ui, uj + 1]], axis=1))
        dn = i + j <= n - 2
        di, dj = i[dn], j[dn]
        tris.append(np.stack([G[di + 1, dj], G[di + 1, dj + 1], G[di, dj + 1]], axis=1))
    verts = np.concatenate(pts)
    corners = np.concatenate(tris)
    verts.flags.writeable = False
    corners.flags.writeable = False
    return verts, corners


def perturbed_geodesic(n: int, radius: float, center, seed: int, radial: float = 0.15,
                       axis_scale=(0.5, 1.5)) -> np.ndarray:
    """Geodesic sphere of frequency n (20 n^2 triangles) with vertex radii
    scaled by U(1-radial, 1+radial) and axes by U(axis_scale), as
    perturbed_icosphere. Returns float32 [ntri, 9]."""
    uniq, corners = geodesic_unit(n)
    scales = uniform_array(seed, 3, axis_scale[0], axis_scale[1])
    rad = uniform_array(seed, len(uniq), 1.0 - radial, 1.0 + radial, skip=3)
    pts = uniq * rad[:, None] * scales[None, :] * radius + np.asarray(center, np.float64)
    return pts[corners].reshape(-1, 9).astype(np.float32)


def face_normals(tris: np.ndarray, center=None) -> np.ndarray:
    """Per-vertex normals as an STL file carries them: each triangle's unit
    face normal (FP64 cross product of its FP32 vertices) on its three
    vertices, 9 floats per triangle. With `center`, oriented away from it."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    if center is not None:
        out = np.einsum("ij,ij->i", n, t.mean(axis=1) - np.asarray(center, np.float64)) < 0
        n[out] = -n[out]
    return np.repeat(n[:, None, :], 3, axis=1).astype(np.float32).reshape(-1, 9)


@functools.lru_cache(maxsize=8)
def _unit_icosphere_vertices(level: int):
    """Distinct vertices of the unit icosphere and each triangle corner's index."""
    base = icosphere(level, 1.0).reshape(-1, 3).astype(np.float64)
    uniq, inv = np.unique(base.round(9), axis=0, return_inverse=True)
    uniq.flags.writeable = False
    inv = inv.reshape(-1)
    inv.flags.writeable = False
    return uniq, inv


def perturbed_icosphere(level: int, radius: float, center, seed: int, radial: float = 0.15,
                        axis_scale=(0.5, 1.5)) -> np.ndarray:
    """Icosphere whose vertex radii are scaled by U(1-radial, 1+radial) and whose
    axes are scaled by U(axis_scale) — the batched design-sweep obstacle."""
    uniq, inv = _unit_icosphere_vertices(level)
    scales = uniform_array(seed, 3, axis_scale[0], axis_scale[1])
    rad = uniform_array(seed, len(uniq), 1.0 - radial, 1.0 + radial, skip=3)
    pts = uniq * rad[:, None] * scales[None, :] * radius + np.asarray(center, np.float64)
    return pts[inv].reshape(-1, 9).astype(np.float32)


def uv_sphere(r: float, n_lat: int, n_lon: int, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """UV sphere as aeros/tests/voxel_headless.cpp:56-72 builds it (float32 trig)."""
    tris = []
    pi = np.float32(math.pi)

    def P(i, j):
        th = pi * np.float32(i) / np.float32(n_lat)
        ph = np.float32(2.0) * pi * np.float32(j) / np.float32(n_lon)
        return np.array([r * np.sin(th) * np.cos(ph), r * np.cos(th), r * np.sin(th) * np.sin(ph)], np.float32)

    for i in range(n_lat):
        for j in range(n_lon):
            a, b, c, d = P(i, j), P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)
            if i > 0:
                tris.append(np.concatenate([a, b, d]))
            if i + 1 < n_lat:
                tris.append(np.concatenate([b, c, d]))
    return (np.array(tris, np.float32).reshape(-1, 3) + np.asarray(center, np.float32)).reshape(-1, 9)


def box(half, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    x, y, z = half
    p = np.array([(-x, -y, -z), (x, -y, -z), (x, y, -z), (-x, y, -z), (-x, -y, z), (x, -y, z), (x, y, z), (-x, y, z)],
                 np.float32) + np.asarray(center, np.float32)
    faces = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (3, 7, 6, 2), (0, 4, 7, 3), (1, 2, 6, 5)]
    tris = []
    for a, b, c, d in faces:
        tris.append(np.concatenate([p[a], p[b], p[c]]))
        tris.append(np.concatenate([p[a], p[c], p[d]]))
    return np.array(tris, np.float32)


def torus(R: float, r: float, nu: int, nv: int) -> np.ndarray:
    tris = []

    def P(i, j):
        u = 2 * math.pi * i / nu
        w = 2 * math.pi * j / nv
        return np.array([(R + r * math.cos(w)) * math.cos(u), r * math.sin(w), (R + r * math.cos(w)) * math.sin(u)],
                        np.float32)

    for i in range(nu):
        for j in range(nv):
            a, b, c, d = P(i, j), P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)
            tris.append(np.concatenate([a, b, c]))
            tris.append(np.concatenate([a, c, d]))
    return np.array(tris, np.float32)


# ---- solver configurations ---------------------------------------------------
def channel_mask(nx: int, ny: int, nz: int) -> np.ndarray:
    """Solid rows y = 0 and y = ny-1 (aeros/tests/physics_ref_headless.cpp:75-79)."""
    m = np.zeros((nz, ny, nx), np.uint8)
    m[:, 0, :] = capi.AEROS_CELL_SOLID
    m[:, ny - 1, :] = capi.AEROS_CELL_SOLID
    return m


def poiseuille(nx=64, ny=32, nz=32, tau=0.8, force=1e-6, storage="fp32"):
    """Plain BGK Poiseuille channel: x, z periodic, walls y = 0 and y = ny-1,
    Guo body force, fluid at rest. Returns (params, mask)."""
    p = capi.make_params(nx, ny, nz, tau=tau, periodic_x=True, periodic_z=True, u_in=(0.08, 0.0, 0.0),
                         u_init=(0.0, 0.0, 0.0), body_force=(force, 0.0, 0.0), vel_scale=1.0 / 0.08, storage=storage)
    return p, channel_mask(nx, ny, nz)


def poiseuille_exact(ny: int, tau: float, force: float) -> np.ndarray:
    """u(y) = F/(2 nu) (H^2/4 - (y - yc)^2), H = ny - 2, yc = (ny-1)/2, for y in 1..ny-2."""
    nu = (tau - 0.5) / 3.0
    H = ny - 2.0
    yc = 0.5 * (ny - 1)
    y = np.arange(1, ny - 1, dtype=np.float64)
    return force / (2.0 * nu) * (0.25 * H * H - (y - yc) ** 2)


SPHERE_GRID = (240, 120, 115)
SPHERE_CENTER = (60.0, 60.0, 57.5)
SPHERE_RADIUS = 12.0


def sphere_config(storage="fp32", u_in=0.05, re=100.0, smag=0.1, grid=SPHERE_GRID, center=SPHERE_CENTER,
                  radius=SPHERE_RADIUS, level=6, mask=None):
    """External flow past a sphere: TRT + Smagorinsky, inlet on x = 0,
    zero-gradient outlet, free-slip lateral walls. tau from Re with D = 2r
    (aeros/tests/validation_headless.cpp:119). Returns (params, mask, tris)."""
    nx, ny, nz = grid
    D = 2.0 * radius
    tau = 0.5 + 3.0 * u_in * D / re
    tris = None
    if mask is None:
        from .solver import voxel_grid, voxelize
        tris = icosphere(level, radius, center)
        mask = voxelize(tris, voxel_grid((nx, ny, nz), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)))
    p = capi.make_params(nx, ny, nz, tau=tau, smagorinsky_c=smag, les=True, trt=True, convective_outlet=False,
                         u_in=(u_in, 0.0, 0.0), vel_scale=1.0 / u_in, storage=storage,
                         lateral_bc=capi.AEROS_LATERAL_FREESLIP, outlet_bc=capi.AEROS_OUTLET_ZEROGRAD)
    return p, np.asarray(mask, np.uint8).reshape(nz, ny, nx), tris


BATCH_SIZES = ((32, 32, 32), (64, 32, 32), (96, 48, 48), (128, 64, 64), (160, 80, 80))


def batch_domain(i: int, storage="fp16", u_in=0.04, level=4, smag=0.1, sizes=BATCH_SIZES, re_range=(50.0, 400.0)):
    """Domain i of the batched design sweep: size drawn from `sizes`, one
    perturbed icosphere (radius ny/6, vertex radii x U(0.85, 1.15), axis
    scales U(0.5, 1.5)) at (nx/3, ny/2, nz/2), Re ~ U(re_range) on the channel
    height ny, TRT + Smagorinsky, uniform inlet, zero-gradient outlet, free-slip
    lateral walls. Returns (params, mask, info)."""
    from .solver import voxel_grid, voxelize
    g = splitmix64(i)
    nx, ny, nz = sizes[min(len(sizes) - 1, int(uniform(g, 0.0, float(len(sizes)))))]
    re = uniform(g, re_range[0], re_range[1])
    tau = 0.5 + 3.0 * u_in * ny / re
    tris = perturbed_icosphere(level, ny / 6.0, (nx / 3.0, ny / 2.0, nz / 2.0), seed=1000 + i)
    mask = voxelize(tris, voxel_grid((nx, ny, nz), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)))
    p = capi.make_params(nx, ny, nz, tau=tau, smagorinsky_c=smag, les=True, trt=True, u_in=(u_in, 0.0, 0.0),
                         vel_scale=1.0 / u_in, storage=storage, lateral_bc=capi.AEROS_LATERAL_FREESLIP,
                         outlet_bc=capi.AEROS_OUTLET_ZEROGRAD)
    return p, np.asarray(mask, np.uint8).reshape(nz, ny, nx), dict(re=re, size=(nx, ny, nz), tau=tau, tris=len(tris))


def rb_config(ra: float, nx=128, nz=128, fluid_rows=32, pr=0.71, tau=0.56, storage="fp32"):
    """Rayleigh-Benard: the reference's vertical axis is y (thermal_lbm.cpp:60-65),
    so the config's 128 x 128 x 32 (z up) maps to nx = 128, ny = 32 + 2 wall
    rows, nz = 128, periodic in x and z, hot wall y = 0, cold wall y = ny-1."""
    ny = fluid_rows + 2
    p = capi.make_params(nx, ny, nz, tau=tau, periodic_x=True, periodic_z=True, u_in=(0.08, 0.0, 0.0),
                         u_init=(0.0, 0.0, 0.0), vel_scale=1.0 / 0.08, storage=storage)
    nu = np.float32((np.float32(tau) - np.float32(0.5)) * np.float32(1.0 / 3.0))
    tp = capi.make_thermal(rayleigh=ra, prandtl=pr, fixed_wall_temps=True, hot=0.5, cold=-0.5, perturbation=0.0,
                           nu_lb=float(nu))
    return p, channel_mask(nx, ny, nz), tp


def rb_initial_T(nx, ny, nz, ra: float, amp: float = 1e-3, hot=0.5, cold=-0.5) -> np.ndarray:
    """Linear conduction profile between the walls plus U(-amp, amp) noise from
    splitmix64(0x5EED + Ra) on the fluid rows."""
    noise = uniform_array(0x5EED + int(ra), nx * (ny - 2) * nz, -amp, amp).astype(np.float32)
    T = np.zeros((nz, ny, nx), np.float32)
    T[:, 0, :] = hot
    T[:, ny - 1, :] = cold
    y = np.arange(1, ny - 1, dtype=np.float32)
    prof = hot + (cold - hot) * (y - 0.5) / np.float32(ny - 2)
    T[:, 1:ny - 1, :] = prof[None, :, None] + noise.reshape(nz, ny - 2, nx)
    return T
