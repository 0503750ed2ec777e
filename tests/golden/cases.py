"""Parity cases shared by the golden-fixture generator and the tests.

Each case is a small grid the reference finishes in well under a second per
hundred steps; ``make_golden.py`` runs it through the reference's own solver
(oracle/_ref) and records SHA-256 digests of every output field, and the
tests rerun it through the oracle (CPU) and the CUDA library (GPU).
Geometry is built in code as the reference's headless tests do.
"""
from __future__ import annotations

import hashlib

import numpy as np

from aeros_gb300 import capi


def sphere_mask(nx, ny, nz, cx, cy, cz, r) -> np.ndarray:
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx]
    return (((x + 0.5 - cx) ** 2 + (y + 0.5 - cy) ** 2 + (z + 0.5 - cz) ** 2) <= r * r).astype(np.uint8)


def channel(nx, ny, nz) -> np.ndarray:
    m = np.zeros((nz, ny, nx), np.uint8)
    m[:, 0, :] = 1
    m[:, ny - 1, :] = 1
    return m


# name -> dict(grid, solid, ground_rows, u_init, steps, harness kwargs, thermal)
CASES = {
    "channel_bgk": dict(grid=(16, 34, 8), solid=lambda: channel(16, 34, 8), u_init=(0.0, 0.0, 0.0), steps=600,
                        kw=dict(tau=0.65, u0=0.0, periodic_x=True, periodic_z=True, body_force=(7.8e-6, 0.0, 0.0))),
    "channel_trt": dict(grid=(16, 34, 8), solid=lambda: channel(16, 34, 8), u_init=(0.0, 0.0, 0.0), steps=600,
                        kw=dict(tau=0.65, u0=0.0, trt=True, periodic_x=True, periodic_z=True,
                                body_force=(7.8e-6, 0.0, 0.0))),
    "channel_force3": dict(grid=(16, 16, 12), solid=lambda: channel(16, 16, 12), u_init=(0.0, 0.0, 0.0), steps=200,
                           kw=dict(tau=0.7, u0=0.0, trt=True, les=True, smag=0.15, periodic_x=True, periodic_z=True,
                                   body_force=(1e-5, 2e-6, -3e-6), flow_speed=5.0)),
    "sphere_bgk_conv": dict(grid=(40, 24, 24), solid=lambda: sphere_mask(40, 24, 24, 12, 12, 12, 4), steps=150,
                            kw=dict(tau=0.56, u0=0.08, convective=True, flow_speed=20.0)),
    "sphere_trt_les_conv": dict(grid=(40, 24, 24), solid=lambda: sphere_mask(40, 24, 24, 12, 12, 12, 4), steps=150,
                                kw=dict(tau=0.536, u0=0.05, les=True, trt=True, smag=0.1, convective=True,
                                        flow_speed=20.0)),
    "sphere_les_ground_copy": dict(grid=(40, 24, 24), solid=lambda: sphere_mask(40, 24, 24, 12, 12, 12, 4),
                                   ground_rows=2, steps=100,
                                   kw=dict(tau=0.56, u0=0.08, les=True, flow_speed=10.0)),
    "sphere_minus_x": dict(grid=(40, 24, 24), solid=lambda: sphere_mask(40, 24, 24, 26, 12, 12, 4), steps=80,
                           kw=dict(tau=0.56, u0=0.08, les=True, trt=True, convective=True, flow_axis=0, flow_sign=-1)),
    "sphere_plus_y": dict(grid=(24, 40, 24), solid=lambda: sphere_mask(24, 40, 24, 12, 12, 12, 4), steps=80,
                          kw=dict(tau=0.56, u0=0.08, les=True, convective=True, flow_axis=1, flow_sign=1)),
    "sphere_minus_z_perx": dict(grid=(24, 24, 40), solid=lambda: sphere_mask(24, 24, 40, 12, 12, 20, 4), steps=80,
                                kw=dict(tau=0.56, u0=0.08, les=True, convective=True, flow_axis=2, flow_sign=-1)),
    "rb_small": dict(grid=(32, 18, 8), solid=lambda: channel(32, 18, 8), u_init=(0.0, 0.0, 0.0), steps=400,
                     kw=dict(tau=0.65, u0=0.0, periodic_x=True, periodic_z=True),
                     thermal=dict(rayleigh=2500.0, prandtl=1.0, fixed=True, hot=1.0, cold=0.0, perturbation=0.02)),
    "rb_pm": dict(grid=(32, 18, 8), solid=lambda: channel(32, 18, 8), u_init=(0.0, 0.0, 0.0), steps=200,
                  kw=dict(tau=0.6, u0=0.0, periodic_x=True, periodic_z=True),
                  thermal=dict(rayleigh=5000.0, prandtl=0.71, fixed=True, hot=0.5, cold=-0.5, perturbation=0.05)),
    "thermal_body": dict(grid=(24, 18, 16), solid=lambda: np.maximum(channel(24, 18, 16),
                                                                     sphere_mask(24, 18, 16, 12, 9, 8, 3)),
                         u_init=(0.0, 0.0, 0.0), steps=150,
                         kw=dict(tau=0.6, u0=0.0, periodic_x=True, periodic_z=False),
                         thermal=dict(rayleigh=20000.0, prandtl=1.0, fixed=True, hot=1.0, cold=0.0,
                                      perturbation=0.02)),
}


def thermal_diffusion_T(nx, ny, nz) -> np.ndarray:
    T = np.zeros((nz, ny, nx), np.float32)
    T[:] = (0.5 + 0.5 * np.cos(2 * np.pi / nx * np.arange(nx))).astype(np.float32)
    return T


CASES["thermal_diffusion"] = dict(grid=(32, 16, 8), solid=lambda: np.zeros((8, 16, 32), np.uint8), steps=200,
                                  kw=dict(tau=0.65, u0=0.0, periodic_x=True, periodic_z=True),
                                  thermal=dict(rayleigh=0.0, prandtl=1.0, fixed=False, hot=1.0, cold=0.0,
                                               perturbation=0.0),
                                  upload=lambda: thermal_diffusion_T(32, 16, 8))


def solver_mask(case) -> np.ndarray:
    nx, ny, nz = case["grid"]
    m = case["solid"]().astype(np.uint8).reshape(nz, ny, nx).copy()
    g = case.get("ground_rows", 0)
    if g:
        ground = np.zeros_like(m)
        ground[:, :g, :] = 1
        m = np.where((m == 0) & (ground == 1), capi.AEROS_CELL_GROUND, m).astype(np.uint8)
    return m


def params_for(case, u_in, storage="fp32"):
    """LbmParams equal to the reference's set-up of the case; u_in is the inlet
    velocity the reference derived (recorded in the golden file)."""
    kw = case["kw"]
    nx, ny, nz = case["grid"]
    u_in = np.asarray(u_in, np.float32)
    mag = np.float32(np.sqrt(np.float32(u_in[0] * u_in[0] + u_in[1] * u_in[1] + u_in[2] * u_in[2])))
    if not np.isfinite(mag) or mag < 1e-6:
        mag = np.float32(0.08)
    vs = np.float32(np.float32(kw.get("flow_speed", 1.0)) / mag)
    if not np.isfinite(vs) or vs > 1000.0:
        vs = np.float32(20.0)
    if vs < 0.01:
        vs = np.float32(0.01)
    return capi.make_params(nx, ny, nz, tau=kw.get("tau", 0.6), smagorinsky_c=kw.get("smag", 0.12),
                            les=kw.get("les", False), trt=kw.get("trt", False),
                            periodic_x=kw.get("periodic_x", False), periodic_z=kw.get("periodic_z", False),
                            convective_outlet=kw.get("convective", False), flow_axis=kw.get("flow_axis", 0),
                            flow_sign=kw.get("flow_sign", 1), u_in=u_in,
                            u_init=case.get("u_init", u_in), body_force=kw.get("body_force", (0.0, 0.0, 0.0)),
                            vel_scale=float(vs), storage=storage)


def thermal_params_for(case, tau):
    t = case["thermal"]
    nu = np.float32((np.float32(tau) - np.float32(0.5)) * np.float32(1.0 / 3.0))
    return capi.make_thermal(rayleigh=t["rayleigh"], prandtl=t["prandtl"], fixed_wall_temps=t["fixed"], hot=t["hot"],
                             cold=t["cold"], perturbation=t["perturbation"], nu_lb=float(nu))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def outputs_digest(fields: dict, f: np.ndarray | None, mask: np.ndarray, T=None, buoy=None) -> dict:
    d = {k: digest(np.asarray(fields[k], np.float32) + np.float32(0.0)) for k in ("rho", "ux", "uy", "uz", "strain", "tke")}
    if f is not None:
        fl = mask.reshape(-1) == 0
        d["f"] = digest(np.ascontiguousarray(f[:, fl]) + np.float32(0.0))
    if T is not None:
        d["T"] = digest(np.asarray(T, np.float32) + np.float32(0.0))
        d["buoy"] = digest(np.asarray(buoy, np.float32) + np.float32(0.0))
    return d


EQ_MOMENT_CASES = [(1.0, 0.0, 0.0, 0.0), (1.0, 0.05, 0.0, 0.0), (0.7, 0.04, -0.03, 0.02), (1.35, -0.02, 0.05, 0.01),
                   (0.55, 0.1, 0.1, 0.0), (1.6, 0.0, 0.0, -0.08), (1.1, 0.28, 0.0, 0.0)]


# ---- readback and post-processing fixtures ------------------------------------
# Cases whose world fields, vorticity / Q / strain and sampler outputs are
# recorded from the reference (tests/golden/post.json); the freestream speed
# they are scaled with; the sample points are drawn from splitmix64.
POST_CASES = ("sphere_trt_les_conv", "channel_force3", "sphere_les_ground_copy", "sphere_plus_y")
POST_FLOW_SPEED = 12.5
POST_NPTS = 300


def post_points(grid, seed: int = 0x9057) -> np.ndarray:
    """Sample points in and around the grid (world units = cells): 60 % of the
    extent around the centre, so some fall outside and next to walls."""
    from aeros_gb300 import geometry
    u = geometry.uniform_array(seed, 3 * POST_NPTS, -1.0, 1.0).reshape(-1, 3)
    g = np.asarray(grid, np.float64)
    return (u * g * 0.6 + g * 0.5).astype(np.float32)


def fdigest(a) -> str:
    """Digest of a float32 array with -0 folded into +0."""
    return digest(np.asarray(a, np.float32) + np.float32(0.0))


# ---- voxel-grid distance field fixtures --------------------------------------
# Meshes voxelized by the reference's buildVoxelGrid (its grid plan, mask and
# distance field, voxel_grid.cpp:224-553); tests/golden/sdf.json keeps the
# mask (packed), the field's digest and the reference samplers' outputs at
# seeded points.
SDF_CASES = {
    "icosphere_l4_res64": dict(mesh=("icosphere", 4), res=64),
    "torus_res80": dict(mesh=("torus", 1.0, 0.3, 48, 24), res=80),
    "box_res48": dict(mesh=("box", (1.0, 0.4, 0.6)), res=48),
    "perturbed_l4_res96": dict(mesh=("perturbed_icosphere", 4, 1.0, (0.0, 0.0, 0.0), 11), res=96),
    # the "binary_exact" STL file of stl_files() as the reference's loadSTL reads it
    "stl_binary_exact_res40": dict(mesh=("stl", "binary_exact"), res=40),
}
SDF_NPTS = 400


def sdf_mesh(case, R=None) -> np.ndarray:
    """The case's triangles; STL cases are read by the reference harness R."""
    from aeros_gb300 import geometry
    kind, *args = case["mesh"]
    if kind == "stl":
        import os
        import tempfile
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, args[0] + ".stl")
            with open(path, "wb") as fh:
                fh.write(stl_files()[args[0]])
            n, v, _ = R.stl_load(path)
        return v.reshape(n, 9)
    return getattr(geometry, kind)(*args)


def sdf_points(lo, hi, seed: int = 0x5DF) -> np.ndarray:
    """Points over the grid box widened by 10 % on each side (some outside)."""
    from aeros_gb300 import geometry
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    u = geometry.uniform_array(seed, 3 * SDF_NPTS, 0.0, 1.0).reshape(-1, 3)
    return (lo - 0.1 * (hi - lo) + u * 1.2 * (hi - lo)).astype(np.float32)


def pack_mask(mask: np.ndarray) -> str:
    import base64
    import zlib
    return base64.b64encode(zlib.compress(np.packbits(np.asarray(mask, np.uint8).reshape(-1)).tobytes(), 9)).decode()


def unpack_mask(s: str, n: int) -> np.ndarray:
    import base64
    import zlib
    return np.unpackbits(np.frombuffer(zlib.decompress(base64.b64decode(s)), np.uint8))[:n].astype(np.uint8)


# ---- STL ingest fixtures -------------------------------------------------------
# Synthetic STL files (bytes built here from seeded meshes); tests/golden/stl.json
# keeps what the reference's loadSTL and stlformat::detect make of each.

def _stl_binary(tris, normals, header=b"aeros-gb300 binary STL", count=None, tail=b""):
    import struct
    tris = np.asarray(tris, np.float32).reshape(-1, 9)
    normals = np.asarray(normals, np.float32).reshape(-1, 3)
    n = tris.shape[0] if count is None else count
    rec = np.zeros(tris.shape[0], dtype=[("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")])
    rec["n"] = normals
    rec["v"] = tris
    return header.ljust(80, b" ")[:80] + struct.pack("<I", n) + rec.tobytes() + tail


def _face_normals(tris):
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    return (n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)).astype(np.float32)


def _stl_ascii(tris, fmt="%.9g", kw=("facet normal", "outer loop", "vertex", "endloop", "endfacet"),
               newline="\n", indent="  ", solid=True, extra_vertices=()):
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    nrm = _face_normals(tris)
    out = ["solid synthetic"] if solid else []
    for t, n in zip(tris, nrm):
        out.append(f"{indent}{kw[0]} " + " ".join(fmt % v for v in n))
        out.append(f"{indent * 2}{kw[1]}")
        for v in t:
            out.append(f"{indent * 3}{kw[2]} " + " ".join(fmt % c for c in v))
        out.append(f"{indent * 2}{kw[3]}")
        out.append(f"{indent}{kw[4]}")
        out.append("")
    for v in extra_vertices:
        out.append(f"{indent}{kw[2]} " + " ".join(fmt % c for c in v))
    if solid:
        out.append("endsolid synthetic")
    return newline.join(out).encode()


def stl_files() -> dict:
    """name -> file bytes."""
    from aeros_gb300 import geometry
    ico3 = geometry.icosphere(3, 1.5, (0.25, -0.5, 2.0))
    ico2 = geometry.icosphere(2, 0.75)
    files = {}
    files["binary_exact"] = _stl_binary(ico3, _face_normals(ico3))
    # "solid" header on a binary file, a tail, normals to fix, a triangle with a NaN vertex
    t = geometry.perturbed_icosphere(2, 1.0, (0.0, 0.0, 0.0), 5).copy()
    n = _face_normals(t) * np.float32(3.5)
    n[0] = np.nan
    n[1] = 0.0
    n[2] = [np.inf, 0.0, 1.0]
    n[3] = [1e-8, 0.0, 0.0]
    t[4, 2] = np.nan
    t[5, 7] = -np.inf
    files["binary_solid_header_tail_fixups"] = _stl_binary(t, n, header=b"solid exported by a CAD tool", tail=b"\0" * 137)
    files["ascii_plain"] = _stl_ascii(ico2)
    files["ascii_mixed_case_crlf"] = _stl_ascii(
        ico2, fmt="%.6e", kw=("Facet Normal", "OUTER LOOP", "VERTEX", "EndLoop", "ENDFACET"), newline="\r\n",
        indent="\t", extra_vertices=[(1.0, 2.0, 3.0), (4.0, 5.0, 6.0)])
    deg = np.array([[0, 0, 0, 1, 1, 1, 2, 2, 2], [0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    files["ascii_no_solid_degenerate"] = _stl_ascii(deg, fmt="%.3f", solid=False)
    nums = "solid n\nfacet normal 0 0 1\nouter loop\nvertex 1.5e-3 -0 +2.25\nvertex .5 7. 1E2\n" \
           "vertex -3.25e+1 0.1 0.2\nendloop\nendfacet\nendsolid n\n"
    files["ascii_number_forms"] = nums.encode()
    files["binary_truncated"] = _stl_binary(ico2[:50], _face_normals(ico2[:50]), count=100)
    files["text_without_keywords"] = b"this is a plain text file\nwith two lines of words\n"
    files["too_small"] = b"solid x"
    return files


# ---- surface-pressure lift and drag fixtures ----------------------------------
# computeLiftDrag (forces.cpp:401-688) of the reference on the post cases'
# stepped states: a level-3 icosphere on the solver's sphere (radius 4 cells
# around (12, 12, 12)) with radial vertex normals, optionally the solver
# mask's distance field, and the aerodynamic options of the reference's globals.
SURFACE_CENTER = (12.0, 12.0, 12.0)
SURFACE_RADIUS = 4.0


def surface_mesh(kind: str = "sphere") -> tuple[np.ndarray, np.ndarray]:
    """(vertices, normals), 9 floats per triangle each. kinds: "sphere";
    "degenerate" adds triangles the pass skips (zero area, NaN first vertex,
    zero normal, NaN second vertex, a 1e-11 sliver) and one whose sample point
    lies outside the grid; "huge" adds a triangle above the 1e6 area limit
    (still counted by the projected area, which then falls back to the box);
    "empty" has none."""
    from aeros_gb300 import geometry
    if kind == "empty":
        z = np.zeros((0, 9), np.float32)
        return z, z
    t = geometry.icosphere(3, SURFACE_RADIUS, SURFACE_CENTER).astype(np.float64).reshape(-1, 9)
    extra = []
    if kind == "degenerate":
        extra = [[12, 12, 17, 12, 12, 17, 12, 12, 17],
                 [np.nan, 1, 1, 1, 2, 1, 1, 1, 2],
                 [12, 17, 12, 13, 17, 12, 12, 17, 13],
                 [12, 12, 20, np.nan, 12, 20, 12, 13, 20],
                 [12, 7, 12, 12 + 1e-6, 7, 12, 12, 7, 12 + 1e-5],
                 [-5, -5, -5, -4, -5, -5, -5, -4, -5]]
    elif kind == "huge":
        extra = [[0, 0, 30, 2000, 0, 30, 0, 2000, 30]]
    if extra:
        t = np.concatenate([t, np.asarray(extra, np.float64)])
    v = t.reshape(-1, 3, 3)
    c = np.asarray(SURFACE_CENTER, np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        n = v - c
        n = n / np.linalg.norm(n, axis=2, keepdims=True)
    n = np.nan_to_num(n, nan=0.0)
    if kind == "degenerate":
        n[-4] = 0.0                       # the zero-normal triangle
        n[-1] = (0.0, 0.0, -1.0)          # the outside one
    return v.astype(np.float32).reshape(-1, 9), n.astype(np.float32).reshape(-1, 9)


SURFACE_DEFAULTS = dict(flow_speed=12.5, azimuth=0.0, elevation=0.0, altitude=0.0, use_real_density=1,
                        auto_ref_area=1, ref_area=1.0, mach_effects=0, ground_effect=0, ground_height=0.0,
                        re_number=1e5, bb_min=(8.0, 8.0, 8.0), bb_max=(16.0, 16.0, 16.0), center=SURFACE_CENTER,
                        max_dim=13.856406)
SURFACE_CASES = {
    "plain": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=False, aero={}),
    "sdf": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=True, aero={}),
    "karman_tsien_m044": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=True,
                              aero=dict(mach_effects=1, flow_speed=150.0)),
    "karman_tsien_wave_m082": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=True,
                                   aero=dict(mach_effects=1, flow_speed=280.0)),
    "wave_m097": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=True, aero=dict(mach_effects=1, flow_speed=330.0)),
    "fixed_area_ground_angles": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=True,
                                     aero=dict(auto_ref_area=0, ref_area=30.0, ground_effect=1, ground_height=3.0,
                                               azimuth=20.0, elevation=10.0)),
    "degenerate": dict(case="sphere_trt_les_conv", mesh="degenerate", sdf=True, aero=dict(azimuth=-35.0)),
    "huge_box_area": dict(case="sphere_trt_les_conv", mesh="huge", sdf=False, aero={}),
    "ground_altitude": dict(case="sphere_les_ground_copy", mesh="sphere", sdf=True,
                            aero=dict(ground_effect=1, ground_height=1.5, altitude=3000.0, use_real_density=0,
                                      elevation=-20.0)),
    "plus_y_low_density": dict(case="sphere_plus_y", mesh="sphere", sdf=True,
                               aero=dict(altitude=11000.0, azimuth=90.0, elevation=60.0, flow_speed=40.0)),
    "no_flow": dict(case="sphere_trt_les_conv", mesh="sphere", sdf=False, aero=dict(flow_speed=0.0)),
    "empty_mesh": dict(case="sphere_trt_les_conv", mesh="empty", sdf=False, aero={}),
}


# computeLBMRefArea (lbm.cpp:2111-2160) settings: (mesh kind, azimuth, elevation, automatic, fixed area)
REF_AREA_CASES = [("sphere", 0.0, 0.0, 1, 1.0), ("sphere", 37.0, -20.0, 1, 1.0), ("degenerate", 90.0, 45.0, 1, 1.0),
                  ("huge", 90.0, 0.0, 1, 1.0), ("empty", 15.0, 5.0, 1, 1.0), ("sphere", 0.0, 0.0, 0, 30.0),
                  ("sphere", 0.0, 0.0, 0, -1.0)]

# computeLBMRe (lbm.cpp:2094-2108) inputs: (air temperature K, air density, flow speed, maxDim, previous aeroReNumber)
RE_CASES = [(288.15, 1.225, 12.5, 13.856406, 0.0), (216.65, 0.3639, 250.0, 40.0, 0.0), (30.0, 1.0, 5.0, 1e-9, 0.0),
            (3000.0, 0.5, 20.0, 2.0, 0.0), (300.0, 1.2, 1e9, 10.0, 0.0), (300.0, 1.2, float("inf"), 10.0, 123.0)]
