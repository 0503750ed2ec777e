"""The C++17 facade (aeros-engine_gb300/facade): a caller written against the
reference's lbm.h names builds against it (CPU) and gets, through it, the
state the C ABI gives directly (GPU)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "aeros-engine_gb300")
LIB = os.path.join(PKG, "lib")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    import __graft_entry__
    __graft_entry__._paths()
    import build as cuda_build
    cuda_build.build()
    exe = str(tmp_path_factory.mktemp("facade") / "channel_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                           "-I", os.path.join(PKG, "facade"), os.path.join(ROOT, "tests", "facade", "channel_driver.cpp"),
                           "-o", exe, "-L" + LIB, "-laeros_facade", "-laeros_gb300", "-Wl,-rpath," + LIB])
    return exe


@pytest.fixture(scope="module")
def voxel_driver(driver, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("facade_voxel") / "voxel_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                           "-I", os.path.join(PKG, "facade"), os.path.join(ROOT, "tests", "facade", "voxel_driver.cpp"),
                           "-o", exe, "-L" + LIB, "-laeros_facade", "-laeros_gb300", "-Wl,-rpath," + LIB])
    return exe


def test_facade_builds_and_links(driver, voxel_driver):
    assert os.path.exists(driver) and os.path.exists(voxel_driver)


def test_facade_ref_area_equals_reference(driver, tmp_path):
    """computeLBMRefArea through the facade (host FP32) equals the reference's
    own (tests/golden/surface.json) on every setting: frontal areas along
    oblique directions, skipped triangles, the box fallback, the fixed area."""
    import json
    from golden.cases import REF_AREA_CASES, SURFACE_DEFAULTS, surface_mesh
    exe = str(tmp_path / "refarea_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                           "-I", os.path.join(PKG, "facade"), os.path.join(ROOT, "tests", "facade", "refarea_driver.cpp"),
                           "-o", exe, "-L" + LIB, "-laeros_facade", "-laeros_gb300", "-Wl,-rpath," + LIB])
    want = json.load(open(os.path.join(ROOT, "tests", "golden", "surface.json")))["ref_area_cases"]
    d = SURFACE_DEFAULTS
    for (kind, az, el, auto, area), w in zip(REF_AREA_CASES, want):
        v, _ = surface_mesh(kind)
        f = tmp_path / f"{kind}.bin"
        np.ascontiguousarray(v, np.float32).tofile(f)
        args = [exe, str(f), repr(az), repr(el), str(auto), repr(area), *[repr(x) for x in d["bb_min"]],
                *[repr(x) for x in d["bb_max"]], repr(d["max_dim"])]
        got = np.float32(subprocess.check_output(args, text=True).strip())
        assert got == np.float32(w), (kind, az, el, got, w)


def test_facade_reynolds_equals_reference(driver, tmp_path):
    """computeLBMRe through the facade equals the reference's own
    (tests/golden/surface.json): sea level, the stratosphere, the clamps of
    the Sutherland viscosity and of the length, the 1e9 cap, a non-finite
    result falling back to the previous number."""
    import json
    from golden.cases import RE_CASES
    exe = str(tmp_path / "re_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                           "-I", os.path.join(PKG, "facade"), os.path.join(ROOT, "tests", "facade", "re_driver.cpp"),
                           "-o", exe, "-L" + LIB, "-laeros_facade", "-laeros_gb300", "-Wl,-rpath," + LIB])
    want = json.load(open(os.path.join(ROOT, "tests", "golden", "surface.json")))["re_cases"]
    for c, w in zip(RE_CASES, want):
        out = subprocess.check_output([exe, *[repr(float(x)) for x in c]], text=True).split()
        assert [np.float32(v) for v in out] == [np.float32(w)] * 3, (c, out, w)


NPTS = 64   # tests/facade/channel_driver.cpp


@pytest.mark.gpu
def test_facade_channel_equals_c_abi(driver, tmp_path):
    """The facade's globals after stepLBMCPU and computeLBMVorticityAndQ and
    its samplers equal, bit for bit, what the C ABI gives for the same calls:
    a world readback after every stepping call (the residuals compare
    consecutive readbacks), then vorticity / Q / strain, then the samplers."""
    from aeros_gb300 import capi, geometry, solver
    out = tmp_path / "fields.bin"
    r = subprocess.run([driver, "200", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    blob = np.fromfile(out, np.float32)
    n = 64 * 32 * 32
    got = {k: blob[i * n:(i + 1) * n] for i, k in
           enumerate(("ux", "uxw", "uyw", "pressure", "vorticity", "q", "strain"))}
    pos = 7 * n
    pts = blob[pos:pos + 3 * NPTS].reshape(NPTS, 3)
    pos += 3 * NPTS

    p = capi.make_params(64, 32, 32, tau=0.8, periodic_x=True, periodic_z=True, u_in=(0.0, 0.0, 0.0),
                         body_force=(1e-6, 0.0, 0.0), convective_outlet=True)
    wp = capi.make_world(10.0, 1.225, (-3.2, -1.6, -1.6), (0.1, 0.1, 0.1))
    s = solver.Solver(p, geometry.channel_mask(64, 32, 32))
    for k in range(100):
        s.step(1)
        s.world_fields(wp, read=False)
        if (k + 1) % 30 == 0:   # updateLBM's vorticity / Q cadence
            s.vorticity_q(read=False)
    s.step(100)
    world, wst = s.world_fields(wp)
    ref = s.fields()
    vq = s.vorticity_q()
    assert np.array_equal(got["ux"], ref["ux"])
    assert np.array_equal(got["uxw"], world["ux"])
    assert np.array_equal(got["uyw"], world["uy"])
    assert np.array_equal(got["pressure"], world["pressure"])
    for k in ("vorticity", "q", "strain"):
        assert np.array_equal(got[k], vq[k]), k
    st = s.stats()
    assert f"step {st['step']} " in r.stdout
    assert np.float32(r.stdout.split("avg_rho ")[1].split()[0]) == np.float32(st["avg_rho"])
    line = r.stdout.split("pmin ")[1].splitlines()[0].split()
    assert np.float32(line[0]) == np.float32(wst["pressure_min"])
    assert np.float32(line[2]) == np.float32(wst["pressure_max"])
    assert np.float32(line[4]) == np.float32(wst["residual_rho"])
    assert np.float32(line[6]) == np.float32(wst["residual_u"])
    for f in range(8):
        per = 3 if f == capi.AEROS_FIELD_VELOCITY_LB else 1
        v = blob[pos:pos + per * NPTS]
        pos += per * NPTS
        ok = blob[pos:pos + NPTS]
        pos += NPTS
        rv, rok = s.sample(wp, f, pts)
        assert np.array_equal(v, rv.reshape(-1)), f
        assert np.array_equal(ok, rok.astype(np.float32)), f
    # the one-point getters agree with the many-point call (point 20 lies inside)
    probe = r.stdout.split("probe ")[1].splitlines()[0].split()
    pv, pok = s.sample(wp, capi.AEROS_FIELD_PRESSURE, pts[20:21])
    assert probe[3] == "1" and pok[0] == 1 and np.float32(probe[1]) == pv[0]
    wall = np.array([[-3.0, -1.58, 0.0]], np.float32)   # cell (2, 0, 16): the y = 0 wall row
    sv, _ = s.sample(wp, capi.AEROS_FIELD_SOLID, np.concatenate([pts[20:21], wall]))
    assert sv.tolist() == [0.0, 1.0], sv
    assert probe[-2:] == ["0", "1"], r.stdout   # the mid point is fluid, the wall point solid
    # world velocity: the lattice velocity times flowSpeed / 0.08 (no inlet velocity), within 2 flowSpeed
    uv, _ = s.sample(wp, capi.AEROS_FIELD_VELOCITY_LB, pts[20:21])
    world = r.stdout.split("world ")[1].splitlines()[0].split()
    scale = np.float32(10.0) / np.float32(0.08)
    assert np.float32(world[1]) == np.float32(uv[0, 0] * scale)
    assert np.float32(world[3]) == np.float32(uv[0, 1] * scale)
    assert np.float32(world[9]) == np.float32(np.float32(0.1) / scale)   # lbmLatticeDtWorld
    assert np.float32(world[11]) == np.float32(10.0)   # outside the grid: the freestream
    # the self-checks: the channel is initialised and stable, conserves mass, its solid rows are at
    # rest and its fields are bounded; its inlet velocity is zero (a forced channel), which the
    # inlet check rejects as the reference's does
    val = r.stdout.split("validate ")[1].splitlines()[0].split()
    assert val == ["1", "1", "0", "1", "1", "1"], val
    # computeLiftDrag through the facade: the C ABI's surface pass on the same state and mesh
    verts = blob[pos:pos + 108]
    nrms = blob[pos + 108:pos + 216]
    assert pos + 216 == blob.size
    sp = capi.make_surface(velocity=(10.0, 0.0, 0.0), air_temperature=288.15, air_density=1.225,
                           speed_of_sound=340.0, bb_min=(-0.5, -0.5, -0.5), bb_max=(0.5, 0.5, 0.5),
                           center=(0.0, 0.0, 0.0), max_dim=1.7320508, reynolds=3e5)
    so, _ = s.surface_forces(wp, sp, solver.SurfaceMesh(verts, nrms))
    fl = r.stdout.split("forces ")[1].splitlines()[0].split()
    want = [so.drag, so.lift, so.lift_to_drag, so.moment_magnitude, *so.center_of_pressure, so.ref_area]
    got_f = [np.float32(fl[i]) for i in (1, 3, 5, 7, 9, 10, 11, 13)]
    assert got_f == [np.float32(v) for v in want], (got_f, want)
    assert so.drag > 0 and fl[15] == "0"
    from golden.cases import EQ_MOMENT_CASES
    from post_common import GOLD
    eq = [ln.split()[1:] for ln in r.stdout.splitlines() if ln.startswith("eq ")]
    assert len(eq) == len(EQ_MOMENT_CASES)
    for row, ref in zip(eq, GOLD["eq_moments"]):
        assert row[0] == "1" and [np.float32(v) for v in row[1:]] == list(np.float32(ref))


@pytest.mark.gpu
def test_facade_stl_to_voxel_grid_equals_reference(voxel_driver, tmp_path):
    """loadSTL + buildVoxelGrid + sampleSDFCPU / sdfNormalCPU through the
    facade: the reference's grid and mask bit for bit, the distance field
    bit for bit the least-fixed-point oracle (and within the distance-field
    tolerance of the reference), the samplers the oracle's on that field."""
    import json
    import oracle
    from golden.cases import fdigest, sdf_points, stl_files, unpack_mask
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "sdf.json")))["stl_binary_exact_res40"]
    stl = tmp_path / "model.stl"
    stl.write_bytes(stl_files()["binary_exact"])
    dims = tuple(g["dims"])
    mn = np.asarray(g["min"], np.float32)
    cs = np.asarray(g["cs"], np.float32)
    pts = sdf_points(mn, mn + cs * np.array(dims, np.float32))
    ptf = tmp_path / "pts.bin"
    pts.tofile(ptf)
    out = tmp_path / "grid.bin"
    r = subprocess.run([voxel_driver, str(stl), "40", str(out), str(ptf)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = out.read_bytes()
    got_dims = tuple(np.frombuffer(raw[:12], np.int32))
    box = np.frombuffer(raw[12:36], np.float32)
    n = dims[0] * dims[1] * dims[2]
    mask = np.frombuffer(raw[36:36 + n], np.uint8)
    field = np.frombuffer(raw[36 + n:36 + 5 * n], np.float32)
    samples = np.frombuffer(raw[36 + 5 * n:], np.float32).reshape(-1, 4)
    assert got_dims == dims and np.array_equal(box[:3], mn)
    assert np.array_equal(mask, unpack_mask(g["mask"], n))
    ex = oracle.sdf(mask, dims, cs, exact=True)
    assert np.array_equal(field, ex)
    ref = oracle.sdf(mask, dims, cs)
    assert fdigest(ref) == g["sdf"]
    d = np.abs(field - ref)
    assert np.array_equal(np.sign(field), np.sign(ref)) and np.mean(d <= 1e-4) >= 0.9999 and d.max() <= 2e-3
    dist, nrm = oracle.sdf_sample(ex, dims, mn, cs, pts)
    assert np.array_equal(samples[:, 0], dist) and np.array_equal(samples[:, 1:], nrm)
