"""GPU parity: the CUDA library (through the C ABI) against the reference.

FP32 storage is the drop-in form. Its fields must match the reference within
1e-5 max-relative (max |a-b| / max |b|); because the kernels keep the
reference's operation order without contraction they are expected to match
bit for bit, which the digest tests check against the reference's own
digests. Every case is also run live through the oracle.
"""
import json
import os

import numpy as np
import pytest

from golden.cases import (CASES, digest, outputs_digest, params_for, solver_mask, thermal_params_for)

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))
MASKS = np.load(os.path.join(HERE, "golden", "masks.npz"))
FIELD_TOL = 1e-5


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-30)
    return float(np.max(np.abs(a - b)) / scale)


@pytest.fixture(scope="module")
def gpu():
    from aeros_gb300 import solver
    return solver


def run_gpu(solver, name, storage="fp32", chunks=None):
    case = CASES[name]
    g = GOLD["cases"][name]
    mask = solver_mask(case)
    p = params_for(case, g["u_in"], storage)
    s = solver.Solver(p, mask)
    if case.get("thermal"):
        s.thermal_init(thermal_params_for(case, p.tau))
        if "upload" in case:
            s.thermal_upload(case["upload"]())
    for n in (chunks or [case["steps"]]):
        s.step(n)
    return s, mask, p


def run_oracle(O, name, precision="f32"):
    case = CASES[name]
    g = GOLD["cases"][name]
    mask = solver_mask(case)
    o = O.OracleLBM(params_for(case, g["u_in"]), mask, precision)
    if case.get("thermal"):
        o.thermal_init(thermal_params_for(case, params_for(case, g["u_in"]).tau))
        if "upload" in case:
            o.thermal_upload(case["upload"]())
    o.step(case["steps"])
    return o


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_fields_within_tolerance_of_oracle(gpu, oracle_built, name):
    s, mask, _ = run_gpu(gpu, name)
    o = run_oracle(oracle_built, name)
    a, b = s.fields(), o.fields()
    for k in ("rho", "ux", "uy", "uz", "strain", "tke"):
        if np.max(np.abs(b[k])) > 0:
            assert max_rel(a[k], b[k]) <= FIELD_TOL, (k, max_rel(a[k], b[k]))
    fl = mask.reshape(-1) == 0
    assert max_rel(s.populations()[:, fl], o.populations()[:, fl]) <= FIELD_TOL
    if CASES[name].get("thermal"):
        Ta, ba = s.thermal()
        Tb, bb = o.thermal()
        assert max_rel(Ta, Tb) <= FIELD_TOL
        assert max_rel(ba, bb) <= FIELD_TOL or np.max(np.abs(bb)) == 0


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_bitwise_equals_reference(gpu, name):
    s, mask, _ = run_gpu(gpu, name)
    g = GOLD["cases"][name]
    T = b = None
    if CASES[name].get("thermal"):
        T, b = s.thermal()
    d = outputs_digest(s.fields(), s.populations(), mask, T, b)
    assert d == g["digest"], {k: d[k] == g["digest"][k] for k in d}
    st = s.stats()
    for k in ("negative_pops", "bad_pops", "rho_out_of_range", "rho_non_finite", "u_limited", "step"):
        assert st[k] == g["stats"][k], k
    assert np.float32(st["avg_rho"]) == np.float32(g["stats"]["avg_rho"])
    assert np.float32(st["max_velocity_lb"]) == np.float32(g["stats"]["max_velocity_lb"])
    assert np.array_equal(s.cv_force(0.3, 0.3, 0.3).astype(np.float32), np.asarray(g["cv_force"], np.float32))
    assert [s.projected_area(a) for a in range(3)] == g["area"]
    if CASES[name].get("thermal"):
        assert np.float32(st["nusselt"]) == np.float32(g["nusselt"])
        assert abs(st["mean_t"] - g["mean_t"]) <= 1e-6 * max(1.0, abs(g["mean_t"]))


@pytest.mark.parametrize("name", ["sphere_trt_les_conv", "rb_small", "channel_force3"])
def test_chunked_stepping_is_identical(gpu, name):
    """step(1) x n, uneven chunks and step(n) give the same state (AA parity,
    side buffers and observable writes are bookkept across calls)."""
    n = CASES[name]["steps"]
    a, mask, _ = run_gpu(gpu, name)
    b, _, _ = run_gpu(gpu, name, chunks=[1, 2, 3, n - 6])
    fa, fb = a.fields(), b.fields()
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k
    assert np.array_equal(a.populations(), b.populations())


def test_population_roundtrip_mid_run(gpu, oracle_built):
    """Read the pre-collision state after an odd number of steps, write it back
    (checkpoint restore), continue: identical to an uninterrupted run."""
    name = "sphere_trt_les_conv"
    a, _, _ = run_gpu(gpu, name, chunks=[37])
    f = a.populations()
    a.write_populations(f)
    a.step(40)
    b, _, _ = run_gpu(gpu, name, chunks=[77])
    assert np.array_equal(a.populations(), b.populations())
    assert np.array_equal(a.fields()["ux"], b.fields()["ux"])


def test_divergence_guard_reequilibrates(gpu, oracle_built):
    """Fault injection on the host: NaN populations in > 10 % of the cells trip
    the NaN guard (lbm.cpp:1313-1319); the solver re-equilibrates to the inlet
    state exactly as the oracle does."""
    name = "sphere_bgk_conv"
    s, mask, p = run_gpu(gpu, name, chunks=[20])
    o = oracle_built.OracleLBM(p, mask)
    o.step(20)
    f = s.populations()
    rng = np.random.default_rng(7)
    bad = rng.random(f.shape[1]) < 0.2
    f[:, bad] = np.nan
    s.write_populations(f)
    o.set_populations(f)
    s.step(5)
    o.step(5)
    st, so = s.stats(), o.stats()
    assert st["diverged"] == 1 and so["diverged"] == 1
    assert st["step"] == so["step"]
    fl = mask.reshape(-1) == 0
    assert np.array_equal(s.populations()[:, fl], o.populations()[:, fl])
    a, b = s.fields(), o.fields()
    assert np.array_equal(a["rho"], b["rho"]) and np.array_equal(a["ux"], b["ux"])
    s.step(10)
    o.step(10)
    assert max_rel(s.fields()["ux"], o.fields()["ux"]) <= FIELD_TOL


def test_force_queued_behind_a_diverging_step(gpu, oracle_built):
    """aeros_lbm_cv_force queued behind a pending step whose divergence guard
    trips: the force is taken again on the re-equilibrated state, so it equals
    the force read after the step has been finished on its own."""
    name = "sphere_bgk_conv"
    forces = []
    for queued in (True, False):
        s, mask, p = run_gpu(gpu, name, chunks=[20])
        f = s.populations()
        bad = np.random.default_rng(7).random(f.shape[1]) < 0.2
        f[:, bad] = np.nan
        s.write_populations(f)
        if queued:
            s.step_async(5)
            forces.append(s.cv_force(0.3, 0.3, 0.3))   # one wait: the steps, the guard, the force
        else:
            s.step(5)
            s.stats()
            forces.append(s.cv_force(0.3, 0.3, 0.3))
        assert s.stats()["diverged"] == 1
        s.close()
    assert np.array_equal(forces[0], forces[1])
    assert np.all(np.isfinite(forces[0]))


def test_run_twice_bitwise_deterministic(gpu):
    a, _, _ = run_gpu(gpu, "sphere_trt_les_conv")
    b, _, _ = run_gpu(gpu, "sphere_trt_les_conv")
    assert np.array_equal(a.populations(), b.populations())
    assert a.stats()["sum_rho"] == b.stats()["sum_rho"]


@pytest.mark.parametrize("key", ["bgk_40k", "trt_40k"])
def test_poiseuille_reference_values(gpu, key):
    """physics_ref_headless.cpp:192-272: 8x34x8 channel, tau 0.65, F 7.8e-6,
    40k steps: L2 and centre velocity equal the reference's to its digits."""
    from aeros_gb300 import capi, geometry
    nx, ny, nz = 8, 34, 8
    p = capi.make_params(nx, ny, nz, tau=0.65, trt=key.startswith("trt"), periodic_x=True, periodic_z=True,
                         u_in=(0.08, 0, 0), u_init=(0.08, 0, 0), body_force=(7.8e-6, 0, 0), vel_scale=12.5)
    s = gpu.Solver(p, geometry.channel_mask(nx, ny, nz))
    s.step(40000)
    ux = s.fields()["ux"].reshape(nz, ny, nx)
    prof = ux[nz // 2, 1:ny - 1, :].astype(np.float64).mean(axis=1)
    exact = geometry.poiseuille_exact(ny, 0.65, 7.8e-6)
    l2 = np.sqrt(np.sum((prof - exact) ** 2) / np.sum(exact ** 2))
    ref = GOLD["physref"][key]
    assert round(100 * l2, 3) == round(100 * ref["l2"], 3)
    assert abs(l2 - ref["l2"]) <= 1e-5 * ref["l2"] + 1e-9
    assert np.array_equal(np.asarray(ref["profile"]), prof) or max_rel(prof, ref["profile"]) <= FIELD_TOL


def test_poiseuille_config_4000_steps(gpu):
    """64x32x32, tau 0.8, F 1e-6, fluid at rest, 4000 steps: fields equal the
    reference's; L2 against the parabola as the reference's."""
    from aeros_gb300 import geometry
    p, mask = geometry.poiseuille()
    s = gpu.Solver(p, mask)
    s.step(4000)
    g = GOLD["poiseuille_config"]
    d = outputs_digest(s.fields(), s.populations(), mask)
    assert d == g["digest"]
    ux = s.fields()["ux"].reshape(32, 32, 64)
    prof = ux[:, 1:31, :].astype(np.float64).mean(axis=(0, 2))
    exact = geometry.poiseuille_exact(32, 0.8, 1e-6)
    l2 = np.sqrt(np.sum((prof - exact) ** 2) / np.sum(exact ** 2))
    assert abs(l2 - g["l2"]) <= 1e-6


def test_validation_sphere_cd(gpu):
    """validation_headless.cpp:206-251: Re = 100 sphere, D = 20 cells, the
    reference's own padded 92x84x84 mask, BGK, convective outlet, 500 + 50
    steps: Cd equals the reference's 1.128 to the reported digits."""
    from aeros_gb300 import capi
    v = GOLD["validation_sphere"]
    nx, ny, nz = v["dims"]
    mask = np.unpackbits(MASKS["validation_sphere_mask"])[: nx * ny * nz].astype(np.uint8)
    u = np.asarray(v["u_in"], np.float32)
    p = capi.make_params(nx, ny, nz, tau=v["tau"], convective_outlet=True, u_in=u, u_init=u,
                         vel_scale=float(np.float32(20.0) / np.float32(0.08)))
    s = gpu.Solver(p, mask)
    s.step(v["warm"])
    area = s.projected_area(0)
    assert area == v["area"]
    q = np.float32(0.5 * 0.08 * 0.08 * area)
    cds = []
    for _ in range(v["meas"]):
        s.step(1)
        F = s.cv_force(0.3, 0.3, 0.3)
        cds.append(np.float32(np.float32(F[0]) / q))
    cd = float(np.mean(np.array(cds, np.float64)))
    assert round(cd, 3) == round(v["cd"], 3) == 1.128
    assert abs(cd - v["cd"]) <= 1e-5 * v["cd"]
    assert outputs_digest(s.fields(), s.populations(), mask) == v["digest"]


def _validation_cd(make, storage="fp32"):
    """Mean Cd of the validation sphere (the set-up of test_validation_sphere_cd)
    on a domain made by make(params, mask); FP64 force, q as the reference."""
    from aeros_gb300 import capi
    v = GOLD["validation_sphere"]
    nx, ny, nz = v["dims"]
    mask = np.unpackbits(MASKS["validation_sphere_mask"])[: nx * ny * nz].astype(np.uint8)
    u = np.asarray(v["u_in"], np.float32)
    p = capi.make_params(nx, ny, nz, tau=v["tau"], convective_outlet=True, u_in=u, u_init=u,
                         vel_scale=float(np.float32(20.0) / np.float32(0.08)), storage=storage)
    s = make(p, mask)
    s.step(v["warm"])
    q = 0.5 * 0.08 * 0.08 * float(v["area"])
    cds = []
    for _ in range(v["meas"]):
        s.step(1)
        cds.append(float(s.cv_force(0.3, 0.3, 0.3)[0]) / q)
    return float(np.mean(cds))


def test_shifted_storage_cd_vs_plain_and_fp64(gpu, oracle_built):
    """Precision form on the Re = 100 validation sphere (649 k cells, 550
    steps), against the plain FP32 path (1.127719, the reference's 1.128) and
    the FP64 oracle (1.128573). Tolerance: 0.5 % for FP16 and BF16 storage
    shifted by the freestream equilibrium (the w shift gave FP16 +0.64 % /
    +0.56 %, BF16 +4.1 %)."""
    cd32 = _validation_cd(lambda p, m: gpu.Solver(p, m))
    cd16 = _validation_cd(lambda p, m: gpu.Solver(p, m), "fp16")
    cdbf = _validation_cd(lambda p, m: gpu.Solver(p, m), "bf16")
    oracle_built.set_threads(os.cpu_count() or 1, "f64")
    cd64 = _validation_cd(lambda p, m: oracle_built.OracleLBM(p, m, "f64"))
    print(f"Cd: fp32 {cd32:.6f} fp16 {cd16:.6f} bf16 {cdbf:.6f} fp64 {cd64:.6f}")
    assert abs(cd32 - cd64) <= 0.001 * abs(cd64)
    assert abs(cd16 - cd32) <= 0.005 * abs(cd32)
    assert abs(cd16 - cd64) <= 0.005 * abs(cd64)
    assert abs(cdbf - cd32) <= 0.005 * abs(cd32)
    assert abs(cdbf - cd64) <= 0.005 * abs(cd64)


def test_voxelizer_bit_exact(gpu):
    from aeros_gb300 import geometry
    from aeros_gb300.solver import voxel_grid, voxelize
    nx, ny, nz = geometry.SPHERE_GRID
    tris = geometry.icosphere(6, geometry.SPHERE_RADIUS, geometry.SPHERE_CENTER)
    assert tris.shape[0] == 81920
    m = voxelize(tris, voxel_grid((nx, ny, nz), (0, 0, 0), (1, 1, 1)))
    ref = np.unpackbits(MASKS["sphere_config_mask"])[: nx * ny * nz]
    assert np.array_equal(m, ref)
    v = GOLD["voxel"]
    for k, tv in {"uv_sphere_40": geometry.uv_sphere(0.35, 32, 48), "torus_48": geometry.torus(0.3, 0.11, 64, 32),
                  "box_32": geometry.box((0.3, 0.2, 0.25)), "plate_64": geometry.box((0.3, 0.003, 0.2))}.items():
        n = v[k]["n"]
        mk = voxelize(tv, voxel_grid((n, n, n), v[k]["min"], (np.float32(v[k]["cell"]),) * 3))
        assert digest(mk) == v[k]["digest"], k


def test_voxelizer_matches_brute_force_oracle(gpu, oracle_built):
    from aeros_gb300 import geometry
    from aeros_gb300.solver import voxel_grid, voxelize
    tris = geometry.perturbed_icosphere(3, 9.0, (16.5, 15.2, 14.9), seed=11)
    g = voxel_grid((33, 30, 29), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    assert np.array_equal(voxelize(tris, g), oracle_built.voxelize_brute(tris, g))
    # degenerate and non-finite triangles are dropped, empty meshes give empty masks
    bad = np.concatenate([tris, np.full((3, 9), np.nan, np.float32), np.zeros((2, 9), np.float32)])
    assert np.array_equal(voxelize(bad, g), oracle_built.voxelize_brute(bad, g))
    assert voxelize(np.zeros((0, 9), np.float32), g).sum() == 0


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_shifted_storage_error_vs_fp64(gpu, oracle_built, storage):
    """Precision form: populations stored as f - w in 16 bits, FP32 arithmetic.
    Error against the FP64 run of the same algorithm stays bounded."""
    name = "sphere_trt_les_conv"
    s, _, _ = run_gpu(gpu, name, storage)
    o = run_oracle(oracle_built, name, "f64")
    a, b = s.fields(), o.fields_f64()
    tol = 2e-3 if storage == "fp16" else 2e-2
    for k in ("ux", "uy", "uz"):
        assert np.max(np.abs(a[k] - b[k])) <= tol * np.max(np.abs(b["ux"])), (k, storage)
    assert np.max(np.abs(a["rho"] - b["rho"])) <= tol


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("name", ["rb_small", "rb_pm", "thermal_body", "thermal_diffusion"])
def test_thermal_single_launch_matches_two_launches(gpu, monkeypatch, name, storage):
    """Thermal domains step in one launch (shell and interior blocks side by
    side); the two-launch form (AEROS_FUSED=0: shell, then interior) gives the
    same populations, fields and temperatures bit for bit, and the same
    statistics up to the order of their sums."""
    out = []
    for fused in ("0", "1"):
        monkeypatch.setenv("AEROS_FUSED", fused)
        s, _, _ = run_gpu(gpu, name, storage)
        st = s.stats()
        out.append((s.populations(), s.fields(), s.thermal(), st, s.last_launch_count()))
        s.close()
    (fa, va, ta, sa, la), (fb, vb, tb, sb, lb) = out
    assert la == 2 * lb > 0   # kernels of the last call: shell + interior per step, then one
    assert np.array_equal(fa, fb)
    for k in va:
        assert np.array_equal(va[k], vb[k]), k
    assert np.array_equal(ta[0], tb[0]) and np.array_equal(ta[1], tb[1])
    assert sa["step"] == sb["step"]
    assert abs(sa["sum_rho"] - sb["sum_rho"]) <= 1e-12 * abs(sa["sum_rho"])
    assert abs(sa["nusselt"] - sb["nusselt"]) <= 1e-6 * max(1.0, abs(sa["nusselt"]))
    assert abs(sa["mean_t"] - sb["mean_t"]) <= 1e-6


FREESLIP_CASES = {   # name: (golden case whose mask and flow it reuses, LES, TRT, lateral, outlet)
    "sphere_freeslip_zerograd_trt_les": ("sphere_trt_les_conv", True, True, "freeslip", "zerograd"),
    "sphere_freeslip_zerograd_bgk": ("sphere_bgk_conv", False, False, "freeslip", "zerograd"),
    "sphere_copy_zerograd_les": ("sphere_les_ground_copy", True, False, "copy", "zerograd"),
    "sphere_freeslip_reference_outlet": ("sphere_trt_les_conv", True, True, "freeslip", "reference"),
    "sphere_plus_y_freeslip_zerograd": ("sphere_plus_y", True, True, "freeslip", "zerograd"),
    "sphere_minus_z_freeslip_zerograd": ("sphere_minus_z_perx", True, False, "freeslip", "zerograd"),
}


@pytest.mark.parametrize("name", sorted(FREESLIP_CASES))
def test_freeslip_and_zero_gradient_equal_restatement(gpu, oracle_built, name):
    """Boundary modes the reference does not have (free-slip lateral walls,
    zero-gradient outlet: the headline sphere's) against their C restatement:
    FP32 populations and fields bit for bit."""
    from aeros_gb300 import capi
    base, les, trt, lateral, outlet = FREESLIP_CASES[name]
    case = CASES[base]
    g = GOLD["cases"][base]
    mask = solver_mask(case)
    p = params_for(case, g["u_in"])
    p.use_les, p.use_trt = int(les), int(trt)
    p.lateral_bc = capi.AEROS_LATERAL_FREESLIP if lateral == "freeslip" else capi.AEROS_LATERAL_COPY
    p.outlet_bc = capi.AEROS_OUTLET_ZEROGRAD if outlet == "zerograd" else capi.AEROS_OUTLET_REFERENCE
    p.convective_outlet = 0 if outlet == "zerograd" else p.convective_outlet
    s = gpu.Solver(p, mask)
    o = oracle_built.OracleLBM(p, mask)
    for n in (case["steps"] // 2, case["steps"] - case["steps"] // 2):
        s.step(n)
        o.step(n)
    fl = mask.reshape(-1) == 0
    assert np.array_equal(s.populations()[:, fl], o.populations()[:, fl])
    a, b = s.fields(), o.fields()
    for k in ("rho", "ux", "uy", "uz", "strain", "tke"):
        assert np.array_equal(a[k], b[k]), k
    assert s.stats()["step"] == o.stats()["step"]
    assert np.array_equal(s.cv_force(0.3, 0.3, 0.3).astype(np.float32), o.cv_force(0.3, 0.3, 0.3).astype(np.float32))


@pytest.mark.parametrize("storage,tol", [("fp32", 5e-5), ("fp16", 2e-3)])
def test_full_size_sphere_keeps_its_mirror_symmetry(gpu, storage, tol):
    """The headline sphere at its full 240 x 120 x 115 size: the mask is
    mirror-symmetric about the sphere's y and z planes (cell centres i + 0.5
    mirror about 60 and 57.5), the inflow is along x, the lateral walls are
    free-slip, so the flow keeps that symmetry: u_x even, u_y odd in y, u_z odd
    in z, up to rounding: mirrored cells sum their populations in opposite
    orders (measured in FP32 after 600 steps: 1.3e-5 of max |u|; tolerance
    5e-5; FP16 2e-3)."""
    from aeros_gb300 import geometry
    p, mask, _ = geometry.sphere_config(storage=storage)
    m = mask.reshape(115, 120, 240)
    assert np.array_equal(m, m[:, ::-1, :]) and np.array_equal(m, m[::-1, :, :])
    s = gpu.Solver(p, mask)
    s.step(600)
    f = s.fields()
    ux, uy, uz = (f[k].reshape(115, 120, 240) for k in ("ux", "uy", "uz"))
    umax = float(np.abs(ux).max())
    assert umax > 0.04
    assert np.abs(ux - ux[:, ::-1, :]).max() <= tol * umax
    assert np.abs(ux - ux[::-1, :, :]).max() <= tol * umax
    assert np.abs(uy + uy[:, ::-1, :]).max() <= tol * umax
    assert np.abs(uz + uz[::-1, :, :]).max() <= tol * umax
    assert s.stats()["diverged"] == 0


def test_voxelizer_half_million_triangles_no_holes_no_extras(gpu):
    """voxel_headless.cpp's large-mesh checks on a 512,000-triangle mesh (four
    disjoint icospheres, levels 7, 6, 6, 5) at 128^3: built and voxelized in
    under 5 s; no cell whose centre lies inside a sphere by more than the
    polyhedron's inscribed gap is fluid, no cell outside by more than that is
    solid; the solid volume is within 2 % of the spheres' volume."""
    import time

    from aeros_gb300 import geometry
    from aeros_gb300.solver import voxel_grid, voxelize
    spheres = [(7, 0.30, (-0.40, 0.0, 0.0)), (6, 0.20, (0.35, 0.25, 0.0)), (6, 0.20, (0.35, -0.25, 0.0)),
               (5, 0.10, (0.0, 0.45, 0.35))]
    tris = np.concatenate([geometry.icosphere(lv, r, c) for lv, r, c in spheres])
    assert tris.shape[0] == 512000
    n = 128
    g = voxel_grid((n, n, n), (-0.8, -0.8, -0.8), (1.6 / n,) * 3)
    t = time.perf_counter()
    m = voxelize(tris, g).reshape(n, n, n)
    assert time.perf_counter() - t < 5.0
    c = (np.arange(n, dtype=np.float64) + 0.5) * (1.6 / n) - 0.8
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    inside = np.zeros(m.shape, bool)
    outside = np.ones(m.shape, bool)
    for lv, r, (cx, cy, cz) in spheres:
        d = np.sqrt((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2)
        gap = r * (1.0 - np.cos(1.2 / 2 ** lv)) + 1e-6   # faces lie within this of the sphere
        inside |= d < r - gap
        outside &= d > r + 1e-6
    assert not np.any(inside & (m == 0)), "holes"
    assert not np.any(outside & (m != 0)), "extras"
    vol = sum(4.0 / 3.0 * np.pi * r ** 3 for _, r, _ in spheres)
    assert abs(m.sum() * (1.6 / n) ** 3 - vol) <= 0.02 * vol


def test_mass_conserved_in_a_closed_periodic_domain(gpu, oracle_built):
    """lbm_physics_headless.cpp's conservation check: a periodic channel with
    a body and walls conserves its mass. Without a force the sum of rho over
    the fluid moves by rounding only (< 1e-6 of it in 2000 steps). With the
    Guo force the reference's FP32 arithmetic drifts by about 4e-5 (its FP64
    run by 1.6e-13): the GPU's FP32 sum equals the FP32 restatement's to the
    last bit, and FP16 storage stays within 1e-4."""
    from aeros_gb300 import capi, geometry
    nx, ny, nz = 64, 34, 24
    mask = geometry.channel_mask(nx, ny, nz).reshape(nz, ny, nx).copy()
    mask[8:16, 12:22, 20:30] = 1
    for force in (0.0, 2e-6):
        for storage in ("fp32", "fp16"):
            p = capi.make_params(nx, ny, nz, tau=0.7, les=True, trt=True, periodic_x=True, periodic_z=True,
                                 u_in=(0.0, 0.0, 0.0), body_force=(force, 0.0, 0.0), storage=storage)
            s = gpu.Solver(p, mask)
            s.step(1)
            m0 = s.stats()["sum_rho"]
            s.step(2000)
            st = s.stats()
            assert st["diverged"] == 0
            drift = abs(st["sum_rho"] - m0) / m0
            assert drift <= (1e-6 if force == 0.0 else 1e-4), (force, storage, drift)
            if storage == "fp32" and force > 0.0:
                o = oracle_built.OracleLBM(p, mask)
                o.step(2001)
                assert st["sum_rho"] == o.stats()["sum_rho"]
            s.close()
