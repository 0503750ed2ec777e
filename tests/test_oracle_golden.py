"""The oracle (CPU restatement) against the reference's golden fixtures.

Bit-exact: every field digest of every case equals the one recorded from the
reference's own solver (tests/golden/make_golden.py). These run on the CPU.
"""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, EQ_MOMENT_CASES, outputs_digest, params_for, solver_mask, thermal_params_for

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def run_oracle(O, name, precision="f32"):
    case = CASES[name]
    g = GOLD["cases"][name]
    mask = solver_mask(case)
    p = params_for(case, g["u_in"])
    o = O.OracleLBM(p, mask, precision)
    if case.get("thermal"):
        o.thermal_init(thermal_params_for(case, p.tau))
        if "upload" in case:
            o.thermal_upload(case["upload"]())
    o.step(case["steps"])
    return o, mask


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_bitwise_equals_reference(oracle_built, name):
    O = oracle_built
    o, mask = run_oracle(O, name)
    g = GOLD["cases"][name]
    T = b = None
    if CASES[name].get("thermal"):
        T, b = o.thermal()
    d = outputs_digest(o.fields(), o.populations(), mask, T, b)
    assert d == g["digest"], {k: d[k] == g["digest"][k] for k in d}
    s = o.stats()
    for k in ("negative_pops", "bad_pops", "rho_out_of_range", "rho_non_finite", "u_limited", "step"):
        assert s[k] == g["stats"][k], k
    for k in ("avg_rho", "max_velocity_lb"):
        assert np.float32(s[k]) == np.float32(g["stats"][k]), k
    cv = o.cv_force(0.3, 0.3, 0.3)
    assert np.array_equal(cv.astype(np.float32), np.asarray(g["cv_force"], np.float32))
    assert [o.projected_area(a) for a in range(3)] == g["area"]
    if CASES[name].get("thermal"):
        assert np.float32(s["nusselt"]) == np.float32(g["nusselt"])
        assert np.float32(s["mean_t"]) == np.float32(g["mean_t"])


def test_oracle_wall_distance(oracle_built):
    from golden.cases import digest
    o, _ = run_oracle(oracle_built, "sphere_les_ground_copy")
    assert digest(o.wall_dist()) == GOLD["cases"]["sphere_les_ground_copy"]["wall_digest"]


def test_oracle_equilibrium_moments(oracle_built):
    for c, ref in zip(EQ_MOMENT_CASES, GOLD["eq_moments"]):
        ok, got = oracle_built.equilibrium_moments(*c)
        assert ok and list(np.float32(got)) == list(np.float32(ref))
    ok, _ = oracle_built.equilibrium_moments(1.0, float("nan"), 0.0, 0.0)
    assert not ok


def test_oracle_f64_close_to_f32(oracle_built):
    """The FP64 build runs the same algorithm: after 150 steps the FP32 fields
    differ from it by FP32 rounding only (|du| <= 1e-4 max|u|, |drho| <= 2e-5)."""
    a, _ = run_oracle(oracle_built, "sphere_trt_les_conv", "f32")
    b, _ = run_oracle(oracle_built, "sphere_trt_les_conv", "f64")
    fa, fb = a.fields(), b.fields_f64()
    for k in ("ux", "uy", "uz"):
        assert np.max(np.abs(fa[k] - fb[k])) <= 1e-4 * np.max(np.abs(fb["ux"])), k
    assert np.max(np.abs(fa["rho"] - fb["rho"])) <= 2e-5


def test_oracle_voxel_equals_reference(oracle_built):
    from aeros_gb300 import geometry
    from aeros_gb300.solver import voxel_grid
    from golden.cases import digest
    v = GOLD["voxel"]
    cases = {"uv_sphere_40": geometry.uv_sphere(0.35, 32, 48), "box_32": geometry.box((0.3, 0.2, 0.25)),
             "torus_48": geometry.torus(0.3, 0.11, 64, 32)}
    for k, tris in cases.items():
        n = v[k]["n"]
        g = voxel_grid((n, n, n), v[k]["min"], (np.float32(v[k]["cell"]),) * 3)
        m = oracle_built.voxelize_brute(tris, g)
        assert digest(m) == v[k]["digest"], k


def test_oracle_voxel_plan(oracle_built):
    p = oracle_built.voxel_plan([1, 0.5, 0.25], 64, 8 << 30)
    assert [p.nx, p.ny, p.nz, p.fits, p.suggested_res, p.cells] == GOLD["voxel_plan"]["1x0.5x0.25@64/8G"]
    p = oracle_built.voxel_plan([1, 1, 1], 512, 512 << 20)
    ref = GOLD["voxel_plan"]["1@512/512M"]
    assert [p.nx, p.ny, p.nz, p.fits, p.suggested_res] == ref[:5]


def test_golden_published_values():
    """The fixtures carry the reference's published validation numbers."""
    pr = GOLD["physref"]
    assert round(100 * pr["bgk_40k"]["l2"], 3) == 0.053
    assert round(pr["bgk_40k"]["u_center"], 6) == 0.019951
    assert round(100 * pr["trt_40k"]["l2"], 3) == 0.051
    p = np.log(abs(pr["h16_15k"]["l2"] - pr["h8_4k"]["l2"]) / abs(pr["bgk_40k"]["l2"] - pr["h16_15k"]["l2"])) / np.log(2)
    assert p > 1.5
    assert round(GOLD["validation_sphere"]["cd"], 3) == 1.128
    assert GOLD["validation_sphere"]["area"] == 316.0


@pytest.mark.parametrize("name", ["sphere_trt_les_conv", "channel_force3", "sphere_les_ground_copy", "sphere_plus_y"])
def test_oracle_post_processing_equals_reference(oracle_built, name):
    """World fields, readback statistics, vorticity / Q / strain and the
    samplers of the C restatement, bitwise the reference's."""
    from post_common import check_post
    O = oracle_built
    check_post(name, lambda p, m: O.OracleLBM(p, m), lambda o, n: o.step(n), lambda o, wp: o.world_fields(wp),
               lambda o, wp: o.vorticity_q(wp), lambda o, wp, f, pts: o.sample(wp, f, pts))
