"""The surface-force restatement (oracle/surface_oracle.c) against the
reference's own computeLiftDrag (forces.cpp:401-688), recorded in
tests/golden/surface.json by make_golden.py --surface: with FP32 sums in
triangle order it is the reference bit for bit; with the FP64 sums the device
uses, within the FP32 rounding of the reference's order."""
import numpy as np
import pytest

import oracle as O
from golden.cases import SURFACE_CASES, params_for
from post_common import GOLD
from surface_common import SURF, check_status, out_vector, ref_vector, surface_inputs, surface_world

_STATES = {}


def _state(case_name):
    """The oracle's LBM state of a post case after its steps (shared by the
    surface cases on that case)."""
    if case_name not in _STATES:
        from post_common import post_case
        from golden.cases import solver_mask
        case = post_case(case_name)
        dom = O.OracleLBM(params_for(case, GOLD["cases"][case_name]["u_in"]), solver_mask(case))
        dom.step(case["steps"])
        _STATES[case_name] = dom
    return _STATES[case_name]


@pytest.mark.parametrize("name", list(SURFACE_CASES))
def test_surface_oracle_bitwise_reference(name):
    case, v, n, sp, sdf, grid = surface_inputs(name)
    dom = _state(SURFACE_CASES[name]["case"])
    w = surface_world(name)
    dom.world_fields(w)
    o, cp = dom.surface_forces(w, sp, v, n, sdf, grid, f32_sums=True)
    if check_status(name, o):
        return
    r = ref_vector(name)
    assert np.array_equal(out_vector(o).view(np.int32), r.view(np.int32)), (out_vector(o), r)
    assert o.cp_non_finite == SURF[name]["result"]["cp_bad"]


@pytest.mark.parametrize("name", list(SURFACE_CASES))
def test_surface_oracle_fp64_sums(name):
    """The FP64-sum form stays within the reference's FP32 summation error."""
    case, v, n, sp, sdf, grid = surface_inputs(name)
    dom = _state(SURFACE_CASES[name]["case"])
    w = surface_world(name)
    dom.world_fields(w)
    o, cp = dom.surface_forces(w, sp, v, n, sdf, grid, f32_sums=False)
    if check_status(name, o):
        return
    r = ref_vector(name).astype(np.float64)
    got = out_vector(o).astype(np.float64)
    scale = np.maximum(np.abs(r), 1e-3 * np.abs(r[0]))
    assert np.all(np.abs(got - r) <= 2e-5 * scale + 1e-6), np.abs(got - r) / scale


def test_surface_cases_cover_the_branches():
    """The fixtures reach every branch the pass has: Karman-Tsien only, with
    wave drag, wave drag only, ground effect on a downforce, the box fallback
    of the reference area, skipped triangles, and both early returns."""
    res = {k: SURF[k]["result"] for k in SURFACE_CASES}
    assert res["karman_tsien_wave_m082"]["drag"] > 3 * res["karman_tsien_m044"]["drag"]
    assert res["fixed_area_ground_angles"]["lift"] < 0 and res["fixed_area_ground_angles"]["ref_area"] == 30.0
    assert res["huge_box_area"]["drag"] != res["plain"]["drag"]
    assert res["degenerate"]["drag"] != res["sdf"]["drag"]
    assert res["no_flow"]["drag"] == 0.0 and res["empty_mesh"]["drag"] == 7.0


@pytest.mark.skipif(not O.RefHarness.available(), reason="reference build not present")
def test_surface_fixtures_match_live_reference():
    """Where the reference tree is present: its build reproduces the fixtures."""
    from golden.cases import CASES, POST_FLOW_SPEED, SURFACE_DEFAULTS, surface_mesh
    R = O.RefHarness()
    for name in ("sdf", "degenerate"):
        sc = SURFACE_CASES[name]
        case = CASES[sc["case"]]
        nx, ny, nz = case["grid"]
        kw = dict(case["kw"], flow_speed=POST_FLOW_SPEED)
        R.L.ref_set_air_density(SURF[name]["world"][1])   # the atmosphere the fixture's run had
        R.setup(nx, ny, nz, case["solid"]().astype(np.uint8).reshape(-1), ground_rows=case.get("ground_rows", 0), **kw)
        R.step(case["steps"])
        v, n = surface_mesh(sc["mesh"])
        sdf = surface_inputs(name)[4]
        r = R.lift_drag(v, n, sdf, **dict(SURFACE_DEFAULTS, **sc["aero"]))
        assert np.float32(r.drag) == np.float32(SURF[name]["result"]["drag"])
        assert np.float32(r.lift) == np.float32(SURF[name]["result"]["lift"])


def test_surface_oracle_field_form_equals_state_form():
    """The restatement over a bare pressure array and wall mask (the form the
    full-size device check uses) gives the state form's results bit for bit."""
    from golden.cases import solver_mask
    for name in ("sdf", "ground_altitude", "degenerate"):
        case, v, n, sp, sdf, grid = surface_inputs(name)
        dom = _state(SURFACE_CASES[name]["case"])
        w = surface_world(name)
        fields, _ = dom.world_fields(w)
        a, cpa = dom.surface_forces(w, sp, v, n, sdf, grid, f32_sums=False)
        wall = (solver_mask(case).reshape(-1) != 0).astype(np.uint8)
        b, cpb = O.surface_forces_field(fields["pressure"], wall, case["grid"], w, sp, v, n, sdf, grid)
        assert np.array_equal(cpa.view(np.int32), cpb.view(np.int32))
        assert np.array_equal(out_vector(a).view(np.int32), out_vector(b).view(np.int32))
        assert list(a.sums) == list(b.sums)


@pytest.mark.skipif(not O.RefHarness.available(), reason="reference build not present")
def test_surface_non_finite_cp_counted_as_reference():
    """A Cp that overflows FP32 (a huge finite pressure in front of the body
    at a low freestream speed): the reference zeroes that Cp and counts it in
    aeroCpNonFinite; the restatement over the same poked field does the same,
    bit for bit."""
    from aeros_gb300 import capi
    from golden.cases import CASES, POST_FLOW_SPEED, SURFACE_DEFAULTS, surface_mesh
    name = "plain"
    sc = SURFACE_CASES[name]
    case = CASES[sc["case"]]
    nx, ny, nz = case["grid"]
    R = O.RefHarness()
    R.L.ref_set_air_density(SURF[name]["world"][1])
    R.setup(nx, ny, nz, case["solid"]().astype(np.uint8).reshape(-1), **dict(case["kw"], flow_speed=POST_FLOW_SPEED))
    R.step(case["steps"])
    fields, _, wp8 = R.world()
    # a block of cells just upstream of the sphere (centre 12, 12, 12, radius 4), where the front
    # triangles sample
    p = fields["pressure"].copy()
    for z in range(11, 14):
        for y in range(11, 14):
            for x in (6, 7):
                c = (z * ny + y) * nx + x
                R.L.ref_poke_pressure(c, 3e38)
                p[c] = np.float32(3e38)
    v, n = surface_mesh(sc["mesh"])
    aero = dict(SURFACE_DEFAULTS, flow_speed=0.1)   # q = 0.006 Pa: 3e38 / q overflows
    r = R.lift_drag(v, n, None, **aero)
    assert r.cp_bad > 0
    sp = capi.make_surface(velocity=list(r.vel), air_temperature=r.air_temperature, air_density=r.air_density,
                           use_real_density=aero["use_real_density"], speed_of_sound=r.speed_of_sound,
                           mach_effects=aero["mach_effects"], auto_ref_area=aero["auto_ref_area"],
                           ref_area=aero["ref_area"], azimuth=aero["azimuth"], elevation=aero["elevation"],
                           bb_min=aero["bb_min"], bb_max=aero["bb_max"], center=aero["center"],
                           max_dim=aero["max_dim"], reynolds=r.re_number, ground_effect=aero["ground_effect"],
                           ground_height=aero["ground_height"], vox_min_y=r.vox_min_y)
    w = capi.make_world(wp8[0], wp8[1], wp8[2:5], wp8[5:8])
    wall = (R.mask().reshape(-1) != 0).astype(np.uint8)
    o, cp = O.surface_forces_field(p, wall, (nx, ny, nz), w, sp, v, n, f32_sums=True)
    assert o.cp_non_finite == r.cp_bad
    print(f"non-finite Cp: {r.cp_bad} triangles")
    got = out_vector(o)
    want = np.array([r.drag, r.lift, r.ld, r.moment_mag, *r.drag_vec, *r.lift_vec, *r.moment, *r.cop, r.ref_area],
                    np.float32)
    assert np.array_equal(got.view(np.int32), want.view(np.int32)), (got, want)
