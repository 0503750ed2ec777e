"""Readback and post-processing on the GPU (aeros_lbm_world_fields,
aeros_lbm_vorticity_q, aeros_lbm_sample): FP32, bitwise the reference's
functions on the golden cases."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sphere_trt_les_conv", "channel_force3", "sphere_les_ground_copy", "sphere_plus_y"])
def test_gpu_post_processing_equals_reference(name):
    from aeros_gb300 import solver
    from post_common import check_post
    check_post(name, lambda p, m: solver.Solver(p, m), lambda s, n: s.step(n), lambda s, wp: s.world_fields(wp),
               lambda s, wp: s.vorticity_q(), lambda s, wp, f, pts: s.sample(wp, f, pts))


def test_gpu_post_processing_shifted_storage_is_close():
    """FP16 storage: the world fields and the vorticity stay within the
    storage error of the FP32 ones."""
    from aeros_gb300 import capi, solver
    from golden.cases import params_for, solver_mask
    from post_common import GOLD, post_case, world_of
    name = "sphere_trt_les_conv"
    case = post_case(name)
    wp = world_of(name)
    out = {}
    for storage in ("fp32", "fp16"):
        s = solver.Solver(params_for(case, GOLD["cases"][name]["u_in"], storage), solver_mask(case))
        s.step(case["steps"])
        f, st = s.world_fields(wp)
        out[storage] = (f, s.vorticity_q())
    (f32, v32), (f16, v16) = out["fp32"], out["fp16"]
    umax = np.abs(f32["ux"]).max()
    assert np.abs(f16["ux"] - f32["ux"]).max() <= 2e-3 * umax
    pmax = np.abs(f32["pressure"]).max()
    assert np.abs(f16["pressure"] - f32["pressure"]).max() <= 2e-2 * pmax


def test_gpu_equilibrium_moments_equal_reference():
    """aeros_equilibrium_moments on the reference test's seven states equals
    lbmEquilibriumMoments bit for bit, keeps mass and momentum within that
    test's tolerances (3e-5), limits |u| to 0.3 and rejects non-finite input."""
    from aeros_gb300 import solver
    from golden.cases import EQ_MOMENT_CASES
    from post_common import GOLD
    st = np.array(EQ_MOMENT_CASES, np.float32)
    out, ok = solver.equilibrium_moments(st)
    assert ok.all()
    assert out.tolist() == np.array(GOLD["eq_moments"], np.float32).tolist()
    for (rho, ux, uy, uz), (m, px, py, pz) in zip(st, out):
        assert abs(m - rho) <= 3e-5 * max(1.0, rho)
        if ux * ux + uy * uy + uz * uz <= 0.09:
            assert max(abs(px - rho * ux), abs(py - rho * uy), abs(pz - rho * uz)) <= 3e-5
    bad = np.array([[1.0, np.nan, 0.0, 0.0], [np.nan, 0.0, 0.0, 0.0], [1.0, 0.0, np.inf, 0.0]], np.float32)
    out, ok = solver.equilibrium_moments(bad)
    assert not ok.any() and not out.any()
    # above the limiter: the momentum is that of |u| = 0.3 along u, the mass is kept
    out, ok = solver.equilibrium_moments(np.array([[1.0, 0.5, 0.0, 0.0]], np.float32))
    assert ok[0] and abs(out[0, 0] - 1.0) <= 3e-5 and abs(out[0, 1] - 0.3) <= 3e-5


def test_pinned_readback_equals_pageable():
    """Fields read into page-locked mirrors (aeros_host_alloc) equal the ones
    read into ordinary numpy arrays, twice in a row into the same mirrors."""
    import json
    import os
    from aeros_gb300 import solver
    from golden.cases import CASES, params_for, solver_mask
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
    case = CASES["sphere_trt_les_conv"]
    mask = solver_mask(case)
    s = solver.Solver(params_for(case, gold["cases"]["sphere_trt_les_conv"]["u_in"]), mask)
    host = solver.pinned_fields(s.n)
    for _ in range(2):
        s.step(7)
        a = s.fields()
        b = s.fields(out=host)
        for k in a:
            assert np.array_equal(a[k], b[k]), k
    s.close()
