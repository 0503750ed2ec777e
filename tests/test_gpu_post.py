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
