"""GPU: the precision form (FP16 / BF16 storage, FP32 arithmetic).

Slots hold f - s_r with s = f_eq(1, u_shift) (the freestream equilibrium),
r the direction the next gather reads the value as; the D3Q7 lattice holds
g - w_i Tc(y) with Tc the conduction profile between fixed wall
temperatures. Tolerances are written beside each check; every figure is
against the plain FP32 path (the drop-in) and the FP64 run of the oracle.
"""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, params_for, solver_mask

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from aeros_gb300 import solver
    return solver


def _uniform_box(flow_axis, flow_sign, lateral, outlet, storage, shift):
    from aeros_gb300 import capi
    dims = [24, 24, 24]
    dims[flow_axis] = 48
    u = [0.0, 0.0, 0.0]
    u[flow_axis] = 0.05 * flow_sign
    p = capi.make_params(*dims, tau=0.56, les=True, trt=True, smagorinsky_c=0.1, u_in=u, u_init=u,
                         vel_scale=20.0, storage=storage, storage_shift=shift, flow_axis=flow_axis, flow_sign=flow_sign,
                         lateral_bc=capi.AEROS_LATERAL_FREESLIP if lateral == "freeslip" else capi.AEROS_LATERAL_COPY,
                         outlet_bc=capi.AEROS_OUTLET_ZEROGRAD if outlet == "zerograd" else capi.AEROS_OUTLET_REFERENCE,
                         convective_outlet=outlet == "convective")
    return p, np.zeros(dims[0] * dims[1] * dims[2], np.uint8), np.asarray(u, np.float32)


UNIFORM = [(0, 1, "freeslip", "zerograd"), (0, 1, "copy", "convective"), (0, 1, "copy", "copy"),
           (0, 1, "freeslip", "convective"), (1, 1, "freeslip", "zerograd"), (2, -1, "freeslip", "zerograd"),
           (2, -1, "copy", "convective")]


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
@pytest.mark.parametrize("axis,sign,lateral,outlet", UNIFORM)
def test_uniform_flow_is_a_fixed_point_of_the_freestream_shift(gpu, axis, sign, lateral, outlet, storage):
    """A uniform stream at the inlet velocity through an empty box is the
    state the freestream shift stores as zeros: every link kind (regular,
    copy-own, free slip, the inlet and the outlets) must hand each value to
    its reader with the reader's shift, or the stream picks up errors of
    6 w c.u ~ 1.7e-2 on the faces. Tolerance: 1e-6 of |u| in FP16 (the
    rounding residue of 1 + sum(s - w) ~ 1e-9 falls below its range), 2e-5 in
    BF16 (which keeps that residue)."""
    p, mask, u = _uniform_box(axis, sign, lateral, outlet, storage, 0)
    s = gpu.Solver(p, mask)
    s.step(301)
    f = s.fields()
    err = max(float(np.max(np.abs(f[k] - u[i]))) for i, k in enumerate(("ux", "uy", "uz")))
    tol = 1e-6 if storage == "fp16" else 2e-5
    assert err <= tol, err
    assert float(np.max(np.abs(f["rho"] - 1.0))) <= tol


def _fp64_fields(oracle, p, mask, steps):
    o = oracle.OracleLBM(p, mask, "f64")
    o.step(steps)
    return o.fields_f64()


def _case(name, storage, **mod):
    from aeros_gb300 import capi
    import json
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
    case = CASES[name]
    mask = solver_mask(case)
    p = params_for(case, gold["cases"][name]["u_in"], storage)
    for k, v in mod.items():
        setattr(p, k, v)
    if mod.get("outlet_bc") == capi.AEROS_OUTLET_ZEROGRAD:
        p.convective_outlet = 0
    return case, mask, p


PRECISION_CASES = ["sphere_trt_les_conv", "sphere_les_ground_copy", "sphere_plus_y", "sphere_minus_x",
                   "freeslip_zerograd", "freeslip_minus_z"]


def _precision_case(name, storage):
    from aeros_gb300 import capi
    fs = dict(lateral_bc=capi.AEROS_LATERAL_FREESLIP, outlet_bc=capi.AEROS_OUTLET_ZEROGRAD)
    if name == "freeslip_zerograd":
        return _case("sphere_trt_les_conv", storage, **fs)
    if name == "freeslip_minus_z":
        return _case("sphere_minus_z_perx", storage, **fs)
    return _case(name, storage)


@pytest.mark.parametrize("storage,tol", [("fp16", 5e-4), ("bf16", 5e-3)])
@pytest.mark.parametrize("name", PRECISION_CASES)
def test_shifted_storage_fields_vs_fp64(gpu, oracle_built, name, storage, tol):
    """Velocity and density against the FP64 run of the same set-up, on every
    boundary kind (bounce-back on a body and on ground rows, copy-own and free
    slip lateral faces, convective and zero-gradient outlets, flow along x, -x,
    y, -z). Tolerances: FP16 5e-4, BF16 5e-3 of max |u| (the w shift needed
    2e-3 / 2e-2 on the first case)."""
    case, mask, p = _precision_case(name, storage)
    s = gpu.Solver(p, mask)
    s.step(case["steps"])
    a = s.fields()
    b = _fp64_fields(oracle_built, p, mask, case["steps"])   # the oracle reads no storage field
    umax = max(float(np.max(np.abs(b[k]))) for k in ("ux", "uy", "uz"))
    err = max(float(np.max(np.abs(a[k] - b[k]))) for k in ("ux", "uy", "uz"))
    print(f"{name} {storage}: max |du| / max |u| = {err / umax:.2e}")
    assert err <= tol * umax, (name, storage, err / umax)
    assert float(np.max(np.abs(a["rho"] - b["rho"]))) <= tol


def test_weights_shift_remains_available(gpu, oracle_built):
    """storage_shift = WEIGHTS stores f - w (the earlier form): still within
    its own bound (2e-3 of max |u| in FP16) and not equal to the default."""
    from aeros_gb300 import capi
    case, mask, p = _case("sphere_trt_les_conv", "fp16", storage_shift=capi.AEROS_SHIFT_WEIGHTS)
    s = gpu.Solver(p, mask)
    s.step(case["steps"])
    a = s.fields()
    _, _, p2 = _case("sphere_trt_les_conv", "fp16")
    s2 = gpu.Solver(p2, mask)
    s2.step(case["steps"])
    assert not np.array_equal(a["ux"], s2.fields()["ux"])
    b = _fp64_fields(oracle_built, p, mask, case["steps"])
    assert float(np.max(np.abs(a["ux"] - b["ux"]))) <= 2e-3 * float(np.max(np.abs(b["ux"])))


HEADLINE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "headline_cd.json")


def test_headline_sphere_cd_against_fp64(gpu):
    """The configuration's 20,000 steps (240 x 120 x 115 sphere, icosphere
    level 6 of radius 12, TRT + Smagorinsky, inlet 0.05, zero-gradient outlet,
    free-slip walls): Cd by the FP64 control-volume balance, mean of the 50
    readings over the last 1,000 steps, against the FP64 run of the oracle
    (tests/golden/headline_cd.json, generated by tests/golden/headline_cd.py).
    Tolerances:
      FP16 storage against FP64: 0.5 % (measured +0.04 %);
      the plain FP32 form against FP64: 1 %. It is the reference's float
        arithmetic bit for bit, and its rounding drifts the mean density and
        Cd (measured -0.6 %): a property of the reference, bounded here;
      FP16 against the plain form: 0.5 % plus the plain form's own distance
        to FP64 (FP16 sits on the FP64 side);
      BF16 against FP64: 1 % (measured -0.3 %)."""
    from golden import headline_cd as H
    ref = json.load(open(HEADLINE))["cd_window_mean"]
    cd = {st: H.run(lambda p, m: gpu.Solver(p, m), st)["cd_window_mean"] for st in ("fp32", "fp16", "bf16")}
    print("headline Cd (mean of steps 19020..20000): fp64 %.6f fp32 %.6f (%+.3f %%) fp16 %.6f (%+.3f %%) "
          "bf16 %.6f (%+.3f %%)" % (ref, cd["fp32"], 100 * (cd["fp32"] / ref - 1), cd["fp16"], 100 * (cd["fp16"] / ref - 1),
                                    cd["bf16"], 100 * (cd["bf16"] / ref - 1)))
    assert abs(cd["fp16"] - ref) <= 0.005 * ref
    assert abs(cd["fp32"] - ref) <= 0.01 * ref
    assert abs(cd["fp16"] - cd["fp32"]) <= 0.005 * ref + abs(cd["fp32"] - ref)
    assert abs(cd["bf16"] - ref) <= 0.01 * ref


def _rb_nusselt(gpu, ra, storage, steps):
    from aeros_gb300 import geometry
    p, mask, tp = geometry.rb_config(ra, storage=storage)
    s = gpu.Solver(p, mask)
    s.thermal_init(tp)
    s.thermal_upload(geometry.rb_initial_T(p.nx, p.ny, p.nz, ra))
    s.step(steps)
    st = s.stats()
    s.close()
    return float(st["nusselt"]), int(st["diverged"])


def test_rayleigh_benard_ra1e4_convects_in_fp16(gpu):
    """Rayleigh-Benard at Ra = 1e4 (128 x 32 fluid rows x 128, Pr 0.71, linear
    profile + 1e-3 seeded noise, 50,000 steps): the FP16 form convects as the
    FP32 one does (with the w T_ref thermal shift it stayed conductive, Nu
    1.000). The Nusselt number of this wide box still wanders by a few per
    cent between readings while its rolls settle, so one reading of FP16 is
    held within 5 % of FP32 (measured -2.0 %); the quantitative check of the
    thermal lattice in FP16 is the reference's validation runs
    (test_validation.py)."""
    nu32, d32 = _rb_nusselt(gpu, 1e4, "fp32", 50000)
    nu16, d16 = _rb_nusselt(gpu, 1e4, "fp16", 50000)
    print(f"RB Ra 1e4 Nu: fp32 {nu32:.5f} fp16 {nu16:.5f} ({nu16 / nu32 - 1:+.3%})")
    assert d32 == 0 and d16 == 0
    assert nu32 > 2.0 and nu16 > 2.0
    assert abs(nu16 - nu32) <= 0.05 * nu32
