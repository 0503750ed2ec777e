"""Shared driver of the post-processing parity checks (CPU oracle and GPU):
step a golden case, read the world fields after the last two steps (the
residuals compare consecutive readbacks), then vorticity / Q / strain and the
samplers, and compare everything with tests/golden/post.json, recorded from
the reference's own functions."""
import json
import os

import numpy as np

from golden.cases import CASES, POST_CASES, POST_FLOW_SPEED, fdigest, params_for, post_points, solver_mask

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))
POST = json.load(open(os.path.join(HERE, "golden", "post.json")))


def post_case(name):
    """The golden case as the post-processing fixtures ran it (their
    freestream speed sets the TKE velocity scale too)."""
    case = CASES[name]
    return dict(case, kw=dict(case["kw"], flow_speed=POST_FLOW_SPEED))


def world_of(name):
    from aeros_gb300 import capi
    w = POST[name]["world"]
    return capi.make_world(w[0], w[1], w[2:5], w[5:8])


def check_post(name, make, step, world_fields, vorticity_q, sample):
    """make(params, mask) -> domain; step(dom, n); world_fields(dom, wp) ->
    (fields, stats); vorticity_q(dom, wp) -> fields; sample(dom, wp, f, pts)."""
    case = post_case(name)
    ref = POST[name]
    wp = world_of(name)
    dom = make(params_for(case, GOLD["cases"][name]["u_in"]), solver_mask(case))
    n = case["steps"]
    step(dom, n - 1)
    world_fields(dom, wp)
    step(dom, 1)
    fields, stats = world_fields(dom, wp)
    assert {k: fdigest(v) for k, v in fields.items()} == ref["fields"]
    for k in ("pressure_min", "pressure_max", "residual_u", "pressure_non_finite"):
        assert np.float32(stats[k]) == np.float32(ref["stats"][k]), k
    # the density residual is a double sum reduced in another order: to 1 ulp
    a, b = np.float32(stats["residual_rho"]), np.float32(ref["stats"]["residual_rho"])
    assert abs(int(a.view(np.int32)) - int(b.view(np.int32))) <= 1
    vq = vorticity_q(dom, wp)
    assert {k: fdigest(v) for k, v in vq.items()} == ref["vorticity"]
    pts = post_points(case["grid"])
    for f in range(8):
        v, ok = sample(dom, wp, f, pts)
        assert fdigest(v) == ref["samples"][str(f)]["value"], f
        if f not in (0, 7):   # the reference's velocity and solid samplers report no validity
            assert fdigest(ok.astype(np.float32)) == ref["samples"][str(f)]["valid"], f
    return dom
