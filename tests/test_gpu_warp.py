"""GPU: the schedules of the single-launch step against each other, bit for
bit. The warp-tiled interior (each warp's tiles brought into shared memory by
16-byte cp.async copies, double buffered, k_lbm_warp; AEROS_WARP=1) and the
direct step (k_lbm_fused) with the boundary shell on dedicated blocks
(AEROS_SHELL_BLOCKS=1) or first in the tile queue (AEROS_SHELL_BLOCKS=0) do
the same arithmetic, so populations and fields must be equal in every storage
form and on every boundary kind; the statistics are exact fixed-point sums of
per-cell values, so they are equal too although the schedules group cells
differently."""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, params_for, solver_mask

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def _run(monkeypatch, env, name, storage, steps, **mod):
    from aeros_gb300 import solver
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    case = CASES[name]
    mask = solver_mask(case)
    p = params_for(case, GOLD["cases"][name]["u_in"], storage)
    for k, v in mod.items():
        setattr(p, k, v)
    s = solver.Solver(p, mask)
    out = []
    for n in steps:   # odd and even call lengths: both kernels' parities and layouts
        s.step(n)
        f = s.fields()
        out.append((s.populations(), {k: f[k] for k in ("rho", "ux", "uy", "uz", "strain", "tke")}, s.stats()))
    s.close()
    return out


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("name,mod", [
    ("sphere_trt_les_conv", {}),
    ("sphere_les_ground_copy", {}),
    ("sphere_plus_y", {}),
    ("sphere_minus_z_perx", {}),
    ("channel_force3", {}),
    ("sphere_trt_les_conv", {"lateral_bc": 1, "outlet_bc": 1, "convective_outlet": 0}),
])
@pytest.mark.parametrize("env", [{"AEROS_WARP": "1", "AEROS_SHELL_BLOCKS": "1"},
                                 {"AEROS_WARP": "0", "AEROS_SHELL_BLOCKS": "0"}], ids=["warp", "shell_queue"])
def test_schedules_equal_direct(monkeypatch, env, name, mod, storage):
    steps = [CASES[name]["steps"] // 2 + 1, 6, 7]
    a = _run(monkeypatch, env, name, storage, steps, **mod)
    b = _run(monkeypatch, {"AEROS_WARP": "0", "AEROS_SHELL_BLOCKS": "1"}, name, storage, steps, **mod)
    for (fa, va, sa), (fb, vb, sb) in zip(a, b):
        assert np.array_equal(fa, fb)
        for k in va:
            assert np.array_equal(va[k], vb[k]), k
        for k in ("sum_rho", "sum_kinetic", "sum_tke", "max_velocity_lb", "step", "negative_pops", "u_limited"):
            assert sa[k] == sb[k], k
