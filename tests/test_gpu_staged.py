"""GPU: the staged interior step (populations brought into a shared-memory
ring by bulk copies, k_lbm_staged) against the direct single-launch step
(k_lbm_fused). Same arithmetic, so populations and fields must be bit for bit
equal, in every storage form and on every boundary kind; the statistics are
exact fixed-point sums of per-cell values, so they are equal too although the
two kernels group cells differently."""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, params_for, solver_mask

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def _run(monkeypatch, staged, name, storage, steps, **mod):
    from aeros_gb300 import solver
    monkeypatch.setenv("AEROS_STAGED", "1" if staged else "0")
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
def test_staged_equals_direct(monkeypatch, name, mod, storage):
    steps = [CASES[name]["steps"] // 2 + 1, 6, 7]
    a = _run(monkeypatch, True, name, storage, steps, **mod)
    b = _run(monkeypatch, False, name, storage, steps, **mod)
    for (fa, va, sa), (fb, vb, sb) in zip(a, b):
        assert np.array_equal(fa, fb)
        for k in va:
            assert np.array_equal(va[k], vb[k]), k
        for k in ("sum_rho", "sum_kinetic", "sum_tke", "max_velocity_lb", "step", "negative_pops", "u_limited"):
            assert sa[k] == sb[k], k
