"""Drag coefficient of the 240 x 120 x 115 sphere configuration from an FP64
run of the C restatement: the yardstick for the plain FP32 form and the
16-bit storage forms over the configuration's 20,000 steps.

Set-up (aeros_gb300.geometry.sphere_config): icosphere level 6, radius 12
cells, centre (60, 60, 57.5); TRT (magic 3/16) + Smagorinsky Cs 0.1; uniform
inlet u = 0.05 on x = 0; zero-gradient outlet; free-slip lateral walls;
tau from Re 100 on D = 2r. The mask is the committed bit-exact voxel mask
(masks.npz, "sphere_config_mask").

Cd is the control-volume momentum balance (aeros/src/lbm.cpp:2183-2230) on
the box x 30..90, y 30..90, z 27..88 around the sphere, over
0.5 * u^2 * A with A the projected area in cells (lbm.cpp:2232-2256). It is
read every 500 steps from 10,000 on and every 20 steps over the last 1,000;
tests compare the mean over those last 50 readings.

    python tests/golden/headline_cd.py      # ~95 min on 8 threads

writes headline_cd.json beside this file.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "aeros-engine_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

FIXTURE = os.path.join(HERE, "headline_cd.json")
STEPS = 20000
COARSE = 500          # reading interval from 10,000 steps
FINE = 20             # reading interval over the last 1,000 steps
WINDOW = 1000
CV_BOX = [30, 90, 30, 90, 27, 88]
U_IN = 0.05


def readings():
    """Step counts at which Cd is read: every COARSE steps from 10,000, then
    every FINE steps over the last WINDOW steps."""
    coarse = list(range(10000, STEPS - WINDOW + 1, COARSE))
    fine = list(range(STEPS - WINDOW + FINE, STEPS + 1, FINE))
    return coarse, fine


def sphere_mask():
    from aeros_gb300 import geometry
    nx, ny, nz = geometry.SPHERE_GRID
    masks = np.load(os.path.join(HERE, "masks.npz"))
    return np.unpackbits(masks["sphere_config_mask"])[: nx * ny * nz].astype(np.uint8)


def run(make, storage="fp32"):
    """Step the configuration through `make(params, mask)` (a GPU Solver or
    the oracle) and return the Cd and mean-density readings."""
    from aeros_gb300 import geometry
    p, mask, _ = geometry.sphere_config(storage=storage, mask=sphere_mask())
    s = make(p, mask)
    area = s.projected_area(0)
    q = 0.5 * U_IN * U_IN * area
    coarse, fine = readings()
    steps, cd, rho = [], [], []
    k = 0
    for target in coarse + fine:
        s.step(target - k)
        k = target
        steps.append(k)
        cd.append(float(s.cv_force_box(CV_BOX)[0]) / q)
        rho.append(float(s.stats()["avg_rho"]))
    c = getattr(s, "close", None)
    if c:
        c()
    n_fine = len(fine)
    return {"steps": steps, "cd": cd, "avg_rho": rho, "area": float(area),
            "cd_window_mean": float(np.mean(cd[-n_fine:])), "cd_window_std": float(np.std(cd[-n_fine:]))}


def main():
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads, "f64")
    t0 = time.time()
    res = run(lambda p, m: O.OracleLBM(p, m, "f64"))
    res["note"] = ("FP64 run of the C restatement on the 240x120x115 sphere configuration, generated by "
                   "tests/golden/headline_cd.py (%d threads, %.0f s)" % (threads, time.time() - t0))
    with open(FIXTURE, "w") as fh:
        json.dump(res, fh, indent=1)
    print(json.dumps({k: res[k] for k in ("cd_window_mean", "cd_window_std", "area")}))


if __name__ == "__main__":
    main()
