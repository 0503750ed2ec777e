"""The reference's own validation runs, written once for three drivers.

The runs and the quantities they report follow the reference's headless
validation programs:

  viscosity decay   aeros/tests/physics_ref_headless.cpp:168-178, 216-225
  grid order        aeros/tests/physics_ref_headless.cpp:180-185, 227-243
  diffusion         aeros/tests/thermal_headless.cpp:153-186
  advection         aeros/tests/thermal_headless.cpp:188-242
  conduction        aeros/tests/thermal_headless.cpp:244-283
  Rayleigh-Benard   aeros/tests/thermal_headless.cpp:285-334 (Ra 1000, 1700, 2500)
  buoyancy sign     aeros/tests/thermal_headless.cpp:336-355

A run is a case in the format of cases.CASES (grid, solid mask, the
reference's set-up keywords, thermal settings, an uploaded temperature)
plus the step counts at which it is read. Drivers:

  RefDriver     the reference's own solver (oracle/_ref, the fixtures)
  SolverDriver  the GPU library through the C ABI, or the C restatement

Generate the fixtures (validation.json) where the reference tree exists:

    python tests/golden/validation.py
    python tests/golden/validation.py --f64    # the FP64 summary (C restatement)
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "aeros-engine_gb300"), os.path.join(ROOT, "oracle"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

from cases import channel, digest, params_for, thermal_params_for  # noqa: E402

FIXTURE = os.path.join(HERE, "validation.json")
TAU_PHYS = 0.65          # physics_ref_headless.cpp:194
FORCE32 = 7.8e-6         # physics_ref_headless.cpp:201 (H = 32)


def _box(nx, ny, nz, walls=False):
    return (lambda: channel(nx, ny, nz)) if walls else (lambda: np.zeros((nz, ny, nx), np.uint8))


def _wave_T(nx, ny, nz):
    """T = 0.5 + 0.5 cos(2 pi x / L), thermal_headless.cpp:165-169."""
    k = 2.0 * math.pi / nx
    row = np.array([np.float32(0.5 + 0.5 * math.cos(k * x)) for x in range(nx)], np.float32)
    return np.broadcast_to(row, (nz, ny, nx)).copy()


def _thermal(ra, fixed, pert, pr=1.0):
    return dict(rayleigh=ra, prandtl=pr, fixed=fixed, hot=1.0, cold=0.0, perturbation=pert)


PERIODIC = dict(tau=0.65, u0=0.0, periodic_x=True, periodic_z=True)

# name -> case (cases.CASES format) + "reads": the step counts at which the run is read
RUNS = {
    # physics_ref_headless.cpp:65-106 with the force off: the reference's
    # default inlet speed 0.08 (lbm.cpp:195) decays between the walls
    "decay": dict(grid=(8, 34, 8), solid=_box(8, 34, 8, True), reads=(5000, 6000),
                  kw=dict(tau=TAU_PHYS, u0=0.0, periodic_x=True, periodic_z=True, body_force=(0.0, 0.0, 0.0))),
    "diffusion": dict(grid=(32, 16, 8), solid=_box(32, 16, 8), reads=(0, 1500), kw=dict(PERIODIC),
                      thermal=_thermal(0.0, False, 0.0), upload=lambda: _wave_T(32, 16, 8)),
    "advection": dict(grid=(32, 16, 8), solid=_box(32, 16, 8), reads=(0, 1200), kw=dict(PERIODIC, u0=0.05),
                      thermal=_thermal(0.0, False, 0.0), upload=lambda: _wave_T(32, 16, 8)),
    "conduction": dict(grid=(24, 18, 8), solid=_box(24, 18, 8, True), reads=(6000,), kw=dict(PERIODIC),
                       thermal=_thermal(0.0, True, 0.0), upload=lambda: np.full((8, 18, 24), 0.5, np.float32)),
    "rb_1000": dict(grid=(32, 18, 8), solid=_box(32, 18, 8, True), reads=(6000, 24000), kw=dict(PERIODIC),
                    thermal=_thermal(1000.0, True, 0.02)),
    "rb_1700": dict(grid=(32, 18, 8), solid=_box(32, 18, 8, True), reads=(6000, 24000), kw=dict(PERIODIC),
                    thermal=_thermal(1700.0, True, 0.02)),
    "rb_2500": dict(grid=(32, 18, 8), solid=_box(32, 18, 8, True), reads=(6000, 24000), kw=dict(PERIODIC),
                    thermal=_thermal(2500.0, True, 0.02)),
    "buoyancy": dict(grid=(8, 8, 8), solid=_box(8, 8, 8), reads=(1,), kw=dict(PERIODIC),
                     thermal=_thermal(1.0, False, 0.0), upload=lambda: _hot_cold_T()),
}


def _hot_cold_T():
    """thermal_headless.cpp:345-347: 0.5 with a hot cell (4, 5, 0), a cold one (4, 2, 0)."""
    T = np.full((8, 8, 8), 0.5, np.float32)
    T[0, 5, 4] = 1.0
    T[0, 2, 4] = 0.0
    return T


# ---- quantities, as the reference's programs compute them -------------------
def centre_velocity(ux, grid):
    """physics_ref_headless.cpp:122-150: the profile averaged over x at
    z = nz/2; its largest value within 0.75 of the channel centre."""
    nx, ny, nz = grid
    u = ux.reshape(nz, ny, nx)[nz // 2].astype(np.float64)
    yc = 0.5 * (ny - 1)
    best = 0.0
    for y in range(1, ny - 1):
        v = float(np.sum(u[y]) / nx)
        if abs(y - yc) <= 0.75:
            best = max(best, v)
    return best


def harmonic(T, grid):
    """First x harmonic at (ny/2, nz/2): amplitude and phase
    (thermal_headless.cpp:106-132)."""
    nx, ny, nz = grid
    row = T.reshape(nz, ny, nx)[nz // 2, ny // 2].astype(np.float64)
    k = 2.0 * math.pi / nx
    re = im = 0.0
    for x in range(nx):
        re += row[x] * math.cos(k * x)
        im -= row[x] * math.sin(k * x)
    return 2.0 * math.sqrt(re * re + im * im) / nx, math.atan2(im, re)


def perturbation_rms(T, solid, grid, hot=1.0, cold=0.0):
    """RMS deviation from the conduction profile over the fluid rows
    (thermal_headless.cpp:135-150)."""
    nx, ny, nz = grid
    t = T.reshape(nz, ny, nx).astype(np.float64)
    s = solid.reshape(nz, ny, nx)
    span = max(1.0, float(ny - 2))
    acc, n = 0.0, 0
    for y in range(1, ny - 1):
        lin = hot + (cold - hot) * ((y - 0.5) / span)
        d = t[:, y, :][s[:, y, :] == 0] - lin
        acc += float(np.sum(d * d))
        n += d.size
    return math.sqrt(acc / n) if n else 0.0


def conduction_error(T, solid, grid):
    """Largest deviation from the linear profile at x = nx/2
    (thermal_headless.cpp:262-272)."""
    nx, ny, nz = grid
    t = T.reshape(nz, ny, nx)
    s = solid.reshape(nz, ny, nx)
    span = float(ny - 2)
    err = 0.0
    for z in range(nz):
        for y in range(1, ny - 1):
            if s[z, y, nx // 2]:
                continue
            lin = 1.0 + (0.0 - 1.0) * ((y - 0.5) / span)
            err = max(err, abs(float(t[z, y, nx // 2]) - lin))
    return err


def run(name, driver) -> dict:
    """Runs RUNS[name] on `driver` and returns its readings: the quantity the
    reference prints at each read, plus digests of the final fields."""
    case = RUNS[name]
    d = driver(name, case)
    grid = case["grid"]
    out = {"reads": {}}
    done = 0
    for k in case["reads"]:
        d.step(k - done)
        done = k
        fl = d.fields()
        r = {"u_centre": centre_velocity(fl["ux"], grid), "ux_mean": float(np.mean(fl["ux"][d.solid == 0], dtype=np.float64))}
        if case.get("thermal"):
            T, buoy, nu = d.thermal()
            amp, ph = harmonic(T, grid)
            r.update(amplitude=amp, phase=ph, nusselt=nu, rms=perturbation_rms(T, d.solid, grid),
                     conduction_err=conduction_error(T, d.solid, grid),
                     buoy_hot=float(buoy.reshape(grid[2], grid[1], grid[0])[0, 5, 4]) if name == "buoyancy" else None,
                     buoy_cold=float(buoy.reshape(grid[2], grid[1], grid[0])[0, 2, 4]) if name == "buoyancy" else None)
            out["T_digest"] = digest(T)
        out["reads"][str(k)] = r
        out["digest"] = {k2: digest(fl[k2]) for k2 in ("rho", "ux", "uy", "uz")}
    d.close()
    return out


def summarise(res: dict) -> dict:
    """The numbers the reference's programs print, from the readings."""
    s = {}
    dec = res["decay"]["reads"]
    s["decay_lambda"] = math.log(dec["5000"]["u_centre"] / dec["6000"]["u_centre"]) / 1000.0
    s["decay_lambda_exact"] = (TAU_PHYS - 0.5) / 3.0 * math.pi ** 2 / (32.0 * 32.0)
    k = 2.0 * math.pi / 32.0
    dif = res["diffusion"]["reads"]
    s["alpha_diffusion"] = -math.log(max(1e-12, dif["1500"]["amplitude"] / dif["0"]["amplitude"])) / (k * k * 1500)
    adv = res["advection"]["reads"]
    u_act = adv["1200"]["ux_mean"]
    dphi = adv["1200"]["phase"] - (adv["0"]["phase"] - k * u_act * 1200)
    while dphi > math.pi:
        dphi -= 2.0 * math.pi
    while dphi < -math.pi:
        dphi += 2.0 * math.pi
    s["advection_phase_speed"] = u_act * (1.0 + dphi / (k * u_act * 1200))
    s["advection_phase_residual"] = dphi
    s["alpha_advection"] = -math.log(max(1e-12, adv["1200"]["amplitude"] / adv["0"]["amplitude"])) / (k * k * 1200)
    s["conduction_max_err"] = res["conduction"]["reads"]["6000"]["conduction_err"]
    s["conduction_nusselt"] = res["conduction"]["reads"]["6000"]["nusselt"]
    for ra in ("1000", "1700", "2500"):
        r = res["rb_" + ra]["reads"]
        s[f"rb_{ra}_amp_6000"] = r["6000"]["rms"]
        s[f"rb_{ra}_amp_24000"] = r["24000"]["rms"]
        s[f"rb_{ra}_nusselt"] = r["24000"]["nusselt"]
    s["buoyancy_hot"] = res["buoyancy"]["reads"]["1"]["buoy_hot"]
    s["buoyancy_cold"] = res["buoyancy"]["reads"]["1"]["buoy_cold"]
    return s


# ---- drivers ---------------------------------------------------------------------
class RefDriver:
    """The reference's own solver, stepped one call per step."""

    def __init__(self, R, name, case, record):
        self.R = R
        nx, ny, nz = case["grid"]
        self.solid = case["solid"]().astype(np.uint8).reshape(-1)
        u_in = R.setup(nx, ny, nz, self.solid, **case["kw"])
        record["u_in"] = [float(v) for v in u_in]
        th = case.get("thermal")
        if th:
            R.thermal_setup(th["rayleigh"], th["prandtl"], th["fixed"], th["hot"], th["cold"], th["perturbation"])
            if "upload" in case:
                R.thermal_upload(case["upload"]())

    def step(self, n):
        if n:
            self.R.step(n)

    def fields(self):
        return self.R.fields()

    def thermal(self):
        T, b, nu, _ = self.R.thermal()
        return T, b, nu

    def close(self):
        pass


class SolverDriver:
    """A GPU Solver (aeros_gb300.solver) or an oracle OracleLBM on the
    reference's set-up (u_in as the reference derived it)."""

    def __init__(self, make, name, case, u_in, storage="fp32"):
        self.solid = case["solid"]().astype(np.uint8).reshape(-1)
        p = params_for(case, u_in, storage)
        self.s = make(p, self.solid.reshape(case["grid"][::-1]))
        if case.get("thermal"):
            self.s.thermal_init(thermal_params_for(case, p.tau))
            if "upload" in case:
                self.s.thermal_upload(case["upload"]())

    def step(self, n):
        if n:
            self.s.step(n)

    def fields(self):
        return self.s.fields()

    def thermal(self):
        T, b = self.s.thermal()
        return T, b, float(self.s.stats()["nusselt"])

    def close(self):
        c = getattr(self.s, "close", None)
        if c:
            c()


def solver_results(make, fixture=None, names=None, storage="fp32") -> dict:
    fx = fixture or json.load(open(FIXTURE))
    out = {}
    for name in (names or RUNS):
        out[name] = run(name, lambda n, c: SolverDriver(make, n, c, fx["runs"][n]["u_in"], storage))
    return out


def main():
    import oracle as O
    O.build()
    R = O.RefHarness()
    res = {}
    for name in RUNS:
        rec = {}
        res[name] = run(name, lambda n, c: RefDriver(R, n, c, rec))
        res[name]["u_in"] = rec["u_in"]
        print(f"  {name}: {json.dumps(res[name]['reads'])[:160]}")
    s = summarise(res)
    for k, v in s.items():
        print(f"  {k}: {v}")
    with open(FIXTURE, "w") as fh:
        json.dump({"note": "the reference's validation runs, generated by tests/golden/validation.py from the "
                           "reference's own solver", "runs": res, "summary": s}, fh, indent=1, sort_keys=True)


def make_f64_summary():
    """The same runs stepped by the C restatement in FP64: the yardstick the
    16-bit storage forms state their errors against. Added to validation.json
    as "summary_f64" (python tests/golden/validation.py --f64)."""
    import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1, "f64")
    fx = json.load(open(FIXTURE))
    res = solver_results(lambda p, m: O.OracleLBM(p, m, "f64"), fx)
    fx["summary_f64"] = summarise(res)
    for k, v in fx["summary_f64"].items():
        print(f"  {k}: {v}")
    with open(FIXTURE, "w") as fh:
        json.dump(fx, fh, indent=1, sort_keys=True)



# ---- the full-size configurations (C restatement as the checker) -----------------
# The sphere configuration runs free-slip walls and a zero-gradient outlet,
# which the reference does not have, and the Rayleigh-Benard configuration a
# seeded noise start the reference has no loader for in its programs: their
# fixtures come from the C restatement (bitwise the reference on every mode
# the reference has), stepped here.
CONFIG_STEPS = {"sphere_240x120x115": 200, "rb_128x34x128_ra1e4": 2000}
CONFIG_FIXTURE = os.path.join(HERE, "configs.json")


def config_case(name, storage="fp32"):
    """(params, mask, initial T or None) of a full-size configuration."""
    from aeros_gb300 import geometry
    if name == "sphere_240x120x115":
        nx, ny, nz = geometry.SPHERE_GRID
        masks = np.load(os.path.join(HERE, "masks.npz"))
        mask = np.unpackbits(masks["sphere_config_mask"])[: nx * ny * nz].astype(np.uint8)
        p, mask, _ = geometry.sphere_config(storage=storage, mask=mask)
        return p, mask, None, None
    p, mask, tp = geometry.rb_config(1e4, storage=storage)
    return p, mask, tp, geometry.rb_initial_T(p.nx, p.ny, p.nz, 1e4)


def run_config(make, name, storage="fp32") -> dict:
    p, mask, tp, T0 = config_case(name, storage)
    s = make(p, mask)
    if tp is not None:
        s.thermal_init(tp)
        s.thermal_upload(T0)
    s.step(CONFIG_STEPS[name])
    fl = s.fields()
    out = {"steps": CONFIG_STEPS[name], "digest": {k: digest(fl[k]) for k in ("rho", "ux", "uy", "uz")},
           "fields": {k: fl[k] for k in ("rho", "ux", "uy", "uz")}}
    if tp is not None:
        T, _ = s.thermal()
        out["T_digest"] = digest(T)
        out["fields"]["T"] = T
        out["nusselt"] = float(s.stats()["nusselt"])
    c = getattr(s, "close", None)
    if c:
        c()
    return out


def make_config_fixture():
    import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1, "f32")
    res = {}
    for name in CONFIG_STEPS:
        r = run_config(lambda p, m: O.OracleLBM(p, m), name)
        r.pop("fields")
        res[name] = r
        print(f"  {name}: {r}")
    with open(CONFIG_FIXTURE, "w") as fh:
        json.dump({"note": "full-size configurations stepped by the C restatement (tests/golden/validation.py "
                           "--configs)", "configs": res}, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    if "--configs" in sys.argv:
        make_config_fixture()
    elif "--f64" in sys.argv:
        make_f64_summary()
    else:
        main()
