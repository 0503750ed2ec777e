"""Generates tests/golden/golden.json and the mask fixtures from the
reference's OWN solver sources (oracle/_ref/libaeros_ref.so, built in place by
``make -C oracle ref``). Run where the reference tree exists:

    python tests/golden/make_golden.py

Every fixture is small: SHA-256 digests of float32 fields, scalars, and
bit-packed masks. The reference is stepped one call per step (see
oracle/ref_harness.cpp on why).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "aeros-engine_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from cases import CASES, EQ_MOMENT_CASES, outputs_digest, solver_mask  # noqa: E402

from aeros_gb300 import geometry  # noqa: E402


def run_case(R, name, case):
    nx, ny, nz = case["grid"]
    solid = case["solid"]().astype(np.uint8).reshape(-1)
    kw = dict(case["kw"])
    u_in = R.setup(nx, ny, nz, solid, ground_rows=case.get("ground_rows", 0), **kw)
    if "u_init" in case:
        R.set_uniform(*case["u_init"])
    th = case.get("thermal")
    if th:
        R.thermal_setup(th["rayleigh"], th["prandtl"], th["fixed"], th["hot"], th["cold"], th["perturbation"])
        if "upload" in case:
            R.thermal_upload(case["upload"]())
    R.step(case["steps"])
    fields = R.fields()
    f = R.populations()
    mask = solver_mask(case)
    T = buoy = None
    out = {"u_in": [float(v) for v in u_in]}
    if th:
        T, buoy, nu, mt = R.thermal()
        out["nusselt"] = nu
        out["mean_t"] = mt
    out["digest"] = outputs_digest(fields, f, mask, T, buoy)
    out["stats"] = R.stats()
    out["cv_force"] = [float(v) for v in R.cv_force(0.3, 0.3, 0.3)]
    out["area"] = [R.projected_area(a) for a in range(3)]
    out["wall_digest"] = __import__("cases").digest(R.wall_dist())
    out["checksum"] = {k: float(np.sum(fields[k], dtype=np.float64)) for k in ("rho", "ux", "uy", "uz")}
    print(f"  {name}: {case['steps']} steps, rho sum {out['checksum']['rho']:.9f}")
    return out


def channel_profile(R, ny, tau, force, steps, trt=False, nx=8, nz=8):
    """physics_ref_headless.cpp:65-166: profile averaged over x at z = nz/2."""
    solid = geometry.channel_mask(nx, ny, nz).reshape(-1)
    R.setup(nx, ny, nz, solid, tau=tau, u0=0.0, trt=trt, periodic_x=True, periodic_z=True,
            body_force=(force, 0.0, 0.0))
    R.set_uniform(0.0, 0.0, 0.0) if False else None   # reference starts at U0 -> 0.08 (lbm.cpp:196)
    R.step(steps)
    fl = R.fields()
    ux = fl["ux"].reshape(nz, ny, nx)
    prof = ux[nz // 2, 1:ny - 1, :].astype(np.float64).mean(axis=1)
    exact = geometry.poiseuille_exact(ny, tau, force)
    l2 = float(np.sqrt(np.sum((prof - exact) ** 2) / np.sum(exact ** 2)))
    mask = solid.reshape(nz, ny, nx)
    rho = fl["rho"].reshape(nz, ny, nx)
    drift = float(abs(rho[mask == 0].astype(np.float64).mean() - 1.0))
    yc = 0.5 * (ny - 1)
    s = np.arange(1, ny - 1) - yc
    uc = float(prof[np.abs(s) <= 0.75].max())
    return dict(l2=l2, u_center=uc, flux=float(prof.sum()), flux_exact=float(exact.sum()), mass_drift=drift,
                digest=outputs_digest(fl, None, mask), profile=[float(v) for v in prof])


def validation_sphere(R, res=48, d_cells=20, pad=0.15, warm=500, meas=50):
    """validation_headless.cpp:99-183 and :206-251: Cd of the Re = 100 sphere."""
    radius = 3.0 * d_cells / res
    dims, tau, u_in = R.validation_setup(0, res, radius, d_cells, 100.0, pad, 0.08)
    mask = R.mask()
    R.step(warm)
    area = R.projected_area(0)
    q = 0.5 * 0.08 * 0.08 * area
    cds = []
    for _ in range(meas):
        R.step(1)
        F = R.cv_force(0.3, 0.3, 0.3)
        cds.append(np.float32(F[0]) / np.float32(q))
    cd = float(np.mean(np.array(cds, np.float64)))
    fl = R.fields()
    return dict(dims=list(dims), tau=tau, u_in=[float(v) for v in u_in], area=area, cd=cd,
                cd_trace=[float(v) for v in cds], warm=warm, meas=meas,
                digest=outputs_digest(fl, R.populations(), mask.reshape(-1))), mask


def post_fixtures(R) -> dict:
    """World fields + readback statistics of the last step (lbm.cpp:1602-1705),
    computeLBMVorticityAndQ (lbm.cpp:2005-2093) and the samplers
    (lbm.cpp:1782-1969) of the reference, for POST_CASES."""
    from cases import POST_CASES, POST_FLOW_SPEED, fdigest, post_points
    out = {}
    for name in POST_CASES:
        case = CASES[name]
        nx, ny, nz = case["grid"]
        solid = case["solid"]().astype(np.uint8).reshape(-1)
        kw = dict(case["kw"])
        kw["flow_speed"] = POST_FLOW_SPEED
        R.setup(nx, ny, nz, solid, ground_rows=case.get("ground_rows", 0), **kw)
        if "u_init" in case:
            R.set_uniform(*case["u_init"])
        R.step(case["steps"])
        wf, st, wp = R.world()
        vq = R.vorticity_q()
        pts = post_points(case["grid"])
        samples = {}
        for f in range(8):
            v, ok = R.sample(f, pts)
            samples[str(f)] = dict(value=fdigest(v), valid=fdigest(ok.astype(np.float32)))
        out[name] = dict(world=wp, stats=st, fields={k: fdigest(v) for k, v in wf.items()},
                         vorticity={k: fdigest(v) for k, v in vq.items()}, samples=samples)
        print(f"  {name}: p in [{st['pressure_min']:.4g}, {st['pressure_max']:.4g}], residual {st['residual_rho']:.3g}")
    return out


def surface_fixtures(R) -> dict:
    """computeLiftDrag (forces.cpp:401-688) of the reference after the post
    cases' steps, for SURFACE_CASES: its outputs and the flow parameters its
    updateFlowParams resolved (velocity, temperature, density, speed of
    sound, Reynolds number), which the tests feed to the oracle and device."""
    from cases import (POST_FLOW_SPEED, SURFACE_CASES, SURFACE_DEFAULTS, digest, solver_mask, surface_mesh)
    import oracle as O
    out = {}
    for name, sc in SURFACE_CASES.items():
        case = CASES[sc["case"]]
        nx, ny, nz = case["grid"]
        solid = case["solid"]().astype(np.uint8).reshape(-1)
        kw = dict(case["kw"])
        kw["flow_speed"] = POST_FLOW_SPEED
        R.setup(nx, ny, nz, solid, ground_rows=case.get("ground_rows", 0), **kw)
        R.step(case["steps"])
        wp = R.world()[2]   # the step's world parameters (an earlier call's atmosphere update changes airDensity)
        v, n = surface_mesh(sc["mesh"])
        sdf = None
        if sc["sdf"]:
            m = (solver_mask(case).reshape(-1) == 1).astype(np.uint8)
            sdf = O.sdf(m, (nx, ny, nz), (1.0, 1.0, 1.0))
        aero = dict(SURFACE_DEFAULTS, **sc["aero"])
        r = R.lift_drag(v, n, sdf, **aero)
        res = {k: (list(getattr(r, k)) if k in ("drag_vec", "lift_vec", "moment", "cop", "vel")
                   else (int(r.cp_bad) if k == "cp_bad" else float(getattr(r, k)))) for k, _ in r._fields_}
        out[name] = dict(result=res, world=wp, mesh=digest(np.concatenate([v.reshape(-1), n.reshape(-1)])),
                         sdf=digest(sdf) if sdf is not None else None)
        print(f"  {name}: drag {r.drag:.6g} lift {r.lift:.6g} area {r.ref_area:.6g}")
    from cases import REF_AREA_CASES
    areas = []
    for kind, az, el, auto, area in REF_AREA_CASES:
        v, _ = surface_mesh(kind)
        d = SURFACE_DEFAULTS
        bmin, bmax = np.asarray(d["bb_min"], np.float32), np.asarray(d["bb_max"], np.float32)
        areas.append(float(R.L.ref_ref_area(O.fptr(np.ascontiguousarray(v, np.float32).reshape(-1)), v.shape[0], az, el,
                                            auto, area, O.fptr(bmin), O.fptr(bmax), d["max_dim"])))
    out["ref_area_cases"] = areas
    from cases import RE_CASES
    out["re_cases"] = [float(R.L.ref_lbm_re(*c)) for c in RE_CASES]
    print(f"  computeLBMRe: {out['re_cases']}")
    print(f"  computeLBMRefArea: {areas}")
    return out


def sdf_fixtures(R) -> dict:
    """buildVoxelGrid's mask and distance field (voxel_grid.cpp:224-553) and
    sampleSDFCPU / sdfNormalCPU (:32-123) of the reference, for SDF_CASES."""
    from cases import SDF_CASES, fdigest, pack_mask, sdf_mesh, sdf_points
    out = {}
    for name, case in SDF_CASES.items():
        g = R.build_voxel_grid(sdf_mesh(case, R), case["res"])
        nx, ny, nz = g["dims"]
        hi = g["min"] + g["cs"] * np.array([nx, ny, nz], np.float32)
        pts = sdf_points(g["min"], hi)
        dist, nrm = R.sdf_sample(pts)
        out[name] = dict(dims=[nx, ny, nz], min=[float(v) for v in g["min"]], cs=[float(v) for v in g["cs"]],
                         mask=pack_mask(g["mask"]), sdf=fdigest(g["sdf"]),
                         sdf_min=float(g["sdf"].min()), sdf_max=float(g["sdf"].max()),
                         dist=fdigest(dist), normal=fdigest(nrm))
        print(f"  {name}: {nx}x{ny}x{nz}, solid {int(g['mask'].sum())}, sdf [{g['sdf'].min():.4g}, {g['sdf'].max():.4g}]")
    return out


def stl_fixtures(R) -> dict:
    """stlformat::detect and loadSTL (stl_format.h:86-140, stl_loader.cpp:30-223)
    of the synthetic files of cases.stl_files()."""
    import tempfile
    from cases import fdigest, stl_files
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, data in stl_files().items():
            path = os.path.join(tmp, name + ".stl")
            with open(path, "wb") as fh:
                fh.write(data)
            det = R.stl_detect(data)
            n, v, nrm = R.stl_load(path)
            out[name] = dict(detect=det, triangles=n, vertices=fdigest(v) if n > 0 else None,
                             normals=fdigest(nrm) if n > 0 else None)
            print(f"  {name}: detect {det}, triangles {n}")
    return out


def main():
    O.build()
    R = O.RefHarness()
    if "--stl" in sys.argv:   # only the STL fixtures
        with open(os.path.join(HERE, "stl.json"), "w") as fh:
            json.dump(stl_fixtures(R), fh, indent=1, sort_keys=True)
        return
    if "--sdf" in sys.argv:   # only the distance-field fixtures
        with open(os.path.join(HERE, "sdf.json"), "w") as fh:
            json.dump(sdf_fixtures(R), fh, indent=1, sort_keys=True)
        return
    if "--surface" in sys.argv:   # only the surface-force fixtures
        with open(os.path.join(HERE, "surface.json"), "w") as fh:
            json.dump(surface_fixtures(R), fh, indent=1, sort_keys=True)
        return
    if "--post" in sys.argv:   # only the post-processing fixtures
        with open(os.path.join(HERE, "post.json"), "w") as fh:
            json.dump(post_fixtures(R), fh, indent=1, sort_keys=True)
        return
    out = {"cases": {}, "note": "generated from the reference sources by make_golden.py"}
    t0 = time.time()
    for name, case in CASES.items():
        out["cases"][name] = run_case(R, name, case)
    print("physref channels ...")
    out["physref"] = {
        "bgk_40k": channel_profile(R, 34, 0.65, 7.8e-6, 40000),
        "trt_40k": channel_profile(R, 34, 0.65, 7.8e-6, 40000, trt=True),
        "h8_4k": channel_profile(R, 10, 0.65, 7.8e-6 * 16.0, 4000),
        "h16_15k": channel_profile(R, 18, 0.65, 7.8e-6 * 4.0, 15000),
    }
    for k, v in out["physref"].items():
        print(f"  {k}: L2 {100 * v['l2']:.3f} %, u_c {v['u_center']:.6f}")
    # the Poiseuille configuration (64 x 32 x 32, tau 0.8, F 1e-6, u0 = 0, 4000 steps)
    print("poiseuille config ...")
    nx, ny, nz = 64, 32, 32
    solid = geometry.channel_mask(nx, ny, nz).reshape(-1)
    u_in = R.setup(nx, ny, nz, solid, tau=0.8, u0=0.0, periodic_x=True, periodic_z=True, body_force=(1e-6, 0, 0))
    R.set_uniform(0.0, 0.0, 0.0)
    R.step(4000)
    fl = R.fields()
    ux = fl["ux"].reshape(nz, ny, nx)
    prof = ux[:, 1:ny - 1, :].astype(np.float64).mean(axis=(0, 2))
    exact = geometry.poiseuille_exact(ny, 0.8, 1e-6)
    out["poiseuille_config"] = dict(u_in=[float(v) for v in u_in], steps=4000,
                                    l2=float(np.sqrt(np.sum((prof - exact) ** 2) / np.sum(exact ** 2))),
                                    digest=outputs_digest(fl, R.populations(), solid.reshape(nz, ny, nx)),
                                    stats=R.stats())
    print(f"  L2 vs exact {100 * out['poiseuille_config']['l2']:.4f} %")
    print("validation sphere ...")
    val, vmask = validation_sphere(R)
    out["validation_sphere"] = val
    print(f"  Cd {val['cd']:.4f} area {val['area']} dims {val['dims']} tau {val['tau']}")
    masks = {"validation_sphere_mask": np.packbits(vmask)}
    print("voxelizer ...")
    nx, ny, nz = geometry.SPHERE_GRID
    tris = geometry.icosphere(6, geometry.SPHERE_RADIUS, geometry.SPHERE_CENTER)
    t1 = time.time()
    sm = R.voxelize(tris, nx, ny, nz, (0, 0, 0), (1, 1, 1))
    print(f"  sphere config mask: {int(sm.sum())} solid cells in {time.time() - t1:.1f} s")
    masks["sphere_config_mask"] = np.packbits(sm)
    out["voxel"] = {"sphere_config": dict(solid=int(sm.sum()), ntri=int(tris.shape[0]),
                                          digest=__import__("cases").digest(sm))}
    vox_cases = {
        "uv_sphere_40": (geometry.uv_sphere(0.35, 32, 48), 40, (-0.5, -0.5, -0.5), 1.0 / 40),
        "torus_48": (geometry.torus(0.3, 0.11, 64, 32), 48, (-0.45, -0.2, -0.45), 0.9 / 48),
        "box_32": (geometry.box((0.3, 0.2, 0.25)), 32, (-0.4, -0.4, -0.4), 0.8 / 32),
        "plate_64": (geometry.box((0.3, 0.003, 0.2)), 64, (-0.4, -0.4, -0.4), 0.8 / 64),
    }
    for k, (tv, n, mn, cs) in vox_cases.items():
        m = R.voxelize(tv, n, n, n, mn, (np.float32(cs),) * 3)
        out["voxel"][k] = dict(solid=int(m.sum()), digest=__import__("cases").digest(m), n=n, min=list(mn), cell=cs)
        print(f"  {k}: {int(m.sum())} solid")
    out["eq_moments"] = [list(R.equilibrium_moments(*c)[1]) for c in EQ_MOMENT_CASES]
    out["voxel_plan"] = {"1x0.5x0.25@64/8G": list(R.voxel_plan([1, 0.5, 0.25], 64, 8 << 30)),
                         "1@512/512M": list(R.voxel_plan([1, 1, 1], 512, 512 << 20))}
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("post-processing ...")
    with open(os.path.join(HERE, "post.json"), "w") as fh:
        json.dump(post_fixtures(R), fh, indent=1, sort_keys=True)
    print("surface forces ...")
    with open(os.path.join(HERE, "surface.json"), "w") as fh:
        json.dump(surface_fixtures(R), fh, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "masks.npz"), **masks)
    print(f"done in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
