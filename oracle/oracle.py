"""ctypes bindings of the oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` — as the checker, never as the thing measured on the product
path. Two builds of the same C restatement: ``precision="f32"`` (bitwise the
reference's float arithmetic) and ``precision="f64"`` (the FP64 run).
``RefHarness`` drives the reference's own sources (built in place by
``make ref``; only where the reference tree exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "aeros-engine_gb300"))
from aeros_gb300.capi import (AEROS_FIELD_VELOCITY_LB, LbmParams, LbmStats, SurfaceForces,  # noqa: E402
                              SurfaceParams, ThermalParams, VoxelGrid, VoxelPlan, WorldParams, WorldStats)

_FP = C.POINTER(C.c_float)
_U8P = C.POINTER(C.c_uint8)
_DP = C.POINTER(C.c_double)


def build(quiet: bool = True) -> None:
    """Compiles the oracle libraries (and the reference harness when the
    reference tree is present)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE, "all"], stdout=out)
    present = subprocess.call(["make", "-s", "-C", HERE, "has-ref"], stdout=subprocess.DEVNULL,
                              stderr=subprocess.DEVNULL) == 0
    if present:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref"], stdout=out)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_FP)


def u8ptr(a: np.ndarray):
    return a.ctypes.data_as(_U8P)


_libs: dict[str, C.CDLL] = {}


def oracle_lib(precision: str = "f32") -> C.CDLL:
    if precision not in _libs:
        path = os.path.join(HERE, f"liboracle_{precision}.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.ao_lbm_create.restype = C.c_void_p
        L.ao_lbm_create.argtypes = [C.POINTER(LbmParams), _U8P]
        L.ao_lbm_destroy.argtypes = [C.c_void_p]
        L.ao_thermal_init.argtypes = [C.c_void_p, C.POINTER(ThermalParams)]
        L.ao_thermal_upload.argtypes = [C.c_void_p, _FP]
        L.ao_lbm_step.argtypes = [C.c_void_p, C.c_int]
        L.ao_lbm_get_stats.argtypes = [C.c_void_p, C.POINTER(LbmStats)]
        L.ao_lbm_get_fields.argtypes = [C.c_void_p] + [_FP] * 6
        L.ao_lbm_get_fields_f64.argtypes = [C.c_void_p] + [_DP] * 4
        L.ao_lbm_get_populations.argtypes = [C.c_void_p, _FP]
        L.ao_lbm_set_populations.argtypes = [C.c_void_p, _FP]
        L.ao_lbm_set_equilibrium.argtypes = [C.c_void_p, _FP, _FP, _FP, _FP]
        L.ao_lbm_get_wall_dist.argtypes = [C.c_void_p, _U8P]
        L.ao_thermal_get.argtypes = [C.c_void_p, _FP, _FP]
        L.ao_lbm_cv_force.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, _DP]
        L.ao_lbm_cv_force_box.argtypes = [C.c_void_p, C.POINTER(C.c_int32), _DP]
        L.ao_lbm_projected_area.restype = C.c_double
        L.ao_lbm_projected_area.argtypes = [C.c_void_p, C.c_int]
        L.ao_equilibrium_moments.argtypes = [C.c_float] * 4 + [_FP] * 4
        L.ao_voxelize_brute.argtypes = [_FP, C.c_int64, C.POINTER(VoxelGrid), _U8P]
        L.ao_count_hits_brute.argtypes = [_FP, C.c_int64, _FP, C.c_int]
        L.ao_voxel_plan.argtypes = [_FP, C.c_int, C.c_uint64, C.POINTER(VoxelPlan)]
        L.ao_set_threads.argtypes = [C.c_int]
        L.ao_sdf_reference.argtypes = [_U8P, C.c_int, C.c_int, C.c_int, _FP, _FP]
        L.ao_sdf_exact.argtypes = [_U8P, C.c_int, C.c_int, C.c_int, _FP, _FP]
        L.ao_sdf_sample.argtypes = [_FP, C.c_int, C.c_int, C.c_int, _FP, _FP, _FP, C.c_int64, _FP, _FP]
        L.ao_lbm_world_fields.argtypes = [C.c_void_p, C.POINTER(WorldParams), _FP, _FP, _FP, _FP,
                                          C.POINTER(WorldStats)]
        L.ao_lbm_vorticity_q.argtypes = [C.c_void_p, C.POINTER(WorldParams), _FP, _FP, _FP]
        L.ao_lbm_sample.argtypes = [C.c_void_p, C.POINTER(WorldParams), C.c_int, _FP, C.c_int64, _FP, _U8P]
        L.ao_surface_forces.argtypes = [C.c_void_p, C.POINTER(WorldParams), C.POINTER(SurfaceParams), _FP,
                                        C.POINTER(VoxelGrid), _FP, _FP, C.c_int64, C.c_int, C.POINTER(SurfaceForces),
                                        _FP]
        L.ao_surface_forces_field.argtypes = [_FP, _U8P, C.c_int, C.c_int, C.c_int, C.POINTER(WorldParams),
                                              C.POINTER(SurfaceParams), _FP, C.POINTER(VoxelGrid), _FP, _FP,
                                              C.c_int64, C.c_int, C.POINTER(SurfaceForces), _FP]
        _libs[precision] = L
    return _libs[precision]


def set_threads(n: int, precision: str = "f32") -> int:
    return oracle_lib(precision).ao_set_threads(int(n))


class OracleLBM:
    """One domain of the C restatement."""

    def __init__(self, params: LbmParams, mask: np.ndarray, precision: str = "f32"):
        self.L = oracle_lib(precision)
        self.precision = precision
        self.shape = (params.nz, params.ny, params.nx)
        self.n = params.nx * params.ny * params.nz
        self.mask = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        assert self.mask.size == self.n
        self.h = self.L.ao_lbm_create(C.byref(params), u8ptr(self.mask))
        if not self.h:
            raise RuntimeError("oracle create failed")

    def close(self):
        if self.h:
            self.L.ao_lbm_destroy(self.h)
            self.h = None

    __del__ = close

    def thermal_init(self, tp: ThermalParams) -> None:
        if self.L.ao_thermal_init(self.h, C.byref(tp)) != 0:
            raise RuntimeError("oracle thermal init failed")

    def thermal_upload(self, T: np.ndarray) -> None:
        t = np.ascontiguousarray(T, dtype=np.float32).reshape(-1)
        self.L.ao_thermal_upload(self.h, fptr(t))

    def step(self, n: int) -> None:
        self.L.ao_lbm_step(self.h, int(n))

    def stats(self) -> dict:
        s = LbmStats()
        self.L.ao_lbm_get_stats(self.h, C.byref(s))
        return s.as_dict()

    def fields(self) -> dict:
        out = {k: np.empty(self.n, np.float32) for k in ("rho", "ux", "uy", "uz", "strain", "tke")}
        self.L.ao_lbm_get_fields(self.h, *(fptr(out[k]) for k in ("rho", "ux", "uy", "uz", "strain", "tke")))
        return out

    def fields_f64(self) -> dict:
        out = {k: np.empty(self.n, np.float64) for k in ("rho", "ux", "uy", "uz")}
        self.L.ao_lbm_get_fields_f64(self.h, *(out[k].ctypes.data_as(_DP) for k in ("rho", "ux", "uy", "uz")))
        return out

    def populations(self) -> np.ndarray:
        f = np.empty((19, self.n), np.float32)
        self.L.ao_lbm_get_populations(self.h, fptr(f))
        return f

    def set_populations(self, f: np.ndarray) -> None:
        a = np.ascontiguousarray(f, dtype=np.float32)
        self.L.ao_lbm_set_populations(self.h, fptr(a))

    def set_equilibrium(self, rho, ux, uy, uz) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(-1) for a in (rho, ux, uy, uz)]
        self.L.ao_lbm_set_equilibrium(self.h, *(None if a is None else fptr(a) for a in arrs))

    def wall_dist(self) -> np.ndarray:
        w = np.empty(self.n, np.uint8)
        self.L.ao_lbm_get_wall_dist(self.h, u8ptr(w))
        return w

    def thermal(self) -> tuple[np.ndarray, np.ndarray]:
        T = np.empty(self.n, np.float32)
        b = np.empty(self.n, np.float32)
        self.L.ao_thermal_get(self.h, fptr(T), fptr(b))
        return T, b

    def cv_force(self, hx=0.3, hy=0.3, hz=0.3) -> np.ndarray:
        out = np.zeros(3, np.float64)
        self.L.ao_lbm_cv_force(self.h, hx, hy, hz, out.ctypes.data_as(_DP))
        return out

    def cv_force_box(self, box) -> np.ndarray:
        b = (C.c_int32 * 6)(*[int(v) for v in box])
        out = np.zeros(3, np.float64)
        self.L.ao_lbm_cv_force_box(self.h, b, out.ctypes.data_as(_DP))
        return out

    def projected_area(self, axis: int) -> float:
        return float(self.L.ao_lbm_projected_area(self.h, int(axis)))

    def world_fields(self, world: WorldParams) -> tuple[dict, dict]:
        out = {k: np.empty(self.n, np.float32) for k in ("ux", "uy", "uz", "pressure")}
        st = WorldStats()
        if self.L.ao_lbm_world_fields(self.h, C.byref(world), fptr(out["ux"]), fptr(out["uy"]), fptr(out["uz"]),
                                      fptr(out["pressure"]), C.byref(st)) != 0:
            raise RuntimeError("oracle world fields failed")
        return out, st.as_dict()

    def vorticity_q(self, world: WorldParams) -> dict:
        out = {k: np.empty(self.n, np.float32) for k in ("vorticity", "q", "strain")}
        if self.L.ao_lbm_vorticity_q(self.h, C.byref(world), fptr(out["vorticity"]), fptr(out["q"]),
                                     fptr(out["strain"])) != 0:
            raise RuntimeError("oracle vorticity failed")
        return out

    def sample(self, world: WorldParams, field: int, points: np.ndarray):
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        n = pts.shape[0]
        per = 3 if field == AEROS_FIELD_VELOCITY_LB else 1
        out = np.empty(n * per, np.float32)
        valid = np.empty(n, np.uint8)
        if self.L.ao_lbm_sample(self.h, C.byref(world), int(field), fptr(pts), n, fptr(out), u8ptr(valid)) != 0:
            raise RuntimeError("oracle sample failed")
        return (out.reshape(n, 3) if per == 3 else out), valid


    def surface_forces(self, world: WorldParams, sp: SurfaceParams, verts: np.ndarray, normals: np.ndarray,
                       sdf_field: np.ndarray | None = None, sdf_grid: VoxelGrid | None = None, f32_sums: bool = False):
        """computeLiftDrag restated on this state's world pressure (call
        world_fields first). Returns (SurfaceForces, per-triangle Cp)."""
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1)
        nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1)
        ntri = v.size // 9
        out = SurfaceForces()
        cp = np.empty(max(ntri, 1), np.float32)
        f = None if sdf_field is None else np.ascontiguousarray(sdf_field, dtype=np.float32)
        self.L.ao_surface_forces(self.h, C.byref(world), C.byref(sp), fptr(f) if f is not None else None,
                                 C.byref(sdf_grid) if sdf_grid is not None else None, fptr(v), fptr(nn), ntri,
                                 int(bool(f32_sums)), C.byref(out), fptr(cp))
        return out, cp[:ntri]


def surface_forces_field(pressure: np.ndarray, wall: np.ndarray, dims, world: WorldParams, sp: SurfaceParams,
                         verts: np.ndarray, normals: np.ndarray, sdf_field: np.ndarray | None = None,
                         sdf_grid: VoxelGrid | None = None, f32_sums: bool = False):
    """computeLiftDrag restated over a world pressure array and its wall
    cells (1 = solid or ground). Returns (SurfaceForces, per-triangle Cp)."""
    L = oracle_lib("f32")
    nx, ny, nz = dims
    p = np.ascontiguousarray(pressure, dtype=np.float32).reshape(-1)
    w = np.ascontiguousarray(wall, dtype=np.uint8).reshape(-1)
    v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1)
    nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1)
    ntri = v.size // 9
    out = SurfaceForces()
    cp = np.empty(max(ntri, 1), np.float32)
    f = None if sdf_field is None else np.ascontiguousarray(sdf_field, dtype=np.float32)
    L.ao_surface_forces_field(fptr(p), u8ptr(w), nx, ny, nz, C.byref(world), C.byref(sp),
                              fptr(f) if f is not None else None, C.byref(sdf_grid) if sdf_grid is not None else None,
                              fptr(v), fptr(nn), ntri, int(bool(f32_sums)), C.byref(out), fptr(cp))
    return out, cp[:ntri]


def equilibrium_moments(rho, ux, uy, uz):
    L = oracle_lib("f32")
    out = np.zeros(4, np.float32)
    ptrs = [C.cast(out.ctypes.data + 4 * i, _FP) for i in range(4)]
    ok = L.ao_equilibrium_moments(rho, ux, uy, uz, *ptrs)
    return bool(ok), tuple(float(v) for v in out)


def sdf(mask: np.ndarray, dims, cs, exact: bool = False) -> np.ndarray:
    """Distance field of a mask: the reference's sweeps + FIFO restated
    (exact=False) or the least-fixed-point form the device computes."""
    L = oracle_lib("f32")
    nx, ny, nz = dims
    m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
    out = np.empty(m.size, np.float32)
    c = np.asarray(cs, np.float32)
    fn = L.ao_sdf_exact if exact else L.ao_sdf_reference
    if fn(u8ptr(m), nx, ny, nz, fptr(c), fptr(out)) != 0:
        raise RuntimeError("oracle sdf failed")
    return out


def sdf_sample(field: np.ndarray, dims, mn, cs, points: np.ndarray):
    L = oracle_lib("f32")
    nx, ny, nz = dims
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    dist = np.empty(pts.shape[0], np.float32)
    nrm = np.empty((pts.shape[0], 3), np.float32)
    f = np.ascontiguousarray(field, dtype=np.float32)
    L.ao_sdf_sample(fptr(f), nx, ny, nz, fptr(np.asarray(mn, np.float32)), fptr(np.asarray(cs, np.float32)),
                    fptr(pts), pts.shape[0], fptr(dist), fptr(nrm))
    return dist, nrm


def voxelize_brute(tris: np.ndarray, grid: VoxelGrid) -> np.ndarray:
    L = oracle_lib("f32")
    t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
    m = np.zeros(grid.nx * grid.ny * grid.nz, np.uint8)
    rc = L.ao_voxelize_brute(fptr(t), t.size // 9, C.byref(grid), u8ptr(m))
    if rc != 0:
        raise RuntimeError("oracle voxelize failed")
    return m


def count_hits_brute(tris: np.ndarray, origin, axis: int) -> int:
    L = oracle_lib("f32")
    t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
    o = np.asarray(origin, np.float32)
    return L.ao_count_hits_brute(fptr(t), t.size // 9, fptr(o), int(axis))


def voxel_plan(size, res: int, budget: int = 0) -> VoxelPlan:
    L = oracle_lib("f32")
    s = np.asarray(size, np.float32)
    p = VoxelPlan()
    L.ao_voxel_plan(fptr(s), int(res), int(budget), C.byref(p))
    return p


class RefAeroIn(C.Structure):
    _fields_ = [("flow_speed", C.c_float), ("azimuth", C.c_float), ("elevation", C.c_float), ("altitude", C.c_float),
                ("use_real_density", C.c_int), ("auto_ref_area", C.c_int), ("ref_area", C.c_float),
                ("mach_effects", C.c_int), ("ground_effect", C.c_int), ("ground_height", C.c_float),
                ("re_number", C.c_float), ("bb_min", C.c_float * 3), ("bb_max", C.c_float * 3),
                ("center", C.c_float * 3), ("max_dim", C.c_float)]


class RefAeroOut(C.Structure):
    _fields_ = [("drag", C.c_float), ("lift", C.c_float), ("ld", C.c_float), ("moment_mag", C.c_float),
                ("drag_vec", C.c_float * 3), ("lift_vec", C.c_float * 3), ("moment", C.c_float * 3),
                ("cop", C.c_float * 3), ("ref_area", C.c_float), ("cp_bad", C.c_longlong), ("vel", C.c_float * 3),
                ("air_temperature", C.c_float), ("air_density", C.c_float), ("speed_of_sound", C.c_float),
                ("vox_min_y", C.c_float), ("re_number", C.c_float)]


class RefHarness:
    """The reference's own solver sources (oracle/_ref/libaeros_ref.so)."""

    PATH = os.path.join(HERE, "_ref", "libaeros_ref.so")

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(cls.PATH)

    def __init__(self):
        L = C.CDLL(self.PATH)
        L.ref_lbm_setup.argtypes = [C.c_int, C.c_int, C.c_int, _U8P, C.c_int, C.c_float, C.c_float, C.c_float,
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _FP,
                                    C.c_float, _FP]
        L.ref_thermal_setup.argtypes = [C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float]
        L.ref_thermal_upload.argtypes = [_FP]
        L.ref_thermal_get.argtypes = [_FP, _FP, _FP, _FP]
        L.ref_lbm_set_uniform.argtypes = [C.c_float] * 3
        L.ref_lbm_step.argtypes = [C.c_int]
        L.ref_lbm_get_fields.argtypes = [_FP] * 6
        L.ref_lbm_get_populations.argtypes = [_FP]
        L.ref_lbm_set_populations.argtypes = [_FP]
        L.ref_lbm_get_wall_dist.argtypes = [_U8P]
        L.ref_lbm_stats.argtypes = [_FP, C.POINTER(C.c_longlong)]
        L.ref_lbm_cv_force.argtypes = [C.c_float] * 3 + [_FP]
        L.ref_lbm_projected_area.restype = C.c_float
        L.ref_lbm_projected_area.argtypes = [C.c_int]
        L.ref_equilibrium_moments.argtypes = [C.c_float] * 4 + [_FP]
        L.ref_voxelize.argtypes = [_FP, C.c_longlong, C.c_int, C.c_int, C.c_int, _FP, _FP, _U8P]
        L.ref_count_hits.argtypes = [_FP, C.c_longlong, _FP, C.c_int]
        L.ref_voxel_plan.argtypes = [_FP, C.c_int, C.c_ulonglong, C.POINTER(C.c_int)]
        L.ref_validation_setup.argtypes = [C.c_int, C.c_int, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float,
                                           C.POINTER(C.c_int), _FP, _FP]
        L.ref_get_mask.argtypes = [_U8P]
        L.ref_world_get.argtypes = [_FP, _FP, _FP, _FP, _FP, C.POINTER(C.c_longlong), _FP]
        L.ref_vorticity_q.argtypes = [_FP, _FP, _FP]
        L.ref_sample.argtypes = [C.c_int, _FP, C.c_longlong, _FP, _U8P]
        L.ref_build_voxel_grid.restype = C.c_longlong
        L.ref_build_voxel_grid.argtypes = [_FP, C.c_longlong, C.c_int]
        L.ref_voxel_get.argtypes = [C.POINTER(C.c_int), _FP, _FP, _U8P, _FP]
        L.ref_sdf_sample.argtypes = [_FP, C.c_longlong, _FP, _FP]
        L.ref_stl_detect.argtypes = [C.c_char_p, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
        L.ref_stl_load.restype = C.c_longlong
        L.ref_stl_load.argtypes = [C.c_char_p]
        L.ref_stl_get.argtypes = [_FP, _FP]
        L.ref_set_air_density.argtypes = [C.c_float]
        L.ref_poke_pressure.argtypes = [C.c_longlong, C.c_float]
        L.ref_lbm_re.restype = C.c_float
        L.ref_lbm_re.argtypes = [C.c_float] * 5
        L.ref_ref_area.restype = C.c_float
        L.ref_ref_area.argtypes = [_FP, C.c_longlong, C.c_float, C.c_float, C.c_int, C.c_float, _FP, _FP, C.c_float]
        L.ref_lift_drag.argtypes = [_FP, _FP, C.c_longlong, _FP, C.POINTER(RefAeroIn), C.POINTER(RefAeroOut)]
        self.L = L
        self.n = 0

    def setup(self, nx, ny, nz, solid, *, ground_rows=0, tau=0.6, u0=0.08, smag=0.12, les=False, trt=False,
              periodic_x=False, periodic_z=False, convective=False, flow_axis=0, flow_sign=1,
              body_force=(0.0, 0.0, 0.0), flow_speed=1.0):
        s = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        bf = np.asarray(body_force, np.float32)
        uin = np.zeros(3, np.float32)
        rc = self.L.ref_lbm_setup(nx, ny, nz, u8ptr(s), int(ground_rows), tau, u0, smag, int(les), int(trt),
                                  int(periodic_x), int(periodic_z), int(convective), int(flow_axis),
                                  int(flow_sign), fptr(bf), flow_speed, fptr(uin))
        if rc != 0:
            raise RuntimeError(f"reference setup failed: {rc}")
        self.n = nx * ny * nz
        return uin

    def thermal_setup(self, rayleigh, prandtl, fixed, hot, cold, perturbation):
        if self.L.ref_thermal_setup(rayleigh, prandtl, int(fixed), hot, cold, perturbation) != 0:
            raise RuntimeError("reference thermal setup failed")

    def thermal_upload(self, T):
        t = np.ascontiguousarray(T, dtype=np.float32).reshape(-1)
        self.L.ref_thermal_upload(fptr(t))

    def thermal(self):
        T = np.empty(self.n, np.float32)
        b = np.empty(self.n, np.float32)
        nu = np.zeros(1, np.float32)
        mt = np.zeros(1, np.float32)
        self.L.ref_thermal_get(fptr(T), fptr(b), fptr(nu), fptr(mt))
        return T, b, float(nu[0]), float(mt[0])

    def set_uniform(self, ux, uy, uz):
        self.L.ref_lbm_set_uniform(ux, uy, uz)

    def step(self, n):
        self.L.ref_lbm_step(int(n))

    def fields(self) -> dict:
        out = {k: np.empty(self.n, np.float32) for k in ("rho", "ux", "uy", "uz", "strain", "tke")}
        self.L.ref_lbm_get_fields(*(fptr(out[k]) for k in ("rho", "ux", "uy", "uz", "strain", "tke")))
        return out

    def populations(self):
        f = np.empty((19, self.n), np.float32)
        self.L.ref_lbm_get_populations(fptr(f))
        return f

    def set_populations(self, f):
        a = np.ascontiguousarray(f, dtype=np.float32)
        self.L.ref_lbm_set_populations(fptr(a))

    def wall_dist(self):
        w = np.empty(self.n, np.uint8)
        self.L.ref_lbm_get_wall_dist(u8ptr(w))
        return w

    def stats(self) -> dict:
        fs = np.zeros(6, np.float32)
        is_ = (C.c_longlong * 6)()
        self.L.ref_lbm_stats(fptr(fs), is_)
        keys_f = ("avg_rho", "avg_kinetic", "max_velocity_lb", "avg_tke", "convergence", "converged")
        keys_i = ("step", "negative_pops", "bad_pops", "rho_out_of_range", "rho_non_finite", "u_limited")
        d = {k: float(v) for k, v in zip(keys_f, fs)}
        d.update({k: int(v) for k, v in zip(keys_i, is_)})
        return d

    def cv_force(self, hx=0.3, hy=0.3, hz=0.3):
        out = np.zeros(3, np.float32)
        self.L.ref_lbm_cv_force(hx, hy, hz, fptr(out))
        return out

    def projected_area(self, axis):
        return float(self.L.ref_lbm_projected_area(int(axis)))

    def build_voxel_grid(self, tris: np.ndarray, res: int) -> dict:
        """buildVoxelGrid (voxel_grid.cpp:224-553) of a mesh: dims, grid
        minimum, cell sizes, mask and distance field."""
        v = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
        n = self.L.ref_build_voxel_grid(fptr(v), v.size, res)
        if n <= 0:
            raise RuntimeError("the reference refused the voxel grid")
        dims = (C.c_int * 3)()
        mn = np.zeros(3, np.float32)
        cs = np.zeros(3, np.float32)
        mask = np.zeros(n, np.uint8)
        field = np.zeros(n, np.float32)
        self.L.ref_voxel_get(dims, fptr(mn), fptr(cs), u8ptr(mask), fptr(field))
        return dict(dims=tuple(dims), min=mn, cs=cs, mask=mask, sdf=field)

    def stl_detect(self, data: bytes) -> list:
        out = (C.c_ulonglong * 4)()
        self.L.ref_stl_detect(data, len(data), out)
        return [int(v) for v in out]

    def stl_load(self, path: str):
        n = self.L.ref_stl_load(path.encode())
        if n <= 0:
            return int(n), None, None
        v = np.empty(9 * n, np.float32)
        nrm = np.empty(9 * n, np.float32)
        self.L.ref_stl_get(fptr(v), fptr(nrm))
        return int(n), v, nrm

    def sdf_sample(self, points: np.ndarray):
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        dist = np.empty(pts.shape[0], np.float32)
        nrm = np.empty((pts.shape[0], 3), np.float32)
        self.L.ref_sdf_sample(fptr(pts), pts.shape[0], fptr(dist), fptr(nrm))
        return dist, nrm

    def equilibrium_moments(self, rho, ux, uy, uz):
        out = np.zeros(4, np.float32)
        ok = self.L.ref_equilibrium_moments(rho, ux, uy, uz, fptr(out))
        return bool(ok), tuple(float(v) for v in out)

    def voxelize(self, tris, nx, ny, nz, mn, cs):
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
        m = np.zeros(nx * ny * nz, np.uint8)
        self.L.ref_voxelize(fptr(t), t.size // 9, nx, ny, nz, fptr(np.asarray(mn, np.float32)),
                            fptr(np.asarray(cs, np.float32)), u8ptr(m))
        return m

    def count_hits(self, tris, origin, axis):
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
        return self.L.ref_count_hits(fptr(t), t.size // 9, fptr(np.asarray(origin, np.float32)), int(axis))

    def validation_setup(self, shape, res, radius, diameter_cells, re_lat, pad, u0):
        dims = (C.c_int * 3)()
        tau = np.zeros(1, np.float32)
        uin = np.zeros(3, np.float32)
        rc = self.L.ref_validation_setup(int(shape), int(res), radius, int(diameter_cells), re_lat, pad, u0, dims,
                                         fptr(tau), fptr(uin))
        if rc != 0:
            raise RuntimeError("reference validation setup failed")
        self.n = dims[0] * dims[1] * dims[2]
        return tuple(dims), float(tau[0]), uin

    def mask(self):
        m = np.empty(self.n, np.uint8)
        self.L.ref_get_mask(u8ptr(m))
        return m

    def voxel_plan(self, size, res, budget):
        out = (C.c_int * 6)()
        self.L.ref_voxel_plan(fptr(np.asarray(size, np.float32)), int(res), int(budget), out)
        return tuple(out)

    def world(self):
        """The readback prep of the last step: fields, stats and the world
        parameters (flowSpeed, airDensity, lbmMin, lbmCellSize) it used."""
        out = {k: np.empty(self.n, np.float32) for k in ("ux", "uy", "uz", "pressure")}
        st = np.zeros(4, np.float32)
        bad = C.c_longlong()
        wp = np.zeros(8, np.float32)
        self.L.ref_world_get(fptr(out["ux"]), fptr(out["uy"]), fptr(out["uz"]), fptr(out["pressure"]), fptr(st),
                             C.byref(bad), fptr(wp))
        stats = dict(pressure_min=float(st[0]), pressure_max=float(st[1]), residual_rho=float(st[2]),
                     residual_u=float(st[3]), pressure_non_finite=int(bad.value))
        return out, stats, [float(v) for v in wp]

    def vorticity_q(self) -> dict:
        out = {k: np.empty(self.n, np.float32) for k in ("vorticity", "q", "strain")}
        self.L.ref_vorticity_q(fptr(out["vorticity"]), fptr(out["q"]), fptr(out["strain"]))
        return out

    def lift_drag(self, verts: np.ndarray, normals: np.ndarray, sdf_field: np.ndarray | None = None, **kw):
        """computeLiftDrag on the last step's state. kw: RefAeroIn fields."""
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1)
        nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1)
        a = RefAeroIn()
        for k, val in kw.items():
            if k in ("bb_min", "bb_max", "center"):
                for i in range(3):
                    getattr(a, k)[i] = float(val[i])
            else:
                setattr(a, k, val)
        out = RefAeroOut()
        f = None if sdf_field is None else np.ascontiguousarray(sdf_field, dtype=np.float32)
        self.L.ref_lift_drag(fptr(v), fptr(nn), v.size // 9, fptr(f) if f is not None else None, C.byref(a),
                             C.byref(out))
        return out

    def sample(self, field: int, points: np.ndarray):
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        n = pts.shape[0]
        per = 3 if field == AEROS_FIELD_VELOCITY_LB else 1
        out = np.empty(n * per, np.float32)
        valid = np.empty(n, np.uint8)
        self.L.ref_sample(int(field), fptr(pts), n, fptr(out), u8ptr(valid))
        return (out.reshape(n, 3) if per == 3 else out), valid
