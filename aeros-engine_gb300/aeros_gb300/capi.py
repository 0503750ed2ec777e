"""ctypes mirror of include/aeros_lbm.h and the loader of the CUDA library.

The structures below are byte-for-byte the C structs of the ABI. The shared
library (libaeros_gb300.so, built in-tree by ``build.py``) is loaded lazily
on first use and the load fails loudly when it is missing: there is no CPU
fallback on the product path.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_PKG_DIR), "lib", "libaeros_gb300.so")

AEROS_OK = 0
AEROS_CELL_FLUID, AEROS_CELL_SOLID, AEROS_CELL_GROUND = 0, 1, 2
AEROS_STORE_FP32, AEROS_STORE_FP16, AEROS_STORE_BF16 = 0, 1, 2
AEROS_LATERAL_COPY, AEROS_LATERAL_FREESLIP = 0, 1
AEROS_OUTLET_REFERENCE, AEROS_OUTLET_ZEROGRAD = 0, 1
AEROS_SHIFT_FREESTREAM, AEROS_SHIFT_WEIGHTS = 0, 1
STORAGE_NAMES = {"fp32": AEROS_STORE_FP32, "fp16": AEROS_STORE_FP16, "bf16": AEROS_STORE_BF16}


class LbmParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("tau", C.c_float), ("smagorinsky_c", C.c_float),
        ("use_les", C.c_int32), ("use_trt", C.c_int32),
        ("periodic_x", C.c_int32), ("periodic_z", C.c_int32),
        ("convective_outlet", C.c_int32),
        ("flow_axis", C.c_int32), ("flow_sign", C.c_int32),
        ("u_in", C.c_float * 3), ("u_init", C.c_float * 3), ("body_force", C.c_float * 3),
        ("vel_scale", C.c_float), ("convergence_threshold", C.c_float),
        ("storage", C.c_int32), ("lateral_bc", C.c_int32), ("outlet_bc", C.c_int32),
        ("storage_shift", C.c_int32), ("reserved", C.c_int32 * 7),
    ]


class ThermalParams(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("rayleigh", C.c_float), ("prandtl", C.c_float),
        ("fixed_wall_temps", C.c_int32), ("hot_temp", C.c_float), ("cold_temp", C.c_float),
        ("perturbation", C.c_float), ("nu_lb", C.c_float), ("reserved", C.c_int32 * 4),
    ]


class LbmStats(C.Structure):
    _fields_ = [
        ("step", C.c_int64),
        ("avg_rho", C.c_float), ("avg_kinetic", C.c_float), ("avg_tke", C.c_float),
        ("max_velocity_lb", C.c_float), ("convergence", C.c_float),
        ("converged", C.c_int32), ("diverged", C.c_int32), ("pad0", C.c_int32),
        ("negative_pops", C.c_int64), ("bad_pops", C.c_int64),
        ("rho_out_of_range", C.c_int64), ("rho_non_finite", C.c_int64),
        ("u_limited", C.c_int64), ("nan_count", C.c_int64),
        ("sum_rho", C.c_double), ("sum_kinetic", C.c_double), ("sum_tke", C.c_double),
        ("nusselt", C.c_float), ("mean_t", C.c_float),
        ("fluid_cells", C.c_int32), ("pad1", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if not name.startswith("pad")}


class VoxelGrid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("min", C.c_float * 3), ("cell", C.c_float * 3)]


class VoxelPlan(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("fits", C.c_int32),
                ("cells", C.c_int64), ("bytes", C.c_uint64),
                ("requested_res", C.c_int32), ("suggested_res", C.c_int32)]


class WorldParams(C.Structure):
    _fields_ = [("flow_speed", C.c_float), ("air_density", C.c_float), ("min", C.c_float * 3),
                ("cell", C.c_float * 3), ("reserved", C.c_int32 * 4)]


class WorldStats(C.Structure):
    _fields_ = [("pressure_min", C.c_float), ("pressure_max", C.c_float), ("residual_rho", C.c_float),
                ("residual_u", C.c_float), ("pressure_non_finite", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


AEROS_FIELD_VELOCITY_LB, AEROS_FIELD_DENSITY, AEROS_FIELD_PRESSURE, AEROS_FIELD_VORTICITY = 0, 1, 2, 3
AEROS_FIELD_Q, AEROS_FIELD_STRAIN, AEROS_FIELD_TKE, AEROS_FIELD_SOLID = 4, 5, 6, 7


def make_world(flow_speed=1.0, air_density=1.225, mn=(0.0, 0.0, 0.0), cell=(1.0, 1.0, 1.0)) -> WorldParams:
    w = WorldParams()
    w.flow_speed, w.air_density = float(flow_speed), float(air_density)
    for i in range(3):
        w.min[i] = float(mn[i])
        w.cell[i] = float(cell[i])
    return w


class BatchTuning(C.Structure):
    _fields_ = [("blocks_per_sm", C.c_int32), ("tiles_per_item", C.c_int32), ("shell_tiles_per_item", C.c_int32),
                ("chunk_steps", C.c_int32), ("reserved", C.c_int32 * 4)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


def make_params(nx, ny, nz, *, tau=0.6, smagorinsky_c=0.12, les=False, trt=False,
                periodic_x=False, periodic_z=False, convective_outlet=False,
                flow_axis=0, flow_sign=1, u_in=(0.08, 0.0, 0.0), u_init=None,
                body_force=(0.0, 0.0, 0.0), vel_scale=1.0, convergence_threshold=1e-5,
                storage="fp32", lateral_bc=AEROS_LATERAL_COPY, outlet_bc=AEROS_OUTLET_REFERENCE,
                storage_shift=AEROS_SHIFT_FREESTREAM) -> LbmParams:
    """Builds an LbmParams with the reference's LBMParams defaults where not given."""
    p = LbmParams()
    p.nx, p.ny, p.nz = int(nx), int(ny), int(nz)
    p.tau = float(tau)
    p.smagorinsky_c = float(smagorinsky_c)
    p.use_les, p.use_trt = int(bool(les)), int(bool(trt))
    p.periodic_x, p.periodic_z = int(bool(periodic_x)), int(bool(periodic_z))
    p.convective_outlet = int(bool(convective_outlet))
    p.flow_axis, p.flow_sign = int(flow_axis), int(flow_sign)
    for i in range(3):
        p.u_in[i] = float(u_in[i])
        p.u_init[i] = float((u_init if u_init is not None else u_in)[i])
        p.body_force[i] = float(body_force[i])
    p.vel_scale = float(vel_scale)
    p.convergence_threshold = float(convergence_threshold)
    p.storage = STORAGE_NAMES[storage] if isinstance(storage, str) else int(storage)
    p.lateral_bc, p.outlet_bc = int(lateral_bc), int(outlet_bc)
    p.storage_shift = int(storage_shift)
    return p


def make_thermal(*, rayleigh, prandtl, fixed_wall_temps=True, hot=1.0, cold=0.0,
                 perturbation=0.02, nu_lb) -> ThermalParams:
    t = ThermalParams()
    t.enabled = 1
    t.rayleigh, t.prandtl = float(rayleigh), float(prandtl)
    t.fixed_wall_temps = int(bool(fixed_wall_temps))
    t.hot_temp, t.cold_temp = float(hot), float(cold)
    t.perturbation, t.nu_lb = float(perturbation), float(nu_lb)
    return t


_lib = None

_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_U8P = C.POINTER(C.c_uint8)
_DP = C.POINTER(C.c_double)

class StlInfo(C.Structure):
    _fields_ = [("format", C.c_int32), ("reason", C.c_int32), ("declared_triangles", C.c_uint32),
                ("reserved0", C.c_uint32), ("payload_bytes", C.c_uint64), ("trailing_bytes", C.c_uint64),
                ("triangles", C.c_int64), ("dropped", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_ if k != "reserved0"}


AEROS_STL_UNKNOWN, AEROS_STL_BINARY, AEROS_STL_ASCII = 0, 1, 2


class SurfaceParams(C.Structure):
    _fields_ = [("velocity", C.c_float * 3), ("air_temperature", C.c_float), ("air_density", C.c_float),
                ("use_real_density", C.c_int32), ("speed_of_sound", C.c_float), ("mach_effects", C.c_int32),
                ("auto_ref_area", C.c_int32), ("ref_area", C.c_float), ("flow_azimuth_deg", C.c_float),
                ("flow_elevation_deg", C.c_float), ("bb_min", C.c_float * 3), ("bb_max", C.c_float * 3),
                ("center", C.c_float * 3), ("max_dim", C.c_float), ("reynolds", C.c_float),
                ("ground_effect", C.c_int32), ("ground_height", C.c_float), ("vox_min_y", C.c_float),
                ("reserved", C.c_int32 * 4)]


AEROS_SURFACE_NOT_RUN, AEROS_SURFACE_NO_FLOW, AEROS_SURFACE_DONE = 0, 1, 2
SURFACE_SUM_NAMES = ("force_x", "force_y", "force_z", "cp_x", "cp_y", "cp_z", "moment_x", "moment_y", "moment_z",
                     "area", "pressure_weight", "frontal", "base_area", "base_force", "projected")


class SurfaceForces(C.Structure):
    _fields_ = [("status", C.c_int32), ("reserved0", C.c_int32), ("drag", C.c_float), ("lift", C.c_float),
                ("lift_to_drag", C.c_float), ("moment_magnitude", C.c_float), ("drag_vector", C.c_float * 3),
                ("lift_vector", C.c_float * 3), ("moment", C.c_float * 3), ("center_of_pressure", C.c_float * 3),
                ("ref_area", C.c_float), ("ref_area_used", C.c_float), ("cp_non_finite", C.c_int64),
                ("sums", C.c_double * 15)]

    def as_dict(self) -> dict:
        d = {}
        for k, _ in self._fields_:
            if k == "reserved0":
                continue
            v = getattr(self, k)
            d[k] = list(v) if not isinstance(v, (int, float)) else v
        return d


def make_surface(*, velocity, air_temperature=288.15, air_density=1.225, use_real_density=True,
                 speed_of_sound=340.29, mach_effects=False, auto_ref_area=True, ref_area=1.0, azimuth=0.0,
                 elevation=0.0, bb_min, bb_max, center=None, max_dim=None, reynolds=1e5, ground_effect=False,
                 ground_height=0.0, vox_min_y=0.0) -> SurfaceParams:
    sp = SurfaceParams()
    for i in range(3):
        sp.velocity[i] = float(velocity[i])
        sp.bb_min[i], sp.bb_max[i] = float(bb_min[i]), float(bb_max[i])
        sp.center[i] = float(center[i]) if center is not None else 0.5 * (float(bb_min[i]) + float(bb_max[i]))
    sp.air_temperature, sp.air_density = float(air_temperature), float(air_density)
    sp.use_real_density, sp.speed_of_sound = int(bool(use_real_density)), float(speed_of_sound)
    sp.mach_effects, sp.auto_ref_area, sp.ref_area = int(bool(mach_effects)), int(bool(auto_ref_area)), float(ref_area)
    sp.flow_azimuth_deg, sp.flow_elevation_deg = float(azimuth), float(elevation)
    if max_dim is None:
        max_dim = sum((float(bb_max[i]) - float(bb_min[i])) ** 2 for i in range(3)) ** 0.5
    sp.max_dim, sp.reynolds = float(max_dim), float(reynolds)
    sp.ground_effect, sp.ground_height, sp.vox_min_y = int(bool(ground_effect)), float(ground_height), float(vox_min_y)
    return sp

_SIGS = {
    "aeros_consume_error": (C.c_int, [C.c_char_p, C.c_int]),
    "aeros_lbm_create": (C.c_int, [C.POINTER(LbmParams), _U8P, C.POINTER(_P)]),
    "aeros_lbm_destroy": (C.c_int, [_P]),
    "aeros_lbm_set_stream": (C.c_int, [_P, _P]),
    "aeros_lbm_synchronize": (C.c_int, [_P]),
    "aeros_lbm_thermal_init": (C.c_int, [_P, C.POINTER(ThermalParams)]),
    "aeros_lbm_step": (C.c_int, [_P, C.c_int]),
    "aeros_lbm_step_async": (C.c_int, [_P, C.c_int]),
    "aeros_lbm_get_stats": (C.c_int, [_P, C.POINTER(LbmStats)]),
    "aeros_lbm_read_fields": (C.c_int, [_P, _FP, _FP, _FP, _FP, _FP, _FP]),
    "aeros_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_P)]),
    "aeros_host_free": (C.c_int, [_P]),
    "aeros_lbm_device_fields": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "aeros_lbm_read_populations": (C.c_int, [_P, _FP]),
    "aeros_lbm_write_populations": (C.c_int, [_P, _FP]),
    "aeros_lbm_set_equilibrium": (C.c_int, [_P, _FP, _FP, _FP, _FP]),
    "aeros_lbm_read_mask": (C.c_int, [_P, _U8P, _U8P]),
    "aeros_lbm_thermal_upload": (C.c_int, [_P, _FP]),
    "aeros_lbm_thermal_read": (C.c_int, [_P, _FP, _FP]),
    "aeros_lbm_cv_force": (C.c_int, [_P, C.c_float, C.c_float, C.c_float, _DP]),
    "aeros_lbm_cv_force_box": (C.c_int, [_P, C.POINTER(C.c_int32), _DP]),
    "aeros_lbm_projected_area": (C.c_int, [_P, C.c_int, _DP]),
    "aeros_voxelize": (C.c_int, [_FP, C.c_int64, C.POINTER(VoxelGrid), _U8P]),
    "aeros_voxelize_device": (C.c_int, [_FP, C.c_int64, C.POINTER(VoxelGrid), _P]),
    "aeros_voxelize_device_noalloc": (C.c_int, [_FP, C.c_int64, C.POINTER(VoxelGrid), _P, _P]),
    "aeros_voxel_plan": (C.c_int, [_FP, C.c_int, C.c_uint64, C.POINTER(VoxelPlan)]),
    "aeros_lbm_last_step_ms": (C.c_int, [_P, _FP]),
    "aeros_lbm_last_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "aeros_lbm_device_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "aeros_lbm_world_fields": (C.c_int, [_P, C.POINTER(WorldParams), _FP, _FP, _FP, _FP, C.POINTER(WorldStats)]),
    "aeros_lbm_vorticity_q": (C.c_int, [_P, _FP, _FP, _FP]),
    "aeros_lbm_sample": (C.c_int, [_P, C.POINTER(WorldParams), C.c_int, _FP, C.c_int64, _FP, _U8P]),
    "aeros_equilibrium_moments": (C.c_int, [_FP, C.c_int64, _FP, _U8P]),
    "aeros_sdf_device": (C.c_int, [_P, C.POINTER(VoxelGrid), _P, _P]),
    "aeros_sdf": (C.c_int, [_U8P, C.POINTER(VoxelGrid), _FP]),
    "aeros_sdf_sample": (C.c_int, [_P, C.POINTER(VoxelGrid), _FP, C.c_int64, _FP, _FP]),
    "aeros_sdf_field_create": (C.c_int, [_U8P, C.POINTER(VoxelGrid), C.POINTER(_P)]),
    "aeros_sdf_field_destroy": (C.c_int, [_P]),
    "aeros_sdf_field_device": (_P, [_P]),
    "aeros_sdf_field_read": (C.c_int, [_P, _FP]),
    "aeros_sdf_field_sample": (C.c_int, [_P, _FP, C.c_int64, _FP, _FP]),
    "aeros_sdf_last_stats": (C.c_int, [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "aeros_stl_detect": (C.c_int, [C.c_char_p, C.c_uint64, C.POINTER(StlInfo)]),
    "aeros_stl_parse": (C.c_int, [C.c_char_p, C.c_uint64, C.c_uint64, _FP, _FP, C.c_int64, C.POINTER(StlInfo)]),
    "aeros_stl_read_file": (C.c_int, [C.c_char_p, C.c_uint64, _FP, _FP, C.c_int64, C.POINTER(StlInfo)]),
    "aeros_surface_mesh_create": (C.c_int, [_FP, _FP, C.c_int64, C.POINTER(_P)]),
    "aeros_surface_mesh_destroy": (C.c_int, [_P]),
    "aeros_lbm_surface_forces": (C.c_int, [_P, C.POINTER(WorldParams), C.POINTER(SurfaceParams), _P, _P,
                                           C.POINTER(VoxelGrid), C.POINTER(SurfaceForces), _FP]),
    "aeros_batch_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "aeros_batch_destroy": (C.c_int, [_P]),
    "aeros_batch_add": (C.c_int, [_P, _P]),
    "aeros_batch_remove": (C.c_int, [_P, _P]),
    "aeros_batch_size": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "aeros_batch_step": (C.c_int, [_P, C.c_int]),
    "aeros_batch_set_tuning": (C.c_int, [_P, C.POINTER(BatchTuning)]),
    "aeros_batch_get_tuning": (C.c_int, [_P, C.POINTER(BatchTuning)]),
    "aeros_batch_autotune": (C.c_int, [_P, C.c_int, C.POINTER(BatchTuning)]),
    "aeros_batch_last_step_ms": (C.c_int, [_P, _FP]),
    "aeros_batch_last_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
}


def header_symbols() -> list[str]:
    """Function names declared in include/*.h (parsed from the headers)."""
    import re
    inc = os.path.join(os.path.dirname(os.path.dirname(_PKG_DIR)), "include")
    names = []
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(aeros_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def lib() -> C.CDLL:
    """The CUDA library; raises when it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library missing: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


class AerosError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status != AEROS_OK:
        buf = C.create_string_buffer(1024)
        code = lib().aeros_consume_error(buf, 1024)
        raise AerosError(f"{what}: status {status} (code {code}): {buf.value.decode(errors='replace')}")
