"""Python handle over the C ABI: one solver domain on the GPU.

Mirrors the reference solver's operations (aeros/src/lbm.h:156-202,
aeros/src/thermal_lbm.h:62-72) on an explicit grid: create (initLBM), step
(stepLBMCPU), field / population readback, control-volume force, projected
area, thermal init / upload / readback. Every call goes through
libaeros_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import LbmParams, LbmStats, ThermalParams, VoxelGrid, check, lib

_FP = C.POINTER(C.c_float)
_U8P = C.POINTER(C.c_uint8)
_DP = C.POINTER(C.c_double)


def _f(a: np.ndarray):
    return a.ctypes.data_as(_FP)


class Solver:
    """One lattice domain (D3Q19 + optional D3Q7) resident on the device."""

    def __init__(self, params: LbmParams, mask: np.ndarray, stream: int | None = None):
        self.params = params
        self.n = params.nx * params.ny * params.nz
        self.shape = (params.nz, params.ny, params.nx)
        m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        if m.size != self.n:
            raise ValueError(f"mask has {m.size} cells, grid has {self.n}")
        h = C.c_void_p()
        check(lib().aeros_lbm_create(C.byref(params), m.ctypes.data_as(_U8P), C.byref(h)), "aeros_lbm_create")
        self.h = h
        if stream is not None:
            self.set_stream(stream)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().aeros_lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream: int) -> None:
        check(lib().aeros_lbm_set_stream(self.h, C.c_void_p(stream)), "set_stream")

    def synchronize(self) -> None:
        check(lib().aeros_lbm_synchronize(self.h), "synchronize")

    # ---- stepping --------------------------------------------------------
    def step(self, n: int = 1) -> None:
        check(lib().aeros_lbm_step(self.h, int(n)), "aeros_lbm_step")

    def step_async(self, n: int = 1) -> None:
        check(lib().aeros_lbm_step_async(self.h, int(n)), "aeros_lbm_step_async")

    def stats(self) -> dict:
        s = LbmStats()
        check(lib().aeros_lbm_get_stats(self.h, C.byref(s)), "get_stats")
        return s.as_dict()

    def last_step_ms(self) -> float:
        v = C.c_float()
        check(lib().aeros_lbm_last_step_ms(self.h, C.byref(v)), "last_step_ms")
        return float(v.value)

    def last_launch_count(self) -> int:
        v = C.c_int64()
        check(lib().aeros_lbm_last_launch_count(self.h, C.byref(v)), "last_launch_count")
        return int(v.value)

    def device_bytes(self) -> int:
        v = C.c_uint64()
        check(lib().aeros_lbm_device_bytes(self.h, C.byref(v)), "device_bytes")
        return int(v.value)

    # ---- state I/O -------------------------------------------------------
    def fields(self, out: dict | None = None) -> dict:
        """rho, ux, uy, uz, strain, tke as float32 arrays of nx*ny*nz cells;
        `out` (e.g. from pinned_fields) receives them without a new allocation."""
        if out is None:
            out = {k: np.empty(self.n, np.float32) for k in ("rho", "ux", "uy", "uz", "strain", "tke")}
        check(lib().aeros_lbm_read_fields(self.h, *(_f(out[k]) for k in ("rho", "ux", "uy", "uz", "strain", "tke"))),
              "read_fields")
        return out

    def device_fields(self) -> dict:
        """Device addresses: rho (float32 per cell) and u4 ((ux, uy, uz, 0) per cell)."""
        ptrs = [C.c_void_p() for _ in range(2)]
        check(lib().aeros_lbm_device_fields(self.h, *(C.byref(p) for p in ptrs)), "device_fields")
        return dict(zip(("rho", "u4"), (p.value for p in ptrs)))

    def populations(self) -> np.ndarray:
        f = np.empty((19, self.n), np.float32)
        check(lib().aeros_lbm_read_populations(self.h, _f(f)), "read_populations")
        return f

    def write_populations(self, f: np.ndarray) -> None:
        a = np.ascontiguousarray(f, dtype=np.float32)
        if a.size != 19 * self.n:
            raise ValueError("populations must be [19][cells]")
        check(lib().aeros_lbm_write_populations(self.h, _f(a)), "write_populations")

    def set_equilibrium(self, rho, ux, uy, uz) -> None:
        arr = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(-1) for a in (rho, ux, uy, uz)]
        check(lib().aeros_lbm_set_equilibrium(self.h, *(None if a is None else _f(a) for a in arr)), "set_equilibrium")

    def mask(self) -> tuple[np.ndarray, np.ndarray]:
        m = np.empty(self.n, np.uint8)
        w = np.empty(self.n, np.uint8)
        check(lib().aeros_lbm_read_mask(self.h, m.ctypes.data_as(_U8P), w.ctypes.data_as(_U8P)), "read_mask")
        return m, w

    # ---- thermal ---------------------------------------------------------
    def thermal_init(self, tp: ThermalParams) -> None:
        check(lib().aeros_lbm_thermal_init(self.h, C.byref(tp)), "thermal_init")

    def thermal_upload(self, T: np.ndarray) -> None:
        t = np.ascontiguousarray(T, dtype=np.float32).reshape(-1)
        check(lib().aeros_lbm_thermal_upload(self.h, _f(t)), "thermal_upload")

    def thermal(self) -> tuple[np.ndarray, np.ndarray]:
        T = np.empty(self.n, np.float32)
        b = np.empty(self.n, np.float32)
        check(lib().aeros_lbm_thermal_read(self.h, _f(T), _f(b)), "thermal_read")
        return T, b

    # ---- forces ----------------------------------------------------------
    def cv_force(self, hx: float = 0.3, hy: float = 0.3, hz: float = 0.3) -> np.ndarray:
        out = np.zeros(3, np.float64)
        check(lib().aeros_lbm_cv_force(self.h, hx, hy, hz, out.ctypes.data_as(_DP)), "cv_force")
        return out

    def cv_force_box(self, box) -> np.ndarray:
        b = (C.c_int32 * 6)(*[int(v) for v in box])
        out = np.zeros(3, np.float64)
        check(lib().aeros_lbm_cv_force_box(self.h, b, out.ctypes.data_as(_DP)), "cv_force_box")
        return out

    # ---- readback and post-processing -----------------------------------
    def world_fields(self, world: capi.WorldParams, read=True) -> tuple[dict, dict]:
        """World velocity and pressure of the last step (kept on the device;
        copied to host arrays when `read`) and the readback statistics."""
        out = {k: np.empty(self.n, np.float32) for k in ("ux", "uy", "uz", "pressure")} if read else {}
        st = capi.WorldStats()
        ptr = (lambda k: _f(out[k])) if read else (lambda k: None)
        check(lib().aeros_lbm_world_fields(self.h, C.byref(world), ptr("ux"), ptr("uy"), ptr("uz"),
                                           ptr("pressure"), C.byref(st)), "world_fields")
        return out, st.as_dict()

    def vorticity_q(self, read=True) -> dict:
        out = {k: np.empty(self.n, np.float32) for k in ("vorticity", "q", "strain")} if read else {}
        ptr = (lambda k: _f(out[k])) if read else (lambda k: None)
        check(lib().aeros_lbm_vorticity_q(self.h, ptr("vorticity"), ptr("q"), ptr("strain")), "vorticity_q")
        return out

    def sample(self, world: capi.WorldParams, field: int, points: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        n = pts.shape[0]
        per = 3 if field == capi.AEROS_FIELD_VELOCITY_LB else 1
        out = np.empty(n * per, np.float32)
        valid = np.empty(n, np.uint8)
        check(lib().aeros_lbm_sample(self.h, C.byref(world), int(field), _f(pts), n, _f(out),
                                     valid.ctypes.data_as(_U8P)), "sample")
        return (out.reshape(n, 3) if per == 3 else out), valid

    def projected_area(self, axis: int) -> float:
        v = C.c_double()
        check(lib().aeros_lbm_projected_area(self.h, int(axis), C.byref(v)), "projected_area")
        return float(v.value)

    def surface_forces(self, world: capi.WorldParams, sp: capi.SurfaceParams, mesh: "SurfaceMesh",
                       d_sdf: int = 0, sdf_grid: VoxelGrid | None = None, want_cp: bool = True):
        """computeLiftDrag (aeros/src/forces.cpp:401-688) on the pressure of
        the last world_fields call: (SurfaceForces, per-triangle Cp or None).
        d_sdf: device address of the voxel grid's distance field (0: none)."""
        out = capi.SurfaceForces()
        cp = np.empty(max(mesh.ntri, 1), np.float32) if want_cp else None
        check(lib().aeros_lbm_surface_forces(self.h, C.byref(world), C.byref(sp), mesh.h, C.c_void_p(d_sdf or None),
                                             C.byref(sdf_grid) if sdf_grid is not None else None, C.byref(out),
                                             _f(cp) if cp is not None else None), "surface_forces")
        return out, (cp[:mesh.ntri] if cp is not None else None)


class SurfaceMesh:
    """A triangle soup resident on the device for the surface-force pass:
    vertices and per-vertex normals, 9 floats per triangle each (the
    reference's g_vertices / g_normals)."""

    def __init__(self, vertices: np.ndarray, normals: np.ndarray):
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1)
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1)
        if v.size % 9 or n.size != v.size:
            raise ValueError("vertices and normals need 9 floats per triangle each")
        self.ntri = v.size // 9
        h = C.c_void_p()
        check(lib().aeros_surface_mesh_create(_f(v), _f(n), self.ntri, C.byref(h)), "surface_mesh_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().aeros_surface_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray(np.ndarray):
    """A numpy array over page-locked host memory (aeros_host_alloc): device
    readbacks into it are single direct copies. The memory is released when
    the array (and every view of it) is gone."""

    class _Owner:
        def __init__(self, ptr):
            self.ptr = ptr

        def __del__(self):
            try:
                lib().aeros_host_free(C.c_void_p(self.ptr))
            except Exception:
                pass

    def __new__(cls, n: int, dtype=np.float32):
        dt = np.dtype(dtype)
        ptr = C.c_void_p()
        check(lib().aeros_host_alloc(max(1, n) * dt.itemsize, C.byref(ptr)), "aeros_host_alloc")
        buf = (C.c_char * (max(1, n) * dt.itemsize)).from_address(ptr.value)
        a = np.frombuffer(buf, dtype=dt, count=n).view(cls)
        a._owner = PinnedArray._Owner(ptr.value)
        return a

    def __array_finalize__(self, obj):
        self._owner = getattr(obj, "_owner", None)


def pinned_fields(n: int) -> dict:
    """Page-locked host arrays for Solver.fields(out=...)."""
    return {k: PinnedArray(n) for k in ("rho", "ux", "uy", "uz", "strain", "tke")}


def equilibrium_moments(states) -> tuple[np.ndarray, np.ndarray]:
    """lbmEquilibriumMoments (aeros/src/lbm.cpp:249-267) on the device for
    rows (rho, ux, uy, uz): returns (n, 4) sums (mass, momentum xyz) and the
    (n,) finite flags."""
    st = np.ascontiguousarray(states, dtype=np.float32).reshape(-1, 4)
    n = st.shape[0]
    out = np.empty((n, 4), np.float32)
    ok = np.empty(n, np.uint8)
    check(lib().aeros_equilibrium_moments(_f(st), n, _f(out), ok.ctypes.data_as(capi._U8P)), "equilibrium_moments")
    return out, ok


def sdf(mask: np.ndarray, grid: VoxelGrid) -> np.ndarray:
    """The voxel grid's signed distance field (buildVoxelGrid's distance part,
    aeros/src/voxel_grid.cpp:384-553) computed on the device from a host mask."""
    m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
    if m.size != grid.nx * grid.ny * grid.nz:
        raise ValueError("mask size does not match the grid")
    out = np.empty(m.size, np.float32)
    check(lib().aeros_sdf(m.ctypes.data_as(_U8P), C.byref(grid), _f(out)), "sdf")
    return out


def sdf_last_stats() -> tuple[int, int]:
    """(propagation passes, tile runs) of this thread's last distance field."""
    p, t = C.c_int64(), C.c_int64()
    check(lib().aeros_sdf_last_stats(C.byref(p), C.byref(t)), "sdf_last_stats")
    return p.value, t.value


def sdf_sample(d_sdf: int, grid: VoxelGrid, points: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """sampleSDFCPU / sdfNormalCPU (voxel_grid.cpp:32-123) of the device field
    at address d_sdf (0: no field) at host points (n, 3): (dist, normals)."""
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    n = pts.shape[0]
    dist = np.empty(n, np.float32)
    nrm = np.empty((n, 3), np.float32)
    check(lib().aeros_sdf_sample(C.c_void_p(d_sdf or None), C.byref(grid), _f(pts), n, _f(dist), _f(nrm)),
          "sdf_sample")
    return dist, nrm


def stl_detect(data: bytes) -> dict:
    """stlformat::detect (aeros/src/stl_format.h:86-140) of file bytes."""
    info = capi.StlInfo()
    check(lib().aeros_stl_detect(data, len(data), C.byref(info)), "stl_detect")
    return info.as_dict()


def stl_parse(data: bytes, budget: int = 0) -> tuple[np.ndarray, np.ndarray, dict]:
    """loadSTL's parse (aeros/src/stl_loader.cpp:30-223) of file bytes:
    (triangles [n, 9], per-vertex normals [n, 9], info)."""
    info = capi.StlInfo()
    check(lib().aeros_stl_parse(data, len(data), budget, None, None, 0, C.byref(info)), "stl_parse")
    n = info.triangles
    v = np.empty((n, 9), np.float32)
    nrm = np.empty((n, 9), np.float32)
    check(lib().aeros_stl_parse(data, len(data), budget, _f(v), _f(nrm), n, C.byref(info)), "stl_parse")
    return v, nrm, info.as_dict()


def stl_read(path: str, budget: int = 0) -> tuple[np.ndarray, np.ndarray, dict]:
    """stl_parse of a file on disk (aeros_stl_read_file)."""
    info = capi.StlInfo()
    p = str(path).encode()
    check(lib().aeros_stl_read_file(p, budget, None, None, 0, C.byref(info)), "stl_read")
    n = info.triangles
    v = np.empty((n, 9), np.float32)
    nrm = np.empty((n, 9), np.float32)
    check(lib().aeros_stl_read_file(p, budget, _f(v), _f(nrm), n, C.byref(info)), "stl_read")
    return v, nrm, info.as_dict()


def voxel_grid(n, mn, cell) -> VoxelGrid:
    g = VoxelGrid()
    g.nx, g.ny, g.nz = (int(v) for v in n)
    for i in range(3):
        g.min[i] = float(mn[i])
        g.cell[i] = float(cell[i])
    return g


def voxelize(tris: np.ndarray, grid: VoxelGrid) -> np.ndarray:
    """Solid mask (1 = inside) at the grid's cell centres, computed on the GPU."""
    t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)
    m = np.zeros(grid.nx * grid.ny * grid.nz, np.uint8)
    check(lib().aeros_voxelize(_f(t), t.size // 9, C.byref(grid), m.ctypes.data_as(_U8P)), "voxelize")
    return m


def voxel_plan(size, res: int, budget: int = 0) -> capi.VoxelPlan:
    s = np.asarray(size, np.float32)
    p = capi.VoxelPlan()
    check(lib().aeros_voxel_plan(_f(s), int(res), int(budget), C.byref(p)), "voxel_plan")
    return p
