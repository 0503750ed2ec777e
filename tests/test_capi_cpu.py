"""C ABI checks that need no GPU: the library loads and exports every entry
point declared in include/*.h, the ctypes mirrors have the C compiler's
layout, argument validation reports errors through aeros_consume_error, and
the host-only entry points agree with the oracle."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__._paths()
    import build as cuda_build
    cuda_build.build()
    from aeros_gb300 import capi
    return capi


def test_library_exports_every_declared_symbol(lib):
    names = lib.header_symbols()
    assert len(names) >= 25
    L = lib.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_table_covers_every_declared_symbol(lib):
    """The Python host binds every entry point the headers declare."""
    assert sorted(set(lib.header_symbols()) - set(lib._SIGS)) == []


def test_struct_layout_matches_c(lib):
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "aeros_lbm.h"
#include "aeros_batch.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(aeros_lbm_params), sizeof(aeros_thermal_params),
         sizeof(aeros_lbm_stats), sizeof(aeros_voxel_grid), sizeof(aeros_voxel_plan_t),
         offsetof(aeros_lbm_params, storage), offsetof(aeros_lbm_stats, sum_rho), offsetof(aeros_lbm_stats, nusselt),
         sizeof(aeros_batch_tuning), sizeof(aeros_surface_params), sizeof(aeros_surface_forces),
         offsetof(aeros_surface_forces, cp_non_finite), offsetof(aeros_surface_forces, sums));
  return 0; }
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "l")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        got = [int(v) for v in subprocess.check_output([exe]).split()]
    want = [C.sizeof(lib.LbmParams), C.sizeof(lib.ThermalParams), C.sizeof(lib.LbmStats), C.sizeof(lib.VoxelGrid),
            C.sizeof(lib.VoxelPlan), lib.LbmParams.storage.offset, lib.LbmStats.sum_rho.offset,
            lib.LbmStats.nusselt.offset, C.sizeof(lib.BatchTuning), C.sizeof(lib.SurfaceParams),
            C.sizeof(lib.SurfaceForces), lib.SurfaceForces.cp_non_finite.offset, lib.SurfaceForces.sums.offset]
    assert got == want


def test_invalid_arguments_are_reported(lib):
    L = lib.lib()
    h = C.c_void_p()
    p = lib.make_params(2, 8, 8)
    m = np.zeros(128, np.uint8)
    rc = L.aeros_lbm_create(C.byref(p), m.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(h))
    assert rc == -1 and not h.value
    buf = C.create_string_buffer(512)
    assert L.aeros_consume_error(buf, 512) == -1
    assert b">= 4" in buf.value
    assert L.aeros_consume_error(buf, 512) == 0      # consumed
    p = lib.make_params(8, 8, 8, storage=7)
    assert L.aeros_lbm_create(C.byref(p), m.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(h)) == -1
    assert L.aeros_consume_error(buf, 512) == -1 and b"storage" in buf.value
    assert L.aeros_lbm_step(None, 1) == -1
    L.aeros_consume_error(buf, 512)
    b = C.c_void_p()
    assert L.aeros_batch_create(7, C.byref(b)) == -1 and not b.value
    assert L.aeros_consume_error(buf, 512) == -1 and b"storage" in buf.value
    assert L.aeros_batch_step(None, 2) == -1
    assert L.aeros_batch_add(None, None) == -1
    assert L.aeros_batch_set_tuning(None, None) == -1
    assert L.aeros_batch_autotune(None, 4, None) == -1
    L.aeros_consume_error(buf, 512)
    # surface forces: argument checks come before any device work
    mesh = C.c_void_p()
    assert L.aeros_surface_mesh_create(None, None, 12, C.byref(mesh)) == -1 and not mesh.value
    assert L.aeros_consume_error(buf, 512) == -1 and b"NULL" in buf.value
    assert L.aeros_surface_mesh_create(None, None, -1, C.byref(mesh)) == -1
    assert L.aeros_consume_error(buf, 512) == -1 and b"triangles" in buf.value
    assert L.aeros_surface_mesh_destroy(None) == 0
    out = lib.SurfaceForces()
    assert L.aeros_lbm_surface_forces(None, None, None, None, None, None, C.byref(out), None) == -1
    assert L.aeros_consume_error(buf, 512) == -1 and b"NULL" in buf.value


def test_voxel_plan_matches_oracle(lib, oracle_built):
    from aeros_gb300 import solver
    for size, res, budget in [([1, 0.5, 0.25], 64, 8 << 30), ([1, 1, 1], 512, 512 << 20), ([0.3, 2.0, 0.9], 100, 0),
                              ([1, 1e-9, float("nan")], 3, 1 << 20)]:
        a = solver.voxel_plan(size, res, budget)
        b = oracle_built.voxel_plan(size, res, budget)
        assert [a.nx, a.ny, a.nz, a.fits, a.cells, a.bytes, a.suggested_res] == \
               [b.nx, b.ny, b.nz, b.fits, b.cells, b.bytes, b.suggested_res]


def test_geometry_generators():
    from aeros_gb300 import geometry
    t = geometry.icosphere(6, 12.0, (60, 60, 57.5))
    assert t.shape == (81920, 9)
    r = np.linalg.norm(t.reshape(-1, 3) - np.array([60, 60, 57.5]), axis=1)
    assert np.allclose(r, 12.0, atol=1e-4)
    g = geometry.splitmix64(0)
    assert next(g) == 0xE220A8397B1DCDAF       # published first output for seed 0
    p = geometry.perturbed_icosphere(4, 10.0, (0, 0, 0), seed=3)
    assert p.shape == (5120, 9)
    assert np.array_equal(p, geometry.perturbed_icosphere(4, 10.0, (0, 0, 0), seed=3))


def test_bench_control_block_size_matches_device_struct(tmp_path):
    """bench.py counts the bytes every step call reads back with the size of
    the device control block: keep the two in step."""
    import bench
    src = tmp_path / "t.cu"
    src.write_text('#include <cstdio>\n#include "lbm_step.cuh"\n'
                   'int main() { printf("%zu\\n", sizeof(aeros::Control)); return 0; }\n')
    exe = tmp_path / "t"
    subprocess.check_call(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I",
                           os.path.join(ROOT, "aeros-engine_gb300", "csrc"), str(src), "-o", str(exe)])
    assert int(subprocess.check_output([str(exe)]).decode().strip()) == bench.CONTROL_BYTES


def test_bench_clock_summary_counts_only_samples_under_load():
    """bench.py's clock record: the median SM clock and the throttle reasons
    are taken over the samples inside the marked step windows only."""
    import bench
    c = bench.ClockSampler(0)
    c.windows = [(1.0, 2.0, "steps"), (2.0, 3.0, "after")]
    idle = ["800", "2070", "100", "Not Active", "Not Active", "Not Active", "Not Active"]
    busy = ["2070", "2070", "900", "Not Active", "Not Active", "Not Active", "Active"]
    c.samples = [(0.5, idle), (1.5, busy), (2.5, busy), (2.7, busy), (3.5, ["600"] + idle[1:3] + ["Active"] * 4)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["samples"] == 3 and s["samples_steps"] == 1
    assert s["reasons"] == ["sw_power_cap"]
    c.samples = [(0.5, idle)]
    assert c.summary()["reasons"] == ["unsampled"]
