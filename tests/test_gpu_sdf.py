"""The voxel grid's distance field on the GPU (aeros_sdf, aeros_sdf_device,
aeros_sdf_sample): bit for bit the least-fixed-point oracle, close to the
reference with its signs (99.99 % of cells within 1e-4, all within 2e-3), and the samplers bit for bit the
reference's sampleSDFCPU / sdfNormalCPU on the reference's own field."""
import json
import os

import numpy as np
import pytest

from golden.cases import SDF_CASES, fdigest, sdf_points, unpack_mask

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "sdf.json")))


def case_inputs(name):
    from aeros_gb300 import solver
    g = GOLD[name]
    dims = tuple(g["dims"])
    mask = unpack_mask(g["mask"], dims[0] * dims[1] * dims[2])
    mn = np.asarray(g["min"], np.float32)
    cs = np.asarray(g["cs"], np.float32)
    return g, dims, mask, mn, cs, solver.voxel_grid(dims, mn, cs)


@pytest.mark.parametrize("name", list(SDF_CASES))
def test_gpu_sdf_equals_exact_oracle_and_is_close_to_reference(name):
    import oracle
    from aeros_gb300 import solver
    g, dims, mask, mn, cs, grid = case_inputs(name)
    got = solver.sdf(mask, grid)
    passes, runs = solver.sdf_last_stats()
    assert passes > 0 and runs > 0
    ex = oracle.sdf(mask, dims, cs, exact=True)
    assert np.array_equal(got, ex)
    ref = oracle.sdf(mask, dims, cs)   # bitwise the reference (pinned by the CPU tests)
    assert fdigest(ref) == g["sdf"]
    assert np.array_equal(np.sign(got), np.sign(ref))
    d = np.abs(got - ref)   # the tolerance of tests/test_sdf_oracle.py
    assert np.mean(d <= 1e-4) >= 0.9999 and d.max() <= 2e-3


@pytest.mark.parametrize("name", list(SDF_CASES))
def test_gpu_sdf_samplers_equal_reference(name):
    """Sampling the reference's field (uploaded) gives the reference's
    distances and normals bit for bit."""
    import oracle
    import torch
    from aeros_gb300 import solver
    g, dims, mask, mn, cs, grid = case_inputs(name)
    ref = oracle.sdf(mask, dims, cs)
    d = torch.from_numpy(ref).cuda()
    torch.cuda.synchronize()
    hi = mn + cs * np.array(dims, np.float32)
    dist, nrm = solver.sdf_sample(d.data_ptr(), grid, sdf_points(mn, hi))
    assert fdigest(dist) == g["dist"]
    assert fdigest(nrm) == g["normal"]


def test_gpu_sdf_edge_cases():
    """Grids off the 8-cell tiles, ground values (2) as non-solid, no
    surface at all (every cell stays 1e6), one cell, sampling without a
    field."""
    import oracle
    from aeros_gb300 import geometry, solver
    rng = geometry.uniform_array(0xED6E, 13 * 9 * 21, 0.0, 1.0)
    cases = [
        ((13, 9, 21), (rng > 0.7).astype(np.uint8)),
        ((13, 9, 21), np.where(rng > 0.8, 2, (rng > 0.5).astype(np.uint8)).astype(np.uint8)),
        ((17, 8, 9), np.zeros(17 * 8 * 9, np.uint8)),
        ((17, 8, 9), np.ones(17 * 8 * 9, np.uint8)),
        ((1, 1, 1), np.ones(1, np.uint8)),
        ((2, 3, 1), np.array([1, 0, 0, 1, 0, 0], np.uint8)),
    ]
    cs = np.array([0.1, 0.13, 0.07], np.float32)
    for dims, mask in cases:
        grid = solver.voxel_grid(dims, (0.0, 0.0, 0.0), cs)
        got = solver.sdf(mask, grid)
        assert np.array_equal(got, oracle.sdf(mask, dims, cs, exact=True)), dims
    assert np.all(solver.sdf(np.zeros(17 * 8 * 9, np.uint8), solver.voxel_grid((17, 8, 9), (0, 0, 0), cs)) == 1e6)
    dist, nrm = solver.sdf_sample(0, solver.voxel_grid((4, 4, 4), (0, 0, 0), cs), np.zeros((3, 3), np.float32))
    assert np.all(dist == 1000.0) and np.all(nrm == np.array([0.0, 1.0, 0.0], np.float32))


def test_gpu_sdf_from_device_voxelizer():
    """Mesh -> device mask (aeros_voxelize_device) -> device field
    (aeros_sdf_device), no host round trip in between: equals the host path."""
    import ctypes as C
    import torch
    from aeros_gb300 import capi, geometry, solver
    tris = geometry.icosphere(4, 0.8)
    grid = solver.voxel_grid((40, 36, 44), (-1.0, -1.0, -1.0), (0.05, 0.055, 0.045))
    n = 40 * 36 * 44
    dm = torch.zeros(n, dtype=torch.uint8, device="cuda")
    df = torch.zeros(n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t = np.ascontiguousarray(tris, np.float32)
    L = capi.lib()
    assert L.aeros_voxelize_device(t.ctypes.data_as(C.POINTER(C.c_float)), t.shape[0], C.byref(grid),
                                   C.c_void_p(dm.data_ptr())) == 0
    assert L.aeros_sdf_device(C.c_void_p(dm.data_ptr()), C.byref(grid), C.c_void_p(df.data_ptr()), None) == 0
    mask = solver.voxelize(tris, grid)
    assert np.array_equal(dm.cpu().numpy(), mask)
    assert np.array_equal(df.cpu().numpy(), solver.sdf(mask, grid))


def test_gpu_sdf_full_size_equals_exact_oracle():
    """The distance field at its full benchmarked size (level-6 icosphere on
    the reference's 256^3 grid plan, 16.8 M cells), bit for bit the
    least-fixed-point oracle."""
    import oracle
    from aeros_gb300 import geometry, solver
    tris = geometry.icosphere(6)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    margin = np.float32(0.14) * np.float32(np.sqrt(np.sum((hi - lo) ** 2, dtype=np.float32)))
    mn, mx = lo - margin, hi + margin
    plan = solver.voxel_plan(mx - mn, 256)
    dims = (plan.nx, plan.ny, plan.nz)
    cs = ((mx - mn) / np.array(dims, np.float32)).astype(np.float32)
    grid = solver.voxel_grid(dims, mn, cs)
    mask = solver.voxelize(tris, grid)
    got = solver.sdf(mask, grid)
    assert np.array_equal(got, oracle.sdf(mask, dims, cs, exact=True))
