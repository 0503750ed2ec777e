"""aeros_voxelize_device_noalloc: the fixed-scratch voxelizer gives the masks of
aeros_voxelize_device, call after call, and refuses meshes larger than its
scratch. Collected last so that it also runs after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from aeros_gb300 import capi, geometry, solver
    return torch, capi, geometry, solver


def _run(env, fn, tris, grid, stream=None):
    """Calls fn through the C ABI into a device mask; the no-allocation entry
    point also takes the stream its work runs on (None: the legacy default
    stream)."""
    torch, capi, _, _ = env
    n = grid.nx * grid.ny * grid.nz
    d = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    t = np.ascontiguousarray(tris, np.float32).reshape(-1)
    args = [t.ctypes.data_as(C.POINTER(C.c_float)), t.size // 9, C.byref(grid), C.c_void_p(d.data_ptr())]
    if fn.endswith("_noalloc"):
        args.append(C.c_void_p(stream.cuda_stream if stream is not None else 0))
    rc = getattr(capi.lib(), fn)(*args)
    capi.check(rc, fn)
    return d.cpu().numpy()


def test_noalloc_masks_equal_allocating_entry_point(env):
    _, _, geometry, solver = env
    meshes = [
        (geometry.icosphere(5, 12.0, (30.0, 24.0, 22.0)), solver.voxel_grid((64, 48, 44), (0, 0, 0), (1, 1, 1))),
        (geometry.perturbed_icosphere(4, 9.0, (20.0, 16.0, 16.0), seed=3),
         solver.voxel_grid((48, 32, 32), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))),
        (geometry.torus(10.0, 3.5, 48, 24) + np.float32(20.0), solver.voxel_grid((40, 40, 40), (0, 0, 0), (1, 1, 1))),
    ]
    torch = env[0]
    side = torch.cuda.Stream()   # a stream of the caller's own
    for k, (tris, grid) in enumerate(meshes + meshes):   # two calls in a row for every mesh
        ref = _run(env, "aeros_voxelize_device", tris, grid)
        got = _run(env, "aeros_voxelize_device_noalloc", tris, grid, side if k % 2 else None)
        assert ref.max() == 1 and np.array_equal(got, ref)


def test_noalloc_level7_fits_and_oversize_is_refused(env):
    _, capi, geometry, solver = env
    tris = geometry.icosphere(7, 30.0, (40.0, 40.0, 40.0))
    grid = solver.voxel_grid((80, 80, 80), (0, 0, 0), (1, 1, 1))
    assert np.array_equal(_run(env, "aeros_voxelize_device_noalloc", tris, grid),
                          _run(env, "aeros_voxelize_device", tris, grid))
    big = np.tile(tris, (3, 1))   # 983,040 triangles: their vertices alone exceed the scratch
    with pytest.raises(capi.AerosError, match="scratch"):
        _run(env, "aeros_voxelize_device_noalloc", big, grid)
    # 655,360 triangles: the vertices fit (23.6 MB of 24 MiB), vertices and
    # BVH nodes together do not: refused by the second check
    two = np.concatenate([tris, geometry.icosphere(7, 20.0, (40.0, 40.0, 40.0))])
    with pytest.raises(capi.AerosError, match="scratch"):
        _run(env, "aeros_voxelize_device_noalloc", two, grid)
    # the refusals left nothing behind: the next call is still correct
    assert np.array_equal(_run(env, "aeros_voxelize_device_noalloc", tris, grid),
                          _run(env, "aeros_voxelize_device", tris, grid))
