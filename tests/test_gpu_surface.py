"""Surface-pressure lift and drag on the GPU (aeros_lbm_surface_forces)
against the oracle and the reference's own computeLiftDrag (forces.cpp:401-688,
tests/golden/surface.json). The FP32 step and world pressure are bitwise the
reference's, so the per-triangle Cp is compared bit for bit; the device sums
over 32 triangles in FP32 and above in FP64, the oracle in FP64 (with the
skin friction's log10f / powf a few ulp apart: 2e-6 of each group of sums);
the closing formulas agree with the oracle to 1e-5 and with the reference's
FP32 sums to 2e-5."""
import numpy as np
import pytest

from golden.cases import SURFACE_CASES, params_for, solver_mask
from post_common import GOLD
from surface_common import SURF, check_status, out_vector, ref_vector, surface_inputs, surface_world

pytestmark = pytest.mark.gpu

GROUPS = ((0, 3), (3, 6), (6, 9))   # force, pressure-weighted centre, moment: compared against their group's size


def _close_sums(dev, ora, length, rtol=2e-6):
    """Sums against the oracle's FP64 sums: each group against its largest
    member; the moments (cancelling sums of force x lever arm) against the
    largest force times the body length."""
    dev, ora = np.asarray(dev, np.float64), np.asarray(ora, np.float64)
    scale = np.abs(ora).copy()
    for a, b in GROUPS:
        scale[a:b] = np.abs(ora[a:b]).max()
    scale[6:9] = max(scale[6], scale[0] * length)
    bad = np.abs(dev - ora) > rtol * scale + 1e-9
    assert not bad.any(), (np.nonzero(bad), dev[bad], ora[bad])


MOMENT_ENTRIES = [3, 10, 11, 12]   # out_vector: the moment magnitude and vector


def _close_out(got, want, rtol, length):
    """Results against each one's size, at least 1e-3 of the drag (lift and
    side force of a symmetric body are cancelling sums); moments at least
    1e-3 of the drag times the body length."""
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = np.maximum(np.abs(want), 1e-3 * np.abs(want[0]))
    scale[MOMENT_ENTRIES] = np.maximum(scale[MOMENT_ENTRIES], 1e-3 * np.abs(want[0]) * length)
    assert np.all(np.abs(got - want) <= rtol * scale + 1e-6), np.abs(got - want) / scale


def _device(name, world, steps_done=None):
    import torch
    from aeros_gb300 import solver
    case, v, n, sp, sdf, grid = surface_inputs(name)
    cname = SURFACE_CASES[name]["case"]
    s = solver.Solver(params_for(case, GOLD["cases"][cname]["u_in"]), solver_mask(case))
    s.step(case["steps"])
    fields, _ = s.world_fields(world)
    mesh = solver.SurfaceMesh(v, n)
    d = None
    if sdf is not None:
        d = torch.from_numpy(sdf).cuda()
        torch.cuda.synchronize()
    return s, mesh, d, (case, v, n, sp, sdf, grid), fields


@pytest.mark.parametrize("name", list(SURFACE_CASES))
def test_gpu_surface_forces_equal_oracle_and_reference(name):
    import oracle as O
    w = surface_world(name)
    s, mesh, d, (case, v, n, sp, sdf, grid), fields = _device(name, w)
    o, cp = s.surface_forces(w, sp, mesh, d.data_ptr() if d is not None else 0, grid)
    if check_status(name, o):
        return
    wall = (solver_mask(case).reshape(-1) != 0).astype(np.uint8)
    ro, rcp = O.surface_forces_field(fields["pressure"], wall, case["grid"], w, sp, v, n, sdf, grid)
    assert np.array_equal(cp.view(np.int32), rcp.view(np.int32)), np.nonzero(cp != rcp)
    assert o.cp_non_finite == ro.cp_non_finite == SURF[name]["result"]["cp_bad"]
    _close_sums(o.sums, ro.sums, sp.max_dim)
    _close_out(out_vector(o), out_vector(ro), 1e-5, sp.max_dim)
    _close_out(out_vector(o), ref_vector(name), 2e-5, sp.max_dim)
    assert abs(o.ref_area_used - ro.ref_area_used) <= 1e-6 * abs(ro.ref_area_used)


def test_gpu_surface_forces_repeat_bitwise():
    """The fixed reduction tree: two calls give the same bits."""
    name = "degenerate"
    w = surface_world(name)
    s, mesh, d, (case, v, n, sp, sdf, grid), _ = _device(name, w)
    a, cpa = s.surface_forces(w, sp, mesh, d.data_ptr(), grid)
    b, cpb = s.surface_forces(w, sp, mesh, d.data_ptr(), grid, want_cp=False)
    assert list(a.sums) == list(b.sums) and cpb is None
    assert np.array_equal(out_vector(a).view(np.int32), out_vector(b).view(np.int32))


def test_gpu_surface_forces_errors():
    from aeros_gb300 import capi, solver
    name = "plain"
    case, v, n, sp, sdf, grid = surface_inputs(name)
    cname = SURFACE_CASES[name]["case"]
    s = solver.Solver(params_for(case, GOLD["cases"][cname]["u_in"]), solver_mask(case))
    mesh = solver.SurfaceMesh(v, n)
    with pytest.raises(RuntimeError, match="world fields"):   # no world pressure yet
        s.surface_forces(surface_world(name), sp, mesh)
    s.world_fields(surface_world(name), read=False)
    g = capi.VoxelGrid()
    with pytest.raises(RuntimeError, match="go together"):
        s.surface_forces(surface_world(name), sp, mesh, 0, g)
    with pytest.raises(ValueError):
        solver.SurfaceMesh(v[:, :8], n[:, :8])


def test_gpu_surface_forces_full_size_sphere():
    """The 240 x 120 x 115 sphere (Re 100, FP32) after 300 steps with its
    level-6 icosphere (81,920 triangles, face normals as an STL file carries
    them) and the device distance field of its mask: every triangle's Cp
    equals the oracle's over the device pressure, the sums agree, and the
    mirror-symmetric flow and mesh give no side force or lift."""
    import torch
    import oracle as O
    from aeros_gb300 import capi, geometry, solver
    p, mask, tris = geometry.sphere_config("fp32")
    nx, ny, nz = geometry.SPHERE_GRID
    s = solver.Solver(p, mask)
    s.step(300)
    # the reference's sampler puts cell i's value at min + i * cell (lbm.cpp:1881-1933), the mask's
    # cell centres sit at i + 0.5: min = 0.5 centres the pressure on the mesh
    w = capi.make_world(12.5, 1.225, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0))
    fields, _ = s.world_fields(w)
    v = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    c = np.asarray(geometry.SPHERE_CENTER, np.float64)
    nrm = geometry.face_normals(v, c)
    grid = solver.voxel_grid((nx, ny, nz), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    sdf = solver.sdf((mask.reshape(-1) == 1).astype(np.uint8), grid)
    d = torch.from_numpy(sdf).cuda()
    torch.cuda.synchronize()
    r = geometry.SPHERE_RADIUS
    sp = capi.make_surface(velocity=(12.5, 0.0, 0.0), bb_min=c - r, bb_max=c + r, center=c, reynolds=1e7)
    mesh = solver.SurfaceMesh(v, nrm)
    o, cp = s.surface_forces(w, sp, mesh, d.data_ptr(), grid)
    assert o.status == capi.AEROS_SURFACE_DONE and cp.shape == (81920,)
    wall = (mask.reshape(-1) != 0).astype(np.uint8)
    ro, rcp = O.surface_forces_field(fields["pressure"], wall, (nx, ny, nz), w, sp, v, nrm, sdf, grid)
    assert np.array_equal(cp.view(np.int32), rcp.view(np.int32))
    _close_sums(o.sums, ro.sums, sp.max_dim)
    _close_out(out_vector(o), out_vector(ro), 1e-5, sp.max_dim)
    print(f"full-size sphere: drag {o.drag:.6g} N, force y {o.sums[1]:.4g}, z {o.sums[2]:.4g}, cp max {cp.max():.4f}")
    assert o.drag > 0 and abs(o.sums[1]) < 1e-3 * o.sums[0] and abs(o.sums[2]) < 1e-3 * o.sums[0]
    assert cp.max() > 0.3   # a stagnation region on the upstream side
