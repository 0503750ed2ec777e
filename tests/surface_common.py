"""Shared driver of the surface-force parity checks (CPU oracle and GPU):
the inputs of a SURFACE_CASES entry as the reference ran it (mesh, distance
field, and the flow parameters its updateFlowParams resolved, recorded in
tests/golden/surface.json) and the comparison of results."""
import json
import os

import numpy as np

from golden.cases import SURFACE_CASES, SURFACE_DEFAULTS, digest, solver_mask, surface_mesh
from post_common import post_case

HERE = os.path.dirname(os.path.abspath(__file__))
SURF = json.load(open(os.path.join(HERE, "golden", "surface.json")))


def surface_inputs(name):
    """(case, vertices, normals, SurfaceParams, distance field or None, VoxelGrid or None)."""
    from aeros_gb300 import capi
    import oracle as O
    sc = SURFACE_CASES[name]
    case = post_case(sc["case"])
    v, n = surface_mesh(sc["mesh"])
    assert digest(np.concatenate([v.reshape(-1), n.reshape(-1)])) == SURF[name]["mesh"]
    a = dict(SURFACE_DEFAULTS, **sc["aero"])
    r = SURF[name]["result"]
    sp = capi.make_surface(velocity=r["vel"], air_temperature=r["air_temperature"], air_density=r["air_density"],
                           use_real_density=a["use_real_density"], speed_of_sound=r["speed_of_sound"],
                           mach_effects=a["mach_effects"], auto_ref_area=a["auto_ref_area"], ref_area=a["ref_area"],
                           azimuth=a["azimuth"], elevation=a["elevation"], bb_min=a["bb_min"], bb_max=a["bb_max"],
                           center=a["center"], max_dim=a["max_dim"], reynolds=r["re_number"],
                           ground_effect=a["ground_effect"], ground_height=a["ground_height"],
                           vox_min_y=r["vox_min_y"])
    sdf = grid = None
    if sc["sdf"]:
        nx, ny, nz = case["grid"]
        m = (solver_mask(case).reshape(-1) == 1).astype(np.uint8)
        sdf = O.sdf(m, (nx, ny, nz), (1.0, 1.0, 1.0))
        assert digest(sdf) == SURF[name]["sdf"]
        grid = capi.VoxelGrid()
        grid.nx, grid.ny, grid.nz = nx, ny, nz
        for i in range(3):
            grid.min[i], grid.cell[i] = 0.0, 1.0
    return case, v, n, sp, sdf, grid


def surface_world(name):
    """World parameters of the reference's step before its computeLiftDrag
    (flowSpeed, airDensity, lbmMin, lbmCellSize)."""
    from aeros_gb300 import capi
    w = SURF[name]["world"]
    return capi.make_world(w[0], w[1], w[2:5], w[5:8])


def ref_vector(name) -> np.ndarray:
    r = SURF[name]["result"]
    return np.array([r["drag"], r["lift"], r["ld"], r["moment_mag"], *r["drag_vec"], *r["lift_vec"], *r["moment"],
                     *r["cop"], r["ref_area"]], np.float32)


def out_vector(o) -> np.ndarray:
    return np.array([o.drag, o.lift, o.lift_to_drag, o.moment_magnitude, *o.drag_vector, *o.lift_vector, *o.moment,
                     *o.center_of_pressure, o.ref_area], np.float32)


def check_status(name, o) -> bool:
    """The early returns of computeLiftDrag: True when the case ends there
    (and the outputs the reference writes on that return match)."""
    from aeros_gb300 import capi
    r = SURF[name]["result"]
    if SURFACE_CASES[name]["mesh"] == "empty":   # forces.cpp:403-406: nothing written
        assert o.status == capi.AEROS_SURFACE_NOT_RUN
        assert r["drag"] == 7.0 and r["lift"] == 7.0 and np.float32(o.ref_area) == np.float32(r["ref_area"])
        return True
    if name == "no_flow":                       # forces.cpp:412: lift, drag and L/D zeroed
        assert o.status == capi.AEROS_SURFACE_NO_FLOW
        assert (r["drag"], r["lift"], r["ld"]) == (0.0, 0.0, 0.0)
        assert (o.drag, o.lift, o.lift_to_drag) == (0.0, 0.0, 0.0)
        assert r["moment_mag"] == 7.0 and np.float32(o.ref_area) == np.float32(r["ref_area"])
        return True
    assert o.status == capi.AEROS_SURFACE_DONE
    return False
