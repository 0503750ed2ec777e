"""The C++17 facade (aeros-engine_gb300/facade): a caller written against the
reference's lbm.h names builds against it (CPU) and gets, through it, the
state the C ABI gives directly (GPU)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "aeros-engine_gb300")
LIB = os.path.join(PKG, "lib")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    import __graft_entry__
    __graft_entry__._paths()
    import build as cuda_build
    cuda_build.build()
    exe = str(tmp_path_factory.mktemp("facade") / "channel_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                           "-I", os.path.join(PKG, "facade"), os.path.join(ROOT, "tests", "facade", "channel_driver.cpp"),
                           "-o", exe, "-L" + LIB, "-laeros_facade", "-laeros_gb300", "-Wl,-rpath," + LIB])
    return exe


def test_facade_builds_and_links(driver):
    assert os.path.exists(driver)


@pytest.mark.gpu
def test_facade_channel_equals_c_abi(driver, tmp_path):
    from aeros_gb300 import capi, geometry, solver
    out = tmp_path / "ux.bin"
    r = subprocess.run([driver, "200", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ux = np.fromfile(out, np.float32)
    p = capi.make_params(64, 32, 32, tau=0.8, periodic_x=True, periodic_z=True, u_in=(0.0, 0.0, 0.0),
                         body_force=(1e-6, 0.0, 0.0), convective_outlet=True)
    s = solver.Solver(p, geometry.channel_mask(64, 32, 32))
    for _ in range(100):
        s.step(1)
    s.step(100)
    ref = s.fields()["ux"]
    assert np.array_equal(ux, ref)
    st = s.stats()
    assert f"step {st['step']} " in r.stdout
    assert np.float32(r.stdout.split("avg_rho ")[1].split()[0]) == np.float32(st["avg_rho"])
