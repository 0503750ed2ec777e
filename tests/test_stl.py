"""STL ingest (aeros_stl_detect / aeros_stl_parse / aeros_stl_read_file,
host code of libaeros_gb300.so): format detection and the parsed triangles
and normals equal, bit for bit, what the reference's stlformat::detect and
loadSTL make of the same synthetic files (tests/golden/stl.json)."""
import json
import os

import numpy as np
import pytest

from golden.cases import fdigest, stl_files

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "stl.json")))
FILES = stl_files()


@pytest.fixture(scope="module")
def lib_built():
    import __graft_entry__
    __graft_entry__._paths()
    import build as cuda_build
    cuda_build.build()
    from aeros_gb300 import solver
    return solver


@pytest.mark.parametrize("name", sorted(FILES))
def test_stl_detect_equals_reference(lib_built, name):
    d = lib_built.stl_detect(FILES[name])
    assert [d["format"], d["declared_triangles"], d["payload_bytes"], d["trailing_bytes"]] == GOLD[name]["detect"]


@pytest.mark.parametrize("name", sorted(FILES))
def test_stl_parse_equals_reference(lib_built, name, tmp_path):
    from aeros_gb300.capi import AerosError
    ref = GOLD[name]
    path = tmp_path / (name + ".stl")
    path.write_bytes(FILES[name])
    if ref["triangles"] < 0:   # the reference's loadSTL returns false
        with pytest.raises(AerosError):
            lib_built.stl_parse(FILES[name])
        with pytest.raises(AerosError):
            lib_built.stl_read(path)
        return
    for v, n, info in (lib_built.stl_parse(FILES[name]), lib_built.stl_read(path)):
        assert info["triangles"] == ref["triangles"] == v.shape[0]
        assert fdigest(v) == ref["vertices"]
        assert fdigest(n) == ref["normals"]


def test_stl_parse_counts_and_limits(lib_built):
    import ctypes as C
    from aeros_gb300 import capi
    data = FILES["binary_solid_header_tail_fixups"]
    v, n, info = lib_built.stl_parse(data)
    assert info["dropped"] == 2 and info["triangles"] == 318 and info["trailing_bytes"] == 137
    assert np.allclose(np.linalg.norm(n.reshape(-1, 3), axis=1), 1.0, atol=1e-6)
    # a smaller buffer gets the first triangles, the count stays the total
    part = np.empty((10, 9), np.float32)
    st = capi.StlInfo()
    assert capi.lib().aeros_stl_parse(data, len(data), 0, part.ctypes.data_as(C.POINTER(C.c_float)), None, 10,
                                      C.byref(st)) == 0
    assert st.triangles == 318 and np.array_equal(part, v[:10])
    # a byte budget below 72 B per declared triangle refuses the binary file
    with pytest.raises(capi.AerosError):
        lib_built.stl_parse(data, budget=72 * 320 - 1)
    v2, _, _ = lib_built.stl_parse(data, budget=72 * 320)
    assert np.array_equal(v2, v)
