"""The C++ shim (include/radiosity_shim.hpp) keeps reference-style call sites working.

The CPU test compiles the reference-style driver against the library; the GPU test
runs it and compares the final state with the oracle bit for bit.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _build_driver(lib, tmp_path):
    exe = str(tmp_path / "shim_loop")
    libdir = os.path.dirname(lib.LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_loop.cpp"), "-L", libdir, "-lradiosity_gb300",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    subprocess.check_call(cmd)
    return exe


def test_shim_compiles_and_links(lib, tmp_path):
    assert os.path.exists(_build_driver(lib, tmp_path))


@pytest.mark.gpu
def test_shim_loop_matches_oracle(lib, orc, tmp_path):
    exe = _build_driver(lib, tmp_path)
    out = str(tmp_path / "state.bin")
    subprocess.check_call([exe, "16", "10", "0.5", "40", out])
    raw = np.fromfile(out, np.uint32)
    n, shots = int(raw[0]), int(raw[1])
    vals = raw[2:2 + 6 * n].view(np.float32)
    rad, ill = vals[: 3 * n], vals[3 * n:]
    hid, same = int(raw[2 + 6 * n]), int(raw[3 + 6 * n])
    colors = raw[4 + 6 * n:].view(np.float32)
    sc = lib.reference_scene(0.5)
    orad, oill, ost = orc.shoot(0, 16, 10, sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], 40)
    assert n == sc["n"] and shots == ost.shots_done
    assert np.array_equal(rad.view(np.uint32), orad.view(np.uint32))
    assert np.array_equal(ill.view(np.uint32), oill.view(np.uint32))
    assert same == 1 and colors.size == 12 * n
    with lib.Solver(hemicube_side=16, hemicubes_count=10) as s:  # same state through the Python binding
        s.upload(sc["vertices"], sc["color"], orad, oill, indices=sc["indices"])
        s.upload_neighbours(lib.reference_neighbours(0.5))
        assert s.highest_patch() == hid
        c, _ = s.display_colors(radiative=False)
    assert np.array_equal(c.view(np.uint32), colors.view(np.uint32))
