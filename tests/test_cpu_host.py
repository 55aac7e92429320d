"""CPU-side checks of the product library and the oracle's internal contracts.

No compute call reaches the GPU here: the library is loaded, its exports are
checked against include/radiosity.h, and the host-only entry points (config,
scene builder, argument validation) are exercised.
"""
import ctypes
import hashlib
import os
import re

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "radiosity.h")).read()
    return sorted(set(re.findall(r"\b(rad_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    L = lib.load()
    syms = _header_symbols()
    assert syms, "no declarations found"
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(lib.EXPORTS) == syms


def test_library_is_built_for_sm103a(lib):
    # nvcc embeds the target architecture name in the fatbinary section header
    data = open(lib.LIB_PATH, "rb").read()
    assert b"sm_103a" in data or b"sm_103" in data


def test_config_defaults_and_derived(lib, golden):
    cfg = lib.default_config()
    assert (cfg.hemicube_side, cfg.ocl_workitems_x, cfg.shoots_per_cycle, cfg.hemicubes_count) == (16, 4, 500, 10)
    assert cfg.max_patch_area == 0.5
    for cin, cout in zip(golden["config_in"], golden["config_out"]):
        c = lib.default_config(hemicube_side=int(cin[0]), hemicubes_count=int(cin[1]), ocl_workitems_x=int(cin[2]))
        assert np.array_equal(lib.derived(c), cout)


def test_reference_scene_matches_golden(lib, golden):
    s = lib.reference_scene(0.5)
    for k in ("vertices", "indices", "color", "radiosity", "illumination"):
        assert np.array_equal(np.ascontiguousarray(s[k]).view(np.uint32),
                              np.ascontiguousarray(golden[f"scene05_{k}"]).view(np.uint32)), k
    for d in golden["scene_digests"]:
        area, n, dig = str(d).split(":")
        s = lib.reference_scene(float(area))
        h = hashlib.sha256()
        for k in ("vertices", "indices", "color", "radiosity", "illumination"):
            h.update(np.ascontiguousarray(s[k]).tobytes())
        assert s["n"] == int(n) and h.hexdigest() == dig


def test_invalid_configs_are_rejected_before_touching_a_device(lib):
    L = lib.load()
    for kw in (dict(hemicube_side=15), dict(hemicube_side=0), dict(hemicube_side=4096), dict(hemicubes_count=0),
               dict(hemicubes_count=5000), dict(tile=24), dict(mode=7), dict(ocl_workitems_x=0)):
        cfg = lib.default_config(**kw)
        h = ctypes.c_void_p()
        assert L.rad_create(ctypes.byref(cfg), ctypes.byref(h)) == lib._lib.RAD_E_INVALID
        assert not h.value
    assert L.rad_destroy(None) == lib._lib.RAD_E_INVALID
    assert L.rad_strerror(-3) == b"triangle or bin capacity exceeded"


def test_oracle_exact_vs_record_path(orc, lib):
    """Exact sums (the product contract) vs the ProcessHemicube record path: 1e-5 relative."""
    s = lib.reference_scene(0.045)
    n = s["n"]
    light = int(np.where(s["radiosity"][0::3] > 0)[0][0])
    for W, shooter in ((32, light), (64, 100), (128, 4000)):
        items = orc.render(W, s["vertices"], shooter)
        Fx = orc.ff_exact(W, items, 1, n)[0]
        Fr = orc.ff_records(W, items, 1, n)[0]
        nz = Fx > 0
        assert np.array_equal(nz, Fr > 0)
        assert np.max(np.abs(Fx[nz] - Fr[nz]) / Fx[nz]) <= 1e-5


def test_oracle_process_hemicube_padding(orc):
    """4-slot block allocation with zero padding (source/Kernel_ProcessHemicube.h:52-69)."""
    W = 4
    items = np.zeros(3 * W * W, np.uint32)
    items[0:2] = 5  # one run filling the first span (2 px) of row 0
    items[8:11] = 7  # row 1: a run crossing the span boundary -> two records, two blocks
    rh, ri, re = orc.process_hemicube(W, items, 1, workitems_x=4)
    assert len(rh) == 12  # three blocks of 4 slots
    live = re > 0
    assert live.sum() == 3 and sorted(ri[live]) == [4, 6, 6]
    assert np.all(ri[~live] == 0) and np.all(rh[~live] == 0)


def test_oracle_shoot_phys_energy_balance(orc):
    """PHYS mode conserves power: emitted = unshot + absorbed + escaped (closed room: no escape)."""
    from radiosity_gb300 import scenes

    s = scenes.room_with_boxes(target=3000, seed=3)
    area = orc.patch_areas(s["vertices"])
    rad, ill, st = orc.shoot(1, 32, 8, s["vertices"], s["color"], s["radiosity"], s["illumination"], 20,
                             rho=s["reflectance"])
    assert st.shots_done == 20
    e0 = float(np.sum(area.astype(np.float64) * s["radiosity"].reshape(-1, 3).astype(np.float64).sum(1)))
    unshot = float(np.sum(area.astype(np.float64) * rad.reshape(-1, 3).astype(np.float64).sum(1)))
    assert 0 < unshot < e0 and abs(st.residual - unshot / e0) < 1e-12
