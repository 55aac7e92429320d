"""Scene inputs and checkpoints around the shoot loop, against the reference's own code.

Host-only entry points (no GPU): the display neighbours of the reference scene
(Patch::divide), the Wavefront OBJ loader (WaveFrontModel) and the .rr scene files
(SaveToFile / LoadFromFile + LoadingModel).  Golden fixtures come from the
reference's C++ (tests/golden/make_scene_io_golden.py); the live comparisons run
where the reference sources are present.  Everything is bit-exact.
"""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
OBJ = os.path.join(HERE, "golden", "quads.obj")
FIELDS = ("vertices", "color", "radiosity", "illumination", "neighbours")


@pytest.fixture(scope="module")
def sio():
    return np.load(os.path.join(HERE, "golden", "scene_io_golden.npz"), allow_pickle=False)


def _digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def test_neighbours_match_golden(lib, sio):
    assert _same(lib.reference_neighbours(0.5), sio["nb05"])
    nb = lib.reference_neighbours(0.045)
    assert f"{nb.size // 8}:{_digest(nb)}" == str(sio["nb_0045_digest"])
    # an unsubdivided scene: every patch is its own neighbour
    nb0 = lib.reference_neighbours(0.0).reshape(-1, 8)
    assert np.array_equal(nb0, np.repeat(np.arange(len(nb0), dtype=np.uint32)[:, None], 8, axis=1))


@pytest.mark.parametrize("area,tag", [(0.0, "0"), (0.05, "005"), (0.3, "03")])
def test_obj_loader_matches_golden(lib, sio, area, tag):
    s = lib.obj_scene(open(OBJ, "rb").read(), area)
    for k in FIELDS:
        assert _same(s[k], sio[f"obj{tag}_{k}"]), k
    n = s["n"]
    assert _same(s["indices"], (np.arange(n, dtype=np.int32)[:, None] * 4 + np.array([0, 1, 2, 0, 2, 3], np.int32))
                 .reshape(-1))


def test_obj_loader_edge_cases(lib):
    # the fixture's faces: 3 quads, 1 triangle, 1 pentagon (skipped), 1 missing vertex and
    # 1 negative index (skipped), 1 quad with a doubled space, 2 more quads -> 7 patches
    assert lib.obj_scene(open(OBJ, "rb").read(), 0.0)["n"] == 7
    tri = lib.obj_scene(b"v 0 0 0\nv 1000 0 0\nv 0 1000 0\nf 1 2 3\n")
    q = tri["vertices"].reshape(4, 3)
    assert np.array_equal(q[3], q[2]) and np.allclose(q[1], [1, 0, 0])  # last vertex repeated; 1/1000
    assert lib.obj_scene(b"", 0.0)["n"] == 0
    with pytest.raises(lib.RadError):
        lib.obj_scene(b"v 1 2\nf 1 1 1 1\n")  # vertex line with 2 coordinates: parse error


def test_rr_write_matches_reference_bytes(lib, sio):
    data = lib.rr_write(sio["rr_vertices"], sio["rr_color"], sio["rr_rad"], sio["rr_illum"], sio["rr_neighbours"],
                        pointer_bytes=8)
    assert int(sio["rr_record"]) == 184
    assert data == sio["rr_bytes"].tobytes()


def test_rr_read_matches_reference_scene(lib, sio):
    s = lib.rr_read(sio["rr_bytes"].tobytes())
    assert s["pointer_bytes"] == 8 and s["n"] == sio["rr_rad"].size // 3
    for k, g in (("vertices", "rr_vertices"), ("color", "rr_color"), ("radiosity", "rr_rad"),
                 ("illumination", "rr_illum"), ("neighbours", "rr_neighbours")):
        assert _same(s[k], sio[g]), k


def test_rr_32bit_layout_round_trip_and_errors(lib, sio):
    args = (sio["rr_vertices"], sio["rr_color"], sio["rr_rad"], sio["rr_illum"], sio["rr_neighbours"])
    d4 = lib.rr_write(*args, pointer_bytes=4)
    n = sio["rr_rad"].size // 3
    assert len(d4) == 4 + 148 * n
    s = lib.rr_read(d4)
    assert s["pointer_bytes"] == 4
    for k, a in zip(("vertices", "color", "radiosity", "illumination", "neighbours"), args):
        assert _same(s[k], a), k
    with pytest.raises(lib.RadError):
        lib.rr_read(d4[:-1])  # fits neither build's record size
    bad = bytearray(d4)
    bad[4 + 24:4 + 28] = np.uint32(n).tobytes()  # relative neighbour out of range
    with pytest.raises(lib.RadError):
        lib.rr_read(bytes(bad))
    with pytest.raises(lib.RadError):
        lib.rr_write(*args[:4], np.full(8 * n, n, np.uint32))


# ---- live comparisons against the compiled reference --------------------------------------------

@pytest.mark.parametrize("area", [0.5, 0.1, 0.045, 0.0])
def test_neighbours_live(refl, lib, area):
    refl.scene(area)
    assert _same(lib.reference_neighbours(area), refl.neighbours())


@pytest.mark.parametrize("area", [0.0, 0.02, 0.05, 0.3, 1.0])
def test_obj_loader_live(refl, lib, area):
    ref = refl.obj(OBJ, area)
    s = lib.obj_scene(open(OBJ, "rb").read(), area)
    assert s["n"] == ref["n"]
    for k in FIELDS:
        assert _same(s[k], ref[k]), k


def test_rr_live_round_trip(refl, lib):
    rng = np.random.default_rng(7)
    s = refl.scene(0.5)
    n = s["n"]
    rad, ill = rng.random(3 * n).astype(np.float32), rng.random(3 * n).astype(np.float32)
    ref_bytes, rec = refl.rr_save(rad, ill)
    assert rec == 184
    mine = lib.rr_write(s["vertices"], s["color"], rad, ill, refl.neighbours(), pointer_bytes=8)
    assert mine == ref_bytes
    a, b = lib.rr_read(ref_bytes), refl.rr_load(mine)
    for k in FIELDS:
        assert _same(a[k], b[k]), k
