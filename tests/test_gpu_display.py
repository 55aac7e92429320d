"""GPU parity of the display output, the single-patch selection and checkpoint/resume.

  * rad_display_colors == Colors::smoothShadePatch (source/Colors.cpp:198-262) of every
    patch, bit for bit (golden fixtures from the reference's C++);
  * rad_highest_patch == ModelContainer::getHighestRadiosityPatchId
    (source/ModelContainer.cpp:222-237), ties, zeros, NaN and inf included;
  * a shoot loop saved to a .rr file (SaveToFile's layout) after S1 batches, reloaded into
    a new context with its progress restored and run S2 more batches equals the
    uninterrupted S1 + S2 run bit for bit (REF and PHYS rules).
"""
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def sio():
    return np.load(os.path.join(HERE, "golden", "scene_io_golden.npz"), allow_pickle=False)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def hashed_state(n: int, salt: int) -> np.ndarray:
    """The integer-hash state of tests/golden/make_scene_io_golden.py."""
    i = np.arange(3 * n, dtype=np.uint64) + np.uint64(salt)
    h = (i * np.uint64(2654435761) + np.uint64(12345)) % np.uint64(1 << 32)
    return (h.astype(np.float64) / float(1 << 32)).astype(np.float32)


def solver(lib, scene, W=16, K=4, mode=0, **kw):
    s = lib.Solver(hemicube_side=W, hemicubes_count=K, mode=mode, **kw)
    s.upload(scene["vertices"], scene["color"], scene["radiosity"], scene["illumination"],
             reflectance=scene.get("reflectance"), indices=scene.get("indices"))
    return s


def test_display_colors_bit_exact(lib, sio):
    sc = lib.reference_scene(0.5)
    with solver(lib, sc) as s:
        s.upload_neighbours(lib.reference_neighbours(0.5))
        for rad, ill, want in zip(sio["shade_rad"], sio["shade_illum"], sio["shade_colors"]):
            s.set_state(radiosity=rad, illumination=ill)
            colors, radiative = s.display_colors()
            assert np.array_equal(_bits(colors), _bits(want))
            assert np.array_equal(_bits(radiative), _bits(np.tile(rad.reshape(-1, 1, 3), (1, 4, 1)).reshape(-1)))


def test_display_colors_large_scene_digest(lib, sio):
    sc = lib.reference_scene(0.045)
    n = sc["n"]
    with solver(lib, sc) as s:
        s.upload_neighbours(lib.reference_neighbours(0.045))
        s.set_state(radiosity=hashed_state(n, 1), illumination=hashed_state(n, 2))
        colors, _ = s.display_colors(radiative=False)
    assert hashlib.sha256(colors.tobytes()).hexdigest() == str(sio["shade_0045_digest"])


def test_display_colors_need_neighbours(lib):
    sc = lib.reference_scene(0.5)
    with solver(lib, sc) as s:
        with pytest.raises(lib.RadError):
            s.display_colors()
        _, radiative = s.display_colors(colors=False)  # the radiative buffer needs none
        assert np.array_equal(_bits(radiative), _bits(np.tile(sc["radiosity"].reshape(-1, 1, 3), (1, 4, 1)).ravel()))
        with pytest.raises(lib.RadError):
            s.upload_neighbours(np.full(8 * sc["n"], sc["n"], np.uint32))


def test_highest_patch_matches_reference(lib, sio):
    sc = lib.reference_scene(0.5)
    with solver(lib, sc) as s:
        for rad, want in zip(sio["hi_rad"], sio["hi_id"]):
            s.set_state(radiosity=rad)
            assert s.highest_patch() == int(want)


def test_highest_patch_phys_is_largest_unshot_power(lib):
    from radiosity_gb300 import scenes

    sc = scenes.room_with_boxes(target=3000, seed=5)
    n = sc["n"]
    v = sc["vertices"].reshape(n, 4, 3).astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 3]), axis=1)
    rng = np.random.default_rng(3)
    with solver(lib, sc, mode=lib.MODE_PHYS) as s:
        for _ in range(4):
            rad = rng.random(3 * n).astype(np.float32)
            p = rad.reshape(n, 3).astype(np.float64).sum(1) * area
            top = np.argsort(p)[::-1]
            if p[top[0]] < p[top[1]] * (1 + 1e-5):  # keep the answer away from float rounding
                continue
            s.set_state(radiosity=rad)
            assert s.highest_patch() == int(top[0])


@pytest.mark.parametrize("mode", [0, 1])
def test_checkpoint_resume_through_rr_file_is_bit_exact(lib, tmp_path, mode):
    from radiosity_gb300 import scenes

    sc = lib.reference_scene(0.045) if mode == 0 else scenes.room_with_boxes(target=4000, seed=9)
    W, K, S1, S2 = 32, 8, 6, 9
    with solver(lib, sc, W, K, mode) as s:
        full = s.shoot(S1 + S2)
        rad_full, ill_full = s.download()
    with solver(lib, sc, W, K, mode) as s:
        s.shoot(S1)
        rad, ill = s.download()
        shots, power0 = s.progress()
    assert shots == S1
    path = tmp_path / "state.rr"
    path.write_bytes(lib.rr_write(sc["vertices"], sc["color"], rad, ill))
    back = lib.rr_read(path.read_bytes())
    if mode == 1:
        back["reflectance"] = sc["reflectance"]  # not part of the reference's file format
    with solver(lib, back, W, K, mode) as s:
        s.set_progress(shots, power0)
        st = s.shoot(S2)
        rad2, ill2 = s.download()
        shots2, power2 = s.progress()
    assert shots2 == S1 + S2 and power2 == power0
    assert np.array_equal(_bits(rad2), _bits(rad_full)) and np.array_equal(_bits(ill2), _bits(ill_full))
    if mode == 1:
        assert st.residual == full.residual


def test_display_colors_into_caller_device_buffers(lib, sio):
    torch = pytest.importorskip("torch")
    import ctypes

    sc = lib.reference_scene(0.5)
    n = sc["n"]
    rad, ill, want = sio["shade_rad"][0], sio["shade_illum"][0], sio["shade_colors"][0]
    d_colors = torch.zeros(12 * n, dtype=torch.float32, device="cuda:0")
    d_rad = torch.zeros(12 * n, dtype=torch.float32, device="cuda:0")
    with solver(lib, sc) as s:
        s.upload_neighbours(lib.reference_neighbours(0.5))
        s.set_state(radiosity=rad, illumination=ill)
        rc = s.L.rad_display_colors_device(s.h, ctypes.c_void_p(d_colors.data_ptr()), ctypes.c_void_p(d_rad.data_ptr()))
        assert rc == 0
    assert np.array_equal(_bits(d_colors.cpu().numpy()), _bits(want))
    assert np.array_equal(_bits(d_rad.cpu().numpy()), _bits(np.tile(rad.reshape(-1, 1, 3), (1, 4, 1)).ravel()))
