"""Parity at the benchmarked configurations, against the CPU oracle.

* The large plain configuration: the seeded 20 x 20 x 5 m room with 40 boxes and 4 ceiling
  emitters (50,538 patches, seed 0), hemicube side 512, K = 128 shooters per batch, PHYS
  rule, raster bins of 64 px with every record of extent <= 64 px on the span path (the
  configuration the autotuner picks for it and the one the benchmark times).
  - item buffers of four shooters (a light, a box face, a floor patch, a wall patch),
    bit-exact;
  - fused form-factor rows of the same shooters, bit-exact against the oracle's exact sums
    of its own item buffers, at three raster configurations;
  - two K = 128 shoot batches, bit-exact state and the same FP64 residual.
* The small plain configuration: the reference scene (ModelContainer::load at area 0.045,
  5,171 patches), hemicube side 256, K = 10, REF rule, 20 shots: bit-exact against the
  oracle, and within 1e-4 relative L2 of the oracle's solve through the reference's
  ProcessHemicube record path.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_L2 = 1e-4


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def room50k(lib):
    from radiosity_gb300 import scenes

    return scenes.room_with_boxes(target=50000, seed=0)


def _solver(lib, sc, W, K, mode, **kw):
    s = lib.Solver(hemicube_side=W, hemicubes_count=K, mode=mode, **kw)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc.get("reflectance"),
             indices=sc.get("indices"))
    return s


def _four_shooters(sc):
    """A light, a box face, a floor patch and a wall patch (object ids of scenes.room_with_boxes:
    0..5 the room's faces with 5 = floor, 100.. the boxes, 1000.. the emitters)."""
    oid = sc["object_id"]
    light = np.where(oid >= 1000)[0]
    box = np.where((oid >= 100) & (oid < 1000))[0]
    floor = np.where(oid == 5)[0]
    wall = np.where(oid == 3)[0]
    return np.array([light[len(light) // 2], box[len(box) // 3], floor[len(floor) // 2], wall[len(wall) // 2]],
                    np.uint32)


def test_room50k_sizes(room50k):
    assert room50k["n"] == 50538


def test_room50k_item_buffers_bit_exact(lib, orc, room50k):
    sh = _four_shooters(room50k)
    with _solver(lib, room50k, 512, 4, 1, tile=64, small_tri_pixels=4096) as s:
        items = s.item_buffers(sh).reshape(len(sh), -1)
    for k, p in enumerate(sh):
        ref = orc.render(512, room50k["vertices"], int(p))
        assert np.count_nonzero(ref) > 0
        assert np.array_equal(items[k], ref), f"shooter {p}: {np.count_nonzero(items[k] != ref)} px differ"


@pytest.mark.parametrize("tile,small", [(64, 4096), (32, 64), (16, 1)])
def test_room50k_ff_rows_bit_exact(lib, orc, room50k, tile, small):
    sh = _four_shooters(room50k)
    n = room50k["n"]
    with _solver(lib, room50k, 512, 4, 1, tile=tile, small_tri_pixels=small) as s:
        F = s.ff_rows(sh)
    items = np.concatenate([orc.render(512, room50k["vertices"], int(p)) for p in sh])
    assert np.array_equal(_bits(F), _bits(orc.ff_exact(512, items, len(sh), n)))


def test_room50k_shoot_k128_bit_exact(lib, orc, room50k):
    W, K, S = 512, 128, 2
    sc = room50k
    with _solver(lib, sc, W, K, 1, tile=64, small_tri_pixels=4096) as s:
        st = s.shoot(S)
        rad, ill = s.download()
    assert st.shots_done == S and st.hemicubes == S * K
    orad, oill, ost = orc.shoot(1, W, K, sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], S,
                                rho=sc["reflectance"])
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
    assert abs(st.residual - ost.residual) <= 1e-12 * max(1.0, ost.residual)
    assert 0 < st.residual < 1


def test_small_config_ref_shoot(lib, orc):
    """Reference scene, W=256, K=10, 20 shots (REF rule)."""
    sc = lib.reference_scene(0.045)
    W, K, S = 256, 10, 20
    with _solver(lib, sc, W, K, 0) as s:
        st = s.shoot(S)
        rad, ill = s.download()
    assert st.shots_done == S
    orad, oill, ost = orc.shoot(0, W, K, sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], S)
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
    assert list(st.last_energy) == list(ost.last_energy)
    rrad, rill, _ = orc.shoot(0, W, K, sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], S,
                              ff_kind=1)
    tot, rtot = (rad + ill).astype(np.float64), (rrad + rill).astype(np.float64)
    assert np.linalg.norm(tot - rtot) / np.linalg.norm(rtot) <= REL_L2
