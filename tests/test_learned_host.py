"""Host side of the learned warm start (no GPU): seeded scene descriptions, scene generation
in a spawn-started process pool, the attached patch geometry and the guess decoding."""
import numpy as np

from radiosity_gb300 import learned, scenes


def test_scene_specs_are_seeded_and_keep_the_single_kind_sequence():
    a = learned.scene_specs(12, seed=3, patches=(5000, 50000), kinds=("room", "cornell"))
    assert a == learned.scene_specs(12, seed=3, patches=(5000, 50000), kinds=("room", "cornell"))
    assert [k for k, *_ in a] == ["room", "cornell"] * 6
    assert all(5000 <= t <= 50000 for _, t, *_ in a)
    rooms = [sp for sp in a if sp[0] == "room"]
    assert all(10 <= b < 61 and 1 <= e < 7 for _, _, _, b, e in rooms)
    assert sorted({sp[3] for sp in a if sp[0] == "cornell"}) == [1, 2, 3]  # lights in turn
    # one kind: the draw order of the original Cornell-only generator (target, then seed)
    rng = np.random.default_rng(0)
    t = int(np.exp(rng.uniform(np.log(2000), np.log(6000))))
    s = int(rng.integers(1 << 30))
    assert learned.scene_specs(1, seed=0, patches=(2000, 6000))[0] == ("cornell", t, s, 1, 0)


def test_pooled_generation_matches_sequential():
    specs = learned.scene_specs(4, seed=5, patches=(300, 900), kinds=("room", "cornell"))
    seq = list(learned.generated(specs, workers=0))
    pool = list(learned.generated(specs, workers=2))
    assert len(seq) == len(pool) == 4
    for a, b in zip(seq, pool):
        assert a["n"] == b["n"]
        for k in ("vertices", "color", "reflectance", "radiosity", "illumination"):
            assert np.array_equal(a[k], b[k]), k
        for x, y in zip(a["geometry"], b["geometry"]):
            assert np.array_equal(x, y)


def test_attached_geometry_gives_the_same_features():
    sc = scenes.cornell_variant(800, seed=2)
    rng = np.random.default_rng(1)
    direct = rng.random((sc["n"], 3))
    plain = learned.features(sc, direct)
    sc2 = dict(sc, geometry=learned.patch_geometry(sc["vertices"]))
    assert np.array_equal(plain, learned.features(sc2, direct))


def test_decode_is_always_finite():
    sc = scenes.cornell_variant(600, seed=4)
    n = sc["n"]
    direct = np.full((n, 3), 0.5)
    Y = np.zeros((n, 3), np.float32)
    Y[0] = [np.nan, np.inf, -np.inf]
    Y[1] = [1e4, -5.0, 3.0]
    B = learned.decode(sc, direct, Y)
    assert np.all(np.isfinite(B))
    E = sc["radiosity"].reshape(-1, 3)
    assert np.array_equal(B[0], E[0].astype(np.float32))  # non-finite outputs: emission alone
    assert B[1, 0] == np.float32(E[1, 0] + 0.5 * np.expm1(30.0))  # clipped at y = 30
    assert B[1, 1] == np.float32(E[1, 1])  # negative outputs clip to 0
