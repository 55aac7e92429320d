"""Pins the oracle restatement against the reference's own code.

Golden fixtures (tests/golden/make_golden.py) come from the reference's C++
compiled by oracle/build_ref.sh; the live comparisons run where the reference
sources are present.  Everything here is bit-exact except the printed sum,
which the reference prints with 9 significant digits.
"""
import hashlib

import numpy as np
import pytest


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("W", [16, 32])
def test_ff_table_matches_golden(orc, golden, W):
    assert np.array_equal(_bits(orc.ff_table(W)), _bits(golden[f"ff_table_{W}"]))


def test_ff_sum_known_answer(orc, golden):
    # source/FormFactors.cpp:106: "tady musi byt f_sum == 1, mne to vyjde 1.00435f"
    for W, printed in zip(golden["ff_sum_w"], golden["ff_sum_printed"]):
        assert abs(orc.ff_sum(int(W)) - printed) <= 5e-9 * printed
    assert abs(orc.ff_sum(256) - 1.00435) < 5e-6


def test_mvp_matches_golden(orc, golden, lib):
    s = lib.reference_scene(0.045)
    for k, p in enumerate(golden["mvp_patches"]):
        q = s["vertices"][12 * p:12 * p + 12]
        assert np.array_equal(_bits(orc.patch_frame(q)), _bits(golden["frames"][k]))
        for f in range(5):
            assert np.array_equal(_bits(orc.face_mvp(q, f)), _bits(golden["mvp"][k, f])), (p, f)


def test_topk_matches_golden(orc, golden):
    for rad, K, ids, valid in zip(golden["topk_rad"], golden["topk_k"], golden["topk_ids"], golden["topk_valid"]):
        i, v = orc.topk_ref(rad, int(K))
        assert np.array_equal(i, ids[:K])
        assert np.array_equal(v, valid[:K])


def test_face_rects_follow_reference_tables(orc):
    W = 256
    vp, sc = orc.face_rects(W, 2, 0)  # UP of hemicube 2: row offset int(1.5*W*2)
    assert list(vp) == [0, W + 768, W, W] and list(sc) == [0, W + 768, W, W // 2]
    vp, sc = orc.face_rects(W, 0, 2)  # LEFT renders a full view shifted by -W/2, keeps the right half
    assert list(vp) == [-W // 2, 0, W, W] and list(sc) == [0, 0, W // 2, W]
    vp, sc = orc.face_rects(W, 0, 3)
    assert list(vp) == [3 * W // 2, 0, W, W] and list(sc) == [3 * W // 2, 0, W // 2, W]


# ---- live comparisons against the compiled reference --------------------------------------------

@pytest.mark.parametrize("W", [16, 64, 256, 512])
def test_ff_table_live(orc, refl, W):
    assert np.array_equal(_bits(orc.ff_table(W)), _bits(refl.ff_table(W, 1)))


def test_ff_table_stacked_live(orc, refl):
    assert np.array_equal(_bits(np.tile(orc.ff_table(32), 3)), _bits(refl.ff_table(32, 3)))


def test_mvp_live_many(orc, refl):
    s = refl.scene(0.045)
    for p in range(0, s["n"], 37):
        q = s["vertices"][12 * p:12 * p + 12]
        for f in range(5):
            assert np.array_equal(_bits(orc.face_mvp(q, f)), _bits(refl.face_mvp(q, f)))


def test_topk_live_random(orc, refl):
    s = refl.scene(0.045)
    rng = np.random.default_rng(7)
    n = s["n"]
    for t in range(60):
        m = t % 3
        if m == 0:
            rad = rng.random(3 * n).astype(np.float32)
        elif m == 1:
            rad = np.repeat(rng.integers(0, 3, n), 3).astype(np.float32)
        else:
            rad = s["radiosity"].copy()
            rad[rng.integers(0, n, 20) * 3] = 100.0
        K = int(rng.integers(1, 64))
        a = orc.topk_ref(rad, K)
        b = refl.topk(rad, K)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_golden_digests_live(refl, golden):
    for d in golden["scene_digests"]:
        area, n, dig = str(d).split(":")
        s = refl.scene(float(area))
        h = hashlib.sha256()
        for k in ("vertices", "indices", "color", "radiosity", "illumination"):
            h.update(np.ascontiguousarray(s[k]).tobytes())
        assert s["n"] == int(n) and h.hexdigest() == dig
