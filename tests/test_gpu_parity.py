"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bars (all from the solver's contract):
  * delta-FF table, item buffers, form-factor rows (exact-sum contract),
    shooter selection and the whole shoot loop: bit-exact against the oracle;
  * form factors vs the reference's ProcessHemicube record path on identical
    item buffers: <= 1e-5 relative per patch;
  * final radiosity vs the oracle solve through the record path: <= 1e-4
    relative L2, energy sums in FP64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_FF = 1e-5     # per-patch form factors vs the record path
REL_L2 = 1e-4     # final radiosity vs the record-path solve


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def cornell(lib):
    return lib.reference_scene(0.045)


@pytest.fixture(scope="module")
def small(lib):
    return lib.reference_scene(0.5)


@pytest.fixture(scope="module")
def room(lib):
    from radiosity_gb300 import scenes

    return scenes.room_with_boxes(target=6000, seed=11)


def solver(lib, scene, W, K, mode=0, **kw):
    s = lib.Solver(hemicube_side=W, hemicubes_count=K, mode=mode, **kw)
    s.upload(scene["vertices"], scene["color"], scene["radiosity"], scene["illumination"],
             reflectance=scene.get("reflectance"), indices=scene.get("indices"))
    return s


def light_ids(scene):
    return np.where(scene["radiosity"][0::3] > 0)[0]


@pytest.mark.parametrize("W", [16, 32, 256, 512])
def test_ff_table_bit_exact(lib, orc, golden, W):
    with lib.Solver(hemicube_side=W, hemicubes_count=2) as s:
        t = s.ff_table(2)
    ref = orc.ff_table(W)
    assert np.array_equal(_bits(t), _bits(np.tile(ref, 2)))
    if W in (16, 32):
        assert np.array_equal(_bits(t[: ref.size]), _bits(golden[f"ff_table_{W}"]))


def test_face_cameras_match_reference_golden(lib, golden, cornell):
    """Device MVPs and frames of 24 patches against the reference's own Camera::lookFromPatch
    x Perspective products (golden fixture from the compiled reference)."""
    pids = np.asarray(golden["mvp_patches"], np.uint32)
    with solver(lib, cornell, 16, 4) as s:
        mvp, fr = s.face_cameras(pids)
    assert np.array_equal(_bits(mvp), _bits(np.asarray(golden["mvp"]).reshape(len(pids), 5, 16)))
    assert np.array_equal(_bits(fr), _bits(np.asarray(golden["frames"])[:, :6]))


@pytest.mark.parametrize("W", [16, 32, 256])
def test_item_buffers_bit_exact_cornell(lib, orc, cornell, W):
    sh = np.array([light_ids(cornell)[0], 0, 100, 2500, 3000, cornell["n"] - 1], np.uint32)
    with solver(lib, cornell, W, 4) as s:
        items = s.item_buffers(sh).reshape(len(sh), -1)
    for k, p in enumerate(sh):
        ref = orc.render(W, cornell["vertices"], int(p))
        assert np.array_equal(items[k], ref), f"shooter {p} W {W}: {np.count_nonzero(items[k] != ref)} px differ"


def test_item_buffers_bit_exact_room(lib, orc, room):
    rng = np.random.default_rng(5)
    sh = np.concatenate([light_ids(room)[:2], rng.choice(room["n"], 6, replace=False)]).astype(np.uint32)
    with solver(lib, room, 64, 8, mode=1, tile=16) as s:
        items = s.item_buffers(sh).reshape(len(sh), -1)
    for k, p in enumerate(sh):
        assert np.array_equal(items[k], orc.render(64, room["vertices"], int(p))), p


def test_reduce_on_identical_item_buffers(lib, orc, cornell):
    W, n = 64, cornell["n"]
    sh = [int(light_ids(cornell)[3]), 7, 4242]
    items = np.concatenate([orc.render(W, cornell["vertices"], p) for p in sh])
    with solver(lib, cornell, W, 3) as s:
        F = s.reduce_items(items, len(sh))
    Fx = orc.ff_exact(W, items, len(sh), n)
    Fr = orc.ff_records(W, items, len(sh), n)
    assert np.array_equal(_bits(F), _bits(Fx))
    nz = Fr > 0
    assert np.array_equal(F > 0, nz)
    assert np.max(np.abs(F[nz] - Fr[nz]) / Fr[nz]) <= REL_FF


@pytest.mark.parametrize("W", [2, 4])
def test_reduce_items_small_hemicubes(lib, orc, cornell, W):
    """At W=2 an image is 12 texels, so one warp of the reduction spans several images;
    each image's sums must stay apart (rendered buffers, then ids drawn from 3 patches so
    that every image holds the same ids)."""
    n = cornell["n"]
    sh = [int(light_ids(cornell)[0]), 7, 100, 2500, 4242, 3000]
    rendered = np.concatenate([orc.render(W, cornell["vertices"], p) for p in sh])
    rng = np.random.default_rng(W)
    crowded = rng.integers(0, 4, rendered.size).astype(np.uint32)
    for items in (rendered, crowded):
        with solver(lib, cornell, W, len(sh)) as s:
            F = s.reduce_items(items, len(sh))
        assert np.array_equal(_bits(F), _bits(orc.ff_exact(W, items, len(sh), n)))


@pytest.mark.parametrize("W,tile", [(32, 16), (256, 32), (256, 64)])
def test_ff_rows_fused_bit_exact(lib, orc, cornell, W, tile):
    n = cornell["n"]
    sh = np.array([light_ids(cornell)[0], 12, 1300, 5000], np.uint32)
    with solver(lib, cornell, W, 4, tile=tile) as s:
        F = s.ff_rows(sh)
    items = np.concatenate([orc.render(W, cornell["vertices"], int(p)) for p in sh])
    assert np.array_equal(_bits(F), _bits(orc.ff_exact(W, items, len(sh), n)))


def test_select_ref_golden(lib, orc, golden, small):
    cases = list(zip(golden["topk_rad"], golden["topk_k"], golden["topk_ids"], golden["topk_valid"]))
    for K in sorted(set(int(k) for k in golden["topk_k"])):
        with solver(lib, small, 16, K) as s:
            for rad, k, ids, valid in cases:
                if int(k) != K:
                    continue
                s.set_state(radiosity=rad)
                i, v = s.select()
                assert np.array_equal(v, valid[:K]) and np.array_equal(i[v], ids[:K][v])


@pytest.mark.parametrize("K", [1, 10, 32, 128])
def test_select_ref_random_large(lib, orc, cornell, K):
    rng = np.random.default_rng(K)
    n = cornell["n"]
    with solver(lib, cornell, 16, K) as s:
        for t in range(12):
            m = t % 3
            if m == 0:
                rad = rng.random(3 * n).astype(np.float32)
            elif m == 1:
                rad = np.repeat(rng.integers(0, 3, n), 3).astype(np.float32)
            else:
                rad = np.repeat(np.sort(rng.random(n)).astype(np.float32), 3)
            s.set_state(radiosity=rad)
            i, v = s.select()
            ri, rv = orc.topk_ref(rad, K)
            assert np.array_equal(v, rv) and np.array_equal(i[v], ri[rv])


@pytest.mark.parametrize("K", [1, 8, 33, 128, 512])
def test_select_phys(lib, orc, room, K):
    rng = np.random.default_rng(100 + K)
    n = room["n"]
    area = orc.patch_areas(room["vertices"])
    with solver(lib, room, 16, K, mode=1) as s:
        for t in range(6):
            rad = (rng.integers(0, 4, 3 * n) * (t % 2) + rng.random(3 * n) * (1 - t % 2)).astype(np.float32)
            rad[rng.random(3 * n) < 0.3] = 0
            s.set_state(radiosity=rad)
            i, v = s.select()
            ri, rv = orc.topk_phys(rad, area, K)
            assert np.array_equal(v, rv) and np.array_equal(i[v], ri[rv])


@pytest.mark.parametrize("K", [33, 128])
def test_select_phys_few_candidates(lib, orc, room, K):
    """Fewer patches with unshot power than shooters: a zero state, three lit patches, and
    K - 1 / K + 1 lit patches of one power (one radix bucket taken whole or in part)."""
    rng = np.random.default_rng(300 + K)
    n = room["n"]
    area = orc.patch_areas(room["vertices"])
    vals, cnt = np.unique(area, return_counts=True)
    same = np.flatnonzero(area == vals[np.argmax(cnt)])  # patches of one area: equal powers
    assert same.size > K + 1 and np.all(area > 0)
    with solver(lib, room, 16, K, mode=1) as s:
        for lit in (0, 3, K - 1, K + 1):
            rad = np.zeros(3 * n, np.float32)
            ids = rng.choice(n, lit, replace=False) if lit == 3 else rng.choice(same, lit, replace=False)
            rad[3 * ids] = 1.0
            s.set_state(radiosity=rad)
            i, v = s.select()
            ri, rv = orc.topk_phys(rad, area, K)
            assert np.array_equal(v, rv) and np.array_equal(i[v], ri[rv]), lit
            assert int(v.sum()) == min(lit, K)


def test_shoot_ref_bit_exact_and_record_path(lib, orc, cornell):
    W, K, S = 32, 10, 25
    with solver(lib, cornell, W, K) as s:
        st = s.shoot(S)
        rad, ill = s.download()
    assert st.shots_done == S and st.hemicubes == S * K
    orad, oill, ost = orc.shoot(0, W, K, cornell["vertices"], cornell["color"], cornell["radiosity"],
                                cornell["illumination"], S)
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
    assert list(st.last_energy) == list(ost.last_energy)
    rrad, rill, _ = orc.shoot(0, W, K, cornell["vertices"], cornell["color"], cornell["radiosity"],
                              cornell["illumination"], S, ff_kind=1)
    tot, rtot = (rad + ill).astype(np.float64), (rrad + rill).astype(np.float64)
    assert np.linalg.norm(tot - rtot) / np.linalg.norm(rtot) <= REL_L2


def test_shoot_ref_runs_to_stop_rule(lib, orc, small):
    W, K = 16, 10
    with solver(lib, small, W, K) as s:
        st = s.shoot(2000)
        rad, ill = s.download()
    orad, oill, ost = orc.shoot(0, W, K, small["vertices"], small["color"], small["radiosity"],
                                small["illumination"], 2000)
    assert ost.stopped == 1 and st.stopped == 1 and st.shots_done == ost.shots_done
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
    with solver(lib, small, W, K) as s:  # same result when split into several calls
        done = 0
        while True:
            st2 = s.shoot(7)
            done += st2.shots_done
            if st2.stopped:
                break
        rad2, _ = s.download()
    assert done == ost.shots_done and np.array_equal(_bits(rad2), _bits(orad))


@pytest.mark.parametrize("mode", [0, 1])
def test_shoot_dark_scene(lib, orc, small, room, mode):
    """Nothing left to shoot: the loop stops where the oracle stops, with the same states."""
    sc = small if mode == 0 else room
    W, K, S = 16, 8, 6
    zero = np.zeros(3 * sc["n"], np.float32)
    with solver(lib, sc, W, K, mode=mode) as s:
        s.set_state(radiosity=zero, illumination=zero)
        st = s.shoot(S)
        rad, ill = s.download()
    orad, oill, ost = orc.shoot(mode, W, K, sc["vertices"], sc["color"], zero, zero, S,
                                rho=sc.get("reflectance") if mode else None)
    assert ost.stopped == 1 and st.stopped == 1 and st.shots_done == ost.shots_done
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))


def test_shoot_phys_bit_exact(lib, orc, room):
    W, K, S = 32, 8, 15
    with solver(lib, room, W, K, mode=1) as s:
        st = s.shoot(S)
        rad, ill = s.download()
    orad, oill, ost = orc.shoot(1, W, K, room["vertices"], room["color"], room["radiosity"],
                                room["illumination"], S, rho=room["reflectance"])
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
    assert abs(st.residual - ost.residual) <= 1e-12 * max(1.0, ost.residual)


def test_shoot_phys_tolerance_stop(lib, orc, room):
    W, K = 16, 16
    with solver(lib, room, W, K, mode=1, tolerance=0.2) as s:
        st = s.shoot(500)
    _, _, ost = orc.shoot(1, W, K, room["vertices"], room["color"], room["radiosity"], room["illumination"],
                          500, rho=room["reflectance"], tol=0.2)
    assert st.stopped and ost.stopped and st.shots_done == ost.shots_done and st.residual <= 0.2


def test_capacity_overflow_is_reported(lib, cornell):
    with solver(lib, cornell, 32, 2, tri_capacity=8) as s:
        with pytest.raises(lib.RadError) as e:
            s.ff_rows(np.array([0, 1], np.uint32))
        assert e.value.status == -3
    with solver(lib, cornell, 32, 2, binref_capacity=4) as s:
        with pytest.raises(lib.RadError) as e:
            s.shoot(1)
        assert e.value.status == -3


def test_invalid_arguments(lib, cornell):
    with lib.Solver(hemicube_side=16, hemicubes_count=2) as s:
        with pytest.raises(lib.RadError) as e:
            s.select()
        assert e.value.status == -4
        bad = cornell["indices"].copy()
        bad[7] = 0
        with pytest.raises(lib.RadError) as e:
            s.upload(cornell["vertices"], cornell["color"], cornell["radiosity"], cornell["illumination"],
                     indices=bad)
        assert e.value.status == -1
        s.upload(cornell["vertices"], cornell["color"], cornell["radiosity"], cornell["illumination"])
        with pytest.raises(lib.RadError) as e:
            s.ff_rows(np.array([cornell["n"]], np.uint32))
        assert e.value.status == -1


def test_full_size_properties(lib):
    """50k patches, W=512: closed room => every FF row sums to the table sum; runs are deterministic."""
    from radiosity_gb300 import scenes

    sc = scenes.room_with_boxes(target=50000, seed=0)
    W, K = 512, 32
    with solver(lib, sc, W, K, mode=1) as s:
        tab_sum = float(np.sum(s.ff_table(1).astype(np.float64)))
        rng = np.random.default_rng(0)
        sh = rng.choice(sc["n"], 8, replace=False).astype(np.uint32)
        F = s.ff_rows(sh).astype(np.float64)
        assert np.all(np.abs(F.sum(1) - tab_sum) <= 2e-5 * tab_sum)
        st1 = s.shoot(3)
        r1, i1 = s.download()
    with solver(lib, sc, W, K, mode=1) as s:
        st2 = s.shoot(3)
        r2, i2 = s.download()
    assert np.array_equal(_bits(r1), _bits(r2)) and np.array_equal(_bits(i1), _bits(i2))
    assert st1.residual == st2.residual and 0 < st1.residual < 1


def test_autotune_keeps_results_bit_exact(lib, orc, room):
    """The autotuner only changes the raster's bin side and span/warp split: results stay bit-exact."""
    W, K, S = 64, 16, 6
    with solver(lib, room, W, K, mode=1) as s:
        t = s.autotune(tune_k=False)
        assert t.tile in (16, 32, 64) and t.small_tri_pixels in (64, 256, 1024, 4096) and t.candidates >= 8
        assert t.hemicubes_count == K and t.us_per_hemicube > 0
        st = s.shoot(S)
        rad, ill = s.download()
    orad, oill, _ = orc.shoot(1, W, K, room["vertices"], room["color"], room["radiosity"], room["illumination"], S,
                              rho=room["reflectance"])
    assert st.shots_done == S
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))


@pytest.mark.parametrize("small", [1, 16, 256, 4096])
def test_lane_warp_split_is_exact(lib, orc, cornell, small):
    W, n = 128, cornell["n"]
    sh = np.array([int(light_ids(cornell)[1]), 33, 2048, 5100], np.uint32)
    with solver(lib, cornell, W, 4, tile=32, small_tri_pixels=small) as s:
        F = s.ff_rows(sh)
        s.profile_stages(1)
        c = s.raster_counters()
    assert c["record_bin_pairs"] > 0 and c["small_records"] + c["big_records"] <= c["record_bin_pairs"]
    items = np.concatenate([orc.render(W, cornell["vertices"], int(p)) for p in sh])
    assert np.array_equal(_bits(F), _bits(orc.ff_exact(W, items, len(sh), n)))


def test_multi_scene_graph_matches_single_runs(lib, orc):
    """Scenes of uneven size advanced together in one graph give the same state, bit for
    bit, as each scene solved alone, and each stops at the same shot as alone."""
    from radiosity_gb300 import scenes

    scs = [scenes.cornell_variant(t, seed=s) for t, s in ((600, 1), (1500, 2), (900, 3))]
    solvers = []
    for sc in scs:
        s = solver(lib, sc, 32, 4, mode=1, tolerance=0.05)
        solvers.append(s)
    with lib.Multi(solvers) as mm:
        at, ms, reps, total = mm.shoot(400)
    assert np.all(at > 0) and reps == at.max() and total > 0
    for sc, s, a in zip(scs, solvers, at):
        rad, ill = s.download()
        s.close()
        orad, oill, ost = orc.shoot(1, 32, 4, sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], 400,
                                    rho=sc["reflectance"], tol=0.05)
        assert ost.stopped and ost.shots_done == a
        assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
