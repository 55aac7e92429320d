"""Edge cases of the shoot path through the C ABI, bit-exact against the CPU oracle.

  * the largest hemicube the form-factor exact sums support (W = 2048): item buffers and
    fused form-factor rows;
  * the largest batch (K = 1024 shooters per batch) on a scene with fewer patches than K:
    selection slots beyond the candidates stay empty, as the reference's NULL emitters;
  * degenerate patches (collapsed to a point, to a segment, a bow-tie) and patches lying in
    the shooter's tangent plane, in REF and PHYS modes;
  * an empty scene is rejected before anything reaches the device.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def solver(lib, scene, W, K, mode=0, **kw):
    s = lib.Solver(hemicube_side=W, hemicubes_count=K, mode=mode, **kw)
    s.upload(scene["vertices"], scene["color"], scene["radiosity"], scene["illumination"],
             reflectance=scene.get("reflectance"), indices=scene.get("indices"))
    return s


@pytest.fixture(scope="module")
def small(lib):
    return lib.reference_scene(0.5)


def test_largest_hemicube_w2048(lib, orc, small):
    W, n = 2048, small["n"]
    sh = np.array([int(np.where(small["radiosity"][0::3] > 0)[0][0]), 123], np.uint32)
    with solver(lib, small, W, 2) as s:
        items = s.item_buffers(sh).reshape(len(sh), -1)
        F = s.ff_rows(sh)
    for k, p in enumerate(sh):
        ref = orc.render(W, small["vertices"], int(p))
        assert np.array_equal(items[k], ref), f"shooter {p}: {np.count_nonzero(items[k] != ref)} px differ"
    Fx = orc.ff_exact(W, np.concatenate([orc.render(W, small["vertices"], int(p)) for p in sh]), len(sh), n)
    assert np.array_equal(_bits(F), _bits(Fx))


def test_largest_batch_k1024_more_shooters_than_patches(lib, orc, small):
    W, K, S = 16, 1024, 3
    with solver(lib, small, W, K) as s:
        ids, valid = s.select()
        st = s.shoot(S)
        rad, ill = s.download()
    oids, ovalid = orc.topk_ref(small["radiosity"], K)
    assert np.array_equal(valid, ovalid) and np.array_equal(ids[valid], oids[ovalid])
    assert valid.sum() <= small["n"]
    orad, oill, ost = orc.shoot(0, W, K, small["vertices"], small["color"], small["radiosity"],
                                small["illumination"], S)
    assert st.shots_done == ost.shots_done
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))


def _degenerate(scene):
    """Copies `scene` with degenerate and tangent-plane patches mixed in."""
    sc = {k: (np.array(v, copy=True) if isinstance(v, np.ndarray) else v) for k, v in scene.items()}
    q = sc["vertices"].reshape(-1, 4, 3)
    q[5] = q[5][0]                       # all four corners at one point
    q[6, 1] = q[6, 0]                    # a triangle with a doubled corner
    q[6, 2] = q[6, 3] = (q[6, 0] + q[6, 3]) * 0.5
    q[7, 2], q[7, 3] = q[7, 3].copy(), q[7, 2].copy()   # bow-tie (self-crossing outline)
    q[8, :, 1] = q[8, 0, 1]              # flattened onto one plane of constant y
    sc["vertices"] = q.reshape(-1)
    return sc


@pytest.mark.parametrize("mode", [0, 1])
def test_degenerate_patches_bit_exact(lib, orc, small, mode):
    sc = _degenerate(small)
    n = sc["n"]
    if mode == 1:
        rng = np.random.default_rng(4)
        sc["reflectance"] = rng.uniform(0.1, 0.8, 3 * n).astype(np.float32)
    W, K, S = 32, 8, 6
    sh = np.array([5, 6, 7, 8, 20, 300], np.uint32)  # degenerate shooters too
    with solver(lib, sc, W, len(sh), mode) as s:
        items = s.item_buffers(sh).reshape(len(sh), -1)
    for k, p in enumerate(sh):
        assert np.array_equal(items[k], orc.render(W, sc["vertices"], int(p))), p
    with solver(lib, sc, W, K, mode) as s:
        st = s.shoot(S)
        rad, ill = s.download()
    orad, oill, ost = orc.shoot(mode, W, K, sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], S,
                                rho=sc.get("reflectance"))
    assert st.shots_done == ost.shots_done
    assert np.array_equal(_bits(rad), _bits(orad)) and np.array_equal(_bits(ill), _bits(oill))
    assert np.all(np.isfinite(rad)) and np.all(np.isfinite(ill))


def test_empty_scene_is_rejected(lib):
    with lib.Solver(hemicube_side=16, hemicubes_count=2) as s:
        z = np.zeros(0, np.float32)
        with pytest.raises(lib.RadError) as e:
            s.upload(z, z, z, z)
        assert e.value.status == -1
        with pytest.raises(lib.RadError) as e:
            s.shoot(1)
        assert e.value.status == -4


def test_state_round_trip_through_caller_buffers(lib, small):
    """rad_set_state / rad_download with caller-owned host buffers: fresh pageable arrays
    (pages never touched), reused arrays and page-locked arrays give the same bits."""
    torch = pytest.importorskip("torch")
    n = small["n"]
    rng = np.random.default_rng(8)
    rad = rng.random(3 * n).astype(np.float32)
    ill = rng.random(3 * n).astype(np.float32)
    with solver(lib, small, 16, 4) as s:
        s.set_state(radiosity=rad, illumination=ill)
        r0, i0 = s.download()
        assert np.array_equal(_bits(r0), _bits(rad)) and np.array_equal(_bits(i0), _bits(ill))
        fresh = (np.empty(3 * n, np.float32), np.empty(3 * n, np.float32))
        s.download(out=fresh)
        pinned = tuple(torch.empty(3 * n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(2))
        s.download(out=pinned)
        for a, b in ((fresh, (r0, i0)), (pinned, (r0, i0))):
            assert np.array_equal(_bits(a[0]), _bits(b[0])) and np.array_equal(_bits(a[1]), _bits(b[1]))
        s.set_state(radiosity=pinned[1], illumination=pinned[0])  # pinned sources
        r1, i1 = s.download()
        assert np.array_equal(_bits(r1), _bits(ill)) and np.array_equal(_bits(i1), _bits(rad))


def test_bounded_device_wait_gives_up_and_the_device_stays_usable(lib, small):
    """The failure path of every pipeline wait (tcgen05 GEMM, streaming residual): a wait on
    an mbarrier that nothing completes gives up after its bound, the kernel returns, the host
    reads RAD_E_TIMEOUT, and the device keeps working."""
    rc, ms = lib.selftest_bounded_wait(50_000)  # 50 ms
    assert rc == lib._lib.RAD_E_TIMEOUT
    assert 45.0 <= ms < 2000.0
    with solver(lib, small, 16, 4) as s:  # a full shoot afterwards still runs
        st = s.shoot(2)
        assert st.shots_done == 2
    assert lib.selftest_bounded_wait(0)[0] == lib._lib.RAD_E_INVALID
