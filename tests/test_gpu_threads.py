"""Contexts driven from several host threads at once (one context per thread, as the C ABI
requires) give the same bits as the same calls made one after another: the shoot loop, the
dense capture and the gathering solve (whose split-K sums are reduced in a fixed order)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _shoot(lib, sc, mode):
    with lib.Solver(hemicube_side=64, hemicubes_count=16, mode=mode) as s:
        s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"],
                 reflectance=sc.get("reflectance"))
        s.shoot(12)
        return s.download()


def _gather(lib, sc):
    with lib.Solver(hemicube_side=64, hemicubes_count=16, mode=lib.MODE_PHYS) as s:
        s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"],
                 reflectance=sc["reflectance"])
        s.dense_capture(keep_fp32=True)
        E = np.ascontiguousarray(sc["radiosity"].reshape(-1, 3).T, np.float32)
        B, st = s.gather(E, tol=1e-5, max_outer=50, sweeps=4)
        return B, st.outer


@pytest.fixture(scope="module")
def scenes4():
    from radiosity_gb300 import scenes

    return [scenes.cornell_variant(1500 + 700 * k, seed=50 + k, n_lights=1 + k % 3) for k in range(4)]


def test_threaded_shoot_loops_match_sequential(lib, scenes4):
    modes = [k % 2 for k in range(len(scenes4))]
    seq = [_shoot(lib, sc, m) for sc, m in zip(scenes4, modes)]
    with ThreadPoolExecutor(max_workers=4) as ex:
        par = list(ex.map(lambda a: _shoot(lib, *a), zip(scenes4, modes)))
    for (r0, i0), (r1, i1) in zip(seq, par):
        assert np.array_equal(_bits(r0), _bits(r1)) and np.array_equal(_bits(i0), _bits(i1))


def test_threaded_capture_and_gather_match_sequential(lib, scenes4):
    seq = [_gather(lib, sc) for sc in scenes4]
    with ThreadPoolExecutor(max_workers=4) as ex:
        par = list(ex.map(lambda sc: _gather(lib, sc), scenes4))
    for (b0, o0), (b1, o1) in zip(seq, par):
        assert o0 == o1
        assert np.array_equal(_bits(b0), _bits(b1))
