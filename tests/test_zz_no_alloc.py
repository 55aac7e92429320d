"""rad_reduce_items_noalloc: form-factor rows for callers that cannot allocate.

Callers whose device memory belongs to another allocator's pool (here: torch's
caching allocator owns the input and output buffers) get the same rows as the
context-based rad_reduce_item_buffers, with no device allocation inside the
call.  Two calls in a row, the second smaller than the first, check that each
call clears the shared fixed scratch it uses.  The file sorts last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_rows(L, torch, items, count, W, n):
    d_items = torch.from_numpy(np.ascontiguousarray(items, np.uint32).view(np.int32)).cuda()
    d_rows = torch.full((count * n,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.rad_reduce_items_noalloc(ctypes.c_void_p(d_items.data_ptr()), count, W, n,
                                    ctypes.c_void_p(d_rows.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, L.rad_strerror(rc)
    torch.cuda.synchronize()
    return d_rows.cpu().numpy().reshape(count, n)


def _context_rows(lib, scene, items, count, W):
    with lib.Solver(hemicube_side=W, hemicubes_count=count) as s:
        s.upload(scene["vertices"], scene["color"], scene["radiosity"], scene["illumination"])
        return s.reduce_items(items, count)


def test_noalloc_rows_match_context_entry_point(lib, orc):
    torch = pytest.importorskip("torch")
    L = lib.load()
    sc = lib.reference_scene(0.045)
    n = sc["n"]
    light = int(np.where(sc["radiosity"][0::3] > 0)[0][0])
    # call 1: three hemicubes at W=64
    items1 = np.concatenate([orc.render(64, sc["vertices"], p) for p in (light, 7, 4242)])
    got1 = _noalloc_rows(L, torch, items1, 3, 64, n)
    want1 = _context_rows(lib, sc, items1, 3, 64)
    assert np.array_equal(got1.view(np.uint32), want1.view(np.uint32))
    # call 2: two other hemicubes at W=32 (fewer sums than call 1: stale sums would show)
    items2 = np.concatenate([orc.render(32, sc["vertices"], p) for p in (light + 3, 1500)])
    got2 = _noalloc_rows(L, torch, items2, 2, 32, n)
    want2 = _context_rows(lib, sc, items2, 2, 32)
    assert np.array_equal(got2.view(np.uint32), want2.view(np.uint32))
    assert got2.sum() > 0


@pytest.mark.parametrize("W", [2, 4])
def test_noalloc_rows_small_hemicubes(lib, orc, W):
    """At W=2 one warp of the reduction spans several 12-texel images: against the
    oracle's exact rows, on rendered buffers and on buffers whose images all hold the
    same 3 patch ids."""
    torch = pytest.importorskip("torch")
    L = lib.load()
    sc = lib.reference_scene(0.045)
    n, count = sc["n"], 6
    rendered = np.concatenate([orc.render(W, sc["vertices"], p) for p in (0, 7, 100, 2500, 4242, 3000)])
    crowded = np.random.default_rng(W).integers(0, 4, rendered.size).astype(np.uint32)
    for items in (rendered, crowded):
        got = _noalloc_rows(L, torch, items, count, W, n)
        assert np.array_equal(got.view(np.uint32), orc.ff_exact(W, items, count, n).view(np.uint32))


def test_noalloc_rejects_requests_beyond_the_fixed_scratch(lib):
    torch = pytest.importorskip("torch")
    L = lib.load()
    n = lib._lib.NOALLOC_MAX_SUMS // 4 + 1
    d_items = torch.zeros(3 * 16 * 16 * 4, dtype=torch.int32, device="cuda")
    d_rows = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = L.rad_reduce_items_noalloc(ctypes.c_void_p(d_items.data_ptr()), 4, 16, n,
                                    ctypes.c_void_p(d_rows.data_ptr()), None)
    assert rc == lib._lib.RAD_E_NOALLOC_LIMIT
    assert b"RAD_NOALLOC_MAX_SUMS" in L.rad_strerror(rc)
