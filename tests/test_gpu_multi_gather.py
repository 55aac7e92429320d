"""Many scenes under one captured CUDA graph: learned warm start + BF16 gather (rad_multi_gather).

* Without a network (guess = emission) every scene's result is bit-identical to
  rad_gather_solve on its own context, with the same number of refinements.
* With a network the graph over several scenes gives, bit for bit, what the graph over each
  scene alone gives (branches do not interact), and every scene meets the tolerance on the
  FP64 residual of its captured FP32 rows.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _scenes():
    from radiosity_gb300 import scenes

    return [scenes.cornell_variant(t, seed=s, n_lights=1 + s % 3) for t, s in ((700, 1), (1500, 2), (1100, 3))]


def _ctx(lib, sc, W=32):
    s = lib.Solver(hemicube_side=W, hemicubes_count=16, mode=1)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    return s


def _fp64_residual(ctx, sc, B):
    n = sc["n"]
    F, _, _ = ctx.dense_rows(0, n)
    E = sc["radiosity"].reshape(n, 3).astype(np.float64)
    rho = sc["reflectance"].reshape(n, 3).astype(np.float64)
    Bd = B.T.astype(np.float64)
    r = E + rho * (F.astype(np.float64) @ Bd) - Bd
    nE = np.linalg.norm(E, axis=0)
    return float(np.max(np.linalg.norm(r, axis=0)[nE > 0] / nE[nE > 0]))


def test_graph_without_network_equals_gather_solve(lib):
    scs = _scenes()
    ctxs = [_ctx(lib, sc) for sc in scs]
    with lib.MultiGather(ctxs, tol=TOL, max_outer=100, sweeps=4) as mg:
        out = mg.run()
        res = [mg.result(i) for i in range(len(scs))]
    assert np.all(out["status"] == 1) and out["device_ms"] > 0 and np.all(out["scene_ms"] > 0)
    for k, sc in enumerate(scs):
        with _ctx(lib, sc) as s:
            s.dense_capture(keep_fp32=True)
            E = np.ascontiguousarray(sc["radiosity"].reshape(-1, 3).T, np.float32)
            B, st = s.gather(E, tol=TOL, max_outer=100, sweeps=4)
        assert np.array_equal(res[k].view(np.uint32), B.view(np.uint32)), k
        assert st.outer == out["outer"][k]
        assert _fp64_residual(ctxs[k], sc, res[k]) <= 1.05 * TOL
    for c in ctxs:
        c.close()


def test_graph_with_network_is_per_scene_exact(lib):
    scs = _scenes()
    mlp = lib.MLP(seed=3)
    try:
        ctxs = [_ctx(lib, sc) for sc in scs]
        with lib.MultiGather(ctxs, mlp=mlp, tol=TOL, max_outer=100, sweeps=4) as mg:
            out = mg.run()
            res = [mg.result(i) for i in range(len(scs))]
        assert np.all(out["status"] == 1)
        for k, sc in enumerate(scs):
            assert np.all(np.isfinite(res[k]))
            assert _fp64_residual(ctxs[k], sc, res[k]) <= 1.05 * TOL
            with _ctx(lib, sc) as s1:
                with lib.MultiGather([s1], mlp=mlp, tol=TOL, max_outer=100, sweeps=4) as m1:
                    o1 = m1.run()
                    r1 = m1.result(0)
            assert np.array_equal(r1.view(np.uint32), res[k].view(np.uint32)), k
            assert o1["outer"][0] == out["outer"][k]
        for c in ctxs:
            c.close()
    finally:
        mlp.close()
