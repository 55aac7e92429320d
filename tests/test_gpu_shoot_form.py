"""Shoot form of the gathering solve (RAD_DENSE_SHOOT_FORM).

The progressive shooter spreads patch j's power with F_ij A_j / A_i, so its fixed point is
B = E + rho o (F^T (A o B)) / A.  In the shoot form the gather iterates on that system (the
transposed BF16 rows carry the sweeps, the transposed FP32 rows the residual), so it converges
to the plain shooter's answer.

Bars: the shoot-form residual (streaming kernel for R <= 4, tiled kernel for R > 4) equals an
FP64 evaluation on the same FP32 rows within 1e-6 of the terms' size and agrees with
rad_shoot_residual; the shoot-form gather reaches 1e-6 and agrees with an FP64 dense solve of
the shooter's system to 1e-5 relative L2; the plain shooter run to its unshot tolerance 1e-7
and the shoot-form gather agree within 1e-4 relative L2 (closer than the gather form's answer);
the multi-scene graph in the shoot form equals rad_gather_solve in the shoot form bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def box(lib):
    from radiosity_gb300 import scenes

    return scenes.room_with_boxes(target=1500, seed=21)


def _solver(lib, sc, W=64, K=16, **kw):
    s = lib.Solver(hemicube_side=W, hemicubes_count=K, mode=1, **kw)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    return s


def _area(sc):
    from radiosity_gb300 import learned

    return learned.patch_geometry(sc["vertices"])[2]


@pytest.mark.parametrize("R", [3, 5])
def test_shoot_form_residual_matches_fp64(lib, box, R):
    n = box["n"]
    rng = np.random.default_rng(200 + R)
    E = rng.uniform(0, 5, (R, n)).astype(np.float32)
    B = rng.uniform(0, 10, (R, n)).astype(np.float32)
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True, form="shoot")
        F, _, _ = s.dense_rows(0, n)
        r = s.gather_residual(E, B)
        r_shoot = s.shoot_residual(E, B)
    rho = box["reflectance"].reshape(n, 3).astype(np.float64)
    a = _area(box)
    FT = F.astype(np.float64).T
    for c in range(R):
        rc = rho[:, c % 3]
        b = B[c].astype(np.float64)
        ref = E[c] + rc * (FT @ (a * b)) / a - b
        size = np.abs(E[c]) + rc * (np.abs(FT) @ (a * np.abs(b))) / a + np.abs(b)
        assert np.all(np.abs(r[c] - ref) <= 1e-6 * size), c
        assert np.all(np.abs(r[c] - r_shoot[c]) <= 2e-6 * size), c


def test_shoot_form_gather_matches_fp64_solve(lib, box):
    from radiosity_gb300 import learned

    n = box["n"]
    E = learned.emission_block(box)
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True, form="shoot")
        F, _, _ = s.dense_rows(0, n)
        B, st = s.gather(E, tol=1e-6, max_outer=60, sweeps=6)
    assert st.residual <= 1e-6 and st.sweeps > 0
    rho = box["reflectance"].reshape(n, 3).astype(np.float64)
    a = _area(box)
    M = F.astype(np.float64).T * a[None, :] / a[:, None]  # (M X)_i = sum_j F_ji A_j X_j / A_i
    for c in range(3):
        ref = np.linalg.solve(np.eye(n) - rho[:, c][:, None] * M, E[c].astype(np.float64))
        assert np.linalg.norm(B[c] - ref) <= 1e-5 * np.linalg.norm(ref), c


def test_shoot_form_gather_equals_plain_shooter(lib, box):
    """Final radiosity of the shoot-form gather within 1e-4 relative L2 of the plain FP32
    shooter's (shot + unshot) radiosity, both converged tightly."""
    from radiosity_gb300 import learned

    n = box["n"]
    E = learned.emission_block(box)
    with _solver(lib, box, tolerance=1e-7) as sh:
        st = sh.shoot(40000)
        rad, ill = sh.download()
    assert st.stopped
    Bp = (rad.astype(np.float64) + ill).reshape(n, 3).T
    out = {}
    for form in ("shoot", "gather"):
        with _solver(lib, box) as s:
            s.dense_capture(keep_fp32=True, form=form)
            B, gst = s.gather(E, tol=1e-7, max_outer=80, sweeps=6)
        assert gst.residual <= 1e-7
        out[form] = np.linalg.norm(B.astype(np.float64) - Bp) / np.linalg.norm(Bp)
    assert out["shoot"] <= 1e-4, out
    assert out["shoot"] < out["gather"], out


def test_multi_gather_shoot_form_equals_gather_solve(lib):
    from radiosity_gb300 import learned, scenes

    scs = [scenes.cornell_variant(t, seed=s, n_lights=1 + s % 3) for t, s in ((700, 5), (1300, 6))]
    ctxs = [_solver(lib, sc, W=32) for sc in scs]
    try:
        with lib.MultiGather(ctxs, tol=1e-4, max_outer=100, sweeps=4, form="shoot") as mg:
            out = mg.run()
            res = [mg.result(i) for i in range(len(scs))]
        assert np.all(out["status"] == 1)
        for k, sc in enumerate(scs):
            with _solver(lib, sc, W=32) as s:
                s.dense_capture(keep_fp32=True, form="shoot")
                B, st = s.gather(learned.emission_block(sc), tol=1e-4, max_outer=100, sweeps=4)
            assert np.array_equal(res[k].view(np.uint32), B.view(np.uint32)), k
            assert st.outer == out["outer"][k]
    finally:
        for c in ctxs:
            c.close()
