"""Precision form: tcgen05 BF16 GEMM, dense form-factor capture, gathering solve.

Bars: the tcgen05 GEMM equals an FP64 product of the same BF16 inputs to FP32
accumulation accuracy (1e-5 of sum |a||b|); captured FP32 rows are bit-identical
to the hemicube pipeline's rows and BF16 rows are within one BF16 rounding
(2^-8 relative to the row scale); the gathering solve reaches its tolerance and
agrees with an FP64 dense solve on the same FP32 rows to 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)  # round to nearest even
    return r


def _bf16_val(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("n,k,R", [(128, 64, 16), (200, 130, 3), (300, 257, 40), (513, 1000, 192), (256, 640, 256),
                                   (1000, 4000, 3), (700, 2500, 70), (2000, 3000, 192)])
def test_bf16_gemm_tcgen05(lib, n, k, R):
    """The gathering solve's stream-K sweep kernel on host arrays.  The last three shapes give
    CTAs ranges that end inside tiles (2-5 partial tiles per tile, added by the fixup pass)."""
    rng = np.random.default_rng(n + k + R)
    A = _bf16_bits(rng.uniform(-1, 1, (n, k)).astype(np.float32))
    B = _bf16_bits(rng.uniform(-1, 1, (R, k)).astype(np.float32))
    C = lib.bf16_gemm(A, B)
    C2 = lib.bf16_gemm(A, B)
    assert np.array_equal(C.view(np.uint32), C2.view(np.uint32))  # deterministic
    a = _bf16_val(A).astype(np.float64)
    b = _bf16_val(B).astype(np.float64)
    ref = (a @ b.T).T
    bound = (np.abs(a) @ np.abs(b).T).T
    tol = 1e-5 if k <= 1024 else 3e-5  # FP32 accumulation over k terms
    assert np.all(np.abs(C - ref) <= tol * bound + 1e-30)


@pytest.fixture(scope="module")
def box(lib):
    from radiosity_gb300 import scenes

    return scenes.room_with_boxes(target=1500, seed=21)


def _solver(lib, sc, W=64, K=16):
    s = lib.Solver(hemicube_side=W, hemicubes_count=K, mode=1)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    return s


def test_dense_capture_rows(lib, box):
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True)
        f32, bits, scale = s.dense_rows(0, box["n"])
        sh = np.array([0, 7, box["n"] // 2, box["n"] - 1], np.uint32)
        rows = s.ff_rows(sh)
    assert np.array_equal(f32[sh].view(np.uint32), rows.view(np.uint32))
    mx = f32.max(axis=1)
    assert np.allclose(scale[mx > 0], mx[mx > 0])
    approx = _bf16_val(bits) * scale[:, None]
    assert np.all(np.abs(approx - f32) <= 2.0 ** -8 * scale[:, None] + 1e-30)


@pytest.mark.parametrize("R", [1, 3, 4, 5, 6, 70])
def test_gather_residual_matches_fp64(lib, box, R):
    """r = E + rho o (F B) - B: the narrow kernel (R <= 4) and the tiled one (R > 4) against
    an FP64 evaluation on the same FP32 rows, elementwise within 1e-6 of the terms' size."""
    n = box["n"]
    rng = np.random.default_rng(100 + R)
    E = rng.uniform(0, 5, (R, n)).astype(np.float32)
    B = rng.uniform(0, 10, (R, n)).astype(np.float32)
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True)
        F, _, _ = s.dense_rows(0, n)
        r = s.gather_residual(E, B)
    rho = box["reflectance"].reshape(n, 3).astype(np.float64)
    F64 = F.astype(np.float64)
    for c in range(R):
        rc = rho[:, c % 3]
        ref = E[c] + rc * (F64 @ B[c].astype(np.float64)) - B[c]
        size = np.abs(E[c]) + rc * (np.abs(F64) @ np.abs(B[c].astype(np.float64))) + np.abs(B[c])
        assert np.all(np.abs(r[c] - ref) <= 1e-6 * size), c


@pytest.mark.parametrize("emitters", [1, 2])
def test_gather_solve_matches_fp64(lib, box, emitters):
    n = box["n"]
    rng = np.random.default_rng(3)
    E = np.zeros((3 * emitters, n), np.float32)
    for v in range(emitters):  # emission vectors x RGB
        em = rng.choice(n, 3, replace=False)
        E[3 * v:3 * v + 3, em] = rng.uniform(1, 20, (3, 3)).astype(np.float32)
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True)
        F, _, _ = s.dense_rows(0, n)
        B, st = s.gather(E, tol=1e-6, max_outer=60, sweeps=6)
    assert st.residual <= 1e-6 and st.sweeps > 0
    rho = box["reflectance"].reshape(n, 3).astype(np.float64)
    F64 = F.astype(np.float64)
    for c in range(3 * emitters):
        A = np.eye(n) - rho[:, c % 3][:, None] * F64
        ref = np.linalg.solve(A, E[c].astype(np.float64))
        assert np.linalg.norm(B[c] - ref) <= 1e-5 * np.linalg.norm(ref)


def test_shoot_residual_matches_fp64_and_the_shooter_converges_on_it(lib, box):
    """rad_shoot_residual equals the FP64 reciprocity-form residual, and the plain shooter's
    total radiosity (shot + unshot) drives it down as the unshot fraction falls."""
    from radiosity_gb300 import learned

    n = box["n"]
    rng = np.random.default_rng(9)
    E = learned.emission_block(box)
    X = (E + rng.uniform(0, 0.5, E.shape)).astype(np.float32)
    rho = box["reflectance"].reshape(n, 3).astype(np.float64)
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True)
        F, _, _ = s.dense_rows(0, n)
        r = s.shoot_residual(E, X)
        v = box["vertices"].reshape(n, 4, 3).astype(np.float64)
        area = 0.5 * np.linalg.norm(np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 3]), axis=1)
        y = (X.astype(np.float64) * area[None, :])
        FT = F.astype(np.float64).T @ y.T  # N x 3
        ref = E.astype(np.float64) + (rho * FT / area[:, None]).T - X
        assert np.max(np.abs(r - ref)) <= 1e-5 * np.max(np.abs(ref))
        # the shooter's own system
        res = []
        for tol in (1e-2, 1e-4):
            sh = lib.Solver(hemicube_side=64, hemicubes_count=16, mode=1, tolerance=tol)
            sh.upload(box["vertices"], box["color"], box["radiosity"], box["illumination"],
                      reflectance=box["reflectance"])
            st = sh.shoot(5000)
            rad, ill = sh.download()
            sh.close()
            assert st.stopped
            Bt = (rad.astype(np.float64) + ill).reshape(n, 3).T.astype(np.float32)
            res.append(np.linalg.norm(s.shoot_residual(E, Bt).astype(np.float64)) / np.linalg.norm(E))
        assert res[1] < 0.1 * res[0] and res[1] < 1e-3


def test_gather_rejects_non_finite_inputs(lib, box):
    """A NaN guess or emission is refused before any device work; NaN must never pass the
    convergence test (NaN <= tol is false, but a max() over NaN would hide it)."""
    n = box["n"]
    E = np.zeros((3, n), np.float32)
    E[:, 0] = 5.0
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True)
        g = np.array(E, copy=True)
        g[1, n // 2] = np.nan
        with pytest.raises(lib.RadError) as e:
            s.gather(E, guess=g, tol=1e-6)
        assert e.value.status == lib._lib.RAD_E_INVALID
        bad = np.array(E, copy=True)
        bad[2, 3] = np.inf
        with pytest.raises(lib.RadError) as e:
            s.gather(bad, tol=1e-6)
        assert e.value.status == lib._lib.RAD_E_INVALID
        B, st = s.gather(E, tol=1e-6, max_outer=60, sweeps=6)  # the context stays usable
        assert st.residual <= 1e-6 and np.all(np.isfinite(B))


def test_gather_ignores_leftover_device_memory(lib, box):
    """The solve's device buffers come from cudaMalloc and may hold a previous owner's bits.
    Memory filled with NaN and handed back to the driver must not leak into the result (the
    BF16 operands' row padding is multiplied by F's zero padding, and 0 x NaN = NaN)."""
    torch = pytest.importorskip("torch")
    n = box["n"]
    E = np.zeros((3, n), np.float32)
    E[:, [0, n // 3]] = 7.0
    with _solver(lib, box) as s:
        s.dense_capture(keep_fp32=True)
        for _ in range(3):
            junk = torch.full((64 << 20,), float("nan"), dtype=torch.float32, device="cuda:0")
            torch.cuda.synchronize()
            del junk
            torch.cuda.empty_cache()
            B, st = s.gather(E, tol=1e-6, max_outer=60, sweeps=6)
            assert st.residual <= 1e-6 and np.all(np.isfinite(B))


def test_streaming_residual_over_many_stages(lib):
    """k_resid_stream on a scene wide enough that its 3-stage ring wraps many times (N ~ 4k:
    8 stages of 512 columns per row block) and rows do not fill the last CTA: the residual
    equals an FP64 evaluation on the same FP32 rows within 1e-6 of the terms' size."""
    from radiosity_gb300 import scenes

    sc = scenes.room_with_boxes(target=4000, seed=33)
    n = sc["n"]
    rng = np.random.default_rng(7)
    E = rng.uniform(0, 5, (3, n)).astype(np.float32)
    B = rng.uniform(0, 10, (3, n)).astype(np.float32)
    with _solver(lib, sc) as s:
        s.dense_capture(keep_fp32=True)
        F, _, _ = s.dense_rows(0, n)
        r = s.gather_residual(E, B)
    rho = sc["reflectance"].reshape(n, 3).astype(np.float64)
    F64 = F.astype(np.float64)
    for c in range(3):
        rc = rho[:, c]
        ref = E[c] + rc * (F64 @ B[c].astype(np.float64)) - B[c]
        size = np.abs(E[c]) + rc * (np.abs(F64) @ np.abs(B[c].astype(np.float64))) + np.abs(B[c])
        assert np.all(np.abs(r[c] - ref) <= 1e-6 * size), c
