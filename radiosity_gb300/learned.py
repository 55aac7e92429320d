"""Learned warm start for the gathering solve: features, targets and the training loop.

A per-patch MLP (``radiosity_gb300.MLP``, this library's own BF16 kernels) maps 32
features of a patch to its converged radiosity.  Features, per scene:
  0-2   patch centre, normalised to the scene bounding box
  3-5   unit normal
  6     area / mean area
  7-9   RGB reflectance
  10-12 log1p(first-shot direct light / s), s = per-channel mean direct light
  13-15 log1p(emission / s)
  16-31 sin / cos of 2*pi*(p . b_k) for 8 fixed random directions b_k (Fourier features)
Target: log1p(max(B - E, 0) / s); the guess is B0 = E + s * expm1(max(y, 0)).
The prediction only seeds rad_gather_solve, which still iterates to its tolerance.

The solves run in the shoot form (``FORM``): the gather converges to the fixed point of the
progressive shooter, so the network learns, and seeds, the plain solver's answer.
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import _lib, scenes

_FOURIER = np.random.default_rng(1234).normal(0.0, 2.0, (8, 3)).astype(np.float64)

# The system the training targets solve and the warm start seeds (see Solver.dense_capture).
FORM = "shoot"

# The network trained on solver-generated scenes by ``bench.py --workload learned
# --save-weights`` (its training set and evaluation are recorded in the file's metadata).
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warm_start_mlp.npz")


def save_network(mlp: "_lib.MLP", path: str, meta: dict) -> None:
    """FP32 master parameters and a JSON description of how they were trained."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, params=mlp.params(), meta=np.array(json.dumps(meta)))


def load_network(path: str = WEIGHTS, device: int = 0):
    """(MLP, metadata) of a saved network, or None when the file is absent."""
    if not os.path.exists(path):
        return None
    z = np.load(path, allow_pickle=False)
    m = _lib.MLP(seed=0, device=device)
    m.set_params(z["params"])
    return m, json.loads(str(z["meta"]))


def patch_geometry(vertices: np.ndarray):
    """Centres, unit normals and areas of the quads (N x 3, N x 3, N)."""
    q = vertices.reshape(-1, 4, 3).astype(np.float64)
    c = q.mean(1)
    n = np.cross(q[:, 3] - q[:, 0], q[:, 1] - q[:, 0])
    a = 0.5 * np.linalg.norm(np.cross(q[:, 0] - q[:, 2], q[:, 1] - q[:, 3]), axis=1)
    n = n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-20)
    return c, n, a


def scale_of(direct: np.ndarray) -> np.ndarray:
    """Per-channel normalisation s (3,) of a scene from its direct light (N x 3)."""
    return direct.mean(0) + 1e-12


def features(scene: dict, direct: np.ndarray) -> np.ndarray:
    """32 features per patch; direct is N x 3.  Uses scene["geometry"] (patch_geometry's
    output) when a scene generator attached it."""
    c, n, a = scene["geometry"] if "geometry" in scene else patch_geometry(scene["vertices"])
    lo, hi = c.min(0), c.max(0)
    p = (c - lo) / np.maximum(hi - lo, 1e-9)
    s = scale_of(direct)
    E = scene["radiosity"].reshape(-1, 3).astype(np.float64)
    rho = scene["reflectance"].reshape(-1, 3).astype(np.float64)
    ph = 2 * np.pi * p @ _FOURIER.T
    X = np.concatenate([p, n, (a / a.mean())[:, None], rho, np.log1p(np.maximum(direct, 0) / s),
                        np.log1p(E / s), np.sin(ph), np.cos(ph)], axis=1)
    return X.astype(np.float32)


def targets(scene: dict, B: np.ndarray, direct: np.ndarray) -> np.ndarray:
    """B is N x 3 converged radiosity."""
    E = scene["radiosity"].reshape(-1, 3).astype(np.float64)
    return np.log1p(np.maximum(B - E, 0) / scale_of(direct)).astype(np.float32)


def decode(scene: dict, direct: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """B0 = E + s * expm1(y), y clipped to [0, 30] (a non-finite output counts as 0, i.e. the
    emission alone), so the guess is always finite."""
    E = scene["radiosity"].reshape(-1, 3).astype(np.float64)
    y = np.where(np.isfinite(Y), np.clip(Y, 0.0, 30.0), 0.0)
    return (E + scale_of(direct) * np.expm1(y)).astype(np.float32)


def capture(scene: dict, W: int = 128, form: str = FORM) -> "_lib.Solver":
    """A PHYS solver with the scene's dense form factors captured (FP32 + BF16) in `form`."""
    s = _lib.Solver(hemicube_side=W, hemicubes_count=16, mode=_lib.MODE_PHYS)
    s.upload(scene["vertices"], scene["color"], scene["radiosity"], scene["illumination"],
             reflectance=scene["reflectance"])
    s.dense_capture(keep_fp32=True, form=form)
    return s


def emission_block(scene: dict) -> np.ndarray:
    """The scene's emission as a 3 x N column-major block (one RHS per channel)."""
    return np.ascontiguousarray(scene["radiosity"].reshape(-1, 3).T, np.float32)


def direct_light(solver: "_lib.Solver", E: np.ndarray) -> np.ndarray:
    """First-shot direct light rho o (M E) as N x 3 (M the captured form's operator)."""
    return solver.gather_residual(E, E).T.astype(np.float64)


def scene_specs(n_scenes: int, seed: int = 0, patches=(2000, 6000), kinds=("cornell",)) -> list:
    """Seeded scene descriptions for training: the patch target is log-uniform in `patches`,
    the kinds alternate.  A room varies its box count (10-60) and ceiling emitters (1-6); a
    Cornell variant has one light when it is the only kind, else 1-3 lights in turn."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n_scenes):
        target = int(np.exp(rng.uniform(np.log(patches[0]), np.log(patches[1]))))
        kind = kinds[k % len(kinds)]
        s = int(rng.integers(1 << 30))
        if kind == "room":
            specs.append(("room", target, s, int(rng.integers(10, 61)), int(rng.integers(1, 7))))
        else:
            specs.append(("cornell", target, s, 1 if len(kinds) == 1 else 1 + (k // len(kinds)) % 3, 0))
    return specs


def make_scene(spec) -> dict:
    """The scene of one scene_specs entry, with its patch geometry attached (runs in worker
    processes too: it touches no device)."""
    kind, target, seed, a, b = spec
    if kind == "room":
        sc = scenes.room_with_boxes(target=target, seed=seed, n_boxes=a, n_emitters=b)
    else:
        sc = scenes.cornell_variant(target, seed=seed, n_lights=a)
    sc["geometry"] = patch_geometry(sc["vertices"])
    return sc


def generated(specs, workers: int = 0):
    """Yields make_scene(spec) in order.  With workers > 0 the scenes are made ahead in a
    spawn-started process pool (at most 2 * workers in flight), so host generation overlaps
    the caller's device work."""
    if workers <= 0:
        for sp in specs:
            yield make_scene(sp)
        return
    import collections
    import multiprocessing

    with multiprocessing.get_context("spawn").Pool(workers) as pool:
        pending = collections.deque()
        it = iter(specs)
        for sp in it:
            pending.append(pool.apply_async(make_scene, (sp,)))
            if len(pending) >= 2 * workers:
                break
        while pending:
            sc = pending.popleft().get()
            for sp in it:
                pending.append(pool.apply_async(make_scene, (sp,)))
                break
            yield sc


def training_set(n_scenes: int, seed: int = 0, patches=(2000, 6000), W: int = 128, tol: float = 1e-6,
                 kinds=("cornell",), sample: int | None = None, workers: int = 0, form: str = FORM):
    """Solver-generated (X, T) pairs: each scene of scene_specs is captured at hemicube side W
    and solved by rad_gather_solve in `form` to `tol`; `sample` keeps at most that many random
    patches per scene (a seeded choice)."""
    Xs, Ts = [], []
    for k, sc in enumerate(generated(scene_specs(n_scenes, seed, patches, kinds), workers)):
        with capture(sc, W, form) as s:
            E = emission_block(sc)
            B, _ = s.gather(E, tol=tol, max_outer=80, sweeps=8)
            d = direct_light(s, E)
        X, T = features(sc, d), targets(sc, B.T.astype(np.float64), d)
        if sample is not None and sc["n"] > sample:
            idx = np.random.default_rng((seed, k)).choice(sc["n"], sample, replace=False)
            X, T = X[idx], T[idx]
        Xs.append(X)
        Ts.append(T)
    return np.concatenate(Xs), np.concatenate(Ts)


def warm_start(mlp: "_lib.MLP", scene: dict, direct: np.ndarray) -> np.ndarray:
    """3 x N guess for rad_gather_solve."""
    Y = mlp.predict(features(scene, direct))
    return np.ascontiguousarray(decode(scene, direct, Y).T)
