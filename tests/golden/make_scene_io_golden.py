"""Generates tests/golden/scene_io_golden.npz from the reference's own C++.

Run where the reference sources are present (compiled by oracle/build_ref.sh into
oracle/_ref/).  The fixtures pin, on machines without the reference:
  * Patch::neighbours of the reference scene at max area 0.5 (all) and a SHA-256
    digest at 0.045
  * Colors::smoothShadePatch of every patch for two seeded states at area 0.5, and a
    digest for one hashed state (hashed_state, rebuilt by the tests) at 0.045
  * ModelContainer::getHighestRadiosityPatchId for 12 states (ties, zeros, NaN, inf)
  * WaveFrontModel on tests/golden/quads.obj at areas 0, 0.05 and 0.3
  * SaveToFile's bytes (64-bit build layout) for the unsubdivided scene with a seeded
    state

    python tests/golden/make_scene_io_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import RefLib, build_ref  # noqa: E402

OBJ = os.path.join(HERE, "quads.obj")


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def hashed_state(n: int, salt: int) -> np.ndarray:
    """3n floats in [0, 1) from an integer hash: reproducible bit for bit on any machine."""
    i = np.arange(3 * n, dtype=np.uint64) + np.uint64(salt)
    h = (i * np.uint64(2654435761) + np.uint64(12345)) % np.uint64(1 << 32)
    return (h.astype(np.float64) / float(1 << 32)).astype(np.float32)


def shade_states(n: int, rng: np.random.Generator):
    a = (rng.random(3 * n).astype(np.float32), rng.random(3 * n).astype(np.float32))
    b = (rng.integers(0, 5, 3 * n).astype(np.float32) * np.float32(0.37),
         (rng.random(3 * n) * 100).astype(np.float32))
    return [a, b]


def highest_states(n: int, rng: np.random.Generator):
    out = []
    out.append(rng.random(3 * n).astype(np.float32))                 # distinct values
    out.append(rng.integers(0, 3, 3 * n).astype(np.float32))         # many ties
    out.append(np.zeros(3 * n, np.float32))                          # all zero -> patch 0
    s = rng.random(3 * n).astype(np.float32)
    s[0] = np.nan                                                    # NaN at patch 0 -> patch 0
    out.append(s)
    s = rng.random(3 * n).astype(np.float32)
    s[3 * 17 + 1] = np.nan                                           # NaN elsewhere never wins
    out.append(s)
    s = rng.random(3 * n).astype(np.float32)
    s[3 * (n // 2)] = np.inf                                         # inf wins
    out.append(s)
    out.append(-rng.random(3 * n).astype(np.float32))                # negative radiosity
    s = rng.random(3 * n).astype(np.float32) * 0.5
    s[3 * (n - 1):] = 2.0                                            # maximum at the last patch
    out.append(s)
    s = np.repeat(rng.integers(0, 2, n), 3).astype(np.float32)      # ties at the maximum 3
    out.append(s * 3)
    for _ in range(3):
        out.append((rng.random(3 * n) ** 8).astype(np.float32))
    return out


def main():
    if not build_ref():
        raise SystemExit("reference sources not available: cannot generate golden fixtures")
    R = RefLib()
    rng = np.random.default_rng(2024)
    out = {}
    s = R.scene(0.5)
    n = s["n"]
    out["nb05"] = R.neighbours()
    st = shade_states(n, rng)
    out["shade_rad"] = np.stack([x[0] for x in st])
    out["shade_illum"] = np.stack([x[1] for x in st])
    out["shade_colors"] = np.stack([R.smooth_shade(r, i) for r, i in st])
    hs = highest_states(n, rng)
    out["hi_rad"] = np.stack(hs)
    out["hi_id"] = np.array([R.highest_id(h) for h in hs], np.uint32)
    s = R.scene(0.045)
    n45 = s["n"]
    r45, i45 = hashed_state(n45, 1), hashed_state(n45, 2)  # tests rebuild these with hashed_state
    out["nb_0045_digest"] = np.array(f"{n45}:" + digest(R.neighbours()))
    out["shade_0045_digest"] = np.array(digest(R.smooth_shade(r45, i45)))
    for a, tag in ((0.0, "0"), (0.05, "005"), (0.3, "03")):
        o = R.obj(OBJ, a)
        for k in ("vertices", "color", "radiosity", "illumination", "neighbours"):
            out[f"obj{tag}_{k}"] = o[k]
    s = R.scene(0.0)
    r0 = rng.random(3 * s["n"]).astype(np.float32)
    i0 = rng.random(3 * s["n"]).astype(np.float32)
    data, rec = R.rr_save(r0, i0)
    out["rr_bytes"] = np.frombuffer(data, np.uint8)
    out["rr_record"] = np.uint32(rec)
    out["rr_vertices"] = s["vertices"]
    out["rr_color"] = s["color"]
    out["rr_rad"] = r0
    out["rr_illum"] = i0
    out["rr_neighbours"] = R.neighbours()
    path = os.path.join(HERE, "scene_io_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
