"""Generates tests/golden/reference_golden.npz from the reference's own C++.

Run in a checkout where the reference sources are present (they are compiled by
oracle/build_ref.sh into oracle/_ref/).  The fixtures pin the oracle
restatement and the product's host-side code on machines without the reference:
  * delta form-factor tables W=16, 32 (precomputeHemicubeFormFactors) and the
    reference's own sum self-check printed for W=16, 32, 256, 512
  * Config::freeze derived values for a few configurations
  * the reference scene at max area 0.5 (all arrays) and SHA-256 digests of the
    scene at 0.045 and 0.0225
  * face MVPs of 24 patches x 5 faces of the 0.045 scene
  * top-K selections for 48 seeded radiosity states (ties included)

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from oracle import RefLib, build_ref  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def topk_states(n: int, rng: np.random.Generator):
    states = []
    for t in range(48):
        m = t % 4
        if m == 0:
            rad = rng.random(3 * n).astype(np.float32)
        elif m == 1:
            rad = rng.integers(0, 4, 3 * n).astype(np.float32)
        elif m == 2:
            rad = np.repeat(rng.integers(0, 3, n), 3).astype(np.float32)
        else:
            rad = np.sort(rng.integers(0, 6, n)).repeat(3).astype(np.float32)
        states.append((rad, int(rng.integers(1, 40))))
    return states


def main():
    if not build_ref():
        raise SystemExit("reference sources not available: cannot generate golden fixtures")
    R = RefLib()
    out = {}
    for W in (16, 32):
        out[f"ff_table_{W}"] = R.ff_table(W, 1)
    out["ff_sum_w"] = np.array([16, 32, 256, 512], np.uint32)
    out["ff_sum_printed"] = np.array([R.ff_sum_printed(w) for w in (16, 32, 256, 512)], np.float64)
    cfgs = [(16, 10, 4), (256, 10, 4), (512, 32, 4), (32, 3, 5), (64, 7, 1000)]
    out["config_in"] = np.array(cfgs, np.uint32)
    out["config_out"] = np.stack([R.config(*c) for c in cfgs])
    s = R.scene(0.5)
    for k in ("vertices", "indices", "color", "radiosity", "illumination"):
        out[f"scene05_{k}"] = s[k]
    digests = []
    for a in (0.045, 0.0225):
        s = R.scene(a)
        digests.append(f"{a}:{s['n']}:" + digest(s["vertices"], s["indices"], s["color"], s["radiosity"],
                                                 s["illumination"]))
    out["scene_digests"] = np.array(digests)
    s = R.scene(0.045)
    rng = np.random.default_rng(12345)
    pids = np.sort(rng.choice(s["n"], 24, replace=False)).astype(np.uint32)
    out["mvp_patches"] = pids
    out["mvp"] = np.stack([[R.face_mvp(s["vertices"][12 * p:12 * p + 12], f) for f in range(5)] for p in pids])
    out["frames"] = np.stack([R.patch_frame(s["vertices"][12 * p:12 * p + 12]) for p in pids])
    s = R.scene(0.5)
    states = topk_states(s["n"], rng)
    out["topk_rad"] = np.stack([st[0] for st in states])
    out["topk_k"] = np.array([st[1] for st in states], np.uint32)
    ids, valid = [], []
    for rad, K in states:
        i, v = R.topk(rad, K)
        ids.append(np.pad(i, (0, 40 - K)))
        valid.append(np.pad(v, (0, 40 - K)))
    out["topk_ids"] = np.stack(ids).astype(np.uint32)
    out["topk_valid"] = np.stack(valid)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
