"""ctypes bindings for the oracle restatement and the compiled reference.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
``bench.py`` (CPU baseline / reference arm) as the checker.  The product
package never imports this module.

* ``Oracle`` wraps ``oracle/liboracle.so`` (the C restatement in oracle.c).
* ``RefLib`` wraps ``oracle/_ref/libradref.so`` (the reference's own C++ compiled by
  oracle/build_ref.sh); it exists only where the reference sources were present
  at build time.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libradref.so")
REF_FFSUM = os.path.join(HERE, "_ref", "ffsum")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

MODE_REF, MODE_PHYS = 0, 1
FF_EXACT, FF_RECORDS = 0, 1


def build(force: bool = False) -> None:
    """Compile liboracle.so (and oracle/_ref when the reference is present)."""
    if force or not os.path.exists(ORACLE_SO) or (
        os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "oracle.c"))
    ):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so" if False else "all"])


def build_ref() -> bool:
    """Build oracle/_ref from the reference sources if they exist; returns availability."""
    root = os.environ.get("RADIOSITY_REFERENCE", "/root/reference")
    if os.path.isdir(os.path.join(root, "source")) and not os.path.exists(REF_SO):
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), root])
    return os.path.exists(REF_SO)


class OrcStats(ctypes.Structure):
    _fields_ = [
        ("shots_done", ctypes.c_uint32),
        ("stopped", ctypes.c_uint32),
        ("last_energy", ctypes.c_float * 3),
        ("residual", ctypes.c_double),
        ("hemicubes", ctypes.c_double),
    ]


class Oracle:
    """The C restatement of the reference path (oracle/oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        self.L = L
        L.orc_ff_table.argtypes = [ctypes.c_uint32, _f32p]
        L.orc_ff_sum.argtypes = [ctypes.c_uint32]
        L.orc_ff_sum.restype = ctypes.c_float
        L.orc_face_rects.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _i32p, _i32p]
        L.orc_face_mvp.argtypes = [_f32p, ctypes.c_int, _f32p]
        L.orc_patch_frame.argtypes = [_f32p, _f32p]
        L.orc_render_hemicube.argtypes = [ctypes.c_uint32, _f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p]
        L.orc_process_hemicube.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _u32p, _f32p,
                                           _u32p, _u32p, _f32p, ctypes.c_uint32]
        L.orc_process_hemicube.restype = ctypes.c_uint32
        L.orc_ff_from_records.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _u32p, _u32p,
                                          _f32p, _f32p]
        L.orc_ff_exact.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _u32p, _f32p]
        L.orc_topk_ref.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, _u8p]
        L.orc_topk_phys.argtypes = [_f32p, _f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, _u8p]
        L.orc_patch_areas.argtypes = [_f32p, ctypes.c_uint32, _f32p]
        L.orc_shoot.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_uint32, _f32p, _f32p, _f32p, ctypes.c_uint32, _f32p, _f32p,
                                ctypes.c_uint32, ctypes.c_double, ctypes.c_int, ctypes.POINTER(OrcStats)]
        L.orc_shoot.restype = ctypes.c_int

    def ff_table(self, W: int) -> np.ndarray:
        out = np.zeros(3 * W * W, np.float32)
        self.L.orc_ff_table(W, out)
        return out

    def ff_sum(self, W: int) -> float:
        return float(self.L.orc_ff_sum(W))

    def face_rects(self, W: int, hi: int, face: int):
        vp = np.zeros(4, np.int32)
        sc = np.zeros(4, np.int32)
        self.L.orc_face_rects(W, hi, face, vp, sc)
        return vp, sc

    def face_mvp(self, quad: np.ndarray, face: int) -> np.ndarray:
        out = np.zeros(16, np.float32)
        self.L.orc_face_mvp(np.ascontiguousarray(quad, np.float32), face, out)
        return out

    def patch_frame(self, quad: np.ndarray) -> np.ndarray:
        out = np.zeros(9, np.float32)
        self.L.orc_patch_frame(np.ascontiguousarray(quad, np.float32), out)
        return out

    def render(self, W: int, verts: np.ndarray, shooter: int) -> np.ndarray:
        n = verts.size // 12
        out = np.zeros(3 * W * W, np.uint32)
        self.L.orc_render_hemicube(W, np.ascontiguousarray(verts, np.float32), n, shooter, out)
        return out

    def process_hemicube(self, W: int, items: np.ndarray, k: int, workitems_x: int = 4):
        table = self.ff_table(W)
        cap = items.size + 64
        rh = np.zeros(cap, np.uint32)
        ri = np.zeros(cap, np.uint32)
        re = np.zeros(cap, np.float32)
        n = self.L.orc_process_hemicube(W, k, workitems_x, np.ascontiguousarray(items, np.uint32), table,
                                        rh, ri, re, cap)
        n = min(n, cap)
        return rh[:n], ri[:n], re[:n]

    def ff_from_records(self, k: int, n: int, rh, ri, re) -> np.ndarray:
        F = np.zeros(k * n, np.float32)
        self.L.orc_ff_from_records(k, n, len(rh), np.ascontiguousarray(rh, np.uint32),
                                   np.ascontiguousarray(ri, np.uint32), np.ascontiguousarray(re, np.float32), F)
        return F.reshape(k, n)

    def ff_records(self, W: int, items: np.ndarray, k: int, n: int, workitems_x: int = 4) -> np.ndarray:
        rh, ri, re = self.process_hemicube(W, items, k, workitems_x)
        return self.ff_from_records(k, n, rh, ri, re)

    def ff_exact(self, W: int, items: np.ndarray, k: int, n: int) -> np.ndarray:
        F = np.zeros(k * n, np.float32)
        self.L.orc_ff_exact(W, k, n, np.ascontiguousarray(items, np.uint32), F)
        return F.reshape(k, n)

    def topk_ref(self, rad: np.ndarray, K: int):
        n = rad.size // 3
        ids = np.zeros(K, np.uint32)
        valid = np.zeros(K, np.uint8)
        self.L.orc_topk_ref(np.ascontiguousarray(rad, np.float32), n, K, ids, valid)
        return ids, valid.astype(bool)

    def topk_phys(self, rad: np.ndarray, area: np.ndarray, K: int):
        n = rad.size // 3
        ids = np.zeros(K, np.uint32)
        valid = np.zeros(K, np.uint8)
        self.L.orc_topk_phys(np.ascontiguousarray(rad, np.float32), np.ascontiguousarray(area, np.float32),
                             n, K, ids, valid)
        return ids, valid.astype(bool)

    def patch_areas(self, verts: np.ndarray) -> np.ndarray:
        n = verts.size // 12
        out = np.zeros(n, np.float32)
        self.L.orc_patch_areas(np.ascontiguousarray(verts, np.float32), n, out)
        return out

    def shoot(self, mode: int, W: int, K: int, verts, color, rad, illum, n_shots: int, rho=None,
              ff_kind: int = FF_EXACT, tol: float = 0.0, workitems_x: int = 4, threads: int = 0):
        """Runs the shoot loop; returns (rad, illum, stats) with new arrays."""
        n = verts.size // 12
        rad = np.array(rad, np.float32, copy=True).reshape(-1)
        illum = np.array(illum, np.float32, copy=True).reshape(-1)
        rho_a = np.zeros(3 * n, np.float32) if rho is None else np.ascontiguousarray(rho, np.float32).reshape(-1)
        st = OrcStats()
        rc = self.L.orc_shoot(mode, ff_kind, W, K, workitems_x, np.ascontiguousarray(verts, np.float32).reshape(-1),
                              np.ascontiguousarray(color, np.float32).reshape(-1), rho_a, n, rad, illum,
                              n_shots, tol, threads, ctypes.byref(st))
        if rc != 0:
            raise RuntimeError(f"orc_shoot failed ({rc})")
        return rad, illum, st


class RefLib:
    """The reference's own CPU classes compiled by oracle/build_ref.sh."""

    def __init__(self, path: str = REF_SO):
        L = ctypes.CDLL(path)
        self.L = L
        L.ref_scene_build.argtypes = [ctypes.c_double]
        L.ref_scene_build.restype = ctypes.c_uint
        L.ref_scene_get.argtypes = [_f32p, _i32p, _f32p, _f32p, _f32p]
        L.ref_config.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, _u32p]
        L.ref_ff_table.argtypes = [ctypes.c_uint, ctypes.c_uint, _f32p]
        L.ref_topk.argtypes = [ctypes.c_uint, _f32p, _u32p, _i32p]
        L.ref_face_mvp.argtypes = [_f32p, ctypes.c_int, _f32p]
        L.ref_patch_frame.argtypes = [_f32p, _f32p]
        vp = ctypes.c_void_p
        L.ref_neighbours.argtypes = [_u32p]
        L.ref_smooth_shade.argtypes = [_f32p, _f32p, _f32p]
        L.ref_highest_id.argtypes = [_f32p]
        L.ref_highest_id.restype = ctypes.c_uint
        L.ref_obj_build.argtypes = [ctypes.c_char_p, ctypes.c_double]
        L.ref_obj_build.restype = ctypes.c_uint
        L.ref_obj_get.argtypes = [vp, vp, vp, vp, vp]
        L.ref_rr_save.argtypes = [_f32p, _f32p, vp, ctypes.POINTER(ctypes.c_uint)]
        L.ref_rr_save.restype = ctypes.c_ulonglong
        L.ref_rr_load.argtypes = [vp]
        L.ref_rr_load.restype = ctypes.c_uint

    def scene(self, area: float):
        n = self.L.ref_scene_build(area)
        self._n = n
        v = np.zeros(12 * n, np.float32)
        idx = np.zeros(6 * n, np.int32)
        col = np.zeros(3 * n, np.float32)
        rad = np.zeros(3 * n, np.float32)
        ill = np.zeros(3 * n, np.float32)
        self.L.ref_scene_get(v, idx, col, rad, ill)
        return dict(n=n, vertices=v, indices=idx, color=col, radiosity=rad, illumination=ill)

    def config(self, W: int, K: int, wx: int = 4):
        out = np.zeros(9, np.uint32)
        self.L.ref_config(W, K, wx, out)
        return out

    def ff_table(self, W: int, K: int = 1) -> np.ndarray:
        out = np.zeros(3 * W * W * K, np.float32)
        self.L.ref_ff_table(W, K, out)
        return out

    def topk(self, rad: np.ndarray, K: int):
        """Needs a prior scene(area) call with the same patch count."""
        ids = np.zeros(K, np.uint32)
        valid = np.zeros(K, np.int32)
        self.L.ref_topk(K, np.ascontiguousarray(rad, np.float32).reshape(-1), ids, valid)
        return ids, valid.astype(bool)

    def face_mvp(self, quad: np.ndarray, face: int) -> np.ndarray:
        out = np.zeros(16, np.float32)
        self.L.ref_face_mvp(np.ascontiguousarray(quad, np.float32), face, out)
        return out

    def patch_frame(self, quad: np.ndarray) -> np.ndarray:
        out = np.zeros(9, np.float32)
        self.L.ref_patch_frame(np.ascontiguousarray(quad, np.float32), out)
        return out

    def neighbours(self) -> np.ndarray:
        """Display neighbours of the last scene(area), N x 8 scene indices."""
        out = np.zeros(8 * self._n, np.uint32)
        self.L.ref_neighbours(out)
        return out

    def smooth_shade(self, rad: np.ndarray, illum: np.ndarray) -> np.ndarray:
        """Colors::smoothShadePatch of every patch of the last scene(area), N x 12."""
        out = np.zeros(12 * self._n, np.float32)
        self.L.ref_smooth_shade(np.ascontiguousarray(rad, np.float32), np.ascontiguousarray(illum, np.float32), out)
        return out

    def highest_id(self, rad: np.ndarray) -> int:
        return int(self.L.ref_highest_id(np.ascontiguousarray(rad, np.float32)))

    def _container(self, n: int) -> dict:
        out = dict(n=n, vertices=np.zeros(12 * n, np.float32), color=np.zeros(3 * n, np.float32),
                   radiosity=np.zeros(3 * n, np.float32), illumination=np.zeros(3 * n, np.float32),
                   neighbours=np.zeros(8 * n, np.uint32))
        self.L.ref_obj_get(*[out[k].ctypes.data_as(ctypes.c_void_p)
                             for k in ("vertices", "color", "radiosity", "illumination", "neighbours")])
        return out

    def obj(self, path: str, area: float) -> dict:
        """WaveFrontModel(path) in a ModelContainer subdivided to `area`."""
        return self._container(self.L.ref_obj_build(path.encode(), area))

    def rr_save(self, rad: np.ndarray, illum: np.ndarray):
        """SaveToFile's bytes for the last scene(area) with the given state, and sizeof(Patch)."""
        rec = ctypes.c_uint(0)
        r = np.ascontiguousarray(rad, np.float32)
        i = np.ascontiguousarray(illum, np.float32)
        size = self.L.ref_rr_save(r, i, None, ctypes.byref(rec))
        buf = np.zeros(size, np.uint8)
        self.L.ref_rr_save(r, i, buf.ctypes.data_as(ctypes.c_void_p), ctypes.byref(rec))
        return buf.tobytes(), rec.value

    def rr_load(self, data: bytes) -> dict:
        """LoadFromFile + LoadingModel on this build's layout."""
        raw = np.frombuffer(data, np.uint8).copy()
        return self._container(self.L.ref_rr_load(raw.ctypes.data_as(ctypes.c_void_p)))

    @staticmethod
    def ff_sum_printed(W: int) -> float:
        out = subprocess.check_output([REF_FFSUM, str(W)], text=True)
        return float(out.strip().split(":")[1])
