"""ctypes binding of the C ABI in include/radiosity.h.

This is the binding a Python caller of the reference-facing boundary uses; the
library is always the in-tree CUDA build (radiosity_gb300/libradiosity_gb300.so).
There is no fallback: if the library is missing or CUDA is unavailable, the
calls fail with an exception.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

RAD_OK = 0
RAD_E_INVALID = -1
RAD_E_CUDA = -2
RAD_E_OVERFLOW = -3
RAD_E_STATE = -4
RAD_E_NOMEM = -5
RAD_E_TIMEOUT = -6
RAD_E_NOALLOC_LIMIT = -7
RAD_E_NUMERIC = -8
NOALLOC_MAX_SUMS = 1 << 20
MODE_REF, MODE_PHYS = 0, 1
DENSE_FP32, DENSE_SHOOT_FORM = 1, 2
FORMS = {"gather": 0, "shoot": DENSE_SHOOT_FORM}

# Every symbol include/radiosity.h declares.
EXPORTS = [
    "rad_config_default", "rad_config_derived", "rad_create", "rad_destroy", "rad_upload_scene",
    "rad_set_state", "rad_download", "rad_ff_table", "rad_select_shooters", "rad_render_item_buffers",
    "rad_reduce_item_buffers", "rad_ff_rows", "rad_shoot", "rad_profile_stages", "rad_scene_reference",
    "rad_reduce_items_noalloc", "rad_raster_counters", "rad_autotune", "rad_dense_capture",
    "rad_dense_rows", "rad_gather_solve", "rad_gather_residual", "rad_shoot_residual", "rad_bf16_gemm", "rad_mlp_create", "rad_mlp_destroy",
    "rad_mlp_param_count", "rad_mlp_get_params", "rad_mlp_set_params", "rad_mlp_predict", "rad_mlp_gradients",
    "rad_mlp_train", "rad_multi_create", "rad_multi_shoot", "rad_multi_destroy", "rad_strerror", "rad_last_error",
    "rad_scene_reference_neighbours", "rad_scene_obj", "rad_rr_size", "rad_rr_write", "rad_rr_read",
    "rad_upload_neighbours", "rad_display_colors", "rad_display_colors_device", "rad_highest_patch", "rad_progress",
    "rad_set_progress", "rad_selftest_bounded_wait", "rad_face_cameras", "rad_profile_raster_phases",
    "rad_multi_gather_create", "rad_multi_gather_run", "rad_multi_gather_result", "rad_multi_gather_destroy",
    "rad_mlp_set_tensor_cores",
]
STAGES = ["select", "camera", "setup", "bins", "raster", "update", "emitters"]
STAGE_KERNELS = [1, 1, 1, 2, 1, 1, 1]


class RadConfig(ctypes.Structure):
    _fields_ = [
        ("hemicube_side", ctypes.c_uint32),
        ("ocl_workitems_x", ctypes.c_uint32),
        ("shoots_per_cycle", ctypes.c_uint32),
        ("hemicubes_count", ctypes.c_uint32),
        ("max_patch_area", ctypes.c_double),
        ("mode", ctypes.c_uint32),
        ("tile", ctypes.c_uint32),
        ("tolerance", ctypes.c_double),
        ("tri_capacity", ctypes.c_uint32),
        ("binref_capacity", ctypes.c_uint32),
        ("device", ctypes.c_int32),
        ("small_tri_pixels", ctypes.c_uint32),
    ]


class RadGatherStats(ctypes.Structure):
    _fields_ = [
        ("outer", ctypes.c_uint32),
        ("sweeps", ctypes.c_uint32),
        ("initial_residual", ctypes.c_double),
        ("residual", ctypes.c_double),
        ("device_ms", ctypes.c_double),
        ("sweep_ms", ctypes.c_double),
        ("resid_ms", ctypes.c_double),
    ]


class RadTuning(ctypes.Structure):
    _fields_ = [
        ("tile", ctypes.c_uint32),
        ("small_tri_pixels", ctypes.c_uint32),
        ("hemicubes_count", ctypes.c_uint32),
        ("candidates", ctypes.c_uint32),
        ("us_per_hemicube", ctypes.c_double),
    ]


class RadStats(ctypes.Structure):
    _fields_ = [
        ("shots_done", ctypes.c_uint32),
        ("stopped", ctypes.c_uint32),
        ("last_energy", ctypes.c_float * 3),
        ("residual", ctypes.c_double),
        ("hemicubes", ctypes.c_double),
        ("device_ms", ctypes.c_double),
    ]


_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

_LIB = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads (building first if needed) the in-tree library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run radiosity_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    P = ctypes.POINTER
    L.rad_config_default.argtypes = [P(RadConfig)]
    L.rad_config_derived.argtypes = [P(RadConfig), _u32p]
    L.rad_create.argtypes = [P(RadConfig), P(vp)]
    L.rad_destroy.argtypes = [vp]
    L.rad_upload_scene.argtypes = [vp, _f32p, vp, _f32p, vp, _f32p, _f32p, ctypes.c_uint32]
    L.rad_set_state.argtypes = [vp, vp, vp]
    L.rad_download.argtypes = [vp, vp, vp]
    L.rad_ff_table.argtypes = [vp, _f32p, ctypes.c_uint32]
    L.rad_select_shooters.argtypes = [vp, _u32p, _u8p]
    L.rad_render_item_buffers.argtypes = [vp, _u32p, ctypes.c_uint32, _u32p]
    L.rad_reduce_item_buffers.argtypes = [vp, _u32p, ctypes.c_uint32, _f32p]
    L.rad_ff_rows.argtypes = [vp, _u32p, ctypes.c_uint32, _f32p]
    L.rad_face_cameras.argtypes = [vp, _u32p, ctypes.c_uint32, _f32p, vp]
    L.rad_profile_raster_phases.argtypes = [vp, ctypes.c_uint32, np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS"),
                                            P(RadStats)]
    L.rad_shoot.argtypes = [vp, ctypes.c_uint32, P(RadStats)]
    L.rad_profile_stages.argtypes = [vp, ctypes.c_uint32, np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS"),
                                     P(RadStats)]
    L.rad_dense_capture.argtypes = [vp, ctypes.c_uint32, P(ctypes.c_double)]
    L.rad_dense_rows.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp]
    L.rad_gather_solve.argtypes = [vp, _f32p, ctypes.c_uint32, vp, ctypes.c_double, ctypes.c_uint32,
                                   ctypes.c_uint32, _f32p, P(RadGatherStats)]
    L.rad_gather_residual.argtypes = [vp, _f32p, ctypes.c_uint32, _f32p, _f32p]
    L.rad_shoot_residual.argtypes = [vp, _f32p, ctypes.c_uint32, _f32p, _f32p]
    L.rad_bf16_gemm.argtypes = [ctypes.c_int, vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _f32p]
    L.rad_selftest_bounded_wait.argtypes = [ctypes.c_int, ctypes.c_uint32, P(ctypes.c_double)]
    L.rad_mlp_create.argtypes = [ctypes.c_int, ctypes.c_uint64, P(vp)]
    L.rad_mlp_destroy.argtypes = [vp]
    L.rad_mlp_param_count.argtypes = []
    L.rad_mlp_set_tensor_cores.argtypes = [vp, ctypes.c_int]
    L.rad_mlp_get_params.argtypes = [vp, _f32p]
    L.rad_mlp_set_params.argtypes = [vp, _f32p]
    L.rad_mlp_predict.argtypes = [vp, _f32p, ctypes.c_uint32, _f32p]
    L.rad_mlp_gradients.argtypes = [vp, _f32p, _f32p, ctypes.c_uint32, _f32p, P(ctypes.c_double)]
    L.rad_mlp_train.argtypes = [vp, _f32p, _f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                P(ctypes.c_double), P(ctypes.c_double)]
    L.rad_multi_create.argtypes = [P(vp), ctypes.c_uint32, P(vp)]
    L.rad_multi_shoot.argtypes = [vp, ctypes.c_uint32, vp, vp, P(ctypes.c_uint32), P(ctypes.c_double)]
    L.rad_multi_destroy.argtypes = [vp]
    L.rad_multi_gather_create.argtypes = [P(vp), ctypes.c_uint32, vp, vp, ctypes.c_double, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_uint32, P(vp)]
    L.rad_multi_gather_run.argtypes = [vp, P(ctypes.c_double), vp, vp, vp, vp, vp]
    L.rad_multi_gather_result.argtypes = [vp, ctypes.c_uint32, _f32p]
    L.rad_multi_gather_destroy.argtypes = [vp]
    L.rad_autotune.argtypes = [vp, ctypes.c_uint32, P(RadTuning)]
    L.rad_raster_counters.argtypes = [vp, np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")]
    L.rad_reduce_items_noalloc.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp, vp]
    L.rad_scene_reference.argtypes = [ctypes.c_double, ctypes.c_uint32, P(ctypes.c_uint32), vp, vp, vp, vp, vp]
    L.rad_scene_reference_neighbours.argtypes = [ctypes.c_double, ctypes.c_uint32, P(ctypes.c_uint32), vp]
    L.rad_scene_obj.argtypes = [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_uint32,
                                P(ctypes.c_uint32), vp, vp, vp, vp, vp, vp]
    L.rad_rr_size.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P(ctypes.c_uint64)]
    L.rad_rr_write.argtypes = [ctypes.c_uint32, vp, vp, vp, vp, vp, ctypes.c_uint32, vp, ctypes.c_uint64]
    L.rad_rr_read.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint32, P(ctypes.c_uint32), vp, vp, vp, vp, vp, vp,
                              P(ctypes.c_uint32)]
    L.rad_upload_neighbours.argtypes = [vp, _u32p]
    L.rad_display_colors.argtypes = [vp, vp, vp]
    L.rad_display_colors_device.argtypes = [vp, vp, vp]
    L.rad_highest_patch.argtypes = [vp, P(ctypes.c_uint32)]
    L.rad_progress.argtypes = [vp, P(ctypes.c_uint32), P(ctypes.c_double)]
    L.rad_set_progress.argtypes = [vp, ctypes.c_uint32, ctypes.c_double]
    L.rad_strerror.argtypes = [ctypes.c_int]
    L.rad_strerror.restype = ctypes.c_char_p
    L.rad_last_error.argtypes = [vp]
    L.rad_last_error.restype = ctypes.c_char_p
    for name in EXPORTS:
        getattr(L, name).restype = getattr(L, name).restype if name in ("rad_strerror", "rad_last_error") \
            else ctypes.c_int
    L.rad_mlp_param_count.restype = ctypes.c_uint32
    _LIB = L
    return L


class RadError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"radiosity status {status}: {msg}")
        self.status = status


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def reference_scene(max_patch_area: float) -> dict:
    """rad_scene_reference: the reference Cornell scene subdivided to max_patch_area."""
    L = load()
    n = ctypes.c_uint32(0)
    rc = L.rad_scene_reference(max_patch_area, 0, ctypes.byref(n), None, None, None, None, None)
    if rc:
        raise RadError(rc, "rad_scene_reference")
    N = n.value
    out = dict(vertices=np.zeros(12 * N, np.float32), indices=np.zeros(6 * N, np.int32),
               color=np.zeros(3 * N, np.float32), radiosity=np.zeros(3 * N, np.float32),
               illumination=np.zeros(3 * N, np.float32))
    rc = L.rad_scene_reference(max_patch_area, N, ctypes.byref(n), _ptr(out["vertices"]), _ptr(out["indices"]),
                               _ptr(out["color"]), _ptr(out["radiosity"]), _ptr(out["illumination"]))
    if rc:
        raise RadError(rc, "rad_scene_reference")
    out["n"] = N
    return out


def _scene_arrays(N: int, neighbours: bool = True) -> dict:
    out = dict(vertices=np.zeros(12 * N, np.float32), indices=np.zeros(6 * N, np.int32),
               color=np.zeros(3 * N, np.float32), radiosity=np.zeros(3 * N, np.float32),
               illumination=np.zeros(3 * N, np.float32))
    if neighbours:
        out["neighbours"] = np.zeros(8 * N, np.uint32)
    return out


def reference_neighbours(max_patch_area: float) -> np.ndarray:
    """rad_scene_reference_neighbours: N x 8 display neighbours of the reference scene."""
    L = load()
    n = ctypes.c_uint32(0)
    rc = L.rad_scene_reference_neighbours(max_patch_area, 0, ctypes.byref(n), None)
    if rc:
        raise RadError(rc, "rad_scene_reference_neighbours")
    nb = np.zeros(8 * n.value, np.uint32)
    rc = L.rad_scene_reference_neighbours(max_patch_area, n.value, ctypes.byref(n), _ptr(nb))
    if rc:
        raise RadError(rc, "rad_scene_reference_neighbours")
    return nb


def obj_scene(text: bytes, max_patch_area: float = 0.0) -> dict:
    """rad_scene_obj: quads of a Wavefront OBJ file (bytes), subdivided to max_patch_area."""
    L = load()
    n = ctypes.c_uint32(0)
    rc = L.rad_scene_obj(text, len(text), max_patch_area, 0, ctypes.byref(n), None, None, None, None, None, None)
    if rc:
        raise RadError(rc, "rad_scene_obj")
    out = _scene_arrays(n.value)
    rc = L.rad_scene_obj(text, len(text), max_patch_area, n.value, ctypes.byref(n), _ptr(out["vertices"]),
                         _ptr(out["indices"]), _ptr(out["color"]), _ptr(out["radiosity"]), _ptr(out["illumination"]),
                         _ptr(out["neighbours"]))
    if rc:
        raise RadError(rc, "rad_scene_obj")
    out["n"] = n.value
    return out


def rr_write(vertices, color, radiosity, illumination, neighbours=None, pointer_bytes: int = 8) -> bytes:
    """rad_rr_write: the reference's .rr scene file (SaveToFile) as bytes."""
    L = load()
    v = np.ascontiguousarray(vertices, np.float32)
    n = v.size // 12
    arrs = [np.ascontiguousarray(a, np.float32) for a in (color, radiosity, illumination)]
    nb = None if neighbours is None else np.ascontiguousarray(neighbours, np.uint32)
    size = ctypes.c_uint64(0)
    rc = L.rad_rr_size(n, pointer_bytes, ctypes.byref(size))
    if rc:
        raise RadError(rc, "rad_rr_size")
    buf = np.zeros(size.value, np.uint8)
    rc = L.rad_rr_write(n, _ptr(v), _ptr(arrs[0]), _ptr(arrs[1]), _ptr(arrs[2]), _ptr(nb), pointer_bytes, _ptr(buf),
                        size.value)
    if rc:
        raise RadError(rc, "rad_rr_write")
    return buf.tobytes()


def rr_read(data: bytes) -> dict:
    """rad_rr_read: the scene of a .rr file (LoadFromFile + LoadingModel)."""
    L = load()
    raw = np.frombuffer(data, np.uint8)
    n = ctypes.c_uint32(0)
    ptr = ctypes.c_uint32(0)
    rc = L.rad_rr_read(_ptr(raw), raw.size, 0, ctypes.byref(n), None, None, None, None, None, None, ctypes.byref(ptr))
    if rc:
        raise RadError(rc, "rad_rr_read")
    out = _scene_arrays(n.value)
    rc = L.rad_rr_read(_ptr(raw), raw.size, n.value, ctypes.byref(n), _ptr(out["vertices"]), _ptr(out["indices"]),
                       _ptr(out["color"]), _ptr(out["radiosity"]), _ptr(out["illumination"]), _ptr(out["neighbours"]),
                       ctypes.byref(ptr))
    if rc:
        raise RadError(rc, "rad_rr_read")
    out["n"] = n.value
    out["pointer_bytes"] = ptr.value
    return out


def selftest_bounded_wait(limit_us: int, device: int = 0):
    """rad_selftest_bounded_wait: (status, waited_ms) of a device wait that nothing completes;
    the expected status is RAD_E_TIMEOUT."""
    L = load()
    ms = ctypes.c_double(0.0)
    rc = L.rad_selftest_bounded_wait(device, limit_us, ctypes.byref(ms))
    return rc, ms.value


def bf16_gemm(A_bits: np.ndarray, Bt_bits: np.ndarray, device: int = 0) -> np.ndarray:
    """rad_bf16_gemm: C (R x n, column-major rows of C^T) = A (n x k) * Bt (R x k)^T on tcgen05."""
    L = load()
    A = np.ascontiguousarray(A_bits, np.uint16)
    B = np.ascontiguousarray(Bt_bits, np.uint16)
    n, k = A.shape
    R = B.shape[0]
    C = np.zeros(R * n, np.float32)
    rc = L.rad_bf16_gemm(device, A.ctypes.data_as(ctypes.c_void_p), B.ctypes.data_as(ctypes.c_void_p), n, k, R, C)
    if rc:
        raise RadError(rc, L.rad_strerror(rc).decode())
    return C.reshape(R, n)


def default_config(**kw) -> RadConfig:
    L = load()
    cfg = RadConfig()
    L.rad_config_default(ctypes.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def derived(cfg: RadConfig) -> np.ndarray:
    out = np.zeros(9, np.uint32)
    load().rad_config_derived(ctypes.byref(cfg), out)
    return out


class Solver:
    """One rad_ctx: a device-resident scene and its shoot loop."""

    def __init__(self, cfg: RadConfig | None = None, **kw):
        self.L = load()
        self.cfg = cfg if cfg is not None else default_config(**kw)
        h = ctypes.c_void_p()
        rc = self.L.rad_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if rc:
            raise RadError(rc, self.L.rad_strerror(rc).decode())
        self.h = h
        self.n = 0

    def _check(self, rc: int, what: str):
        if rc:
            raise RadError(rc, f"{what}: {self.L.rad_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.L.rad_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def K(self) -> int:
        return int(self.cfg.hemicubes_count)

    @property
    def W(self) -> int:
        return int(self.cfg.hemicube_side)

    def upload(self, vertices, color, radiosity, illumination, reflectance=None, indices=None):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1)
        n = v.size // 12
        c = np.ascontiguousarray(color, np.float32).reshape(-1)
        r = np.ascontiguousarray(radiosity, np.float32).reshape(-1)
        i = np.ascontiguousarray(illumination, np.float32).reshape(-1)
        rho = None if reflectance is None else np.ascontiguousarray(reflectance, np.float32).reshape(-1)
        idx = None if indices is None else np.ascontiguousarray(indices, np.int32).reshape(-1)
        self._check(self.L.rad_upload_scene(self.h, v, _ptr(idx), c, _ptr(rho), r, i, n), "rad_upload_scene")
        self.n = n

    def set_state(self, radiosity=None, illumination=None):
        r = None if radiosity is None else np.ascontiguousarray(radiosity, np.float32).reshape(-1)
        i = None if illumination is None else np.ascontiguousarray(illumination, np.float32).reshape(-1)
        self._check(self.L.rad_set_state(self.h, _ptr(r), _ptr(i)), "rad_set_state")

    def download(self, out=None):
        """rad_download: (radiosity, illumination) as N x 3 float32 arrays, written into
        `out` = (r, i) when given (contiguous float32 arrays of 3N, e.g. pinned buffers)."""
        if out is None:
            r = np.empty(3 * self.n, np.float32)
            i = np.empty(3 * self.n, np.float32)
        else:
            r, i = out
            for a in (r, i):
                if a.dtype != np.float32 or a.size != 3 * self.n or not a.flags.c_contiguous:
                    raise ValueError("download(out=...) needs two contiguous float32 arrays of 3N")
        self._check(self.L.rad_download(self.h, _ptr(r), _ptr(i)), "rad_download")
        return r, i

    def upload_neighbours(self, neighbours):
        """rad_upload_neighbours: N x 8 display neighbours for display_colors."""
        nb = np.ascontiguousarray(neighbours, np.uint32).reshape(-1)
        self._check(self.L.rad_upload_neighbours(self.h, nb), "rad_upload_neighbours")

    def display_colors(self, colors: bool = True, radiative: bool = True):
        """rad_display_colors: smoothShadePatch corner colours and corner radiosities (N x 12 each)."""
        c = np.zeros(12 * self.n, np.float32) if colors else None
        r = np.zeros(12 * self.n, np.float32) if radiative else None
        self._check(self.L.rad_display_colors(self.h, _ptr(c), _ptr(r)), "rad_display_colors")
        return c, r

    def highest_patch(self) -> int:
        """rad_highest_patch: getHighestRadiosityPatchId on the device state."""
        out = ctypes.c_uint32(0)
        self._check(self.L.rad_highest_patch(self.h, ctypes.byref(out)), "rad_highest_patch")
        return out.value

    def progress(self):
        """rad_progress: (batches done, initial unshot power)."""
        shots = ctypes.c_uint32(0)
        p0 = ctypes.c_double(0)
        self._check(self.L.rad_progress(self.h, ctypes.byref(shots), ctypes.byref(p0)), "rad_progress")
        return shots.value, p0.value

    def set_progress(self, shots_done: int, initial_power: float):
        self._check(self.L.rad_set_progress(self.h, shots_done, initial_power), "rad_set_progress")

    def ff_table(self, copies: int = 1) -> np.ndarray:
        out = np.zeros(3 * self.W * self.W * copies, np.float32)
        self._check(self.L.rad_ff_table(self.h, out, copies), "rad_ff_table")
        return out

    def select(self):
        ids = np.zeros(self.K, np.uint32)
        valid = np.zeros(self.K, np.uint8)
        self._check(self.L.rad_select_shooters(self.h, ids, valid), "rad_select_shooters")
        return ids, valid.astype(bool)

    def item_buffers(self, shooters) -> np.ndarray:
        s = np.ascontiguousarray(shooters, np.uint32).reshape(-1)
        out = np.zeros(s.size * 3 * self.W * self.W, np.uint32)
        self._check(self.L.rad_render_item_buffers(self.h, s, s.size, out), "rad_render_item_buffers")
        return out

    def reduce_items(self, items, count: int) -> np.ndarray:
        it = np.ascontiguousarray(items, np.uint32).reshape(-1)
        out = np.zeros(count * self.n, np.float32)
        self._check(self.L.rad_reduce_item_buffers(self.h, it, count, out), "rad_reduce_item_buffers")
        return out.reshape(count, self.n)

    def ff_rows(self, shooters) -> np.ndarray:
        s = np.ascontiguousarray(shooters, np.uint32).reshape(-1)
        out = np.zeros(s.size * self.n, np.float32)
        self._check(self.L.rad_ff_rows(self.h, s, s.size, out), "rad_ff_rows")
        return out.reshape(s.size, self.n)

    def face_cameras(self, shooters):
        """Device face MVPs (count x 5 x 16, column-major) and frames (count x 6: center, normal)."""
        s = np.ascontiguousarray(shooters, np.uint32).reshape(-1)
        mvp = np.zeros(s.size * 80, np.float32)
        fr = np.zeros(s.size * 6, np.float32)
        self._check(self.L.rad_face_cameras(self.h, s, s.size, mvp, fr.ctypes.data_as(ctypes.c_void_p)),
                    "rad_face_cameras")
        return mvp.reshape(s.size, 5, 16), fr.reshape(s.size, 6)

    def profile_stages(self, n_shots: int):
        """Per-stage device milliseconds (summed over the batches) and the stats."""
        ms = np.zeros(len(STAGES), np.float64)
        st = RadStats()
        self._check(self.L.rad_profile_stages(self.h, n_shots, ms, ctypes.byref(st)), "rad_profile_stages")
        return dict(zip(STAGES, ms.tolist())), st

    def autotune(self, tune_k: bool = False) -> RadTuning:
        """rad_autotune: picks bin side and span/warp split (and K when tune_k) by timing."""
        t = RadTuning()
        self._check(self.L.rad_autotune(self.h, 1 if tune_k else 0, ctypes.byref(t)), "rad_autotune")
        self.cfg.tile = t.tile
        self.cfg.small_tri_pixels = t.small_tri_pixels
        self.cfg.hemicubes_count = t.hemicubes_count
        return t

    def dense_capture(self, keep_fp32: bool = True, form: str = "gather") -> float:
        """rad_dense_capture: every form-factor row; returns device ms.  form "gather" solves
        B = E + rho o (F B); "shoot" (RAD_DENSE_SHOOT_FORM) the progressive shooter's fixed point
        B = E + rho o (F^T (A o B)) / A."""
        ms = ctypes.c_double()
        flags = (DENSE_FP32 if keep_fp32 else 0) | FORMS[form]
        self._check(self.L.rad_dense_capture(self.h, flags, ctypes.byref(ms)), "rad_dense_capture")
        return ms.value

    def dense_rows(self, first: int, count: int):
        f = np.zeros(count * self.n, np.float32)
        h = np.zeros(count * self.n, np.uint16)
        sc = np.zeros(count, np.float32)
        self._check(self.L.rad_dense_rows(self.h, first, count, _ptr(f), _ptr(h), _ptr(sc)), "rad_dense_rows")
        return f.reshape(count, self.n), h.reshape(count, self.n), sc

    def gather(self, emission, guess=None, tol: float = 1e-6, max_outer: int = 50, sweeps: int = 8):
        """rad_gather_solve on column-major N x R blocks (given as R x N arrays)."""
        E = np.ascontiguousarray(emission, np.float32)
        R = E.shape[0]
        out = np.zeros_like(E)
        st = RadGatherStats()
        g = None if guess is None else np.ascontiguousarray(guess, np.float32)
        self._check(self.L.rad_gather_solve(self.h, E.reshape(-1), R, _ptr(g), tol, max_outer, sweeps,
                                            out.reshape(-1), ctypes.byref(st)), "rad_gather_solve")
        return out, st

    def gather_residual(self, emission, radiosity):
        """rad_gather_residual: r = E + rho o (M B) - B (R x N arrays), M the captured form's
        operator (F, or F^T with the area weights in the shoot form)."""
        E = np.ascontiguousarray(emission, np.float32)
        B = np.ascontiguousarray(radiosity, np.float32)
        r = np.zeros_like(E)
        self._check(self.L.rad_gather_residual(self.h, E.reshape(-1), E.shape[0], B.reshape(-1), r.reshape(-1)),
                    "rad_gather_residual")
        return r

    def shoot_residual(self, emission, radiosity):
        """rad_shoot_residual: r = E + rho o (F^T (A o B)) / A - B, the shooter's own system."""
        E = np.ascontiguousarray(emission, np.float32)
        B = np.ascontiguousarray(radiosity, np.float32)
        r = np.zeros_like(E)
        self._check(self.L.rad_shoot_residual(self.h, E.reshape(-1), E.shape[0], B.reshape(-1), r.reshape(-1)),
                    "rad_shoot_residual")
        return r

    RASTER_COUNTERS = ["record_bin_pairs", "small_records", "small_box_px", "big_records", "big_stamps",
                       "stamps_visited", "stamps_inside", "big_px_written"]
    RASTER_PHASES = ["setup", "stage", "rows", "spans", "pixels", "pass_sync", "big", "end"]

    def raster_counters(self) -> dict:
        out = np.zeros(8, np.uint64)
        self._check(self.L.rad_raster_counters(self.h, out), "rad_raster_counters")
        return dict(zip(self.RASTER_COUNTERS, [int(x) for x in out]))

    def raster_phases(self, n_shots: int) -> dict:
        """SM cycles per raster phase (summed over warps) over n_shots batches (advances the state)."""
        out = np.zeros(8, np.uint64)
        st = RadStats()
        self._check(self.L.rad_profile_raster_phases(self.h, n_shots, out, ctypes.byref(st)),
                    "rad_profile_raster_phases")
        return dict(zip(self.RASTER_PHASES, [int(x) for x in out]))

    def shoot(self, n_shots: int) -> RadStats:
        st = RadStats()
        self._check(self.L.rad_shoot(self.h, n_shots, ctypes.byref(st)), "rad_shoot")
        return st


class MLP:
    """rad_mlp: the per-patch warm-start network (BF16 weights, FP32 accumulation)."""

    IN, HID, OUT = 32, 128, 3
    DIMS = [32, 128, 128, 128, 128, 3]

    def __init__(self, seed: int = 0, device: int = 0):
        self.L = load()
        h = ctypes.c_void_p()
        rc = self.L.rad_mlp_create(device, seed, ctypes.byref(h))
        if rc:
            raise RadError(rc, "rad_mlp_create")
        self.h = h
        self.nparams = int(self.L.rad_mlp_param_count())

    def close(self):
        if self.h:
            self.L.rad_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tensor_cores(self, on: bool) -> None:
        """tcgen05 BF16 engine (default) or the CUDA-core FP32-activation engine."""
        rc = self.L.rad_mlp_set_tensor_cores(self.h, 1 if on else 0)
        if rc:
            raise RadError(rc, "rad_mlp_set_tensor_cores")

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams, np.float32)
        rc = self.L.rad_mlp_get_params(self.h, out)
        if rc:
            raise RadError(rc, "rad_mlp_get_params")
        return out

    def set_params(self, p):
        rc = self.L.rad_mlp_set_params(self.h, np.ascontiguousarray(p, np.float32))
        if rc:
            raise RadError(rc, "rad_mlp_set_params")

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], 3), np.float32)
        rc = self.L.rad_mlp_predict(self.h, X.reshape(-1), X.shape[0], Y.reshape(-1))
        if rc:
            raise RadError(rc, "rad_mlp_predict")
        return Y

    def gradients(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = ctypes.c_double()
        rc = self.L.rad_mlp_gradients(self.h, X.reshape(-1), T.reshape(-1), X.shape[0], g, ctypes.byref(loss))
        if rc:
            raise RadError(rc, "rad_mlp_gradients")
        return g, loss.value

    def train(self, X, T, epochs: int, batch: int = 4096, lr: float = 1e-3):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        loss, ms = ctypes.c_double(), ctypes.c_double()
        rc = self.L.rad_mlp_train(self.h, X.reshape(-1), T.reshape(-1), X.shape[0], epochs, batch, lr,
                                  ctypes.byref(loss), ctypes.byref(ms))
        if rc:
            raise RadError(rc, "rad_mlp_train")
        return loss.value, ms.value


def plan_shooters(patches, hemicubes_per_patch: float = 2.0, replays: int = 128, kmin: int = 8,
                  kmax: int = 128) -> list:
    """Shooters per batch for each scene of an uneven batch solved under one graph.

    Every replay of the graph advances every scene by one batch, so the batch ends when the
    scene that needs the most replays converges.  A scene of N patches needs about
    ``hemicubes_per_patch * N`` hemicubes to reach its tolerance (about 2 for an unshot fraction
    of 1e-2 and 4.5 for 1e-4 on the Cornell-style scenes), hence K = that / ``replays``, rounded
    up to a power of two and clamped to [kmin, kmax], makes the scenes finish together."""
    out = []
    for n in patches:
        want = max(1.0, hemicubes_per_patch * float(n) / replays)
        k = 1
        while k < want:
            k *= 2
        out.append(int(min(max(k, kmin), kmax)))
    return out


class Multi:
    """rad_multi: many solvers advanced together, one CUDA graph replay per batch."""

    def __init__(self, solvers):
        self.L = load()
        self.solvers = list(solvers)
        arr = (ctypes.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = ctypes.c_void_p()
        rc = self.L.rad_multi_create(arr, len(self.solvers), ctypes.byref(h))
        if rc:
            raise RadError(rc, "rad_multi_create")
        self.h = h

    def shoot(self, n_replays: int):
        n = len(self.solvers)
        at = np.zeros(n, np.uint32)
        ms = np.zeros(n, np.float64)
        reps = ctypes.c_uint32()
        total = ctypes.c_double()
        rc = self.L.rad_multi_shoot(self.h, n_replays, at.ctypes.data_as(ctypes.c_void_p),
                                    ms.ctypes.data_as(ctypes.c_void_p), ctypes.byref(reps), ctypes.byref(total))
        if rc:
            raise RadError(rc, "rad_multi_shoot")
        return at, ms, reps.value, total.value

    def close(self):
        if self.h:
            self.L.rad_multi_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class MultiGather:
    """rad_multi_gather: scenes solved together by (learned warm start +) BF16 gather under one
    captured CUDA graph: dense capture, features, network guess and the refinement loop (a
    conditional node) all run on the device; each scene stops at its own tolerance."""

    def __init__(self, solvers, mlp=None, tol: float = 1e-4, max_outer: int = 100, sweeps: int = 4,
                 form: str = "gather"):
        self.L = load()
        self.solvers = list(solvers)
        arr = (ctypes.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        dirs = None
        if mlp is not None:
            from .learned import _FOURIER

            self._dirs = np.ascontiguousarray(_FOURIER, np.float64)
            dirs = self._dirs.ctypes.data_as(ctypes.c_void_p)
        h = ctypes.c_void_p()
        rc = self.L.rad_multi_gather_create(arr, len(self.solvers), mlp.h if mlp is not None else None, dirs, tol,
                                            max_outer, sweeps, FORMS[form], ctypes.byref(h))
        if rc:
            raise RadError(rc, "rad_multi_gather_create")
        self.h = h

    def run(self) -> dict:
        n = len(self.solvers)
        ms = ctypes.c_double()
        scene_ms = np.zeros(n, np.float64)
        outer = np.zeros(n, np.uint32)
        res = np.zeros(n, np.float64)
        res0 = np.zeros(n, np.float64)
        status = np.zeros(n, np.uint32)
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = self.L.rad_multi_gather_run(self.h, ctypes.byref(ms), ptr(scene_ms), ptr(outer), ptr(res), ptr(res0),
                                         ptr(status))
        if rc:
            raise RadError(rc, "rad_multi_gather_run")
        return {"device_ms": ms.value, "scene_ms": scene_ms, "outer": outer, "residual": res,
                "initial_residual": res0, "status": status}

    def result(self, i: int) -> np.ndarray:
        """Scene i's radiosity as a 3 x N array (one row per channel)."""
        n = self.solvers[i].n
        out = np.zeros(3 * n, np.float32)
        rc = self.L.rad_multi_gather_result(self.h, i, out)
        if rc:
            raise RadError(rc, "rad_multi_gather_result")
        return out.reshape(3, n)

    def close(self):
        if self.h:
            self.L.rad_multi_gather_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
