"""ctypes binding of liblbm_gb300.so (the C ABI in include/lbm_gb300.h).

This is the same boundary a C, C++, Go or Java caller binds.  Loading fails
loudly when the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

LBM_D3Q19, LBM_D3Q27 = 19, 27
LBM_F64, LBM_F32, LBM_F16, LBM_BF16 = 0, 1, 2, 3
LBM_PARITY, LBM_PHYSICS = 0, 1
LBM_BC_REF_INLET, LBM_BC_REF_OUTLET_YMAX, LBM_BC_REF_OUTLET_ZMIN, LBM_BC_VELOCITY, LBM_BC_PRESSURE = 1, 2, 3, 4, 5
FACES = {"x-": 0, "x+": 1, "y-": 2, "y+": 3, "z-": 4, "z+": 5}
PRECISIONS = {"f64": LBM_F64, "f32": LBM_F32, "f16": LBM_F16, "bf16": LBM_BF16}
MAX_BC = 256
LBM_COLLISION_BGK = 0
LBM_COLLISION_REGULARIZED = 1
MAX_WAVES = 256
LBM_FLAG_NONFINITE, LBM_FLAG_BOUNDS = 1, 4
LBM_NN_ENGINE_AUTO, LBM_NN_ENGINE_MMA_SYNC = 0, 1  # lbm_nn_set_conv_engine (include/lbm_nn.h)

ERRORS = {-1: "LBM_ERR_ARG", -2: "LBM_ERR_CUDA", -3: "LBM_ERR_STATE", -4: "LBM_ERR_NONFINITE",
          -5: "LBM_ERR_ALLOC", -6: "LBM_ERR_IO", -7: "LBM_ERR_UNSUPPORTED"}


class LbmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class VoxDesc(C.Structure):
    _fields_ = [("spacing", C.c_double), ("reference_bbox", C.c_int), ("bbox", C.c_double * 6),
                ("origin", C.c_double * 3), ("dims", C.c_int * 3), ("fluid_count", C.c_int64),
                ("ray_tests", C.c_int64)]


class Desc(C.Structure):
    _fields_ = [("Q", C.c_int), ("precision", C.c_int), ("mode", C.c_int), ("tau", C.c_double),
                ("spacing", C.c_double), ("origin", C.c_double * 3), ("wss_scale", C.c_double),
                ("tawss_div", C.c_double), ("device", C.c_int), ("collision", C.c_int)]


class BCSpec(C.Structure):
    _fields_ = [("kind", C.c_int), ("face", C.c_int), ("plane", C.c_int), ("value", C.c_double),
                ("profile", C.c_int), ("c1", C.c_double), ("c2", C.c_double), ("R", C.c_double),
                ("region", C.c_int), ("coord", C.c_double), ("tol", C.c_double), ("lo", C.c_double * 2),
                ("hi", C.c_double * 2), ("wave", C.c_int)]


class Counts(C.Structure):
    _fields_ = [("points", C.c_int64), ("active", C.c_int64), ("fluid", C.c_int64), ("wall", C.c_int64),
                ("bc", C.c_int64 * MAX_BC), ("next_to_wall", C.c_int64), ("special", C.c_int64),
                ("segments", C.c_int64), ("steps", C.c_int64), ("device_bytes", C.c_int64)]


_lib = None
EXPORTS = [
    "lbm_voxelize", "lbm_read_stl_ascii", "lbm_create", "lbm_destroy", "lbm_last_error", "lbm_last_global_error",
    "lbm_set_geometry", "lbm_set_normals_from_surface", "lbm_set_normals_from_surface_box", "lbm_set_inlet_table",
    "lbm_set_waveform", "lbm_init_equilibrium",
    "lbm_init_from_macro", "lbm_step", "lbm_step_async", "lbm_check_status", "lbm_sync", "lbm_get_counts", "lbm_get_classes", "lbm_get_distributions",
    "lbm_set_distributions", "lbm_get_macro", "lbm_get_wss", "lbm_get_conservation", "lbm_save", "lbm_load",
    "lbm_get_stream", "lbm_get_launch_count", "lbm_set_graph_steps", "lbm_set_persistent", "lbm_preset_barrier",
    "lbm_preset_flags", "lbm_autotune", "lbm_set_variant",
    "lbm_moment_sums_noalloc",
    "lbm_nn_conv3d_fwd", "lbm_nn_conv3d_bwd", "lbm_nn_set_conv_engine", "lbm_nn_conv_status",
    "lbm_nn_relu_bwd", "lbm_nn_upsample2", "lbm_nn_add", "lbm_nn_mse",
    "lbm_nn_adam", "lbm_sdf_from_mask", "lbm_ws_prior", "lbm_ws_smooth", "lbm_ws_features", "lbm_ws_output", "lbm_ws_gather",
    "lbm_init_from_macro_device", "lbm_nearest_next_to_wall", "lbm_set_wall_distances", "lbm_get_wall_distances",
    "lbm_get_macro_async", "lbm_get_wss_async", "lbm_wait_outputs",
]
NUM_VARIANTS = 8  # LBM_NUM_VARIANTS: lbm_autotune writes this many floats


def lib_path() -> str:
    """The library this process binds: $LBM_LIBRARY when set (e.g. the
    bounds-checked build), else the in-tree build."""
    return os.environ.get("LBM_LIBRARY") or _build.LIB


def load(build_if_missing: bool = True):
    """Load liblbm_gb300.so (building it in-tree when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise LbmError(-7, f"{path} is not built (run pv_dec_original_gb300.build)")
        _build.build()
    L = C.CDLL(path)
    P = C.c_void_p
    dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
    i64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
    L.lbm_voxelize.argtypes = [P, C.c_int64, C.POINTER(VoxDesc), P]
    L.lbm_read_stl_ascii.argtypes = [C.c_char_p, P, C.POINTER(C.c_int64)]
    L.lbm_create.argtypes = [C.POINTER(Desc), C.POINTER(P)]
    L.lbm_destroy.argtypes = [P]
    L.lbm_last_error.argtypes = [P]
    L.lbm_last_error.restype = C.c_char_p
    L.lbm_last_global_error.restype = C.c_char_p
    L.lbm_set_geometry.argtypes = [P, u8, C.POINTER(C.c_int), C.POINTER(BCSpec), C.c_int]
    L.lbm_set_normals_from_surface.argtypes = [P, dp, C.c_int64]
    L.lbm_set_inlet_table.argtypes = [P, dp, C.c_int64]
    L.lbm_set_waveform.argtypes = [P, C.c_int, dp, C.c_int64]
    L.lbm_set_normals_from_surface_box.argtypes = [P, dp, C.c_int64, dp, dp]
    L.lbm_init_equilibrium.argtypes = [P]
    L.lbm_init_from_macro.argtypes = [P, fp, fp, C.c_int]
    L.lbm_step.argtypes = [P, C.c_int]
    L.lbm_step_async.argtypes = [P, C.c_int]
    L.lbm_check_status.argtypes = [P]
    L.lbm_sync.argtypes = [P]
    L.lbm_get_counts.argtypes = [P, C.POINTER(Counts)]
    L.lbm_get_classes.argtypes = [P, u8]
    L.lbm_get_distributions.argtypes = [P, dp]
    L.lbm_set_distributions.argtypes = [P, dp]
    L.lbm_get_macro.argtypes = [P, P, P]
    L.lbm_get_wss.argtypes = [P, P, P, P, P, P, P, P]
    L.lbm_get_wss_async.argtypes = [P, P, P, P, P, P, P, P]
    L.lbm_get_macro_async.argtypes = [P, P, P]
    L.lbm_wait_outputs.argtypes = [P]
    L.lbm_get_conservation.argtypes = [P, P, P, P]
    L.lbm_save.argtypes = [P, C.c_char_p]
    L.lbm_load.argtypes = [P, C.c_char_p]
    L.lbm_get_stream.argtypes = [P, C.POINTER(P)]
    L.lbm_get_launch_count.argtypes = [P, C.POINTER(C.c_int64)]
    L.lbm_set_graph_steps.argtypes = [P, C.c_int]
    L.lbm_set_persistent.argtypes = [P, C.c_int]
    L.lbm_preset_barrier.argtypes = [P, C.c_uint]
    L.lbm_preset_flags.argtypes = [P, C.c_uint]
    L.lbm_autotune.argtypes = [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]
    L.lbm_set_variant.argtypes = [P, C.c_int]
    L.lbm_moment_sums_noalloc.argtypes = [P, C.c_int64, C.c_int, P, P]
    I3 = C.POINTER(C.c_int)
    L.lbm_nn_conv3d_fwd.argtypes = [P, I3, C.c_int, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P]
    L.lbm_nn_conv3d_bwd.argtypes = [P, I3, C.c_int, P, P, C.c_int, C.c_int, C.c_int, P, P, P, P, P]
    L.lbm_nn_set_conv_engine.argtypes = [C.c_int]
    L.lbm_nn_conv_status.argtypes = []
    L.lbm_nn_relu_bwd.argtypes = [P, P, C.c_int64, P]
    L.lbm_nn_upsample2.argtypes = [P, I3, C.c_int, P, C.c_int, P]
    L.lbm_nn_add.argtypes = [P, P, P, C.c_int64, P]
    L.lbm_nn_mse.argtypes = [P, P, P, C.c_int64, C.c_int, C.c_int, C.c_float, P, P, P]
    L.lbm_nn_adam.argtypes = [P, P, P, P, P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int64, P]
    L.lbm_sdf_from_mask.argtypes = [P, I3, P, P, P]
    L.lbm_ws_prior.argtypes = [P, I3, C.c_double, C.c_double, P, P, P, P, P]
    L.lbm_ws_smooth.argtypes = [P, I3, P, P, C.c_int, P]
    L.lbm_ws_features.argtypes = [P, P, P, P, I3, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, P, P]
    L.lbm_ws_output.argtypes = [P, C.c_int, P, P, P, C.c_int64, C.c_float, C.c_float, C.c_float, P, P]
    L.lbm_ws_gather.argtypes = [P, C.c_int64, P, C.c_int64, P, P, P]
    L.lbm_init_from_macro_device.argtypes = [P, P, P, C.c_int, P]
    L.lbm_nearest_next_to_wall.argtypes = [P, P, C.c_int64, C.c_int, P, P]
    L.lbm_set_wall_distances.argtypes = [P, P, C.c_int64]
    L.lbm_get_wall_distances.argtypes = [P, P, P]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(rc, h=None):
    if rc != 0:
        L = load()
        msg = (L.lbm_last_error(h) if h else L.lbm_last_global_error()) or b""
        raise LbmError(rc, msg.decode(errors="replace"))


def read_stl(path: str) -> np.ndarray:
    L = load()
    n = C.c_int64(0)
    _check(L.lbm_read_stl_ascii(path.encode(), None, C.byref(n)))
    out = np.zeros((n.value, 12), np.float64)
    _check(L.lbm_read_stl_ascii(path.encode(), _ptr(out), C.byref(n)))
    return out


def voxelize(tri12, spacing, bbox=None, origin=None, dims=None):
    """GPU voxelization; returns (mask[k, j, i] uint8, desc).  Without bbox /
    origin / dims the reference's bounding-box rule is used."""
    L = load()
    tri = np.ascontiguousarray(tri12, np.float64)
    d = VoxDesc()
    d.spacing = spacing
    if bbox is None:
        d.reference_bbox = 1
    else:
        d.reference_bbox = 0
        d.bbox[:] = list(bbox)
        d.origin[:] = list(origin)
        d.dims[:] = list(dims)
    _check(L.lbm_voxelize(_ptr(tri), len(tri), C.byref(d), None))
    nx, ny, nz = d.dims
    mask = np.zeros(nx * ny * nz, np.uint8)
    _check(L.lbm_voxelize(_ptr(tri), len(tri), C.byref(d), _ptr(mask)))
    return mask.reshape(nz, ny, nx), d


def bc_spec(kind, face=0, plane=-1, value=1.0, profile=0, c1=0.0, c2=0.0, R=1.0, region=None, wave=0):
    """Boundary rule.  region=(coord, tol, (lo1, hi1), (lo2, hi2)) selects
    points by coordinates instead of a lattice plane; wave picks the inlet
    waveform of a velocity rule (0: the inlet table)."""
    if isinstance(face, str):
        face = FACES[face]
    b = BCSpec(kind, face, plane, value, profile, c1, c2, R)
    b.wave = wave
    if region is not None:
        coord, tol, (lo1, hi1), (lo2, hi2) = region
        b.region, b.coord, b.tol = 1, coord, tol
        b.lo[:] = [lo1, lo2]
        b.hi[:] = [hi1, hi2]
    return b


class Solver:
    """One device-resident lattice behind the C ABI."""

    def __init__(self, Q=19, precision=LBM_F32, mode=LBM_PHYSICS, tau=0.8, spacing=1.0, origin=(0.0, 0.0, 0.0),
                 wss_scale=1.0, tawss_div=0.9, device=0, collision=0):
        L = load()
        if isinstance(precision, str):
            precision = PRECISIONS[precision]
        d = Desc(Q, precision, mode, tau, spacing, (C.c_double * 3)(*origin), wss_scale, tawss_div, device,
                 collision)
        h = C.c_void_p()
        _check(L.lbm_create(C.byref(d), C.byref(h)))
        self.h = h
        self.Q = Q
        self.precision = precision
        self.mode = mode
        self.dims = None
        self.nbc = 0

    def close(self):
        if getattr(self, "h", None):
            load().lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        _check(rc, self.h)

    def set_geometry(self, mask, bcs=()):
        L = load()
        nz, ny, nx = mask.shape
        self.dims = (nx, ny, nz)
        arr = (BCSpec * max(1, len(bcs)))(*bcs)
        self.nbc = len(bcs)
        m = np.ascontiguousarray(mask.reshape(-1), np.uint8)
        self._c(L.lbm_set_geometry(self.h, m, (C.c_int * 3)(nx, ny, nz), arr, len(bcs)))

    def set_normals(self, tri12):
        t = np.ascontiguousarray(tri12, np.float64)
        self._c(load().lbm_set_normals_from_surface(self.h, t, len(t)))

    def set_normals_box(self, tri12, lo, hi):
        """Normals of the next-to-wall nodes inside lo <= x < hi from these triangles."""
        t = np.ascontiguousarray(tri12, np.float64)
        self._c(load().lbm_set_normals_from_surface_box(self.h, t, len(t), np.asarray(lo, np.float64),
                                                        np.asarray(hi, np.float64)))

    def set_waveform(self, wave, amp):
        a = np.ascontiguousarray(amp, np.float64)
        self._c(load().lbm_set_waveform(self.h, int(wave), a, len(a)))

    def set_inlet_table(self, amp):
        a = np.ascontiguousarray(np.atleast_1d(amp), np.float64)
        self._c(load().lbm_set_inlet_table(self.h, a, len(a)))

    def init_equilibrium(self):
        self._c(load().lbm_init_equilibrium(self.h))

    def init_from_macro_device(self, rho_ptr, u_ptr, regularized=True, stream=0):
        """Warm start from device arrays (nact and 3 * nact FP32) written on `stream`."""
        self._c(load().lbm_init_from_macro_device(self.h, C.c_void_p(rho_ptr), C.c_void_p(u_ptr), int(regularized),
                                                  C.c_void_p(stream)))

    def init_from_macro(self, rho, u, regularized=True):
        self._c(load().lbm_init_from_macro(self.h, np.ascontiguousarray(rho, np.float32),
                                           np.ascontiguousarray(u, np.float32).reshape(-1), int(regularized)))

    def step(self, n=1):
        self._c(load().lbm_step(self.h, int(n)))

    def step_async(self, n=1):
        self._c(load().lbm_step_async(self.h, int(n)))

    def check_status(self):
        self._c(load().lbm_check_status(self.h))

    def sync(self):
        self._c(load().lbm_sync(self.h))

    def set_graph_steps(self, n):
        self._c(load().lbm_set_graph_steps(self.h, int(n)))

    def set_persistent(self, n):
        """Steps per persistent (cooperative, grid-barrier) launch; 0 = one launch per step."""
        self._c(load().lbm_set_persistent(self.h, int(n)))

    def preset_barrier(self, extra_arrivals):
        """Testing: extra arrivals the persistent barrier waits for (see lbm_preset_barrier)."""
        self._c(load().lbm_preset_barrier(self.h, int(extra_arrivals)))

    def preset_flags(self, flags):
        """Testing: the kernel error flags the next step reports (see lbm_preset_flags)."""
        self._c(load().lbm_preset_flags(self.h, int(flags)))

    def autotune(self, trial_steps=10):
        """Time every launch variant on a snapshot of the state; keep the fastest."""
        best = C.c_int()
        ms = (C.c_float * NUM_VARIANTS)()
        self._c(load().lbm_autotune(self.h, int(trial_steps), C.byref(best), ms))
        return best.value, list(ms)

    def set_variant(self, v):
        self._c(load().lbm_set_variant(self.h, int(v)))

    def counts(self) -> dict:
        c = Counts()
        self._c(load().lbm_get_counts(self.h, C.byref(c)))
        d = {k: getattr(c, k) for k, _ in Counts._fields_ if k != "bc"}
        d["bc"] = list(c.bc)[: self.nbc]
        return d

    def classes(self):
        nx, ny, nz = self.dims
        out = np.zeros(nx * ny * nz, np.uint8)
        self._c(load().lbm_get_classes(self.h, out))
        return out.reshape(nz, ny, nx)

    def distributions(self):
        out = np.zeros(self.counts()["active"] * self.Q, np.float64)
        self._c(load().lbm_get_distributions(self.h, out))
        return out.reshape(-1, self.Q)

    def set_distributions(self, f):
        self._c(load().lbm_set_distributions(self.h, np.ascontiguousarray(f, np.float64).reshape(-1)))

    def macro(self):
        n = self.counts()["active"]
        rho, u = np.zeros(n), np.zeros(3 * n)
        self._c(load().lbm_get_macro(self.h, _ptr(rho), _ptr(u)))
        return rho, u.reshape(-1, 3)

    def wss(self) -> dict:
        n = self.counts()["next_to_wall"]
        pt = np.zeros(n, np.int64)
        nrm, w, acc, accm, osi, tawss = (np.zeros(3 * n), np.zeros(n), np.zeros(3 * n), np.zeros(n), np.zeros(n),
                                         np.zeros(n))
        self._c(load().lbm_get_wss(self.h, _ptr(pt), _ptr(nrm), _ptr(w), _ptr(acc), _ptr(accm), _ptr(osi),
                                   _ptr(tawss)))
        return {"pt": pt, "normal": nrm.reshape(-1, 3), "wss": w, "acc": acc.reshape(-1, 3), "acc_mag": accm,
                "osi": osi, "tawss": tawss}

    def set_wall_distances(self, tri12):
        """Interpolated bounce-back (physics mode) with wall distances from
        the surface; an empty array returns to half-way bounce-back."""
        t = np.ascontiguousarray(tri12, np.float64).reshape(-1, 12)
        self._c(load().lbm_set_wall_distances(self.h, _ptr(t) if len(t) else None, len(t)))

    def wall_distances(self):
        """(boundary-list points, wall distance per entry and arriving population [nsp, Q])."""
        n = self.counts()["special"]
        pt = np.zeros(n, np.int64)
        q = np.zeros(n * self.Q, np.float32)
        self._c(load().lbm_get_wall_distances(self.h, _ptr(pt), _ptr(q)))
        return pt, q.reshape(n, self.Q)

    def nearest_next_to_wall(self, xyz, max_radius=32):
        """(index into wss() arrays or -1, physical distance) of the nearest
        next-to-wall node of each point (physical coordinates, n x 3)."""
        p = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        idx = np.zeros(len(p), np.int64)
        dist = np.zeros(len(p), np.float64)
        self._c(load().lbm_nearest_next_to_wall(self.h, _ptr(p), len(p), int(max_radius), _ptr(idx), _ptr(dist)))
        return idx, dist

    def wss_at_points(self, xyz, max_radius=32):
        """WSS, OSI and TAWSS at points (e.g. STL vertices) from their nearest
        next-to-wall node (NaN where none lies within max_radius)."""
        idx, dist = self.nearest_next_to_wall(xyz, max_radius)
        w = self.wss()
        ok = idx >= 0
        out = {"index": idx, "distance": dist}
        for k in ("wss", "osi", "tawss"):
            v = np.full(len(idx), np.nan)
            v[ok] = w[k][idx[ok]]
            out[k] = v
        return out

    def outputs_async(self, rho, u, wss, osi, tawss):
        """Queue the rho/u and WSS/OSI/TAWSS read-outs into the given arrays
        (float64; pinned memory makes the copies asynchronous); they hold
        the values once wait_outputs returns."""
        L = load()
        self._c(L.lbm_get_wss_async(self.h, None, None, _ptr(wss), None, None, _ptr(osi), _ptr(tawss)))
        self._c(L.lbm_get_macro_async(self.h, _ptr(rho), _ptr(u)))

    def wait_outputs(self):
        self._c(load().lbm_wait_outputs(self.h))

    def conservation(self):
        m, p, fl = np.zeros(1), np.zeros(3), np.zeros(MAX_BC)
        self._c(load().lbm_get_conservation(self.h, _ptr(m), _ptr(p), _ptr(fl)))
        return float(m[0]), p, fl[: self.nbc]

    def save(self, path):
        self._c(load().lbm_save(self.h, path.encode()))

    def load_checkpoint(self, path):
        self._c(load().lbm_load(self.h, path.encode()))

    def stream(self) -> int:
        s = C.c_void_p()
        self._c(load().lbm_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def launches(self) -> int:
        n = C.c_int64()
        self._c(load().lbm_get_launch_count(self.h, C.byref(n)))
        return n.value
