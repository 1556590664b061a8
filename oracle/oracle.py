"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle (``lbm_oracle.c``) restates the reference's hot path on the CPU in
FP64.  Only the tests, the smoke check and the CPU-baseline leg of
``bench.py`` use it, always as the checker.  ``build()`` compiles it with the
Makefile beside this file; ``run_reference_harness`` drives the reference's
own sources compiled unchanged (``make -C oracle ref``) when they are present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblbm_oracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

PARITY, PHYSICS = 0, 1
BC_REF_INLET, BC_REF_OUTLET_YMAX, BC_REF_OUTLET_ZMIN, BC_VELOCITY, BC_PRESSURE = 1, 2, 3, 4, 5
FACES = {"x-": 0, "x+": 1, "y-": 2, "y+": 3, "z-": 4, "z+": 5}


class OracleBC(C.Structure):
    _fields_ = [("kind", C.c_int), ("face", C.c_int), ("value", C.c_double), ("profile", C.c_int),
                ("c1", C.c_double), ("c2", C.c_double), ("R", C.c_double)]


_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = np.ctypeslib.ndpointer
        d, i64, u8, i32 = np.float64, np.int64, np.uint8, np.int32
        L.oracle_lattice.argtypes = [C.c_int, P(i32), P(d), P(i32)]
        L.oracle_bbox_dims.argtypes = [P(d), C.c_int64, C.c_double, P(d), P(i32)]
        L.oracle_voxelize.argtypes = [P(d), C.c_int64, P(d), P(d), C.c_double, P(i32), P(u8), C.c_int, C.c_int]
        L.oracle_voxelize.restype = C.c_int64
        L.oracle_cull_margin.argtypes = [P(d), C.c_double]
        L.oracle_cull_margin.restype = C.c_double
        L.oracle_find_boundary.argtypes = [P(u8), P(i32), C.c_int, P(u8)]
        L.oracle_find_boundary.restype = C.c_int64
        L.oracle_sim_create.argtypes = [C.c_int, C.c_int, P(i32), P(u8), P(d), C.c_double, C.c_double,
                                        C.POINTER(OracleBC), C.c_int]
        L.oracle_sim_create.restype = C.c_void_p
        L.oracle_sim_destroy.argtypes = [C.c_void_p]
        L.oracle_sim_set_amplitude.argtypes = [C.c_void_p, P(d), C.c_int64]
        L.oracle_sim_set_wss.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.oracle_sim_compute_normals.argtypes = [C.c_void_p, P(d), C.c_int64, C.c_int]
        L.oracle_sim_step.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_sim_set_collision.argtypes = [C.c_void_p, C.c_int]
        L.oracle_sim_set_wall_distances.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.float64), C.c_int64]
        L.oracle_sim_get_wall_distances.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.float32)]
        L.oracle_sim_nactive.argtypes = [C.c_void_p]
        L.oracle_sim_nactive.restype = C.c_int64
        L.oracle_sim_nnw.argtypes = [C.c_void_p]
        L.oracle_sim_nnw.restype = C.c_int64
        L.oracle_sim_get_active.argtypes = [C.c_void_p, P(i64), P(u8)]
        L.oracle_sim_get_f.argtypes = [C.c_void_p, P(d), P(d), P(d)]
        L.oracle_sim_set_f.argtypes = [C.c_void_p, P(d)]
        L.oracle_sim_get_macro.argtypes = [C.c_void_p, P(d), P(d)]
        L.oracle_sim_get_nw.argtypes = [C.c_void_p, P(i64), P(d), P(d), P(d), P(d), P(d), P(d)]
        L.oracle_sim_get_wall_normals.argtypes = [C.c_void_p, P(i64), P(d)]
        L.oracle_sim_conservation.argtypes = [C.c_void_p, P(d), P(d), P(d)]
        _lib = L
    return _lib


def lattice(Q: int):
    c = np.zeros(Q * 3, np.int32)
    w = np.zeros(Q, np.float64)
    opp = np.zeros(Q, np.int32)
    assert lib().oracle_lattice(Q, c, w, opp) == 0
    return c.reshape(Q, 3), w, opp


def bbox_dims(tri12: np.ndarray, spacing: float):
    bb = np.zeros(6)
    dims = np.zeros(3, np.int32)
    lib().oracle_bbox_dims(np.ascontiguousarray(tri12, np.float64), len(tri12), spacing, bb, dims)
    return bb, tuple(int(v) for v in dims)


def voxelize(tri12, spacing, bbox=None, origin=None, dims=None, culled=True, nthreads=0):
    """Mask laid out [k, j, i] (x fastest), 1 = Fluid."""
    tri = np.ascontiguousarray(tri12, np.float64)
    bb, d = bbox_dims(tri, spacing)
    if bbox is not None:
        bb = np.asarray(bbox, np.float64)
    if dims is not None:
        d = tuple(dims)
    org = np.asarray(origin if origin is not None else (bb[0], bb[2], bb[4]), np.float64)
    mask = np.zeros(d[0] * d[1] * d[2], np.uint8)
    lib().oracle_voxelize(tri, len(tri), bb, org, spacing, np.asarray(d, np.int32), mask, int(culled), nthreads)
    return mask.reshape(d[2], d[1], d[0]), bb, d


def cull_margin(tri_row, zspan):
    return lib().oracle_cull_margin(np.ascontiguousarray(tri_row, np.float64), zspan)


def find_boundary(mask: np.ndarray, Q: int = 19) -> np.ndarray:
    nz, ny, nx = mask.shape
    out = np.zeros(mask.size, np.uint8)
    lib().oracle_find_boundary(np.ascontiguousarray(mask.reshape(-1), np.uint8),
                               np.array([nx, ny, nz], np.int32), Q, out)
    return out.reshape(mask.shape)


class Sim:
    """FP64 oracle solver over a class array cls[k, j, i] (0 solid, 1 fluid, 2 wall, 3+b bc[b])."""

    def __init__(self, Q, mode, cls, origin, spacing, tau, bcs):
        self.Q = Q
        nz, ny, nx = cls.shape
        self.dims = (nx, ny, nz)
        arr = (OracleBC * max(1, len(bcs)))()
        for b, spec in enumerate(bcs):
            arr[b] = OracleBC(spec.get("kind", BC_VELOCITY), spec.get("face", 0), spec.get("value", 1.0),
                              spec.get("profile", 0), spec.get("c1", 0.0), spec.get("c2", 0.0),
                              spec.get("R", 1.0))
        self.h = lib().oracle_sim_create(Q, mode, np.array(self.dims, np.int32),
                                         np.ascontiguousarray(cls.reshape(-1), np.uint8),
                                         np.asarray(origin, np.float64), spacing, tau, arr, len(bcs))
        if not self.h:
            raise ValueError("oracle_sim_create failed")
        self.nbc = len(bcs)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_sim_destroy(self.h)
            self.h = None

    def set_amplitude(self, amp):
        a = np.ascontiguousarray(np.atleast_1d(amp), np.float64)
        lib().oracle_sim_set_amplitude(self.h, a, len(a))

    def set_wss(self, C, tawss_div):
        lib().oracle_sim_set_wss(self.h, C, tawss_div)

    def compute_normals(self, tri12, nthreads=0):
        t = np.ascontiguousarray(tri12, np.float64)
        lib().oracle_sim_compute_normals(self.h, t, len(t), nthreads)

    def step(self, n=1, nthreads=0):
        lib().oracle_sim_step(self.h, n, nthreads)

    def set_collision(self, regularized):
        """Physics mode: regularized collision (True) or BGK (False)."""
        lib().oracle_sim_set_collision(self.h, int(bool(regularized)))

    def set_wall_distances(self, tri12):
        """Physics mode: interpolated bounce-back with wall distances from
        the triangles (an empty array: half-way bounce-back)."""
        t = np.ascontiguousarray(tri12, np.float64).reshape(-1, 12)
        lib().oracle_sim_set_wall_distances(self.h, t if len(t) else np.zeros((1, 12)), len(t))

    def wall_distances(self):
        """Wall distance per (active node, arriving population), [nact, Q]."""
        q = np.zeros(self.nactive * self.Q, np.float32)
        lib().oracle_sim_get_wall_distances(self.h, q)
        return q.reshape(-1, self.Q)

    @property
    def nactive(self):
        return lib().oracle_sim_nactive(self.h)

    @property
    def nnw(self):
        return lib().oracle_sim_nnw(self.h)

    def active(self):
        pt = np.zeros(self.nactive, np.int64)
        cl = np.zeros(self.nactive, np.uint8)
        lib().oracle_sim_get_active(self.h, pt, cl)
        return pt, cl

    def f(self):
        n = self.nactive * self.Q
        f, fn, fe = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().oracle_sim_get_f(self.h, f, fn, fe)
        return f.reshape(-1, self.Q), fn.reshape(-1, self.Q), fe.reshape(-1, self.Q)

    def set_f(self, f):
        lib().oracle_sim_set_f(self.h, np.ascontiguousarray(f, np.float64).reshape(-1))

    def macro(self):
        r, u = np.zeros(self.nactive), np.zeros(3 * self.nactive)
        lib().oracle_sim_get_macro(self.h, r, u)
        return r, u.reshape(-1, 3)

    def nw(self):
        n = self.nnw
        pt = np.zeros(n, np.int64)
        nrm, wss, acc, accm, osi, tawss = (np.zeros(3 * n), np.zeros(n), np.zeros(3 * n), np.zeros(n),
                                            np.zeros(n), np.zeros(n))
        lib().oracle_sim_get_nw(self.h, pt, nrm, wss, acc, accm, osi, tawss)
        return {"pt": pt, "normal": nrm.reshape(-1, 3), "wss": wss, "acc": acc.reshape(-1, 3),
                "acc_mag": accm, "osi": osi, "tawss": tawss}

    def conservation(self):
        m, p, fl = np.zeros(1), np.zeros(3), np.zeros(max(1, self.nbc))
        lib().oracle_sim_conservation(self.h, m, p, fl)
        return float(m[0]), p, fl[: self.nbc]


# ---------------------------------------------------------------------------
# the reference's own sources (compiled unchanged) as the pinning oracle

def reference_available() -> bool:
    return os.path.exists(REF_HARNESS)


def reference_dir() -> str:
    """Where the reference's sources are read from: $LBM_REFERENCE_DIR, else
    the default the Makefile beside this file gives its REF variable."""
    env = os.environ.get("LBM_REFERENCE_DIR")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as fh:
        for line in fh:
            if line.startswith("REF ?="):
                return line.split("=", 1)[1].strip()
    return ""


def build_reference(ref_dir: str | None = None) -> bool:
    ref_dir = ref_dir or reference_dir()
    if not ref_dir or not os.path.isdir(ref_dir):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_dir}", "-j8"], check=True)
    return os.path.exists(REF_HARNESS)


def read_ref_vox(path):
    b = open(path, "rb").read()
    h = np.frombuffer(b[:16], np.int32)
    nx, ny, nz = (int(v) for v in h[1:4])
    off = 16
    bb = np.frombuffer(b[off:off + 48], np.float64).copy(); off += 48
    ntri = int(np.frombuffer(b[off:off + 8], np.int64)[0]); off += 8
    secs = float(np.frombuffer(b[off:off + 8], np.float64)[0]); off += 8
    mask = np.frombuffer(b[off:off + nx * ny * nz], np.uint8).reshape(nz, ny, nx).copy(); off += nx * ny * nz
    nb = int(np.frombuffer(b[off:off + 8], np.int64)[0]); off += 8
    bidx = np.frombuffer(b[off:off + 12 * nb], np.int32).reshape(nb, 3).copy()
    return {"dims": (nx, ny, nz), "bbox": bb, "ntri": ntri, "seconds": secs, "mask": mask, "boundary_ijk": bidx}


def read_ref_sim(path):
    b = open(path, "rb").read()
    h = np.frombuffer(b[:24], np.int32)
    nx, ny, nz, Q, nsteps = (int(v) for v in h[1:6])
    off = 24
    setup_s, step_s = np.frombuffer(b[off:off + 16], np.float64); off += 16
    na = int(np.frombuffer(b[off:off + 8], np.int64)[0]); off += 8
    rec = np.dtype([("ijk", np.int32, 3), ("type", np.int32), ("f", np.float64, Q), ("fnew", np.float64, Q),
                    ("feq", np.float64, Q), ("rho", np.float64), ("u", np.float64, 3)])
    act = np.frombuffer(b[off:off + rec.itemsize * na], rec).copy(); off += rec.itemsize * na
    nn = int(np.frombuffer(b[off:off + 8], np.int64)[0]); off += 8
    rec2 = np.dtype([("ijk", np.int32, 3), ("normal", np.float64, 3), ("wss", np.float64), ("acc", np.float64, 3),
                     ("acc_mag", np.float64), ("osi", np.float64), ("tawss", np.float64)])
    nw = np.frombuffer(b[off:off + rec2.itemsize * nn], rec2).copy(); off += rec2.itemsize * nn
    nwl = int(np.frombuffer(b[off:off + 8], np.int64)[0]); off += 8
    rec3 = np.dtype([("ijk", np.int32, 3), ("normal", np.float64, 3)])
    wall = np.frombuffer(b[off:off + rec3.itemsize * nwl], rec3).copy()
    return {"dims": (nx, ny, nz), "Q": Q, "nsteps": nsteps, "setup_s": float(setup_s), "step_s": float(step_s),
            "active": act, "nw": nw, "wall": wall}


def run_reference_vox(stl, spacing, out):
    subprocess.run([REF_HARNESS, "vox", stl, repr(float(spacing)), out], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return read_ref_vox(out)


def run_reference_sim(stl, spacing, bc_txt, tau, dt, nsteps, inlet_txt, out):
    subprocess.run([REF_HARNESS, "sim", stl, repr(float(spacing)), bc_txt, repr(float(tau)), repr(float(dt)),
                    str(nsteps), inlet_txt, out], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return read_ref_sim(out)
