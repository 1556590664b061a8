"""lbm_moment_sums_noalloc -- the entry point for callers that cannot allocate.

Callers that run inside CUDA graph capture, real-time loops with memory
fixed up-front, or frameworks whose pool allocator owns the device cannot
call cudaMalloc; this entry point sums mass and momentum of distributions in
caller-owned device memory with its scratch in a fixed array inside the
library.  Here the test plays the caller: it owns the device buffers
(allocated through the CUDA runtime) and checks two calls in a row against
lbm_get_conservation of the same state.  This file is collected last so
that a run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import fixtures, load, sim_bcs

pytestmark = pytest.mark.gpu

MAX_NODES = 4194304


def _cudart():
    rt = C.CDLL("libcudart.so.13")
    for n in ("cudaMalloc", "cudaFree", "cudaMemcpy", "cudaMemset", "cudaDeviceSynchronize"):
        getattr(rt, n).restype = C.c_int
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
    return rt


def _sums(L, rt, d_f, nact, Q, d_out):
    assert rt.cudaMemset(d_out, 0xFF, 4 * 8) == 0  # poison the output
    assert L.lbm_moment_sums_noalloc(d_f, nact, Q, d_out, None) == 0, L.lbm_last_global_error()
    assert rt.cudaDeviceSynchronize() == 0
    out = np.zeros(4)
    assert rt.cudaMemcpy(out.ctypes.data, d_out, 4 * 8, 2) == 0  # device to host
    return out


@pytest.mark.parametrize("Q", [19, 27])
def test_noalloc_sums_match_conservation(gpu_lib, Q):
    """Two calls in a row on the same caller-owned state (D3Q19 parity run of
    a golden case, D3Q27 physics run of the same vessel) against
    lbm_get_conservation; then a size beyond the fixed scratch."""
    capi = gpu_lib
    L = capi.load()
    d = load(fixtures("sim")[0])
    mask, desc = capi.voxelize(d["tri12"], float(d["spacing"]))
    mode = capi.LBM_PARITY if Q == 19 else capi.LBM_PHYSICS
    s = capi.Solver(Q, capi.LBM_F64, mode, float(d["tau"]), float(d["spacing"]))
    s.set_geometry(mask, [capi.bc_spec(**spec) for _, spec in sim_bcs(d)])
    s.set_inlet_table(d["amp"])
    s.step(int(d["nsteps"]))
    mass, mom, _ = s.conservation()
    f = np.ascontiguousarray(s.distributions())
    nact = f.shape[0]
    assert f.shape[1] == Q

    rt = _cudart()
    d_f, d_out = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(d_f), f.nbytes) == 0
    assert rt.cudaMalloc(C.byref(d_out), 4 * 8) == 0
    try:
        assert rt.cudaMemcpy(d_f, f.ctypes.data, f.nbytes, 1) == 0  # host to device
        for call in range(2):
            out = _sums(L, rt, d_f, nact, Q, d_out)
            np.testing.assert_allclose(out[0], mass, rtol=1e-12)
            np.testing.assert_allclose(out[1:], mom, rtol=1e-9, atol=1e-12 * mass)
        # beyond the fixed scratch: a clear error, not a fault
        rc = L.lbm_moment_sums_noalloc(d_f, MAX_NODES + 1, Q, d_out, None)
        assert rc == -1
        assert b"4194304" in L.lbm_last_global_error()
    finally:
        rt.cudaFree(d_f)
        rt.cudaFree(d_out)


def test_noalloc_sums_of_no_nodes(gpu_lib):
    """nact = 0: no partial sums, the final sum reads none; twice in a row,
    after a call on real data left the scratch full."""
    L = gpu_lib.load()
    rt = _cudart()
    d_f, d_out = C.c_void_p(), C.c_void_p()
    f = np.full((300, 19), 1.0 / 19.0)
    assert rt.cudaMalloc(C.byref(d_f), f.nbytes) == 0
    assert rt.cudaMalloc(C.byref(d_out), 4 * 8) == 0
    try:
        assert rt.cudaMemcpy(d_f, f.ctypes.data, f.nbytes, 1) == 0
        full = _sums(L, rt, d_f, 300, 19, d_out)
        np.testing.assert_allclose(full[0], 300.0, rtol=1e-14)
        for call in range(2):
            out = _sums(L, rt, None, 0, 19, d_out)
            assert np.array_equal(out, np.zeros(4))
    finally:
        rt.cudaFree(d_f)
        rt.cudaFree(d_out)
