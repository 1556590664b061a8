"""The C ABI library: loads, exports every declared symbol, host-side paths
work without a GPU (no compute calls here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from helpers import fixtures, load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header=None):
    """Entry points declared in include/*.h (or in one header)."""
    inc = os.path.join(ROOT, "include")
    names = [header] if header else sorted(f for f in os.listdir(inc) if f.endswith(".h"))
    out = set()
    for h in names:
        txt = open(os.path.join(inc, h)).read()
        out |= set(re.findall(r"^(?:lbm_status|const char\*)\s+(lbm_\w+)\s*\(", txt, re.M))
    return sorted(out)


def test_python_binding_constants_match_header():
    """The ctypes binding mirrors the header's constants; a stale mirror of
    LBM_NUM_VARIANTS sizes lbm_autotune's output array too small."""
    from pv_dec_original_gb300 import capi
    txt = "".join(open(os.path.join(ROOT, "include", f)).read() for f in ("lbm_gb300.h", "lbm_nn.h"))
    h = {k: int(v) for k, v in re.findall(r"#define\s+(LBM_\w+)\s+(-?\d+)", txt)}
    mirror = {"LBM_NUM_VARIANTS": capi.NUM_VARIANTS, "LBM_MAX_BC": capi.MAX_BC, "LBM_MAX_WAVES": capi.MAX_WAVES}
    for k in ("LBM_F64", "LBM_F32", "LBM_F16", "LBM_BF16", "LBM_PARITY", "LBM_PHYSICS", "LBM_BC_REF_INLET",
              "LBM_BC_REF_OUTLET_YMAX", "LBM_BC_REF_OUTLET_ZMIN", "LBM_BC_VELOCITY", "LBM_BC_PRESSURE",
              "LBM_COLLISION_BGK", "LBM_COLLISION_REGULARIZED", "LBM_FLAG_NONFINITE", "LBM_FLAG_BOUNDS",
              "LBM_NN_ENGINE_AUTO", "LBM_NN_ENGINE_MMA_SYNC"):
        mirror[k] = getattr(capi, k)
    for face, v in capi.FACES.items():
        mirror["LBM_FACE_" + {"x": "X", "y": "Y", "z": "Z"}[face[0]] + ("MIN" if face[1] == "-" else "MAX")] = v
    for k, v in mirror.items():
        assert h[k] == v, (k, h[k], v)


def test_library_exports_every_declared_symbol(gpu_lib):
    """Every entry point of include/lbm_gb300.h and include/lbm_nn.h is
    exported by the library and bound by the Python layer."""
    L = gpu_lib.load()
    syms = declared_symbols()
    assert len(declared_symbols("lbm_gb300.h")) >= 20 and len(declared_symbols("lbm_nn.h")) >= 14
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    unbound = [s for s in syms if s not in gpu_lib.EXPORTS]
    assert not unbound, unbound


def test_errors_are_status_codes_not_crashes(gpu_lib):
    L = gpu_lib.load()
    bad = gpu_lib.Desc(19, 1, 1, 0.4, 1.0, (C.c_double * 3)(0, 0, 0), 1.0, 0.9, 0)  # tau <= 0.5
    h = C.c_void_p()
    assert L.lbm_create(C.byref(bad), C.byref(h)) == -1
    assert b"tau" in L.lbm_last_global_error()
    assert L.lbm_step(None, 1) == -1
    assert L.lbm_destroy(None) == 0


def test_convolutions_refuse_misaligned_tensors(gpu_lib):
    """The convolution entry points check their arguments on the host before
    any device call: a tensor address that is not 16-byte aligned (the
    tensor-core kernels copy 16-byte rows and tensor-map boxes) is an
    argument error, never a launch."""
    L = gpu_lib.load()
    dims = (C.c_int * 3)(8, 16, 8)
    good, odd = C.c_void_p(1 << 20), C.c_void_p((1 << 20) + 8)
    assert L.lbm_nn_conv3d_fwd(odd, dims, 16, good, None, 16, 3, 1, 0, good, None, None) == -1
    assert b"invalid argument" in L.lbm_last_global_error()
    assert L.lbm_nn_conv3d_fwd(good, dims, 16, odd, None, 16, 3, 1, 0, good, None, None) == -1
    assert L.lbm_nn_conv3d_fwd(good, dims, 16, good, None, 16, 3, 1, 0, good, odd, None) == -1
    assert L.lbm_nn_conv3d_bwd(good, dims, 16, good, good, 16, 3, 1, odd, None, None, None, None) == -1
    assert L.lbm_nn_conv3d_bwd(good, dims, 16, good, good, 16, 3, 1, good, odd, None, None, None) == -1


def test_stl_reader_matches_python_parser(gpu_lib, tmp_path):
    from pv_dec_original_gb300 import geometry as G
    d = load(fixtures("vox")[0])
    tri = d["tri12"]
    p = str(tmp_path / "x.stl")
    G.write_stl_ascii(p, G.Surface(tri[:, :9].reshape(-1, 3, 3).copy(), tri[:, 9:].copy()))
    got = gpu_lib.read_stl(p)
    assert np.array_equal(got, tri)
    assert np.array_equal(G.read_stl_ascii(p), tri)


def test_stl_reader_skips_malformed_facets(gpu_lib, tmp_path):
    p = tmp_path / "bad.stl"
    p.write_text("solid a\n facet normal 0 0 1\n outer loop\n vertex 0 0 0\n vertex 1 0 0\n vertex 0 1 0\n"
                 " endloop\n endfacet\n facet normal 0 0 1\n outer loop\n vertex 0 0\n endloop\n endfacet\n"
                 " facet normal x y z\nendsolid\n")
    got = gpu_lib.read_stl(str(p))
    assert got.shape == (1, 12)
    with pytest.raises(gpu_lib.LbmError):
        gpu_lib.read_stl(str(tmp_path / "missing.stl"))


@pytest.mark.parametrize("path", fixtures("vox"), ids=lambda p: p.split("/")[-1])
def test_reference_bbox_rule_on_host(gpu_lib, path):
    """lbm_voxelize with no mask buffer only sizes the lattice (host code)."""
    d = load(path)
    L = gpu_lib.load()
    desc = gpu_lib.VoxDesc()
    desc.spacing = float(d["spacing"])
    desc.reference_bbox = 1
    tri = np.ascontiguousarray(d["tri12"])
    assert L.lbm_voxelize(tri.ctypes.data_as(C.c_void_p), len(tri), C.byref(desc), None) == 0
    assert tuple(desc.dims) == tuple(d["dims"])
    assert np.array_equal(np.array(desc.bbox[:]), d["bbox"])
