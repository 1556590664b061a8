"""The bounds-checked build (-DLBM_CHECK) and the step kernels' error flags.

* The host's handling of the bounds flag, without any invalid access: the
  flag is preset through lbm_preset_flags, the next step reports it with
  the library's message and clears it, and stepping continues.
* The checked library (pv_dec_original_gb300.build.build_checked), bound in
  a child process through LBM_LIBRARY, steps every kernel family on real
  cases -- the flat and compact kernels, FP64 parity, FP32 / FP16 physics,
  interpolated walls, persistent launches -- with no index outside its array
  and results bit-identical to the normal build (the checks do not change
  the arithmetic).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from pv_dec_original_gb300 import capi, geometry as G
from helpers import fixtures, load, sim_bcs, wss_C
capi.load(build_if_missing=False)
out = {{}}
d = load(fixtures("sim")[0])
mask, desc = capi.voxelize(d["tri12"], float(d["spacing"]))
bb = np.array(desc.bbox[:])
s = capi.Solver(19, capi.LBM_F64, capi.LBM_PARITY, float(d["tau"]), float(d["spacing"]), (bb[0], bb[2], bb[4]),
                wss_C(float(d["dt"]), float(d["spacing"])), 0.9)
s.set_geometry(mask, [capi.bc_spec(**spec) for _, spec in sim_bcs(d)])
s.set_normals(d["tri12"]); s.set_inlet_table(d["amp"]); s.step(int(d["nsteps"]))
out["parity_f64"] = s.distributions(); s.close()
surf = G.stenosed_tube(6.0, 60.0, 0.5, 0.25, center=(8.3, 8.1), z0=1.6, h=1.4, seed=5)
surf = G.add_bbox_anchors(surf, (0.0, 0.0, 0.0), (17.0, 17.0, 64.0))
tri = surf.tri12()
mask, desc = capi.voxelize(tri, 1.0)
bb = np.array(desc.bbox[:])
fl = np.argwhere(mask > 0)
kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
for prec in ("f32", "f16"):
    for v in (0, 6, 7):
        for walls in (False, True):
            if walls and v:
                continue
            s = capi.Solver(19, prec, capi.LBM_PHYSICS, 0.6, 1.0, (bb[0], bb[2], bb[4]), 1.0, 1.0)
            s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, 8.3, 8.1, 6.0),
                                  capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
            s.set_normals(tri); s.set_inlet_table([0.04])
            if walls:
                s.set_wall_distances(tri)
            s.set_variant(v); s.step(24)
            out[f"{{prec}}_v{{v}}_w{{int(walls)}}"] = s.distributions()
            if v == 0 and not walls:
                s.set_persistent(8); s.step(16)
                out[f"{{prec}}_persistent"] = s.distributions()
            s.close()
np.savez({path!r}, **out)
"""


def _child(lib, path):
    env = dict(os.environ)
    if lib:
        env["LBM_LIBRARY"] = lib
    code = CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), path=path)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return dict(np.load(path))


def test_bounds_flag_reported_and_cleared(gpu_lib):
    capi = gpu_lib
    mask = np.zeros((8, 6, 6), np.uint8)
    mask[1:7, 1:5, 1:5] = 1
    s = capi.Solver(19, "f32", capi.LBM_PHYSICS, 0.8, 1.0, (0.0, 0.0, 0.0), 1.0, 1.0)
    s.set_geometry(mask)
    s.step(2)
    s.preset_flags(capi.LBM_FLAG_BOUNDS)
    with pytest.raises(capi.LbmError) as e:
        s.step(1)
    assert "outside its array" in str(e.value)
    s.step(3)  # the flag was cleared
    with pytest.raises(capi.LbmError):
        s.preset_flags(8)  # only the non-finite and bounds flags can be preset
    s.close()


def test_checked_build_runs_clean_and_bit_identical(gpu_lib, tmp_path):
    from pv_dec_original_gb300 import build
    lib = build.build_checked()
    plain = _child(None, str(tmp_path / "plain.npz"))
    checked = _child(lib, str(tmp_path / "checked.npz"))
    assert set(plain) == set(checked) and len(plain) >= 8
    for k in plain:
        assert np.array_equal(plain[k], checked[k]), k
