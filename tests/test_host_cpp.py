"""The C++ host layer (reference class names over the C ABI)."""
import os
import subprocess

import numpy as np
import pytest

from helpers import GOLDEN, fixtures, load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "pv_dec_original_gb300", "_build")
HOST_INC = os.path.join(ROOT, "pv_dec_original_gb300", "csrc", "host")


def _compile(tmp_path, src, name):
    from pv_dec_original_gb300 import build
    build.build()
    exe = str(tmp_path / name)
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I",
                    HOST_INC, src, "-o", exe, f"-L{BUILD}", "-llbm_host", "-llbm_gb300", f"-Wl,-rpath,{BUILD}"],
                   check=True)
    return exe


def test_host_layer_cpu(tmp_path, oracle_lib):
    exe = _compile(tmp_path, os.path.join(ROOT, "tests", "cpp", "host_cpu_test.cpp"), "host_cpu_test")
    cfg = tmp_path / "c.cfg"
    cfg.write_text("# comment\nspacing 0.05\ntau 1.5\n\ndt 8e-6\nConditions: inlet\nu = 1\nEquation\n")
    out = subprocess.run([exe, str(cfg)], capture_output=True, text=True, check=True).stdout.split("\n")
    kv = [l.split() for l in out if l]
    assert ["config_ok", "0"] in kv  # "Conditions: inlet" is not numeric -> the read fails, as the reference's
    cfg.write_text("# comment\nspacing 0.05\ntau 1.5\n\ndt 8e-6\n")
    out = subprocess.run([exe, str(cfg)], capture_output=True, text=True, check=True).stdout.split("\n")
    kv = [l.split() for l in out if l]
    conf = {k[1]: float(k[2]) for k in kv if k[0] == "config"}
    assert conf == {"spacing": 0.05, "tau": 1.5, "dt": 8e-6}
    for Q in (19, 27):
        c, w, opp = oracle_lib.lattice(Q)
        rows = [k for k in kv if k[0] == "lattice" and int(k[1]) == Q]
        assert len(rows) == Q
        for r in rows:
            q = int(r[2])
            assert [int(r[3]), int(r[4]), int(r[5])] == list(c[q])
            assert float(r[6]) == w[q] and int(r[7]) == opp[q]
        assert [int(k[2]) for k in kv if k[0] == "unknowns" and int(k[1]) == Q] == [5 if Q == 19 else 9] * 6
    d = load(os.path.join(GOLDEN, "pulse.npz"))
    pulse = {int(k[1]): float(k[2]) for k in kv if k[0] == "pulse"}
    got = np.array([pulse[int(i)] for i in d["idx"]])
    np.testing.assert_allclose(got, d["v"], rtol=1e-14, atol=1e-15)


@pytest.mark.gpu
def test_lbm_run_end_to_end_vs_oracle(tmp_path, gpu_lib, oracle_lib):
    """lbm_run (the reference's driver on the GPU engine) on a golden elbow:
    FP64 parity with a velocity inlet and a density outlet; the CSV output
    matches the oracle run with the same inlet table."""
    from pv_dec_original_gb300 import build, geometry as G, waveform
    from helpers import classify
    build.build()
    d = load(fixtures("sim")[0])
    tri = d["tri12"]
    stl = str(tmp_path / "e.stl")
    G.write_stl_ascii(stl, G.Surface(tri[:, :9].reshape(-1, 3, 3).copy(), tri[:, 9:].copy()))
    dt, end = 8e-6, 8e-6 * 30.5   # 31 iterations (t = 0 .. 30 dt)
    cfg = tmp_path / "run.cfg"
    cfg.write_text(f"stl {stl}\nspacing 1.0\ntau 0.8\ndt {dt!r}\nend_time {end!r}\noutput_every 30\n"
                   f"output_dir {tmp_path}\nprecision 0\nmode 0\ninlet_face 0\ninlet_plane -1\n"
                   f"outlet_face 4\noutlet_plane -1\nwrite_vertices 1\n")
    r = subprocess.run([os.path.join(BUILD, "lbm_run"), str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "steps 31" in r.stdout
    csv = np.loadtxt(str(tmp_path / "FlowHemodynamics" / "30_FlowHemodynamics.csv"), delimiter=",", skiprows=1)
    assert (tmp_path / "Fluid_Variables" / "30.vtu").exists()
    mask, bb, dims = oracle_lib.voxelize(tri, 1.0)
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 2].min()), int(fl[:, 0].min())
    bcs = [dict(kind=oracle_lib.BC_VELOCITY, face=0, plane=kin, value=1.0),
           dict(kind=oracle_lib.BC_PRESSURE, face=4, plane=kout, value=1.0)]
    cls = classify(mask, [(0, kin), (2, kout)])
    o = oracle_lib.Sim(19, oracle_lib.PARITY, cls, (bb[0], bb[2], bb[4]), 1.0, 0.8, bcs)
    o.set_amplitude(waveform.reference_table(dt, 31))
    o.set_wss(1060.0 * (dt * dt) / ((1.0 * 1.0) * 1e-6), 0.9)
    o.compute_normals(tri)
    o.step(31)
    nw = o.nw()
    assert len(csv) == len(nw["pt"])
    np.testing.assert_allclose(csv[:, 3], nw["wss"], rtol=2e-5, atol=1e-12)
    np.testing.assert_allclose(csv[:, 5], nw["tawss"], rtol=2e-5, atol=1e-12)
    # the STL-vertex read-out: each vertex takes its nearest next-to-wall node's values
    vx = np.loadtxt(str(tmp_path / "STL_Vertices" / "30_Vertices.csv"), delimiter=",", skiprows=1)
    assert len(vx) == 3 * len(tri)
    verts = tri[:, :9].reshape(-1, 3)
    np.testing.assert_allclose(vx[:, :3], verts, rtol=1e-5, atol=1e-5)  # the CSV prints 6 digits
    nx_, ny_, _ = dims
    pt = np.asarray(nw["pt"])
    ijk = np.stack([pt % nx_, (pt // nx_) % ny_, pt // (nx_ * ny_)], 1).astype(np.float64)
    g = (verts - np.array([bb[0], bb[2], bb[4]])) / 1.0
    near = np.argmin(((ijk[None] - g[:, None]) ** 2).sum(-1), 1)
    np.testing.assert_array_equal(vx[:, 3], csv[near, 3])
    np.testing.assert_array_equal(vx[:, 5], csv[near, 5])
    _check_vtu(str(tmp_path / "Fluid_Variables" / "30.vtu"), mask, o)


def _vtu_arrays(path):
    """DataArray name -> (values, components) of an ASCII .vtu file."""
    import re
    txt = open(path).read()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)"([^>]*)>(.*?)</DataArray>', txt, re.S):
        typ, attrs, body = m.groups()
        name = re.search(r'Name="(\w+)"', attrs)
        comp = re.search(r'NumberOfComponents="(\d+)"', attrs)
        key = name.group(1) if name else "Points"
        dt = np.float64 if typ.startswith("Float") else np.int64
        out[key] = (np.array(body.split(), dtype=dt), int(comp.group(1)) if comp else 1)
    piece = re.search(r'NumberOfPoints="(\d+)" NumberOfCells="(\d+)"', txt)
    return out, int(piece.group(1)), int(piece.group(2))


def _check_vtu(path, mask, oracle_sim):
    """The .vtu against the layout of WriteVTK_Collective
    (OutputFile.cpp:259-429): every active node in point order (x fastest)
    at its integer lattice coordinates; a hexahedron (type 12) for every
    lattice cube whose eight corners are active, cubes in z, y, x loop order,
    corners (x,y,z) (x+1,y,z) (x+1,y+1,z) (x,y+1,z) then the same at z+1;
    point fields Velocity, Density and VelocityMagnitude -- here of the
    post-boundary distributions (the oracle's f after the same steps)."""
    arr, npts, ncell = _vtu_arrays(path)
    nz, ny, nx = mask.shape
    act = np.flatnonzero(mask.reshape(-1) > 0)
    assert npts == len(act)
    pts = arr["Points"][0].reshape(-1, 3)
    ijk = np.stack([act % nx, (act // nx) % ny, act // (nx * ny)], 1)
    np.testing.assert_array_equal(pts, ijk)
    pid = np.full(mask.size, -1, np.int64)
    pid[act] = np.arange(len(act))
    pid = pid.reshape(nz, ny, nx)
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    ids = np.stack([pid[dz:nz - 1 + dz, dy:ny - 1 + dy, dx:nx - 1 + dx] for dx, dy, dz in corners], -1)
    cells = ids[(ids >= 0).all(-1)]  # z, y, x order of the cube loop
    assert ncell == len(cells)
    np.testing.assert_array_equal(arr["connectivity"][0].reshape(-1, 8), cells)
    np.testing.assert_array_equal(arr["offsets"][0], 8 * np.arange(1, ncell + 1))
    assert np.all(arr["types"][0] == 12)
    f, _, _ = oracle_sim.f()
    from oracle import oracle as O
    c, _, _ = O.lattice(19)
    rho = f.sum(axis=1)
    u = (f @ c) / rho[:, None]
    vel, ncomp = arr["Velocity"]
    assert ncomp == 3
    np.testing.assert_allclose(arr["Density"][0], rho, rtol=1e-13)
    np.testing.assert_allclose(vel.reshape(-1, 3), u, rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(arr["VelocityMagnitude"][0], np.linalg.norm(u, axis=1), rtol=1e-10, atol=1e-14)


@pytest.mark.gpu
def test_lbm_run_interpolated_walls(tmp_path, gpu_lib):
    """lbm_run's interpolated_walls key: a physics-mode run completes and
    differs from half-way bounce-back; a parity-mode run is refused with the
    library's message (a status, not a fault)."""
    from pv_dec_original_gb300 import build, geometry as G
    build.build()
    d = load(fixtures("sim")[0])
    tri = d["tri12"]
    stl = str(tmp_path / "e.stl")
    G.write_stl_ascii(stl, G.Surface(tri[:, :9].reshape(-1, 3, 3).copy(), tri[:, 9:].copy()))
    runs = {}
    for name, extra in (("half", "mode 1\n"), ("interp", "mode 1\ninterpolated_walls 1\n"),
                        ("parity", "mode 0\ninterpolated_walls 1\n")):
        out = tmp_path / name
        out.mkdir()
        cfg = tmp_path / f"{name}.cfg"
        cfg.write_text(f"stl {stl}\nspacing 1.0\ntau 0.8\ndt 8e-06\nend_time 0.000244\noutput_every 30\n"
                       f"output_dir {out}\nprecision 1\ninlet_face 0\ninlet_plane -1\noutlet_face 4\n"
                       f"outlet_plane -1\n" + extra)
        runs[name] = subprocess.run([os.path.join(BUILD, "lbm_run"), str(cfg)], capture_output=True, text=True,
                                    timeout=300)
    assert runs["half"].returncode == 0, runs["half"].stderr
    assert runs["interp"].returncode == 0, runs["interp"].stderr
    a = np.loadtxt(str(tmp_path / "half" / "FlowHemodynamics" / "30_FlowHemodynamics.csv"), delimiter=",",
                   skiprows=1)
    b = np.loadtxt(str(tmp_path / "interp" / "FlowHemodynamics" / "30_FlowHemodynamics.csv"), delimiter=",",
                   skiprows=1)
    assert a.shape == b.shape and not np.array_equal(a[:, 3], b[:, 3])
    assert runs["parity"].returncode == 1
    assert "physics-mode" in runs["parity"].stderr
