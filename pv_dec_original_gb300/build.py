"""In-tree build of liblbm_gb300.so (CUDA kernels + C ABI) for sm_103a.

Every translation unit is compiled by nvcc in parallel, then linked with
``nvcc -shared``.  Units whose results must round exactly like the reference
(FP64 voxelizer, geometry set-up, FP64 step) are compiled with
``--fmad=false``; host code never contracts (``-ffp-contract=off``), so x86
and aarch64 builds give the same doubles.

    python -m pv_dec_original_gb300.build        # build (incremental)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblbm_gb300.so")
HOST_LIB = os.path.join(OUT, "liblbm_host.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, fmad)
UNITS = [
    ("scan.cu", True),
    ("voxelize.cu", False),
    ("setup.cu", False),
    ("step_f64.cu", False),
    ("step_f32.cu", True),
    ("step_f16.cu", True),
    ("step_bf16.cu", True),
    ("step_fast.cu", True),
    ("capi.cu", False),
    ("noalloc.cu", False),
    ("nn.cu", True),
    ("conv_tc.cu", True),
]
HOST_UNITS = ["host/LatticeModel.cpp", "host/GeometryReader.cpp", "host/ComplexGeometry.cpp",
              "host/Subdomain.cpp", "host/Simulation.cpp", "host/Boundary.cpp", "host/ConfigReader.cpp",
              "host/OutputFile.cpp", "host/pulsatile.cpp"]
RUNNER = os.path.join(OUT, "lbm_run")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps(src: str):
    d = [os.path.join(CSRC, src)]
    for h in os.listdir(CSRC):
        if h.endswith((".cuh", ".h")):
            d.append(os.path.join(CSRC, h))
    d.append(os.path.join(HERE, "..", "include", "lbm_gb300.h"))
    d.append(os.path.join(HERE, "..", "include", "lbm_nn.h"))
    hd = os.path.join(CSRC, "host")
    if os.path.isdir(hd):
        d += [os.path.join(hd, h) for h in os.listdir(hd) if h.endswith(".h")]
    return d


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.exists(x) and os.path.getmtime(x) > t for x in deps)


def _compile(src: str, fmad: bool, verbose: bool, out: str = OUT, defines=()):
    obj = os.path.join(out, os.path.basename(src).replace(".cu", ".o"))
    if not _stale(obj, _deps(src)):
        return obj, None
    cmd = [nvcc(), "-std=c++17", "-O3", *ARCH, "-lineinfo", f"--fmad={'true' if fmad else 'false'}",
           *[f"-D{d}" for d in defines],
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
           "-I", os.path.join(HERE, "..", "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None, f"{src}:\n{r.stderr}"
    if verbose:
        sys.stderr.write(r.stderr)
    return obj, None


def _compile_host(src: str):
    obj = os.path.join(OUT, "host_" + os.path.basename(src).replace(".cpp", ".o"))
    if not _stale(obj, _deps(src)):
        return obj, None
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
           "-I", os.path.join(HERE, "..", "include"), "-I", os.path.join(CSRC, "host"), "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None, f"{src}:\n{r.stderr}"
    return obj, None


def build(verbose: bool = False, jobs: int = 0) -> str:
    os.makedirs(OUT, exist_ok=True)
    jobs = jobs or min(8, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, fm, verbose) for s, fm in UNITS]
        hfuts = [ex.submit(_compile_host, s) for s in HOST_UNITS if os.path.exists(os.path.join(CSRC, s))]
        res = [f.result() for f in futs]
        hres = [f.result() for f in hfuts]
    errs = [e for _, e in res + hres if e]
    if errs:
        raise RuntimeError("build failed:\n" + "\n".join(errs))
    objs = [o for o, _ in res]
    if _stale(LIB, objs):
        cmd = [nvcc(), "-shared", *ARCH, "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    hobjs = [o for o, _ in hres]
    if hobjs and _stale(HOST_LIB, hobjs + [LIB]):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-shared", "-o", HOST_LIB, *hobjs, f"-L{OUT}", "-llbm_gb300", f"-Wl,-rpath,{OUT}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host link failed:\n" + r.stderr)
    drv = os.path.join(CSRC, "host", "LBM.cpp")
    if os.path.exists(drv) and _stale(RUNNER, [drv, HOST_LIB, LIB] + _deps("host/LBM.cpp")):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(HERE, "..", "include"), "-I",
               os.path.join(CSRC, "host"), drv, "-o", RUNNER, f"-L{OUT}", "-llbm_host", "-llbm_gb300",
               f"-Wl,-rpath,{OUT}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("lbm_run link failed:\n" + r.stderr)
    return LIB


CHECK_OUT = os.path.join(HERE, "_build_check")
CHECK_LIB = os.path.join(CHECK_OUT, "liblbm_gb300.so")
# units whose kernels carry the bounds checks (in_bounds, lbm_internal.cuh)
CHECK_UNITS = ("step_f64.cu", "step_f32.cu", "step_f16.cu", "step_bf16.cu", "step_fast.cu", "capi.cu")


def build_checked(jobs: int = 0) -> str:
    """The bounds-checked library (-DLBM_CHECK): the step kernels test every
    population, pull-row and boundary-list index before the access, skip an
    access outside its array and raise a flag the host reports; the other
    units are the normal build's.  Slower; for debugging and its test.
    Bind it with LBM_LIBRARY=<path> (capi.lib_path)."""
    build(jobs=jobs)
    os.makedirs(CHECK_OUT, exist_ok=True)
    jobs = jobs or min(8, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, fm, False, CHECK_OUT, ("LBM_CHECK",)) for s, fm in UNITS if s in CHECK_UNITS]
        res = [f.result() for f in futs]
    errs = [e for _, e in res if e]
    if errs:
        raise RuntimeError("checked build failed:\n" + "\n".join(errs))
    objs = [o for o, _ in res] + [os.path.join(OUT, s.replace(".cu", ".o")) for s, _ in UNITS if s not in CHECK_UNITS]
    if _stale(CHECK_LIB, objs):
        r = subprocess.run([nvcc(), "-shared", *ARCH, "-o", CHECK_LIB, *objs, "-lcudart"], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError("checked link failed:\n" + r.stderr)
    return CHECK_LIB


if __name__ == "__main__":
    if "--checked" in sys.argv:
        print(build_checked())
    else:
        print(build(verbose="-v" in sys.argv))
