"""Build recipe of the GB300 solver libraries (in-tree, no cmake).

Produces, next to this file:
  libss4d.so      the C ABI of include/ss4d.h (CUDA kernels for sm_103a + host code)
  libss4d_seg.so  the reference-named layer for segmentation4D.c drivers
  libss4d_mcf.so  the reference-named layer for mcf_4D.c drivers

`python build.py` or `build.build()`.  Translation units compile in parallel;
a library is rebuilt only when one of its sources or headers is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-Xptxas", "-v"]

# translation unit -> extra nvcc flags.  The reference-order kernels are
# compiled without multiply-add contraction so each voxel update rounds like
# the reference (see the header of ss4d_kernels_ref.cu).
CUDA_UNITS = {
    "ss4d_kernels_ref.cu": ["--fmad=false"],
    "ss4d_kernels_fast.cu": [],
    "ss4d_api.cu": [],
    "ss4d_noalloc.cu": [],
    "ss4d_batch.cu": [],
    "ss4d_ws.cu": [],
    "ss4d_nn.cu": [],
    "ss4d_conv_tc.cu": [],
    "ss4d_assemble_ff.cu": [],
    "ss4d_front_ff.cu": [],
    "ss4d_project.cu": [],
}
C_UNITS = {"ss4d_scene.c": ["-fopenmp"], "ss4d_vtk.c": [], "ss4d_slab.c": []}

LIB = os.path.join(HERE, "libss4d.so")
LIB_SEG = os.path.join(HERE, "libss4d_seg.so")
LIB_MCF = os.path.join(HERE, "libss4d_mcf.so")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the solver")


def _cuda_lib_dir(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def _headers() -> list[str]:
    out = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], log: str | None = None) -> str:
    p = subprocess.run(cmd, capture_output=True, text=True)
    text = p.stdout + p.stderr
    if log:
        with open(log, "w") as fh:
            fh.write(" ".join(cmd) + "\n" + text)
    if p.returncode != 0:
        raise RuntimeError(f"build step failed ({p.returncode}): {' '.join(cmd)}\n{text[-4000:]}")
    return text


def build(verbose: bool = False, force: bool = False) -> dict:
    """Compile every CUDA/C unit for sm_103a and link the three libraries."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for unit, extra in CUDA_UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(([nvcc] + GENCODE + NVCC_FLAGS + extra + ["-c", src, "-o", obj], obj + ".log"))
    for unit, extra in C_UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append((["gcc", "-O2", "-fPIC", "-std=gnu11"] + extra + ["-c", src, "-o", obj], obj + ".log"))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            futs = [ex.submit(_run, c, l) for c, l in jobs]
            for f in futs:
                f.result()
    libdir = _cuda_lib_dir(nvcc)
    if force or _stale(LIB, objs):
        _run([nvcc] + GENCODE + ["-shared", "-o", LIB] + objs +
             ["-cudart", "shared", "-Xcompiler", "-fopenmp", "-Xlinker", f"-rpath,{libdir}", "-lgomp", "-lpthread"],
             os.path.join(BUILD, "link.log"))
    for lib, src in ((LIB_SEG, "ss4d_compat_seg.c"), (LIB_MCF, "ss4d_compat_mcf.c")):
        srcp = os.path.join(CSRC, src)
        if force or _stale(lib, [srcp, LIB] + hdrs):
            _run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-o", lib, srcp, f"-L{HERE}", "-lss4d",
                  "-lpthread", "-Wl,-Bsymbolic", "-Wl,-rpath,$ORIGIN"], os.path.join(BUILD, src + ".log"))
    if verbose:
        print(f"built {LIB}, {LIB_SEG}, {LIB_MCF}")
    return {"lib": LIB, "seg": LIB_SEG, "mcf": LIB_MCF}


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
