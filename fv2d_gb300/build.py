"""Builds the native parts of fv2d_gb300 in-tree for GB300 (sm_103a):

  fv2d_gb300/lib/libfv2d_gpu.so   the C-ABI library (include/fv2d_gpu.h)
  fv2d_gb300/bin/fv2d_gpu         the driver executable (main.cpp's role)
  fv2d_gb300/lib_checked/...      build(bounds_check=True): the same library
                                  with -DFV2D_BOUNDS_CHECK (index checks in
                                  the FP64 step, for the tests)

Translation units are compiled in parallel with nvcc (one -gencode,
arch=compute_103a,code=sm_103a); object files go to fv2d_gb300/_build/.
Rebuilds only what changed (source or any header newer than the object).
The FP64 step is compiled with -fmad=false so that no multiply-add is
contracted: its results are then bit-identical to the reference's
binary64 expressions.  Host C++ uses -ffp-contract=off for the same reason
(GCC contracts by default on aarch64).
"""
import glob
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libfv2d_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fv2d_gb300")


# (source, extra flags)
UNITS = [
    ("fv2d_api.cu", ["-fmad=false"]),
    ("step_dispatch.cu", ["-fmad=false"]),
    ("step_hll.cu", ["-fmad=false"]),
    ("step_hllc.cu", ["-fmad=false"]),
    ("step_fslp.cu", ["-fmad=false"]),
    ("probe.cu", []),
    ("selftest.cu", ["-fmad=false"]),
    ("noalloc.cu", ["-fmad=false"]),
    ("batch_kernels.cu", ["-use_fast_math"]),
    ("batch_march2.cu", ["-use_fast_math"]),
    ("serve.cu", []),
    ("problems.cpp", []),
    ("../host/ini.cpp", []),
    ("../host/h5.cpp", []),
    ("../host/io_api.cpp", []),
]
DRIVER = os.path.join(PKG, "bin", "fv2d_gpu")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(REPO, "include", "*.h"))


def _stale(obj, src, hdr_mtime):
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return os.path.getmtime(src) > m or hdr_mtime > m


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, jobs=None, bounds_check=False):
    """Compile every translation unit and link libfv2d_gpu.so.  Returns the
    library path.  bounds_check=True builds the index-checking variant into
    fv2d_gb300/lib_checked/ (objects in fv2d_gb300/_build_checked/)."""
    BUILD = os.path.join(PKG, "_build_checked" if bounds_check else "_build")
    LIBDIR = os.path.join(PKG, "lib_checked" if bounds_check else "lib")
    LIB = os.path.join(LIBDIR, "libfv2d_gpu.so")
    checked = ["-DFV2D_BOUNDS_CHECK"] if bounds_check else []
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)] +
                    [os.path.getmtime(h) for h in glob.glob(os.path.join(PKG, "host", "*.hpp"))])
    # objects built on another host architecture are never reused
    stamp = os.path.join(BUILD, "host-arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        for f in glob.glob(os.path.join(BUILD, "*.o")) + [LIB, DRIVER]:
            if os.path.exists(f):
                os.unlink(f)
        with open(stamp, "w") as f:
            f.write(arch)
    cmds, objs = [], []
    for src, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(o)
        if not _stale(o, s, hdr_mtime):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   *extra, *checked, "-c", s, "-o", o]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", s, "-o", o]
        cmds.append(cmd)
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(8, len(cmds))) as ex:
            for out in ex.map(_compile, cmds):
                if verbose and out.strip():
                    print(out)
    if cmds or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        _compile([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"])
    if bounds_check:
        return LIB
    # the fv2d_gpu driver executable (main.cpp's role), linked to the library
    drv_src = os.path.join(PKG, "host", "driver.cpp")
    if not os.path.exists(DRIVER) or os.path.getmtime(DRIVER) < max(os.path.getmtime(LIB), os.path.getmtime(drv_src)):
        os.makedirs(os.path.dirname(DRIVER), exist_ok=True)
        _compile(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", drv_src, "-o", DRIVER,
                  "-L" + LIBDIR, "-lfv2d_gpu", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
