"""Build the engine library in-tree with nvcc for sm_103a.

Produces ``pseudoacousticmodeling_gb300/_build/libpam_gb300.so`` (the C ABI of
include/pam.h) and the command-line drivers.  No CMake; one nvcc call per
translation unit, run in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpam_gb300.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code never contracts a * b + c into a fused multiply-add (gcc does on
# aarch64 by default), so host float expressions round as written on every
# machine; device code keeps nvcc's own contraction rules
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-O3",
           "--expt-relaxed-constexpr"]
CU_SOURCES = ["pam_engine.cu", "pam_adjoint.cu", "pam_noalloc.cu", "pam_preprocess.cu"]
CXX_SOURCES = ["survey.cpp", "random_boundary.cpp", "stability.cpp"]
DRIVERS = {"pam_modeling": 1, "pam_migration": 2, "pam_inversion": 3}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "pam.h"))
    return files


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(f) > t for f in _deps() + [os.path.abspath(__file__)])


def build(force=False, verbose=False, extra_flags=(), out_dir=None, drivers=True):
    """Compile every translation unit and link the shared library; returns its
    path.  out_dir / extra_flags build a variant elsewhere (see build_checked)."""
    out = out_dir or OUT
    lib = os.path.join(out, "libpam_gb300.so")
    os.makedirs(out, exist_ok=True)
    if not force and not _stale(lib):
        return lib
    cc = nvcc()
    srcs = [s for s in CU_SOURCES + CXX_SOURCES if os.path.exists(os.path.join(CSRC, s))]

    def comp(src):
        obj = os.path.join(out, src.rsplit(".", 1)[0] + ".o")
        cmd = [cc, *ARCH, *NVFLAGS, *extra_flags, "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [cc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-c",
                   os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(comp, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if drivers:
        _build_drivers(cc, verbose)
    return lib


SDDIV_OUT = os.path.join(HERE, "_build_sddiv")


def build_sd_division(force=False, verbose=False):
    """The library with the pseudo-acoustic Sd ratio divided with correct
    rounding (-DPAM_SD_DIV) instead of the hardware reciprocal: a measurement
    build of the parity tests, in _build_sddiv/."""
    return build(force=force, verbose=verbose, extra_flags=("-DPAM_SD_DIV",), out_dir=SDDIV_OUT, drivers=False)


CHECKED_OUT = os.path.join(HERE, "_build_checked")


def build_checked(force=False, verbose=False):
    """The library with every global access of the stepping, CPML and
    gradient kernels checked against its buffer (-DPAM_BOUNDS_CHECK): a
    violation is printed from the device and the access redirected to a
    small scratch array instead of faulting.  A test build, in _build_checked/."""
    return build(force=force, verbose=verbose, extra_flags=("-DPAM_BOUNDS_CHECK",), out_dir=CHECKED_OUT,
                 drivers=False)


def _build_drivers(cc, verbose=False):
    """The command-line drivers (csrc/drivers.cpp), linked against the library
    with an rpath to _build so they run in place."""
    survey_obj = os.path.join(OUT, "survey.o")

    def one(item):
        name, mode = item
        exe = os.path.join(OUT, name)
        cmd = [cc, "-O2", "-std=c++17", f"-DPAM_DRIVER={mode}", "-I", INCLUDE, os.path.join(CSRC, "drivers.cpp"),
               survey_obj, "-o", exe, "-L", OUT, "-lpam_gb300", "-Xlinker", "-rpath=$ORIGIN"]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed for {name}:\n{r.stdout}\n{r.stderr}")

    with ThreadPoolExecutor(max_workers=len(DRIVERS)) as ex:
        list(ex.map(one, DRIVERS.items()))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
