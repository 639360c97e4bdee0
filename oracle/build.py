"""Build recipe for the CPU oracle (test infrastructure).

Compiles ``oracle/pam_oracle.c`` with gcc into ``oracle/_build/libpam_oracle.so``.
``-ffp-contract=off`` keeps the FP32 restatement free of fused multiply-adds
so each operation rounds exactly as written; no architecture-specific flags,
so the same source builds on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpam_oracle.so")
SOURCES = [os.path.join(HERE, "pam_oracle.c"), os.path.join(HERE, "pam_oracle_impl.h")]


def build(force: bool = False) -> str:
    """Compile the oracle if it is missing or older than its sources; return the .so path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        lib_mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_mtime for s in SOURCES):
            return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", os.path.join(HERE, "pam_oracle.c"), "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


REF_SRC = os.environ.get("PAM_REFERENCE_SRC", "/root/reference/cpp")
REF_DIR = os.path.join(HERE, "_ref")
REF_CUBIN = os.path.join(REF_DIR, "Modeling.cubin")
HARNESS_SRC = os.path.join(HERE, "ref_harness.cpp")
HARNESS_LIB = os.path.join(OUT_DIR, "libpam_refharness.so")


def _cuda_home():
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_ref_cubin(force: bool = False):
    """Compile the reference's unmodified cpp/Modeling.cu into an sm_103a
    cubin (device code only) with the reference's own -std=c++17 -O3, when
    the reference sources are present; the cubin is what travels."""
    src = os.path.join(REF_SRC, "Modeling.cu")
    if not os.path.exists(src):
        return REF_CUBIN if os.path.exists(REF_CUBIN) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if not force and os.path.exists(REF_CUBIN) and os.path.getmtime(REF_CUBIN) >= os.path.getmtime(src):
        return REF_CUBIN
    tmp = REF_CUBIN + f".tmp{os.getpid()}"
    cmd = [os.path.join(_cuda_home(), "bin", "nvcc"), "-cubin", "-std=c++17", "-O3",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I" + REF_SRC, src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_CUBIN)
    return REF_CUBIN


REF_MIG_CUBIN = os.path.join(REF_DIR, "Migration.cubin")


def build_ref_migration_cubin(force: bool = False):
    """Compile the reference's unmodified cpp/Migration.cu into an sm_103a
    cubin (device code only: the adjoint, imaging, adjoint-source and
    normalisation kernels), when the reference sources are present."""
    src = os.path.join(REF_SRC, "Migration.cu")
    if not os.path.exists(src):
        return REF_MIG_CUBIN if os.path.exists(REF_MIG_CUBIN) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if not force and os.path.exists(REF_MIG_CUBIN) and os.path.getmtime(REF_MIG_CUBIN) >= os.path.getmtime(src):
        return REF_MIG_CUBIN
    tmp = REF_MIG_CUBIN + f".tmp{os.getpid()}"
    cmd = [os.path.join(_cuda_home(), "bin", "nvcc"), "-cubin", "-std=c++17", "-O3",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I" + REF_SRC, src, "-o", tmp]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, REF_MIG_CUBIN)
    return REF_MIG_CUBIN


def build_harness(force: bool = False):
    """Compile the driver-API host harness (oracle/ref_harness.cpp) that runs
    the reference's kernels; None when the CUDA headers are absent."""
    cuda = _cuda_home()
    inc = os.path.join(cuda, "include")
    if not os.path.exists(os.path.join(inc, "cuda.h")):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(HARNESS_LIB) and os.path.getmtime(HARNESS_LIB) >= os.path.getmtime(HARNESS_SRC):
        return HARNESS_LIB
    stubs = [d for d in (os.path.join(cuda, "lib64", "stubs"), os.path.join(cuda, "lib", "stubs"))
             if os.path.exists(os.path.join(d, "libcuda.so"))]
    tmp = HARNESS_LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", HARNESS_SRC, "-I" + inc, "-o", tmp]
    cmd += ["-L" + d for d in stubs] + ["-lcuda"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, HARNESS_LIB)
    return HARNESS_LIB


HOST_SRC = os.path.join(HERE, "ref_host.cpp")
HOST_LIB = os.path.join(REF_DIR, "libref_host.so")


def build_ref_host(force: bool = False, ref_src: str = None):
    """Compile the reference's unmodified cpp/Migration.cu and cpp/Modeling.cu
    (its own -std=c++17 -O3 -fopenmp) with the host harness oracle/ref_host.cpp
    into a shared library that runs the reference's host routines (smoothing,
    mute, stability check, padding) on the CPU; None when the reference
    sources are absent."""
    src = ref_src or REF_SRC
    cus = [os.path.join(src, "Migration.cu"), os.path.join(src, "Modeling.cu")]
    if not all(os.path.exists(c) for c in cus):
        return HOST_LIB if os.path.exists(HOST_LIB) else None
    os.makedirs(REF_DIR, exist_ok=True)
    newest = max(os.path.getmtime(f) for f in cus + [HOST_SRC])
    if not force and os.path.exists(HOST_LIB) and os.path.getmtime(HOST_LIB) >= newest:
        return HOST_LIB
    tmp = HOST_LIB + f".tmp{os.getpid()}"
    cmd = [os.path.join(_cuda_home(), "bin", "nvcc"), "-std=c++17", "-O3", "-shared", "-Xcompiler", "-fPIC,-fopenmp",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I" + src] + cus + [HOST_SRC, "-o", tmp, "-lgomp"]
    subprocess.run(cmd, check=True, capture_output=True)   # the reference's own warnings stay quiet
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_ref_cubin(force="--force" in sys.argv))
    print(build_ref_migration_cubin(force="--force" in sys.argv))
    print(build_harness(force="--force" in sys.argv))
    print(build_ref_host(force="--force" in sys.argv))
