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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
