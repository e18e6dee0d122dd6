"""Build recipe for the CPU FP64 oracle (test infrastructure only).

Compiles oracle/ppm_oracle.c into oracle/_build/libppm_oracle.so with FMA
contraction disabled, so that f64 results follow the source's evaluation
order on both x86-64 and aarch64 hosts.  The reference itself (Rust) cannot
be compiled here, so there is no oracle/_ref build.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libppm_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ppm_oracle.c")
    hdr = os.path.join(HERE, "ppm_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    base = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-Wall",
            "-Wno-unused-function", "-Wno-unknown-pragmas", src, "-o", LIB + ".tmp", "-lm"]
    try:
        subprocess.check_call(base[:1] + ["-fopenmp"] + base[1:], stderr=subprocess.DEVNULL)
    except subprocess.CalledProcessError:
        subprocess.check_call(base)   # single-threaded oracle when OpenMP is unavailable
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
