"""Compile the CUDA library (libppmpa_gb300.so) for sm_103a, in-tree.

Translation units are compiled in parallel; the FP64 kernels are built with
--fmad=false so double arithmetic rounds exactly as written.  The host code
is compiled with -ffp-contract=off for the same reason (aarch64 GCC would
otherwise fuse multiply-adds in the camera and material derivations).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libppmpa_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "k_f64.cu": ["--fmad=false"],
    "k_f32.cu": [],
    "k_grid.cu": [],
    "k_bvh.cu": [],
    "scene_file.cpp": [],
    "output.cpp": [],
    "ppm_api.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libppmpa_gb300.so")


def _sources_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(HERE, "cli", f) for f in os.listdir(os.path.join(HERE, "cli"))]
    files.append(os.path.join(ROOT, "include", "ppm_api.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _compile(unit: str, extra, verbose_ptxas: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, os.path.splitext(unit)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           *extra, "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        with open(obj + ".ptxas.txt", "w") as f:
            f.write(res.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose_ptxas), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    _build_cli()
    return LIB


CLI = os.path.join(OUT, "ppmpa")
TOOLS = ("ppmpa", "pm", "rt", "rtc")   # drop-ins for the reference's binaries


def _build_cli() -> str:
    """The command-line programs (same argv and output as the reference's binaries)."""
    def one(name):
        src = os.path.join(HERE, "cli", name + ".cpp")
        out = os.path.join(OUT, name)
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), src,
               "-o", out + ".tmp", "-L", OUT, "-lppmpa_gb300", "-Wl,-rpath,$ORIGIN"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"{name} build failed:\n{res.stderr}")
        os.replace(out + ".tmp", out)
    with cf.ThreadPoolExecutor(max_workers=len(TOOLS)) as ex:
        list(ex.map(one, TOOLS))
    return CLI


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose_ptxas="-v" in sys.argv))
