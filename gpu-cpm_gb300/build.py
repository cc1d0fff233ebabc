"""Build recipe of libgpucpm_gb300.so (the CUDA engine and its C-ABI).

Compiles every translation unit of csrc/ for sm_103a only, in parallel, and
links one shared library next to this file.  No fast-math and no implicit
FMA contraction: the sweep's FP32 ΔH and Metropolis test are written with
explicitly rounded intrinsics and must execute exactly as written.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB_PATH = HERE / "libgpucpm_gb300.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           f"-I{INCLUDE}", f"-I{CSRC}"]
SOURCES = ["cpm_engine.cu", "cpm_kernels.cu", "cpm_sweep2d.cu", "cpm_sweep3d.cu",
           "cpm_static.cu"]
HEADERS = ["cpm_internal.h", "cpm_device.cuh", "cpm_sweep_common.cuh", "cpm_rowtile.cuh"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = [CSRC / s for s in SOURCES + HEADERS] + [INCLUDE / "gpucpm.h"]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile the engine if any source is newer than the library."""
    if not force and not _stale():
        return LIB_PATH
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src: str) -> pathlib.Path:
        obj = BUILD / (pathlib.Path(src).stem + ".o")
        cmd = [nvcc, *ARCH, *NVFLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", str(tmp),
                        *map(str, objs), "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
