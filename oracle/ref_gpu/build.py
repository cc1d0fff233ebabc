"""Build recipe of the reference's own CUDA sweep (test infrastructure only).

* cubin: compiled from the reference sources where they lie (the reference
  checkout's src/kernels.cu, which includes kernels2d.cu, kernels3d.cu and
  random.cu; the directory is --ref-src, else $GPUCPM_REFERENCE_SRC, else
  the checkout at /root/reference/src) with the reference's nvcc flags from its
  setup.py:79-86 (-std=c++17 -use_fast_math -maxrregcount=40), the target
  changed from compute_70/sm_70 (which nvcc 13 rejects) to sm_103a, and
  without -rdc (cooperative grid sync needs no device linking here).  Built
  only where the reference checkout exists; the result in oracle/_ref/
  travels to GPU machines with the working tree.
* driver: oracle/ref_gpu/ref_driver.cpp, this project's host code standing in
  for the reference's host class Cpm, compiled for the local machine and
  linked against the CUDA driver library.
"""
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
DEFAULT_REF_SRC = "/root/reference/src"


def ref_src(path=None):
    """Directory of the reference's CUDA sources: `path`, else the
    GPUCPM_REFERENCE_SRC environment variable, else the default checkout."""
    return pathlib.Path(path or os.environ.get("GPUCPM_REFERENCE_SRC") or DEFAULT_REF_SRC)


CUBIN = OUT / "gpucpm_ref_sm103a.cubin"
DRIVER = OUT / "libref_driver.so"
CUDA = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build_cubin(force=False, src_dir=None):
    """Compile the reference kernels if the checkout is present."""
    REF_SRC = ref_src(src_dir)
    src = REF_SRC / "kernels.cu"
    if not src.exists():
        return CUBIN if CUBIN.exists() else None
    deps = list(REF_SRC.glob("*.cu")) + list(REF_SRC.glob("*.h"))
    if (not force and CUBIN.exists()
            and CUBIN.stat().st_mtime >= max(p.stat().st_mtime for p in deps)):
        return CUBIN
    OUT.mkdir(exist_ok=True)
    nvcc = shutil.which("nvcc") or str(CUDA / "bin" / "nvcc")
    tmp = CUBIN.with_suffix(".tmp")
    subprocess.run([nvcc, f"-I{REF_SRC}", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-cubin", "-std=c++17", "-use_fast_math", "-maxrregcount=40",
                    "-o", str(tmp), str(src)], check=True, capture_output=True)
    os.replace(tmp, CUBIN)
    return CUBIN


def build_driver(force=False):
    src = HERE / "ref_driver.cpp"
    if not force and DRIVER.exists() and DRIVER.stat().st_mtime >= src.stat().st_mtime:
        return DRIVER
    OUT.mkdir(exist_ok=True)
    libdirs = [CUDA / "lib64", CUDA / "lib64" / "stubs", CUDA / "lib" / "stubs"]
    tmp = DRIVER.with_suffix(".tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
           f"-I{CUDA / 'include'}", str(src), "-o", str(tmp)]
    cmd += [f"-L{d}" for d in libdirs if d.exists()] + ["-lcuda"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, DRIVER)
    return DRIVER


def build(force=False, src_dir=None):
    cubin = build_cubin(force, src_dir)
    driver = build_driver(force)
    return cubin, driver


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--ref-src", default=None,
                    help="directory of the reference's src/ (kernels.cu and its includes)")
    print(build(force=True, src_dir=ap.parse_args().ref_src))
