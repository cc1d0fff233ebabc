"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/cpm_oracle.cpp into oracle/_build/libcpm_oracle.so with the
host compiler.  Floating-point contraction is switched off so that the FP32
operation order written in the source is the one executed on x86-64 and on
aarch64 alike.
"""
import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "cpm_oracle.cpp"
OUT_DIR = HERE / "_build"
LIB_PATH = OUT_DIR / "libcpm_oracle.so"

FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
         "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> pathlib.Path:
    """Compile the oracle if the library is missing or older than its source."""
    OUT_DIR.mkdir(exist_ok=True)
    if (not force and LIB_PATH.exists()
            and LIB_PATH.stat().st_mtime >= SRC.stat().st_mtime):
        return LIB_PATH
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB_PATH.with_suffix(".so.tmp")
    subprocess.run([cxx, *FLAGS, str(SRC), "-o", str(tmp)], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True))
