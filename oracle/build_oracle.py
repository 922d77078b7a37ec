"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles ``oracle/sm_oracle.cpp`` — the C++ restatement of NuclearToolkit.jl's
shell-model path — into ``oracle/liboracle_sm.so`` with OpenMP, ``-O3`` and
the host's native instruction set (it is the timed CPU baseline too).  The reference
itself is Julia; Julia is not available on either machine, so there is no
``oracle/_ref`` build: the restatement is the oracle and the CPU baseline.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sm_oracle.cpp")
LIB = os.path.join(HERE, "liboracle_sm.so")


def native_flag() -> str:
    """Tune for the host the oracle runs on (it is rebuilt on each machine):
    -mcpu=native on Arm, -march=native elsewhere."""
    return "-mcpu=native" if platform.machine().lower() in ("aarch64", "arm64") else "-march=native"


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O3", native_flag(), "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
