"""In-tree build of libsmgpu.so for sm_103a (no cmake, parallel nvcc)."""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsmgpu.so")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["hv.cu", "hv_staged.cu", "hv_2b.cu", "hv_multi.cu", "hv_batch.cu", "lanczos.cu", "multi_lanczos.cu", "batch_lanczos.cu", "enum.cu", "capi.cu",
              "multi.cu", "batch.cu", "obtr.cu", "ec.cu", "membw.cu"]
CXX_SOURCES = ["setup.cpp", "wavio.cpp", "obtr.cpp"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources():
    out = [os.path.join(CSRC, f) for f in CU_SOURCES + CXX_SOURCES]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out.append(os.path.join(INCLUDE, "smgpu.h"))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    procs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(objdir, f + ".o")
        cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                               "-I" + INCLUDE, "-c", os.path.join(CSRC, f), "-o", o]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(o)
    for f in CXX_SOURCES:
        o = os.path.join(objdir, f + ".o")
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-I" + INCLUDE,
               "-I" + os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"),
               "-c", os.path.join(CSRC, f), "-o", o]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(o)
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("libsmgpu build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp", "-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
