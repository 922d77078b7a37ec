"""smgpu_matvec_noalloc: the H·v entry point that allocates nothing.

It serves callers that cannot let the library allocate device memory while
they run (a CUDA stream capture, or a host whose device memory belongs to its
own pool allocator).  Its result must equal the ordinary smgpu_matvec.  This
file is collected last (its name sorts last) so that a run stopping at the
first failure has already run every other test; it also passes on its own in
a fresh process.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MATVEC_FP64_RTOL = 1e-12  # the FP64 H·v tolerance used throughout the GPU tests


def _cudart():
    # the same CUDA runtime libsmgpu.so links against; the test (not the
    # entry point) allocates the device buffers
    rt = C.CDLL("libcudart.so.13")
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    return rt


def test_noalloc_matvec_matches_matvec():
    from smgpu import FP64, MIXED, ShellModelProblem
    from smgpu import _lib
    L = _lib.load()
    rt = _cudart()
    G = ShellModelProblem(os.path.join(GOLDEN, "usdb.snt"), "Mg24", FP64)
    n = G.mdim
    nbytes = 8 * n
    dv, dw, dx = C.c_void_p(), C.c_void_p(), C.c_void_p()
    for p, b in ((dv, nbytes), (dw, nbytes), (dx, 8)):
        assert rt.cudaMalloc(C.byref(p), b) == 0
    try:
        rng = np.random.default_rng(11)
        for call in range(2):  # two calls in a row share the static scratch
            v = rng.standard_normal(n)
            assert rt.cudaMemcpy(dv, v.ctypes.data, nbytes, 1) == 0  # host -> device
            rc = L.smgpu_matvec_noalloc(G._h, dv, dw, dx)
            assert rc == _lib.OK, L.smgpu_last_error(G._h)
            w = np.empty(n)
            vhv = np.empty(1)
            assert rt.cudaMemcpy(w.ctypes.data, dw, nbytes, 2) == 0  # device -> host
            assert rt.cudaMemcpy(vhv.ctypes.data, dx, 8, 2) == 0
            ref = G.matvec(v)
            scale = np.abs(ref).max()
            assert np.abs(w - ref).max() <= MATVEC_FP64_RTOL * scale, f"call {call}"
            assert abs(vhv[0] - v @ ref) <= MATVEC_FP64_RTOL * np.abs(v).sum() * scale, f"call {call}"
        # a mixed-precision handle is rejected with a clear error
        M = ShellModelProblem(os.path.join(GOLDEN, "usdb.snt"), "Mg24", MIXED)
        rc = L.smgpu_matvec_noalloc(M._h, dv, dw, None)
        assert rc == _lib.ERR_ARG
        assert b"SMGPU_FP64" in L.smgpu_last_error(M._h)
    finally:
        for p in (dv, dw, dx):
            rt.cudaFree(p)
