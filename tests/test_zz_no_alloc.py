"""smgpu_matvec_noalloc: the H·v entry point that allocates nothing.

Some hosts own all of the device memory through their own pool allocator (a
Julia CuArray pool, PyTorch's caching allocator).  A library that calls
cudaMalloc or cudaFree in the middle of such a host's step can fail for lack
of memory the pool holds, or stall the host's queued work (cudaFree
synchronizes the device).  This entry point serves those callers: they pass
device buffers they allocated themselves, and the only scratch the call needs
is a fixed-size static device array.

Checked here: its result equals the ordinary entry point's (smgpu_matvec) and
the oracle's operate_H!, on two calls in a row (which share that array), and
a problem whose H·v launch needs more partial sums than the array holds is
rejected with SMGPU_ERR_LIMIT.  This file is collected last (its name sorts
last) so that a run stopping at the first failure has already run every other
test; it also passes on its own in a fresh process.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MATVEC_FP64_RTOL = 1e-12  # the FP64 H·v tolerance used throughout the GPU tests
NOALLOC_MAX_CTAS = 65536  # partial sums the static scratch array holds


def _cudart():
    """The CUDA runtime libsmgpu.so is linked against (found among the loaded
    objects), else the unversioned name.  The test, not the entry point,
    allocates the device buffers."""
    from smgpu import _lib
    _lib.load()
    path = "libcudart.so"
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                p = line.split()[-1]
                if "/libcudart.so" in p:
                    path = p
                    break
    except OSError:
        pass
    rt = C.CDLL(path)
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    return rt


def test_noalloc_matvec_matches_matvec_and_oracle():
    from oracle.oracle import OracleProblem
    from smgpu import FP64, MIXED, ShellModelProblem
    from smgpu import _lib
    L = _lib.load()
    rt = _cudart()
    snt = os.path.join(GOLDEN, "usdb.snt")
    G = ShellModelProblem(snt, "Mg24", FP64)
    O = OracleProblem(snt, "Mg24")
    n = G.mdim
    assert O.mdim == n
    nbytes = 8 * n
    dv, dw, dx = C.c_void_p(), C.c_void_p(), C.c_void_p()
    for p, b in ((dv, nbytes), (dw, nbytes), (dx, 8)):
        assert rt.cudaMalloc(C.byref(p), b) == 0
    try:
        rng = np.random.default_rng(11)
        for call in range(2):  # two calls in a row share the static scratch
            v = rng.standard_normal(n)
            assert rt.cudaMemcpy(dv, v.ctypes.data, nbytes, 1) == 0  # host -> device
            # the entry point requires v to be complete on the device
            assert rt.cudaDeviceSynchronize() == 0
            rc = L.smgpu_matvec_noalloc(G._h, dv, dw, dx)
            assert rc == _lib.OK, L.smgpu_last_error(G._h)
            w = np.empty(n)
            vhv = np.empty(1)
            assert rt.cudaMemcpy(w.ctypes.data, dw, nbytes, 2) == 0  # device -> host
            assert rt.cudaMemcpy(vhv.ctypes.data, dx, 8, 2) == 0
            ref = G.matvec(v)
            scale = np.abs(ref).max()
            assert np.abs(w - ref).max() <= MATVEC_FP64_RTOL * scale, f"call {call} vs smgpu_matvec"
            oref = O.operate_H(v)
            assert np.abs(w - oref).max() <= MATVEC_FP64_RTOL * np.abs(oref).max(), f"call {call} vs oracle"
            assert abs(vhv[0] - v @ ref) <= MATVEC_FP64_RTOL * np.abs(v).sum() * scale, f"call {call}"
        # a mixed-precision handle is rejected with a clear error
        M = ShellModelProblem(snt, "Mg24", MIXED)
        rc = L.smgpu_matvec_noalloc(M._h, dv, dw, None)
        assert rc == _lib.ERR_ARG
        assert b"SMGPU_FP64" in L.smgpu_last_error(M._h)
    finally:
        for p in (dv, dw, dx):
            rt.cudaFree(p)


def _sparse_pf_snt(path):
    """A pf-shell interaction with its single-particle energies and only a few
    TBME lines (so that the jump tables of a large basis stay small)."""
    from smgpu import synth
    labels, vals = synth.draw_tbmes("pf", 7777)
    pp = [k for k, l in enumerate(labels) if l[0] <= 4 and l[1] <= 4][:3]
    pn = [k for k, l in enumerate(labels) if l[0] <= 4 < l[1]][:3]
    keep = pp + pn
    with open(path, "w") as f:
        f.write(synth.snt_text("pf", [labels[k] for k in keep], [vals[k] for k in keep], 50, "sparse"))
    return path


def test_noalloc_rejects_launch_larger_than_scratch(tmp_path, monkeypatch):
    """pf shell, 9 protons and 1 neutron (Cu50, M = 0): 110,722 proton rows,
    so the FP64 H·v with one row per CTA has more CTAs than the static
    scratch has partial sums.  The call must fail with SMGPU_ERR_LIMIT and
    name the limit, and the handle must stay usable."""
    from smgpu import FP64, ShellModelProblem
    from smgpu import _lib
    L = _lib.load()
    rt = _cudart()
    snt = _sparse_pf_snt(str(tmp_path / "pf_sparse.snt"))
    monkeypatch.setenv("SMGPU_HV_SHAPE", "128,1,1,0")  # FP64 row-tile, one row per CTA
    G = ShellModelProblem(snt, "Cu50", FP64)
    monkeypatch.delenv("SMGPU_HV_SHAPE")
    assert G.stats()["hv_rows"] == 1
    assert int(G.np_.sum()) > NOALLOC_MAX_CTAS
    nbytes = 8 * G.mdim
    dv, dw = C.c_void_p(), C.c_void_p()
    for p in (dv, dw):
        assert rt.cudaMalloc(C.byref(p), nbytes) == 0
    try:
        rc = L.smgpu_matvec_noalloc(G._h, dv, dw, None)
        assert rc == _lib.ERR_LIMIT
        msg = L.smgpu_last_error(G._h)
        assert b"65536" in msg and b"smgpu_matvec_noalloc" in msg
    finally:
        for p in (dv, dw):
            rt.cudaFree(p)
    # the ordinary entry point still works on this handle
    v = np.random.default_rng(3).standard_normal(G.mdim)
    w = G.matvec(v)
    assert np.isfinite(w).all() and np.abs(w).max() > 0
