"""`.wav` files of eigenvalues, 2J labels and Ritz vectors (the format of the
reference's writeRitzvecs / read_wav / read_appwav,
src/ShellModel/shellmodel_main.jl:967-1003,1215-1229), through the C ABI's
host-only calls."""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check_wav, load


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def write_wav(path, mtot2, evals, twoJ, vecs):
    """Write neig = len(evals) states: energies, 2J labels and the vectors
    (shape (neig, mdim)) — writeRitzvecs."""
    e = np.ascontiguousarray(evals, dtype=np.float64)
    j = np.ascontiguousarray(twoJ, dtype=np.int32)
    v = np.ascontiguousarray(vecs, dtype=np.float64)
    if v.ndim != 2 or v.shape[0] != e.size or j.size != e.size:
        raise ValueError("vecs must have shape (len(evals), mdim) and twoJ len(evals) entries")
    check_wav(load().smgpu_write_wav(os.fsencode(path), v.shape[1], int(mtot2), e.size, _p(e), _p(j), _p(v)))


def read_wav(path, mdim, n=1, all=False):
    """read_wav: (V[n], 2J[n]) for the 1-based state n, or (V, 2J) of all
    states with all=True.  Also returns nothing else; use read_wav_header for
    the energies' count and Mtot."""
    L = load()
    nev, mt = C.c_int(), C.c_int()
    check_wav(L.smgpu_read_wav_header(os.fsencode(path), int(mdim), C.byref(nev), C.byref(mt)))
    k = nev.value
    e = np.zeros(k)
    j = np.zeros(k, dtype=np.int32)
    v = np.zeros((k, int(mdim)))
    check_wav(L.smgpu_read_wav(os.fsencode(path), int(mdim), k, _p(e), _p(j), _p(v)))
    if all:
        return list(v), list(map(int, j))
    return v[n - 1], int(j[n - 1])


def read_wav_full(path, mdim):
    """(energies, 2J labels, vectors (neig, mdim), Mtot doubled)."""
    L = load()
    nev, mt = C.c_int(), C.c_int()
    check_wav(L.smgpu_read_wav_header(os.fsencode(path), int(mdim), C.byref(nev), C.byref(mt)))
    k = nev.value
    e = np.zeros(k)
    j = np.zeros(k, dtype=np.int32)
    v = np.zeros((k, int(mdim)))
    check_wav(L.smgpu_read_wav(os.fsencode(path), int(mdim), k, _p(e), _p(j), _p(v)))
    return e, j, v, int(mt.value)


__all__ = ["write_wav", "read_wav", "read_wav_full"]
_ = _lib
