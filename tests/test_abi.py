"""C ABI surface and host-side logic that needs no GPU."""
import ctypes
import inspect
import os
import re
import subprocess

import pytest

from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "smgpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|double|const char\*)\s+(smgpu_\w+)\s*\(", txt, re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    L = _lib.load()
    decl = declared_symbols()
    assert len(decl) >= 12
    for name in decl:
        assert hasattr(L, name), name
    assert set(decl) == set(_lib.SIGNATURES)
    out = subprocess.run(["nm", "-D", "--defined-only", b.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (smgpu_\w+)", out))
    assert set(decl) <= exported


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_loudly():
    from smgpu import SmgpuError, ShellModelProblem
    from smgpu import _lib
    with pytest.raises(SmgpuError) as ei:
        ShellModelProblem(os.path.join(ROOT, "tests", "golden", "ckpot.snt"), "Be8")
    assert ei.value.code == _lib.ERR_CUDA
    assert "no CUDA device" in str(ei.value)


def test_multi_create_without_gpu_fails_loudly():
    from smgpu import MultiSampleProblem, SmgpuError
    from smgpu import _lib
    ck = os.path.join(ROOT, "tests", "golden", "ckpot.snt")
    with pytest.raises(SmgpuError) as ei:
        MultiSampleProblem([ck, ck], "Be8")
    assert ei.value.code == _lib.ERR_CUDA
    assert "no CUDA device" in str(ei.value)
    # argument checks come before any device work
    with pytest.raises(SmgpuError) as ei:
        MultiSampleProblem([ck] * 17, "Be8")
    assert ei.value.code == _lib.ERR_LIMIT
    with pytest.raises(SmgpuError) as ei:
        MultiSampleProblem([], "Be8")
    assert ei.value.code == _lib.ERR_ARG


def test_batch_create_without_gpu_fails_loudly():
    from smgpu import BatchProblem, SmgpuError
    from smgpu import _lib
    ck = os.path.join(ROOT, "tests", "golden", "ckpot.snt")
    with pytest.raises(SmgpuError) as ei:
        BatchProblem([(ck, "Be8"), (ck, "Li7")])
    assert ei.value.code == _lib.ERR_CUDA
    assert "no CUDA device" in str(ei.value)
    with pytest.raises(SmgpuError) as ei:
        BatchProblem([(ck, "Be8")] * 4097)
    assert ei.value.code == _lib.ERR_LIMIT
    with pytest.raises(SmgpuError) as ei:
        BatchProblem([])
    assert ei.value.code == _lib.ERR_ARG


def test_main_sm_keeps_reference_signature():
    """shellmodel_main.jl:89-92 argument names."""
    from smgpu import main_sm
    names = list(inspect.signature(main_sm).parameters)
    ref = ["sntf", "target_nuc", "num_ev", "target_J", "save_wav", "q", "is_block", "is_show", "num_history", "lm",
           "ls", "tol", "in_wf", "mdimmode", "print_evec", "calc_moment", "calc_entropy", "visualize_occ",
           "gfactors", "effcharge", "truncation_scheme", "truncated_jocc", "debugmode"]
    assert names[:len(ref)] == ref
    assert inspect.signature(main_sm).parameters["lm"].default == 300
    assert inspect.signature(main_sm).parameters["ls"].default == 20
    assert inspect.signature(main_sm).parameters["tol"].default == 1e-8


def test_main_sm_rejects_unsupported_paths():
    from smgpu import main_sm
    with pytest.raises(ValueError):
        main_sm("x.snt", "Be8", 1, [0, 2])  # one target J only (shellmodel_main.jl:109)
    with pytest.raises(NotImplementedError):
        main_sm("x.snt", "Be8", 1, [], calc_entropy=True)


def test_synthetic_recipe_counts():
    from smgpu import synth
    sd = synth.tbme_labels(synth.SD_ORBITS)
    pf = synth.tbme_labels(synth.PF_ORBITS)
    assert len(sd) == 158 and len(pf) == 518
    k = len(synth.SD_ORBITS)
    assert sum(1 for l in sd if l[1] <= k) == 30  # pp lines, as in usdb.snt
    assert sum(1 for l in sd if l[0] <= k < l[1]) == 98  # pn lines
    for (a, b, c, d, J) in sd + pf:
        assert (a, b) <= (c, d)
    l1, v1 = synth.draw_tbmes("pf", 5)
    l2, v2 = synth.draw_tbmes("pf", 5)
    assert l1 == l2 and (v1 == v2).all()


def test_synthetic_snt_is_readable_by_the_oracle(tmp_path):
    from oracle.oracle import OracleProblem
    from smgpu import synth
    p = synth.write_snt(str(tmp_path / "s.snt"), "sd", 11, 2, 1)
    P = OracleProblem(p, synth.nucleus_name("sd", 2, 1))
    assert P.vp == 2 and P.vn == 1 and P.Mtot == 1
    H = P.dense_H()
    import numpy as np
    assert np.abs(H - H.T).max() < 1e-12


def test_wav_round_trip_and_layout(tmp_path):
    """smgpu_write_wav / smgpu_read_wav (host-only calls) against the byte
    layout of writeRitzvecs (shellmodel_main.jl:1215-1229)."""
    import struct
    import numpy as np
    from smgpu import SmgpuError
    from smgpu import _lib
    from smgpu.wav import read_wav, read_wav_full, write_wav
    rng = np.random.default_rng(1)
    mdim, nev = 37, 3
    e = np.array([-31.119, -27.3, -19.162])
    j = [0, 4, 8]
    v = rng.standard_normal((nev, mdim))
    p = tmp_path / "Be8_ckpot.wav"
    write_wav(str(p), 0, e, j, v)
    raw = p.read_bytes()
    ref = struct.pack("<ii", nev, 0) + struct.pack("<3d", *e) + struct.pack("<3i", *j) + v.astype("<f8").tobytes()
    assert raw == ref
    e2, j2, v2, mt = read_wav_full(str(p), mdim)
    assert mt == 0 and np.array_equal(e2, e) and list(j2) == j and np.array_equal(v2, v)
    x, jj = read_wav(str(p), mdim, 2)
    assert np.array_equal(x, v[1]) and jj == 4
    with pytest.raises(SmgpuError) as ei:
        read_wav(str(p), mdim + 1, 1)
    assert ei.value.code == _lib.ERR_PARSE
    with pytest.raises(SmgpuError) as ei:
        read_wav(str(tmp_path / "missing.wav"), mdim, 1)
    assert ei.value.code == _lib.ERR_IO


def test_wigner_symbols_of_the_library_equal_the_oracle():
    """smgpu_wigner3j / smgpu_wigner6j (host code) against the oracle's
    restatement: both square exactly and round once, so they agree bit for
    bit."""
    import itertools
    from smgpu import _lib
    from oracle.oracle import wigner3j, wigner6j
    L = _lib.load()
    for js in itertools.product(range(0, 7), repeat=6):
        assert L.smgpu_wigner6j(*js) == wigner6j(*js)
    for a, b, c in itertools.product(range(0, 9), range(0, 5), range(0, 9)):
        for ma in range(-a, a + 1, 2):
            for mb in range(-b, b + 1, 2):
                assert L.smgpu_wigner3j(a, b, c, ma, mb, -ma - mb) == wigner3j(a, b, c, ma, mb, -ma - mb)
