"""Host-side mirror of NuclearToolkit.jl's ShellModel entry point over libsmgpu.

``main_sm`` keeps the reference's signature and return value
(src/ShellModel/shellmodel_main.jl:89-281): it reads the snt file, sets the
problem up for the target nucleus and returns the lowest ``num_ev``
eigenvalues (MeV) — all compute on the GPU through the C ABI.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import FP64, MIXED, check, load


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class ShellModelProblem:
    """One M-scheme problem resident on the GPU (an ``smgpu_problem`` handle)."""

    def __init__(self, sntf: str, target_nuc: str, precision: int = FP64, twoJ=None):
        """twoJ: build the basis of Mtot = twoJ for the J-projected solve
        (main_sm's target_J = [twoJ]); None: Mtot = A mod 2."""
        L = load()
        h = C.c_void_p()
        if twoJ is None:
            rc = L.smgpu_problem_create_from_snt(os.fsencode(sntf), target_nuc.encode(), int(precision), C.byref(h))
        else:
            rc = L.smgpu_problem_create_from_snt_J(os.fsencode(sntf), target_nuc.encode(), int(twoJ), int(precision),
                                                   C.byref(h))
        check(rc, None)
        self._h = h
        self.precision = precision
        md = C.c_longlong()
        nb = C.c_int()
        check(L.smgpu_dims(h, C.byref(md), C.byref(nb), None), h)
        self.mdim = int(md.value)
        self.nblocks = int(nb.value)
        self.tdims = np.zeros(self.nblocks + 1, dtype=np.int64)
        check(L.smgpu_dims(h, None, None, _p(self.tdims)), h)
        self.np_ = np.zeros(self.nblocks, dtype=np.int32)
        self.nn_ = np.zeros(self.nblocks, dtype=np.int32)
        self.Mp = np.zeros(self.nblocks, dtype=np.int32)
        self.Mn = np.zeros(self.nblocks, dtype=np.int32)
        check(L.smgpu_blocks(h, _p(self.np_), _p(self.nn_), _p(self.Mp), _p(self.Mn)), h)
        self.mtot2 = int(self.Mp[0] + self.Mn[0]) if self.nblocks else 0  # doubled total M

    def close(self):
        if getattr(self, "_h", None):
            load().smgpu_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- exports for parity checks
    def basis(self):
        p = np.zeros(int(self.np_.sum()), dtype=np.uint64)
        n = np.zeros(int(self.nn_.sum()), dtype=np.uint64)
        check(load().smgpu_export_basis(self._h, _p(p), _p(n)), self._h)
        return p, n

    def jumps(self, which: int):
        L = load()
        cnt = C.c_longlong()
        check(L.smgpu_export_jumps(self._h, which, C.byref(cnt), None, None), self._h)
        width = 7 if which in (0, 1) else 3
        ints = np.zeros((cnt.value, width), dtype=np.int64)
        coef = np.zeros(cnt.value)
        check(L.smgpu_export_jumps(self._h, which, C.byref(cnt), _p(ints), _p(coef)), self._h)
        return (ints, coef) if which in (2, 3) else ints

    def stats(self):
        s = np.zeros(12, dtype=np.int64)
        check(load().smgpu_stats(self._h, _p(s)), self._h)
        keys = ["updates", "pn_proton_entries", "pn_neutron_entries", "pp_entries", "nn_entries", "table_bytes",
                "len_pad", "links", "hv_threads", "hv_rows", "hv_min_ctas", "hv_staged"]
        return dict(zip(keys, map(int, s)))

    def tune_report(self):
        """The H·v autotuner's candidates: list of dicts (threads, rows, min_ctas, staged, ms)."""
        n = C.c_int(0)
        check(load().smgpu_tune_report(self._h, 0, None, None, C.byref(n)), self._h)
        shapes = np.zeros(4 * max(n.value, 1), dtype=np.int32)
        ms = np.zeros(max(n.value, 1))
        check(load().smgpu_tune_report(self._h, n.value, _p(shapes), _p(ms), C.byref(n)), self._h)
        return [dict(threads=int(shapes[4 * k]), rows=int(shapes[4 * k + 1]), min_ctas=int(shapes[4 * k + 2]),
                     staged=int(shapes[4 * k + 3]), ms=float(ms[k])) for k in range(n.value)]

    def timings(self):
        t = np.zeros(8)
        check(load().smgpu_timings(self._h, _p(t)), self._h)
        keys = ["setup", "lanczos", "matvec", "capture", "ritz", "solve_wall", "setup_tables", "setup_upload"]
        return dict(zip(keys, map(float, t)))

    def time_matvec(self, reps=20, flush_l2=True):
        """Mean ms per H·v launch, CUDA events on the library's stream."""
        ms = C.c_double()
        check(load().smgpu_time_matvec(self._h, int(reps), 1 if flush_l2 else 0, C.byref(ms)), self._h)
        return float(ms.value)

    def jj(self, vecs):
        """<v|J^2|v>/<v|v> for each row of vecs (shape (n, mdim) or (mdim,))."""
        v = np.ascontiguousarray(vecs, dtype=np.float64)
        n = 1 if v.ndim == 1 else v.shape[0]
        out = np.zeros(n)
        check(load().smgpu_jj(self._h, _p(v), n, _p(out)), self._h)
        return out

    def obtr(self, op, vl, vr=None, right=None, symmetric=True, gfactors=None, effcharge=None):
        """<vl_a| O |vr_b> for the one-body M1 (op 0) / E2 (op 1) operator on
        the GPU.  symmetric: eval_moment's expectation-value form on this
        basis (vr defaults to vl); otherwise transit_main's operator from the
        basis of ``right`` (vr) to this one (vl), ΔM = (Mtot - right.Mtot)/2."""
        R = self if right is None else right
        vl = np.ascontiguousarray(np.atleast_2d(np.asarray(vl, dtype=np.float64)))
        vr = vl if vr is None else np.ascontiguousarray(np.atleast_2d(np.asarray(vr, dtype=np.float64)))
        if vl.shape[1] != self.mdim or vr.shape[1] != R.mdim:
            raise ValueError("vector length does not match the basis dimension")
        out = np.zeros((vl.shape[0], vr.shape[0]))
        g = None if gfactors is None else np.ascontiguousarray(gfactors, dtype=np.float64)
        e = None if effcharge is None else np.ascontiguousarray(effcharge, dtype=np.float64)
        check(load().smgpu_obtr(self._h, R._h, int(op), 1 if symmetric else 0, _p(g), _p(e), _p(vl), vl.shape[0],
                                _p(vr), vr.shape[0], _p(out)), self._h)
        return out

    def ec_td(self, vecs):
        """Overlap matrix and transition densities of the sample vectors
        (rows of vecs): prepEC mode "TD" (eigenvector_continuation.jl:212-310)
        on the GPU.  Returns (Nmat, TDs) with TDs[pair] = [OBTD_p, OBTD_n,
        TBTD per snt line] for the pairs i <= j in idx_from_ij order."""
        v = np.ascontiguousarray(np.atleast_2d(np.asarray(vecs, dtype=np.float64)))
        if v.shape[1] != self.mdim:
            raise ValueError("vector length does not match the basis dimension")
        n = v.shape[0]
        ltd = C.c_int()
        check(load().smgpu_ec_td_length(self._h, C.byref(ltd)), self._h)
        nmat = np.zeros((n, n))
        td = np.zeros((n * (n + 1) // 2, ltd.value))
        check(load().smgpu_ec_td(self._h, _p(v), n, _p(nmat), _p(td)), self._h)
        return nmat, td

    # --- compute
    def matvec(self, v, accumulate: bool = False, out=None):
        v = np.ascontiguousarray(v, dtype=np.float64)
        ncols = 1 if v.ndim == 1 else v.shape[0]
        w = np.zeros_like(v) if out is None else out
        check(load().smgpu_matvec(self._h, _p(v), _p(w), ncols, 1 if accumulate else 0), self._h)
        return w

    def solve(self, num_ev, lm=300, ls=20, tol=1e-8, max_restarts=10000, v1=None, want_vecs=False, twoJ=None,
              block=None):
        """Lowest num_ev eigenvalues; twoJ: J-projected (double) Lanczos for
        total angular momentum twoJ/2 (the handle must have Mtot = twoJ);
        block = q: block Lanczos with q vectors per block (TRBL)."""
        nev = min(num_ev, self.mdim)
        ev = np.zeros(nev)
        vecs = np.zeros((nev, self.mdim)) if want_vecs else None
        stats = np.zeros(8, dtype=np.int32)
        v1a = None if v1 is None else np.ascontiguousarray(v1, dtype=np.float64)
        if block is not None:
            rc = load().smgpu_solve_block(self._h, int(block), int(num_ev), int(lm), int(ls), float(tol),
                                          int(max_restarts), _p(v1a), _p(ev), _p(vecs), _p(stats))
        elif twoJ is None:
            rc = load().smgpu_solve(self._h, int(num_ev), int(lm), int(ls), float(tol), int(max_restarts), _p(v1a),
                                    _p(ev), _p(vecs), _p(stats))
        else:
            rc = load().smgpu_solve_J(self._h, int(twoJ), int(num_ev), int(lm), int(ls), float(tol),
                                      int(max_restarts), _p(v1a), _p(ev), _p(vecs), _p(stats))
        if rc not in (_lib.OK, _lib.ERR_NOCONV):
            check(rc, self._h)
        return dict(evals=ev, evecs=vecs, elit=int(stats[0]), n_matvec=int(stats[1]), n_restart=int(stats[2]),
                    converged=bool(stats[3]) and rc == _lib.OK, n_second_pass=int(stats[5]),
                    kernel_launches=int(stats[6]), status=rc)


class MultiSampleProblem:
    """Interaction samples sharing one basis, solved together (an
    ``smgpu_multi`` handle): the sample loop of the reference's ``prepEC``
    (src/ShellModel/eigenvector_continuation.jl:140-177) with one
    multi-sample H·V per Lanczos iteration, FP32-mixed."""

    def __init__(self, snt_files, target_nuc: str):
        L = load()
        files = [os.fsencode(f) for f in snt_files]
        arr = (C.c_char_p * len(files))(*files)
        h = C.c_void_p()
        rc = L.smgpu_multi_create_from_snt(arr, len(files), target_nuc.encode(), C.byref(h))
        _lib.check_multi(rc, None)
        self._h = h
        md, ns, lanes = C.c_longlong(), C.c_int(), C.c_int()
        _lib.check_multi(L.smgpu_multi_dims(h, C.byref(md), C.byref(ns), C.byref(lanes)), h)
        self.mdim = int(md.value)
        self.nsamples = int(ns.value)
        self.lanes = int(lanes.value)

    def close(self):
        if getattr(self, "_h", None):
            load().smgpu_multi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        s = np.zeros(8, dtype=np.int64)
        _lib.check_multi(load().smgpu_multi_stats(self._h, _p(s)), self._h)
        keys = ["updates", "lanes", "table_bytes", "len_pad", "hv_ctas", "hv_threads", "hv_min_ctas", "hv_entry_cache"]
        return dict(zip(keys, map(int, s)))

    def timings(self):
        t = np.zeros(8)
        _lib.check_multi(load().smgpu_multi_timings(self._h, _p(t)), self._h)
        keys = ["setup", "lanczos", "matvec", "capture", "ritz", "solve_wall", "r6", "r7"]
        return dict(zip(keys, map(float, t)))

    def time_matvec(self, reps=20, flush_l2=True):
        """Mean ms per multi-sample H·V launch (all samples), CUDA events."""
        ms = C.c_double()
        _lib.check_multi(load().smgpu_multi_time_matvec(self._h, int(reps), 1 if flush_l2 else 0, C.byref(ms)),
                         self._h)
        return float(ms.value)

    def matvec(self, v, accumulate: bool = False, out=None):
        """w_s = H_s v_s; v has shape (nsamples, mdim)."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        if v.shape != (self.nsamples, self.mdim):
            raise ValueError(f"v must have shape {(self.nsamples, self.mdim)}")
        w = np.zeros_like(v) if out is None else out
        _lib.check_multi(load().smgpu_multi_matvec(self._h, _p(v), _p(w), 1 if accumulate else 0), self._h)
        return w

    def solve(self, num_ev, lm=300, ls=20, tol=1e-8, max_restarts=10000, v1=None, want_vecs=False):
        nev = min(num_ev, self.mdim)
        ev = np.zeros((self.nsamples, nev))
        vecs = np.zeros((self.nsamples, nev, self.mdim)) if want_vecs else None
        stats = np.zeros(8 + 4 * self.nsamples, dtype=np.int32)
        v1a = None if v1 is None else np.ascontiguousarray(v1, dtype=np.float64)
        rc = load().smgpu_multi_solve(self._h, int(num_ev), int(lm), int(ls), float(tol), int(max_restarts),
                                      _p(v1a), _p(ev), _p(vecs), _p(stats))
        if rc not in (_lib.OK, _lib.ERR_NOCONV):
            _lib.check_multi(rc, self._h)
        per = stats[8:].reshape(self.nsamples, 4)
        return dict(evals=ev, evecs=vecs, n_matvec=int(stats[0]), n_restart=int(stats[1]),
                    converged=bool(stats[2]) and rc == _lib.OK, kernel_launches=int(stats[4]),
                    lanes=int(stats[5]), elit=per[:, 0].astype(int), sample_converged=per[:, 1].astype(bool),
                    n_second_pass=per[:, 2].astype(int), status=rc)


class BatchProblem:
    """Independent problems of uneven dimension solved together (an
    ``smgpu_batch`` handle): many ``main_sm`` set-ups
    (src/ShellModel/shellmodel_main.jl:89-281), one per (snt, nucleus) pair,
    iterated in lockstep in the FP32-mixed form."""

    def __init__(self, problems):
        """problems: sequence of (snt path, nucleus name)."""
        L = load()
        snts = [os.fsencode(p[0]) for p in problems]
        nucs = [p[1].encode() for p in problems]
        a = (C.c_char_p * len(snts))(*snts)
        b = (C.c_char_p * len(nucs))(*nucs)
        h = C.c_void_p()
        rc = L.smgpu_batch_create_from_snt(a, b, len(snts), C.byref(h))
        _lib.check_batch(rc, None)
        self._h = h
        tot, n = C.c_longlong(), C.c_int()
        _lib.check_batch(L.smgpu_batch_dims(h, C.byref(tot), C.byref(n), None), h)
        self.nprob = int(n.value)
        self.total_mdim = int(tot.value)
        self.mdims = np.zeros(self.nprob, dtype=np.int64)
        _lib.check_batch(L.smgpu_batch_dims(h, None, None, _p(self.mdims)), h)
        self.moff = np.concatenate([[0], np.cumsum(self.mdims)[:-1]]).astype(np.int64)

    def close(self):
        if getattr(self, "_h", None):
            load().smgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def split(self, x):
        """Concatenated vector -> list of per-problem vectors."""
        return [x[o:o + m] for o, m in zip(self.moff, self.mdims)]

    def stats(self):
        s = np.zeros(9, dtype=np.int64)
        _lib.check_batch(load().smgpu_batch_stats(self._h, _p(s)), self._h)
        keys = ["updates", "problems", "chunks", "hv_tasks", "hv_threads", "hv_rows", "hv_min_ctas", "table_bytes",
                "hv_staged"]
        return dict(zip(keys, map(int, s)))

    def timings(self):
        t = np.zeros(8)
        _lib.check_batch(load().smgpu_batch_timings(self._h, _p(t)), self._h)
        keys = ["setup", "lanczos", "matvec", "capture", "ritz", "solve_wall", "r6", "r7"]
        return dict(zip(keys, map(float, t)))

    def time_matvec(self, reps=20, flush_l2=True):
        """Mean ms per batched H·v launch (all problems), CUDA events."""
        ms = C.c_double()
        _lib.check_batch(load().smgpu_batch_time_matvec(self._h, int(reps), 1 if flush_l2 else 0, C.byref(ms)),
                         self._h)
        return float(ms.value)

    def matvec(self, v, accumulate: bool = False, out=None):
        """w_p = H_p v_p on the concatenated vector (total_mdim entries)."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        if v.shape != (self.total_mdim,):
            raise ValueError(f"v must have shape ({self.total_mdim},)")
        w = np.zeros_like(v) if out is None else out
        _lib.check_batch(load().smgpu_batch_matvec(self._h, _p(v), _p(w), 1 if accumulate else 0), self._h)
        return w

    def solve(self, num_ev, lm=300, ls=20, tol=1e-8, max_restarts=10000, v1=None, want_vecs=False):
        ev = np.zeros((self.nprob, num_ev))
        vecs = np.zeros(num_ev * self.total_mdim) if want_vecs else None
        stats = np.zeros(8 + 4 * self.nprob, dtype=np.int32)
        v1a = None if v1 is None else np.ascontiguousarray(v1, dtype=np.float64)
        rc = load().smgpu_batch_solve(self._h, int(num_ev), int(lm), int(ls), float(tol), int(max_restarts),
                                      _p(v1a), _p(ev), _p(vecs), _p(stats))
        if rc not in (_lib.OK, _lib.ERR_NOCONV):
            _lib.check_batch(rc, self._h)
        per = stats[8:].reshape(self.nprob, 4)
        evecs = None
        if want_vecs:
            evecs = [vecs[num_ev * o:num_ev * (o + m)].reshape(num_ev, m) for o, m in zip(self.moff, self.mdims)]
        return dict(evals=ev, evecs=evecs, n_matvec=int(stats[0]), n_restart=int(stats[1]),
                    converged=bool(stats[2]) and rc == _lib.OK, kernel_launches=int(stats[4]),
                    elit=per[:, 0].astype(int), problem_converged=per[:, 1].astype(bool),
                    n_second_pass=per[:, 2].astype(int), status=rc)


def l2_read_bandwidth(nbytes=32 << 20, reps=50):
    """GB/s of the library's read kernel on an L2-resident device buffer of
    nbytes (the ceiling of the L2-resident H·v kernels)."""
    g = C.c_double()
    check(load().smgpu_l2_read_bandwidth(int(nbytes), int(reps), C.byref(g)), None)
    return float(g.value)


def J_from_JJ1(JJ, tol=1.0e-6):
    """J from <J^2> = J(J+1) (shellmodel_main.jl:1105-1113): the first
    half-integer J in 0..50 within tol, else -1."""
    for J2 in range(0, 101):
        hJ = 0.5 * J2
        if abs(hJ * (hJ + 1.0) - JJ) < tol:
            return hJ
    return -1.0


def main_sm(sntf, target_nuc, num_ev, target_J, save_wav=False, q=1, is_block=False, is_show=False,
            num_history=3, lm=300, ls=20, tol=1.0e-8, in_wf="", mdimmode=False, print_evec=False,
            calc_moment=False, calc_entropy=False, visualize_occ=False, gfactors=(1.0, 0.0, 5.586, -3.826),
            effcharge=(1.5, 0.5), truncation_scheme="", truncated_jocc=None, debugmode="", precision=FP64,
            max_restarts=10000, verbose=True):
    """Lowest ``num_ev`` eigenvalues of the valence-space Hamiltonian.

    Same positional arguments and keyword names as the reference's ``main_sm``
    (src/ShellModel/shellmodel_main.jl:89-92).  ``precision`` selects the
    plain FP64 form or the FP32-mixed form.  Features of the reference outside
    the eigensolver path raise ``NotImplementedError``.
    """
    tJ = None
    if target_J is not None and len(target_J) > 0:
        # shellmodel_main.jl:109-116: one target 2J; the basis has Mtot = 2J
        if len(target_J) > 1:
            raise ValueError("Invalid `target_J` Multiple J is not supported now.")
        tJ = int(target_J[0])
    unsupported = dict(block_with_target_J=is_block and tJ is not None, calc_entropy=calc_entropy,
                       visualize_occ=visualize_occ, print_evec=print_evec, truncation=bool(truncation_scheme),
                       debugmode=bool(debugmode))
    bad = [k for k, v in unsupported.items() if v]
    if bad:
        raise NotImplementedError("not supported by the GPU eigensolver: " + ", ".join(bad))
    if num_history != 3:
        raise NotImplementedError("num_history other than 3")
    P = ShellModelProblem(sntf, target_nuc, precision, twoJ=tJ)
    if verbose:
        print(f"{target_nuc:>6s}  mdim: {P.mdim:12d} ({np.log10(max(P.mdim, 1)):5.2f}) "
              + (f" 2J={tJ}" if tJ is not None else ""))
    if mdimmode:
        P.close()
        return None
    v1 = None
    if in_wf:
        # read_appwav: the first vector (q of them for a block) starts the Lanczos
        from .wav import read_wav
        vs, _ = read_wav(in_wf, P.mdim, all=True)
        if is_block:
            if len(vs) < q:
                raise ValueError("#(appwav) must be >= q")
            v1 = np.array(vs[:q])
        else:
            v1 = vs[0]
    r = P.solve(num_ev, lm=lm, ls=ls, tol=tol, max_restarts=max_restarts, v1=v1,
                want_vecs=verbose or save_wav or calc_moment,
                twoJ=tJ, block=int(q) if is_block else None)
    en = list(map(float, r["evals"]))
    totJs = None
    if r["status"] == _lib.OK and r["evecs"] is not None:
        # J labels of the Ritz vectors (shellmodel_main.jl:226-240)
        totJs = [J_from_JJ1(x) for x in P.jj(r["evecs"])]
    tx_mom = ""
    if calc_moment and totJs is not None:
        # eval_moment (:242-246, transit.jl:702-765)
        from .transit import eval_moment
        tx_mom = eval_moment(P, r["evecs"], totJs, gfactors, effcharge)["text"]
    if save_wav and totJs is not None:
        # writeRitzvecs to ./<nucleus>_<interaction>.wav (:248-253)
        from .wav import write_wav
        csnt = os.path.basename(sntf).split(".")[0]
        oupf = f"./{target_nuc}_{csnt}.wav" if tJ is None else f"./{target_nuc}_{csnt}_j{tJ}.wav"
        write_wav(oupf, P.mtot2, en, [int(2 * j) for j in totJs], r["evecs"])
    if verbose and tJ is not None:
        # :261-264
        print(f"2J= {int(2 * totJs[0]) if totJs else tJ}  En." + " ".join(f"{x:12.5f}" for x in en))
    elif verbose:
        if totJs is not None:
            print("J " + str(totJs))
        print("En. " + " ".join(f"{x:10.4f}" for x in en))
        print("Ex. " + " ".join(f"{x - en[0]:10.4f}" for x in en))
        if is_show:
            print(P.timings())
    if verbose and tx_mom != "":
        print(tx_mom)
    P.close()
    if r["status"] == _lib.ERR_NOCONV:
        raise RuntimeError(f"Lanczos did not converge within {max_restarts} restarts")
    return en
