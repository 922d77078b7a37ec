"""ctypes front end of the CPU oracle — test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, and only as the checker / the timed CPU restatement of
NuclearToolkit.jl's ``main_sm`` path (src/ShellModel/shellmodel_main.jl:89-281,
src/ShellModel/lanczos_methods.jl:1-307).  The GPU library never imports it.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_char_p, C.c_char_p]
        L.orc_destroy.argtypes = [vp]
        L.orc_last_error.restype = C.c_char_p
        L.orc_mdim.restype = C.c_longlong
        L.orc_mdim.argtypes = [vp]
        L.orc_nblocks.argtypes = [vp]
        L.orc_info.argtypes = [vp, C.c_void_p]
        L.orc_blocks.argtypes = [vp] + [C.c_void_p] * 5
        L.orc_sds.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.orc_2b_count.restype = C.c_longlong
        L.orc_2b_count.argtypes = [vp, C.c_int]
        L.orc_2b_export.argtypes = [vp, C.c_int] + [C.c_void_p] * 4
        L.orc_pn_count.restype = C.c_longlong
        L.orc_pn_count.argtypes = [vp, C.c_int]
        L.orc_pn_export.argtypes = [vp, C.c_int] + [C.c_void_p] * 6
        L.orc_ndelM.argtypes = [vp]
        L.orc_vpn_count.restype = C.c_longlong
        L.orc_vpn_count.argtypes = [vp]
        L.orc_vpn_export.argtypes = [vp] + [C.c_void_p] * 4
        L.orc_v1_count.restype = C.c_longlong
        L.orc_v1_count.argtypes = [vp, C.c_int]
        L.orc_v1_export.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_spe_diag.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.orc_operate_H.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.orc_jj.argtypes = [vp, C.c_void_p]
        L.orc_jj.restype = C.c_double
        L.orc_nnz.restype = C.c_longlong
        L.orc_nnz.argtypes = [vp]
        L.orc_start_vector.argtypes = [C.c_longlong, C.c_ulonglong, C.c_void_p]
        L.orc_trl.restype = C.c_int
        L.orc_trl.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p,
                              C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.orc_trbl.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p,
                               C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_create_M.restype = vp
        L.orc_create_M.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.orc_sym_eig.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_trl_sample.restype = C.c_int
        L.orc_trl_sample.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p]
        L.orc_clebsch.restype = C.c_double
        L.orc_clebsch.argtypes = [C.c_int] * 6
        L.orc_obtr.restype = C.c_int
        L.orc_obtr.argtypes = [vp, vp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                               C.c_void_p, C.c_int, C.c_void_p]
        for f in ("orc_wigner3j", "orc_wigner6j"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.c_int] * 6
        L.orc_radius_power.restype = C.c_double
        L.orc_radius_power.argtypes = [C.c_int] * 5 + [C.c_double]
        L.orc_ec_td_length.restype = C.c_int
        L.orc_ec_td_length.argtypes = [vp]
        L.orc_ec_td.restype = C.c_int
        L.orc_ec_td.argtypes = [vp, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def clebsch(tj1, tm1, tj2, tm2, tJ, tM):
    return lib().orc_clebsch(tj1, tm1, tj2, tm2, tJ, tM)


def wigner3j(*a):
    return lib().orc_wigner3j(*map(int, a))


def wigner6j(*a):
    return lib().orc_wigner6j(*map(int, a))


def radius_power(k, n1, l1, n2, l2, bpar):
    return lib().orc_radius_power(int(k), int(n1), int(l1), int(n2), int(l2), float(bpar))


def sym_eig(A):
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    w = np.zeros(n)
    Z = np.zeros((n, n), order="F")
    lib().orc_sym_eig(n, _p(A), _p(w), _p(Z))
    return w, Z


def start_vector(mdim: int, seed: int = 1234):
    v = np.zeros(mdim)
    lib().orc_start_vector(mdim, seed, _p(v))
    return v


class OracleProblem:
    """One shell-model problem set up exactly as ``main_sm`` does it
    (readsmsnt → occ → prep_Hamil_T1 → prep_Hamil_pn → prep_pn)."""

    def __init__(self, sntf: str, nuc: str, mtot2=None):
        """mtot2: doubled total M of the basis (None: A mod 2, as main_sm
        without target_J; target_J = [tJ] uses mtot2 = tJ)."""
        L = lib()
        if mtot2 is None:
            self._h = L.orc_create(os.fsencode(sntf), nuc.encode())
        else:
            self._h = L.orc_create_M(os.fsencode(sntf), nuc.encode(), int(mtot2))
        if not self._h:
            raise ValueError("oracle: " + L.orc_last_error().decode())
        self.mdim = int(L.orc_mdim(self._h))
        self.nblocks = int(L.orc_nblocks(self._h))
        info = np.zeros(8, dtype=np.int32)
        L.orc_info(self._h, _p(info))
        self.A, self.Z, self.N, self.vp, self.vn, self.Mtot, self.lp_m, self.ln_m = map(int, info)
        nb = self.nblocks
        self.tdims = np.zeros(nb + 1, dtype=np.int64)
        self.np_ = np.zeros(nb, dtype=np.int32)
        self.nn_ = np.zeros(nb, dtype=np.int32)
        self.Mp = np.zeros(nb, dtype=np.int32)
        self.Mn = np.zeros(nb, dtype=np.int32)
        if nb:
            L.orc_blocks(self._h, _p(self.tdims), _p(self.np_), _p(self.nn_), _p(self.Mp), _p(self.Mn))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def sds(self):
        p = np.zeros(int(self.np_.sum()), dtype=np.int64)
        n = np.zeros(int(self.nn_.sum()), dtype=np.int64)
        lib().orc_sds(self._h, _p(p), _p(n))
        return p, n

    def jumps_2b(self, which: int):
        L = lib()
        c = L.orc_2b_count(self._h, which)
        blk = np.zeros(c, dtype=np.int32)
        i = np.zeros(c, dtype=np.int32)
        f = np.zeros(c, dtype=np.int32)
        coef = np.zeros(c)
        L.orc_2b_export(self._h, which, _p(blk), _p(i), _p(f), _p(coef))
        return blk, i, f, coef

    def jumps_pn(self, which: int):
        L = lib()
        c = L.orc_pn_count(self._h, which)
        arrs = [np.zeros(c, dtype=np.int32) for _ in range(6)]
        L.orc_pn_export(self._h, which, *[_p(a) for a in arrs])
        return tuple(arrs)  # bi, bf, nth, i, f, phase

    def vpn(self):
        L = lib()
        nd = L.orc_ndelM(self._h)
        c = L.orc_vpn_count(self._h)
        delMs = np.zeros(nd, dtype=np.int32)
        idx = np.zeros(c, dtype=np.int32)
        abcd = np.zeros((c, 4), dtype=np.int64)
        V = np.zeros(c)
        L.orc_vpn_export(self._h, _p(delMs), _p(idx), _p(abcd), _p(V))
        return delMs, idx, abcd, V

    def v1(self, which: int):
        L = lib()
        c = L.orc_v1_count(self._h, which)
        abcd = np.zeros((c, 4), dtype=np.int64)
        V = np.zeros(c)
        L.orc_v1_export(self._h, which, _p(abcd), _p(V))
        return abcd, V

    def spe_diag(self):
        ep = np.zeros(int(self.np_.sum()))
        en = np.zeros(int(self.nn_.sum()))
        lib().orc_spe_diag(self._h, _p(ep), _p(en))
        return ep, en

    def operate_H(self, wf):
        wf = np.ascontiguousarray(wf, dtype=np.float64)
        twf = np.zeros_like(wf)
        lib().orc_operate_H(self._h, _p(wf), _p(twf))
        return twf

    def jj(self, v) -> float:
        """<v|J^2|v>/<v|v> by the ladder operator (J^2 = J-J+ + M(M+1))."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        return float(lib().orc_jj(self._h, _p(v)))

    def trbl(self, q, num_ev, lm=300, ls=20, tol=1e-8, max_restart=10000, v1=None, seed=1234, want_vecs=False):
        """Block thick-restart Lanczos (TRBL) with q vectors per block."""
        L = lib()
        k = min(num_ev, self.mdim)
        ev = np.zeros(k)
        vecs = np.zeros((k, self.mdim)) if want_vecs else None
        stats = np.zeros(4, dtype=np.int32)
        v1p = None
        if v1 is not None:
            v1 = np.ascontiguousarray(v1, dtype=np.float64)
            v1p = _p(v1)
        if L.orc_trbl(self._h, q, num_ev, lm, ls, tol, max_restart, v1p, seed, _p(ev),
                      _p(vecs) if want_vecs else None, _p(stats)) != 0:
            raise RuntimeError("oracle TRBL: " + L.orc_last_error().decode())
        return dict(evals=ev, evecs=vecs, elit=int(stats[0]), n_hv=int(stats[1]), n_restart=int(stats[2]),
                    converged=bool(stats[3]))

    def nnz(self) -> int:
        """Structural non-zeros of H (distinct (row, col) pairs, diagonal included)."""
        return int(lib().orc_nnz(self._h))

    def dense_H(self):
        n = self.mdim
        H = np.zeros((n, n))
        e = np.zeros(n)
        for j in range(n):
            e[:] = 0.0
            e[j] = 1.0
            H[:, j] = self.operate_H(e)
        return H

    def trl_sample(self, num_ev, lm, ls, tol, max_hv):
        """Time the first `max_hv` H·v iterations of TRL (restarts included)."""
        out = np.zeros(6)
        if lib().orc_trl_sample(self._h, num_ev, lm, ls, tol, max_hv, _p(out)) != 0:
            raise RuntimeError("oracle TRL sample: " + lib().orc_last_error().decode())
        return dict(t_hv=out[0], t_reorth=out[1], t_restart=out[2], t_total=out[3], n_hv=int(out[4]),
                    n_restart=int(out[5]))

    def trl(self, num_ev, lm=300, ls=20, tol=1e-8, max_restart=10000, v1=None, seed=1234, want_vecs=False,
            eval_jj=None):
        """TRL; eval_jj = J(J+1) turns on the J-projected double Lanczos
        (target_J; the basis must have M = J)."""
        L = lib()
        k = min(num_ev, self.mdim)
        ev = np.zeros(k)
        vecs = np.zeros((k, self.mdim)) if want_vecs else None
        stats = np.zeros(4, dtype=np.int32)
        times = np.zeros(3)
        v1p = None
        if v1 is not None:
            v1 = np.ascontiguousarray(v1, dtype=np.float64)
            v1p = _p(v1)
        rc = L.orc_trl(self._h, num_ev, lm, ls, tol, max_restart, v1p, seed, _p(ev),
                       _p(vecs) if want_vecs else None, _p(stats), _p(times),
                       -1.0 if eval_jj is None else float(eval_jj))
        if rc != 0:
            raise RuntimeError("oracle TRL: " + L.orc_last_error().decode())
        return dict(evals=ev, evecs=vecs, elit=int(stats[0]), n_hv=int(stats[1]), n_restart=int(stats[2]),
                    converged=bool(stats[3]), t_hv=float(times[0]), t_reorth=float(times[1]),
                    t_total=float(times[2]))

    def obtr(self, op, vl, vr=None, right=None, symmetric=True, gfactors=(1.0, 0.0, 5.586, -3.826),
             effcharge=(1.5, 0.5)):
        """<vl_a| O |vr_b> for op 0 (M1) / 1 (E2): symmetric -> eval_moment's
        operator (transit.jl:82-284), else transit_main's between this basis
        (left) and ``right`` (transit.jl:286-531)."""
        R = right if right is not None else self
        vl = np.ascontiguousarray(np.atleast_2d(np.asarray(vl, dtype=np.float64)))
        vr = vl if vr is None else np.ascontiguousarray(np.atleast_2d(np.asarray(vr, dtype=np.float64)))
        out = np.zeros((vl.shape[0], vr.shape[0]))
        g = np.asarray(gfactors, dtype=np.float64)
        e = np.asarray(effcharge, dtype=np.float64)
        rc = lib().orc_obtr(self._h, R._h, int(op), 1 if symmetric else 0, _p(g), _p(e), _p(vl), vl.shape[0], _p(vr),
                            vr.shape[0], _p(out))
        if rc != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return out

    def ec_td(self, vecs):
        """prepEC "TD" (eigenvector_continuation.jl:212-310): the overlap
        matrix and, per pair i <= j (idx_from_ij order), [OBTD_p, OBTD_n,
        TBTD per snt line] from the restatement of calcOBTD / prepTBTD /
        calcTBTD (:1035-1380)."""
        v = np.ascontiguousarray(np.atleast_2d(np.asarray(vecs, dtype=np.float64)))
        n = v.shape[0]
        ltd = lib().orc_ec_td_length(self._h)
        nmat = np.zeros((n, n))
        td = np.zeros((n * (n + 1) // 2, ltd))
        if lib().orc_ec_td(self._h, _p(v), n, _p(nmat), _p(td)) != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return nmat, td
