"""Electromagnetic moments and transitions over libsmgpu — the host side of
NuclearToolkit.jl's src/ShellModel/transit.jl.

The one-body M1 / E2 operators are built and applied by the library
(``smgpu_obtr``: O·v and the overlaps on the GPU in FP64); this module holds
the host arithmetic the reference wraps around them: the 3j selection factors,
reduced matrix elements, B values and the printed lines of ``eval_moment``
(transit.jl:702-765) and ``transit_main`` (:561-700).
"""
import math

import numpy as np

from . import _lib
from .shellmodel import FP64, ShellModelProblem

M1, E2 = 0, 1
GFACTORS = (1.0, 0.0, 5.586, -3.826)  # g_l(p), g_l(n), g_s(p), g_s(n)
EFFCHARGE = (1.5, 0.5)                # e_p, e_n
C_MOM_MU = math.sqrt(4.0 * math.pi / 3.0)
C_MOM_Q = math.sqrt(16.0 * math.pi / 5.0)


def wigner3j(tj1, tj2, tj3, tm1, tm2, tm3):
    """(j1 j2 j3; m1 m2 m3) with doubled arguments (library host code)."""
    return _lib.load().smgpu_wigner3j(int(tj1), int(tj2), int(tj3), int(tm1), int(tm2), int(tm3))


def wigner6j(tj1, tj2, tj3, tj4, tj5, tj6):
    """{j1 j2 j3; j4 j5 j6} with doubled arguments (library host code)."""
    return _lib.load().smgpu_wigner6j(int(tj1), int(tj2), int(tj3), int(tj4), int(tj5), int(tj6))


def tri_relation(tja, tjb, tjc):
    """Triangle condition on doubled angular momenta (transit.jl:33-43)."""
    return not (tja + tjb < tjc or tjb + tjc < tja or tjc + tja < tjb or abs(tja - tjb) > tjc
                or abs(tjb - tjc) > tja or abs(tjc - tja) > tjb)


def _sign(e2):
    """(-1)^(e2/2) for an even doubled exponent."""
    return -1.0 if (e2 // 2) % 2 else 1.0


def eval_moment(P: ShellModelProblem, Rvecs, totJs, gfactors=GFACTORS, effcharge=EFFCHARGE):
    """Magnetic dipole and electric quadrupole moments of the states Rvecs
    (rows) with J labels totJs, as eval_moment (transit.jl:702-765) prints
    them: "mu (n=k) <mu>" and "Q (n=k) <Q>" for every state whose 3j selection
    factor is non-zero (J = -1 states are skipped).  Returns the text and the
    per-state values (NaN where nothing is printed)."""
    V = np.atleast_2d(np.asarray(Rvecs, dtype=np.float64))
    n = V.shape[0]
    m2 = P.mtot2  # Mi = Mf = Mtot/2
    omu = 0
    mu_mat = P.obtr(M1, V, symmetric=True, gfactors=gfactors, effcharge=effcharge)
    q_mat = P.obtr(E2, V, symmetric=True, gfactors=gfactors, effcharge=effcharge)
    mus = np.full(n, np.nan)
    qs = np.full(n, np.nan)
    text = ""
    for k in range(n):
        tJ = int(2 * totJs[k])
        if tJ < 0:
            continue
        tx = ""
        sel = wigner3j(tJ, 2, tJ, -m2, 2 * omu, m2)
        if sel != 0.0:
            cg = wigner3j(tJ, 2, tJ, -tJ, 2 * omu, tJ) / sel
            mus[k] = _sign(tJ - m2) * mu_mat[k, k] * cg * C_MOM_MU
            tx += f"mu (n={k + 1}) " + f"{mus[k]:12.5f} " + "\t"
        sel = wigner3j(tJ, 4, tJ, -m2, 2 * omu, m2)
        if sel != 0.0:
            cg = wigner3j(tJ, 4, tJ, -tJ, 2 * omu, tJ) / sel
            qs[k] = q_mat[k, k] * cg * C_MOM_Q * _sign(tJ - m2)
            tx += f"Q (n={k + 1}) " + f"{qs[k]:12.5f} "
        if tx != "":
            text += tx + "\n"
    return dict(text=text, mu=mus, Q=qs)


def transit_main(sntf, target_nuc, jl2, jr2, in_wfs, num_ev_l=100, num_ev_r=100, q=1, is_block=False, is_show=True,
                 calc_EM=True, gfactors=GFACTORS, eff_charge=EFFCHARGE, verbose=True):
    """M1 and E2 reduced matrix elements and B values between the states of
    two .wav files (transit.jl:561-700): the left states have J = jl2/2 and
    Mtot = jl2, the right ones jr2 (doubled; swapped when jl2 < jr2, as the
    reference does).  Prints the reference's lines and returns them with the
    reduced matrix elements (rows: left states, columns: right states)."""
    from .wav import read_wav

    if len(in_wfs) == 0:
        raise ValueError("input wfs must be specified")
    widx = [0, 1]
    if jl2 < jr2:
        jl2, jr2 = jr2, jl2
        widx = [1, 0]
    lines = []

    def out(s):
        lines.append(s)
        if verbose:
            print(s)

    PL = ShellModelProblem(sntf, target_nuc, FP64, twoJ=jl2)
    PR = ShellModelProblem(sntf, target_nuc, FP64, twoJ=jr2)
    try:
        out(f"wfl: {in_wfs[widx[0]]}")
        if in_wfs[widx[0]] != in_wfs[widx[1]]:
            out(f"wfr: {in_wfs[widx[1]]}")
        out(f"mdims J2={jl2} {PL.mdim} J2={jr2} {PR.mdim} Mtots=({jl2}, {jr2})")
        wfs_l, _ = read_wav(in_wfs[widx[0]], PL.mdim, all=True)
        wfs_r, _ = read_wav(in_wfs[widx[1]], PR.mdim, all=True)
        wfs_l = np.asarray(wfs_l)
        wfs_r = np.asarray(wfs_r)
        omu = (jl2 - jr2) // 2
        if omu > 2:
            out("Only the M1&E2 are supported now")
            return dict(lines=lines)
        same = in_wfs[0] == in_wfs[1]
        nr = min(len(wfs_r), num_ev_r)
        nl = min(len(wfs_l), num_ev_l) if calc_EM else min(len(wfs_l), nr)
        res = dict(lines=lines)
        for lam, op, name, cm, key in ((1, M1, "M1", C_MOM_MU, "gm"), (2, E2, "E2", C_MOM_Q, "eQ")):
            if not tri_relation(jl2, jr2, 2 * lam):
                continue
            Jf, Ji, Mf, Mi = jl2, jr2, jl2, jr2  # doubled
            sel = wigner3j(Jf, 2 * lam, Ji, -Mf, 2 * omu, Mi)
            sign = _sign(Jf - Mf)
            cg = wigner3j(Ji, 2 * lam, Jf, -Ji, 2 * omu, Jf)
            if sel == 0.0 or nr == 0 or nl == 0:
                continue
            mat = PL.obtr(op, wfs_l[:nl], wfs_r[:nr], right=PR, symmetric=False, gfactors=gfactors,
                          effcharge=eff_charge)
            mred = mat / sel
            res["Mred_" + name] = mred
            for r in range(nr):
                if calc_EM:
                    for l_ in range(nl):
                        M = mred[l_, r]
                        B_l = M * M / (Ji + 1)
                        B_r = M * M / (Jf + 1)
                        tx = f"Mred.({name}) ({l_ + 1},{r + 1}) " + f"{M:9.3f} " + "  "
                        tx += (f"B({name}) ({l_ + 1}<={r + 1}) " + f"{B_l:9.3f} " + f" B({name}) ({l_ + 1}=>{r + 1}) "
                               + f"{B_r:9.3f} ")
                        if same and l_ == r:
                            tx += f" <{key}>= " + f"{M * cg * cm * sign:9.3f} "
                        out(tx)
                else:
                    M = mred[r, r]
                    out(f" <{key}>= " + f"{M * cg * cm * sign:9.3f} ")
        return res
    finally:
        PL.close()
        PR.close()
