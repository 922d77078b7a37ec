"""Eigenvector continuation over libsmgpu — the host side of
NuclearToolkit.jl's src/ShellModel/eigenvector_continuation.jl.

``prep_ec`` mode "sample" solves the J-projected eigenproblem of every
interaction on the GPU and writes the sample .wav files; mode "TD" computes
the overlap matrix and the one- and two-body transition densities of all
sample vectors on the GPU (``smgpu_ec_td``) and writes the reference's
tdmat file.  ``solve_ec`` reads it back, forms H = Σ ME·TD for each
interaction and solves the small generalized eigenproblem H v = λ N v on the
host, as the reference does.
"""
import os
import re
import struct

import numpy as np

from .shellmodel import FP64, J_from_JJ1, ShellModelProblem
from .wav import read_wav_full, write_wav


def _mass_number(target_nuc):
    m = re.search(r"[0-9]+", target_nuc)
    if not m:
        raise ValueError("no mass number in nucleus name")
    return int(m.group(0))


def read_snt_mes(sntf, target_nuc):
    """SPEs and the TBMEs of the snt lines in file order, mass-scaled as
    readsmsnt does (shellmodel_main.jl:293-365): (SPE_p, SPE_n, oTBMEs)."""
    A = _mass_number(target_nuc)
    lines = []
    with open(sntf) as f:
        for raw in f:
            t = raw.strip()
            if t.startswith("!") or t.startswith("#"):
                continue
            lines.append(t)
    k = 0
    hd = lines[k].split()
    k += 1
    lp, ln = int(hd[0]), int(hd[1])
    k += lp + ln
    nsp = int(lines[k].split()[0])
    k += 1
    spe_p = np.zeros(lp)
    spe_n = np.zeros(ln)
    for _ in range(nsp):
        t = lines[k].split()
        k += 1
        j = int(t[0])
        if j <= lp:
            spe_p[j - 1] = float(t[2])
        else:
            spe_n[j - lp - 1] = float(t[2])
    ht = lines[k].split()
    k += 1
    ntbme, massop, Aref = int(ht[0]), int(ht[1]), float(ht[2])
    pw = float(ht[3]) if len(ht) > 3 else 0.0
    tb = np.zeros(ntbme)
    for i in range(ntbme):
        v = float(lines[k].split()[5])
        k += 1
        if massop == 1:
            v *= (A / Aref) ** pw
        tb[i] = v
    return spe_p, spe_n, tb


def idx_from_ij(i, j, Dim):
    """shellmodel_main.jl:1297-1299 (1-based)."""
    return (Dim + 1) * (i - 1) - (i * (i - 1)) // 2 + j - i + 1


def read_rvecs(mdim, inpf, tJ, vecs, wfinfos, num=100):
    """readRvecs! (eigenvector_continuation.jl:83-100): the first min(num,
    neig) vectors of a .wav whose 2J label is tJ."""
    e, jj, V, _ = read_wav_full(inpf, mdim)
    n = min(num, len(e))
    for i in range(n):
        if int(jj[i]) == tJ:
            vecs.append(np.array(V[i]))
            wfinfos.append([inpf, i + 1, len(vecs)])


def _print_vec(label, v):
    print(label + " " + " ".join(f"{x:12.5f}" for x in v))


def prep_ec(Hs, target_nuc, num_ev, num_ECsample, tJ, mode, num_history=3, lm=500, ls=30, tol=1.0e-8, q=1,
            path_to_samplewav="", calc_moment=True, save_wav=False, tdmatdir="./tdmat/",
            gfactors=(1.0, 0.0, 5.586, -3.826), effcharge=(1.5, 0.5), debugmode="", doublelanczos=True,
            is_show=False, verbose=True):
    """prepEC (eigenvector_continuation.jl:102-310).  mode "sample": for each
    interaction of Hs, the lowest num_ev states of total angular momentum
    tJ/2 (J-projected Lanczos when doublelanczos), printed with their J
    labels and moments and written to
    <path_to_samplewav><nucleus>_<interaction>_j<tJ>.wav when save_wav.
    mode "TD": reads <path_to_samplewav><nucleus>_tmp_<k>_j<tJ>.wav for
    k < num_ECsample, computes Nmat and the transition densities on the GPU
    and writes <tdmatdir><nucleus>_J<tJ>.dat and the wfinfos file."""
    if not isinstance(tJ, (int, np.integer)):
        raise ValueError("targetJ must be integer!!")
    if num_history != 3 or q != 1 or debugmode:
        raise NotImplementedError("prep_ec supports num_history = 3, q = 1 and no debugmode")
    A = _mass_number(target_nuc)
    Mtot = int(tJ)
    if A % 2 != Mtot % 2:
        raise ValueError("invalid target J")
    out = dict(mode=mode)
    if mode == "sample":
        out["samples"] = []
        for sntf in Hs:
            if verbose:
                print(f"sntf: {sntf}")
            P = ShellModelProblem(sntf, target_nuc, FP64, twoJ=Mtot)
            try:
                r = P.solve(num_ev, lm=lm, ls=ls, tol=tol, twoJ=Mtot if doublelanczos else None, want_vecs=True)
                if not r["converged"]:
                    raise RuntimeError(f"Lanczos did not converge for {sntf}")
                en = list(map(float, r["evals"]))
                totJs = [J_from_JJ1(x) for x in P.jj(r["evecs"])]
                if verbose:
                    print("J " + str(totJs))
                    print("En. " + "".join(f"{x:24.15f} " for x in en))
                csnt = os.path.basename(sntf).split(".")[0]
                oupf = path_to_samplewav + target_nuc + "_" + csnt + ".wav"
                if tJ != -1:
                    oupf = path_to_samplewav + target_nuc + "_" + csnt + "_j" + str(tJ) + ".wav"
                if save_wav:
                    write_wav(oupf, Mtot, en, [int(2 * j) for j in totJs], r["evecs"])
                tx = ""
                if calc_moment:
                    from .transit import eval_moment
                    tx = eval_moment(P, r["evecs"], totJs, gfactors, effcharge)["text"]
                    if verbose and tx != "":
                        print(tx, end="")
                if verbose:
                    print("")
                out["samples"].append(dict(snt=sntf, evals=en, J=totJs, wav=oupf if save_wav else None, moments=tx))
            finally:
                P.close()
        return out
    if mode != "TD":
        raise ValueError(f"unknown prepEC mode {mode}")
    os.makedirs(tdmatdir, exist_ok=True)
    P = ShellModelProblem(Hs[0], target_nuc, FP64, twoJ=Mtot)
    try:
        svecs, wfinfos = [], []
        for fidx in range(num_ECsample):
            inpf = path_to_samplewav + target_nuc + f"_tmp_{fidx}" + "_j" + str(tJ) + ".wav"
            read_rvecs(P.mdim, inpf, tJ, svecs, wfinfos, num=num_ev)
        with open(os.path.join(tdmatdir, "wfinfos_" + target_nuc + "_J" + str(tJ) + ".dat"), "w") as f:
            for inpf, nth, k in wfinfos:
                f.write(f"{os.path.basename(inpf)} nth= {nth} TDmatidx  {k}\n")
        Dim = len(svecs)
        if verbose:
            print(f"Dim {Dim}")
        if Dim == 0:
            raise ValueError("no sample vectors with the target J")
        Nmat, TDs = P.ec_td(np.array(svecs))
        oupf = os.path.join(tdmatdir, target_nuc + "_J" + str(tJ) + ".dat")
        with open(oupf, "wb") as f:
            f.write(struct.pack("<qqq", Dim, TDs.shape[0], TDs.shape[1]))
            for i in range(1, Dim + 1):
                for j in range(i, Dim + 1):
                    Nij = idx_from_ij(i, j, Dim)
                    f.write(struct.pack("<qqqd", i, j, Nij, Nmat[i - 1, j - 1]))
                    f.write(np.ascontiguousarray(TDs[Nij - 1], dtype="<f8").tobytes())
        out.update(Dim=Dim, Nmat=Nmat, TDs=TDs, tdmat=oupf)
        return out
    finally:
        P.close()


def read_tdmat(inpf):
    """read_tdmat (eigenvector_continuation.jl:43-61): Dim, number of pairs,
    lTD, Nmat, the (i, j, Nij) of each pair and its TD vector."""
    with open(inpf, "rb") as f:
        Dim, npair, lTD = struct.unpack("<qqq", f.read(24))
        Nmat = np.zeros((Dim, Dim))
        infos, TDs = [], []
        for _ in range(npair):
            i, j, Nij, tN = struct.unpack("<qqqd", f.read(32))
            infos.append((i, j, Nij))
            Nmat[i - 1, j - 1] = Nmat[j - 1, i - 1] = tN
            TDs.append(np.frombuffer(f.read(8 * lTD), dtype="<f8").copy())
    return Dim, npair, lTD, Nmat, infos, np.array(TDs)


def my_cholesky(A):
    """myCholesky! (eigenvector_continuation.jl:11-30): lower-triangular L
    with L L^T = A; raises ValueError where a pivot is not positive."""
    n = A.shape[0]
    L = np.zeros((n, n))
    for i in range(n):
        for j in range(i):
            L[i, j] = (A[i, j] - L[i, :j] @ L[j, :j]) / L[j, j]
        d = A[i, i] - L[i, :i] @ L[i, :i]
        if not d > 0.0:
            raise ValueError("matrix is not positive definite")
        L[i, i] = np.sqrt(d)
    return L


def solve_ec(Hs, target_nuc, tJNs, write_appwav=False, verbose=False, calc_moment=True, wpath="./", tdmatpath="./",
             is_show=False, gfactors=(1.0, 0.0, 5.586, -3.826), effcharge=(1.5, 0.5), exact_logf="", quiet=False):
    """solveEC (eigenvector_continuation.jl:347-483): for each [tJ, n] of
    tJNs read <tdmatpath><nucleus>_J<tJ>.dat, and for each interaction of Hs
    solve H v = λ N v in the sample space (H = Σ ME·TD); the lowest n values
    are printed and returned.  write_appwav writes the continued vectors of
    the first interaction to ./appwavs/<nucleus>_<interaction>_j<tJ>.appwav,
    built from the sample .wav files named in ./tdmat/wfinfos_*."""
    if len(tJNs) == 0:
        raise ValueError("specify targetJ and # of states")
    sumV = []
    for tJ, num_ev_target in tJNs:
        Mtot = int(tJ)
        inpf = tdmatpath + target_nuc + "_J" + str(tJ) + ".dat"
        Dim, _, lTD, Nmat, infos, TDs = read_tdmat(inpf)
        if Dim + 1 <= num_ev_target:
            raise ValueError(f"Error!: sample number must be larger than {num_ev_target}")
        try:
            L = my_cholesky(Nmat)
        except ValueError:
            u = 1.1 * 1.0e-16
            shift = np.trace(Nmat) * u * ((Dim + 2) / (1.0 - ((Dim + 1) * (Dim + 2)) * u))
            Nmat = Nmat + shift * np.eye(Dim)
            L = my_cholesky(Nmat)
        Linv = np.linalg.inv(L)
        for sntidx, sntf in enumerate(Hs):
            spe_p, spe_n, otb = read_snt_mes(sntf, target_nuc)
            MEs = np.concatenate([spe_p, spe_n, otb])
            if MEs.size != lTD:
                raise ValueError(f"{sntf}: {MEs.size} matrix elements, the TD vectors have {lTD}")
            Hmat = np.zeros((Dim, Dim))
            for (i, j, _), TD in zip(infos, TDs):
                Hmat[i - 1, j - 1] = Hmat[j - 1, i - 1] = TD @ MEs
            # N^{-1} H has the generalized eigenvalues; solved in the symmetric
            # form L^{-1} H L^{-T} y = λ y, v = L^{-T} y.
            S = Linv @ Hmat @ Linv.T
            w, Y = np.linalg.eigh(0.5 * (S + S.T))
            vals = w[:num_ev_target]
            vecs = Linv.T @ Y[:, :num_ev_target]
            if not quiet:
                print(f"vals {list(map(float, vals))} ln {len(vals)} num_ev_target {num_ev_target}")
                if verbose:
                    _print_vec(f"{target_nuc} 2J={tJ}  En(EC)", vals)
            sumV.append([sntf, tJ, vals])
            if write_appwav and sntidx == 0:
                P = ShellModelProblem(sntf, target_nuc, FP64, twoJ=Mtot)
                mdim = P.mdim
                P.close()
                vs = np.zeros((Dim, mdim))
                with open("./tdmat/wfinfos_" + target_nuc + "_J" + str(tJ) + ".dat") as f:
                    for line in f:
                        t = line.split()
                        if not t:
                            continue
                        name, nth, k = t[0], int(t[2]), int(t[4])
                        path = name if wpath in ("./", "") else wpath + "/" + os.path.basename(name)
                        _, _, V, _ = read_wav_full(path, mdim)
                        vs[k - 1] = V[nth - 1]
                R = vecs.T @ vs
                R /= np.sqrt((R * R).sum(axis=1, keepdims=True))
                csnt = os.path.basename(sntf).split(".")[0]
                os.makedirs("./appwavs", exist_ok=True)
                wavname = "./appwavs/" + target_nuc + "_" + csnt + "_j" + str(tJ) + ".appwav"
                # writeRitzvecs stores 2*J of Jlist = [tJ, ...]
                write_wav(wavname, Mtot, list(map(float, vals)), [2 * int(tJ)] * len(vals), R)
    return sumV
