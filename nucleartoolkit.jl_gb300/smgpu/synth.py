"""Seeded synthetic `.snt` interactions for the sd and pf shells.

The benchmark configurations are quoted on synthetic interactions: the
reference's own sd/pf interaction files with published energies are not
available, so every measured problem uses an interaction drawn from a fixed
numpy PCG64 seed.  The file layout is the one ``readsmsnt`` reads
(src/ShellModel/shellmodel_main.jl:293-365, docs/src/fileformat.md):

* header ``lp ln cp cn``; orbit lines ``idx n l 2j 2tz`` (protons first);
* ``nsp 0`` then ``i i SPE`` lines;
* ``ntbme 0 A`` (massop = 0: no mass scaling) then ``a b c d J V`` lines.

TBMEs are one i.i.d. N(0, σ²) draw per Pauli-allowed line, each (ab,cd) pair
listed once — ``readsmsnt`` adds the hermitian partner (shellmodel_main.jl:
354-357), so H comes out symmetric.  pp/nn lines: a≤b, c≤d, (a,b)≤(c,d),
J allowed by both couplings and even when a==b or c==d.  pn lines: a, c
protons and b, d neutrons with (a,b)≤(c,d) and J allowed by both couplings.
"""
import os

import numpy as np

# (n, l, 2j) per orbit, in file order, plus single-particle energies (MeV)
SD_ORBITS = [(0, 2, 5), (1, 0, 1), (0, 2, 3)]
SD_SPE = [-3.9, -3.2, 1.6]
SD_CORE = (8, 8)
PF_ORBITS = [(0, 3, 7), (1, 1, 3), (0, 3, 5), (1, 1, 1)]
PF_SPE = [-8.6, -6.0, -2.0, -4.0]
PF_CORE = (20, 20)

SHELLS = {
    "sd": (SD_ORBITS, SD_SPE, SD_CORE, 1.5),
    "pf": (PF_ORBITS, PF_SPE, PF_CORE, 1.0),
}

ELEMENTS = ["n", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar",
            "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"]


def nucleus_name(shell: str, vp: int, vn: int) -> str:
    """e.g. ('pf', 4, 4) -> 'Cr48'."""
    cp, cn = SHELLS[shell][2]
    Z, N = cp + vp, cn + vn
    return f"{ELEMENTS[Z]}{Z + N}"


def tbme_labels(orbits):
    """Pauli-allowed TBME lines (a,b,c,d,J), 1-based snt indices, protons
    1..k and neutrons k+1..2k, in a fixed order (pp, nn, pn)."""
    k = len(orbits)
    js = [o[2] for o in orbits]

    def jrange(a, b):
        return range(abs(js[a] - js[b]) // 2, (js[a] + js[b]) // 2 + 1)

    out = []
    for off in (0, k):  # pp then nn
        pairs = [(a, b) for a in range(k) for b in range(a, k)]
        for i, (a, b) in enumerate(pairs):
            for (c, d) in pairs[i:]:
                for J in jrange(a, b):
                    if J not in jrange(c, d):
                        continue
                    if (a == b or c == d) and J % 2 == 1:
                        continue
                    out.append((a + 1 + off, b + 1 + off, c + 1 + off, d + 1 + off, J))
    pairs = [(a, b) for a in range(k) for b in range(k)]  # (proton, neutron)
    for i, (a, b) in enumerate(pairs):
        for (c, d) in pairs[i:]:
            for J in jrange(a, b):
                if J not in jrange(c, d):
                    continue
                out.append((a + 1, b + 1 + k, c + 1, d + 1 + k, J))
    return out


def draw_tbmes(shell: str, seed: int, sigma=None, base_seed=None, base_sigma=None):
    """TBME values for ``tbme_labels``.  With ``base_seed`` the values are a
    base draw N(0, base_sigma²) plus a perturbation N(0, sigma²) from ``seed``
    (interaction samples sharing one basis)."""
    orbits, _, _, sig0 = SHELLS[shell]
    labels = tbme_labels(orbits)
    n = len(labels)
    if base_seed is not None:
        base = np.random.Generator(np.random.PCG64(base_seed)).normal(0.0, base_sigma, n)
        pert = np.random.Generator(np.random.PCG64(seed)).normal(0.0, sigma, n)
        return labels, base + pert
    s = sig0 if sigma is None else sigma
    return labels, np.random.Generator(np.random.PCG64(seed)).normal(0.0, s, n)


def snt_text(shell: str, labels, values, A: int, title: str = "") -> str:
    orbits, spe, (cp, cn), _ = SHELLS[shell]
    k = len(orbits)
    lines = [f"! synthetic {shell}-shell interaction {title}".rstrip(), "! model space",
             f"  {k:2d}  {k:2d}   {cp:3d} {cn:3d}"]
    for t, tz in ((0, -1), (1, 1)):
        for i, (n, l, j2) in enumerate(orbits):
            lines.append(f"  {i + 1 + t * k:3d}  {n:3d} {l:3d} {j2:3d} {tz:3d}")
    lines.append("! interaction")
    lines.append(f"  {2 * k:3d}   0")
    for t in range(2):
        for i in range(k):
            idx = i + 1 + t * k
            lines.append(f"  {idx:3d} {idx:3d}  {spe[i]:14.8f}")
    lines.append(f"  {len(labels):5d}   0  {A:3d}")
    for (a, b, c, d, J), v in zip(labels, values):
        lines.append(f"  {a:3d} {b:3d} {c:3d} {d:3d}  {J:3d}  {v:17.12f}")
    return "\n".join(lines) + "\n"


def write_snt(path: str, shell: str, seed: int, vp: int, vn: int, sigma=None, base_seed=None, base_sigma=None) -> str:
    """Write one seeded interaction file and return its path."""
    labels, vals = draw_tbmes(shell, seed, sigma=sigma, base_seed=base_seed, base_sigma=base_sigma)
    cp, cn = SHELLS[shell][2]
    A = cp + cn + vp + vn
    txt = snt_text(shell, labels, vals, A, title=f"seed={seed}")
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        f.write(txt)
    return path


# Named workloads.  Seeds are fixed here.
CONFIG_SEEDS = {
    "sd2p2n": 2020,     # 20Ne, M=0, dim 640
    "sd4p4n": 2424,     # 24Mg, M=0, dim 28,503
    "pf4p4n": 4848,     # 48Cr, M=0, dim 1,963,461
    "pf_multi_base": 48000,  # base draw for the 16 pf samples; sample s uses seed 48001+s
    "sd_batch_base": 128000,  # batch problem k uses seed 128000+k
}


def config_snt(dirpath: str, name: str):
    """Write the interaction of a named workload; returns (snt path, nucleus)."""
    if name == "sd2p2n":
        return write_snt(os.path.join(dirpath, "sd_seed2020.snt"), "sd", CONFIG_SEEDS[name], 2, 2), "Ne20"
    if name == "sd4p4n":
        return write_snt(os.path.join(dirpath, "sd_seed2424.snt"), "sd", CONFIG_SEEDS[name], 4, 4), "Mg24"
    if name == "pf4p4n":
        return write_snt(os.path.join(dirpath, "pf_seed4848.snt"), "pf", CONFIG_SEEDS[name], 4, 4), "Cr48"
    raise KeyError(name)


def multi_snts(dirpath: str, shell: str, vp: int, vn: int, nsamples: int, base_seed: int, base_sigma: float,
               sigma: float, prefix: str):
    """Interaction samples sharing one basis: a base draw N(0, base_sigma²)
    plus a per-sample perturbation N(0, sigma²); sample s uses seed
    base_seed+1+s."""
    return [write_snt(os.path.join(dirpath, f"{prefix}_{s:02d}.snt"), shell, base_seed + 1 + s, vp, vn,
                      sigma=sigma, base_seed=base_seed, base_sigma=base_sigma) for s in range(nsamples)]


def pf_multi_snts(dirpath: str, nsamples: int = 16):
    """The 16 pf samples sharing the 48Cr basis: base N(0,1²) + N(0,0.1²)."""
    return multi_snts(dirpath, "pf", 4, 4, nsamples, CONFIG_SEEDS["pf_multi_base"], 1.0, 0.1, "pf_multi")


def sd_batch_problems(nprob: int = 128):
    """(vp, vn) list for the uneven sd batch: cycles through the 36 (vp,vn)
    combinations with 1..6 particles per species."""
    combos = [(vp, vn) for vp in range(1, 7) for vn in range(1, 7)]
    return [combos[k % len(combos)] for k in range(nprob)]


def sd_batch_snts(dirpath: str, nprob: int = 128):
    out = []
    base = CONFIG_SEEDS["sd_batch_base"]
    for k, (vp, vn) in enumerate(sd_batch_problems(nprob)):
        p = write_snt(os.path.join(dirpath, f"sd_batch_{k:03d}.snt"), "sd", base + k, vp, vn)
        out.append((p, nucleus_name("sd", vp, vn)))
    return out
