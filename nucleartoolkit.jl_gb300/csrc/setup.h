// Host-side problem set-up for libsmgpu: interaction parsing, m-scheme
// matrix elements and the factorised ("pull") tables the GPU kernels read.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace smgpu {

struct Orbit {
  int n, l, j2, tz;
};

// The data of the reference's SMobject (shellmodel_main.jl:38-53) that the
// eigensolver needs.  `tb[k]` holds pp (k=0), nn (1) and pn (2) entries with
// the hermitian partners already added in readsmsnt's order.
struct Interaction {
  int lp = 0, ln = 0, cp = 0, cn = 0;
  std::vector<Orbit> porb, norb;
  std::vector<double> spe_p, spe_n;
  struct TB {
    int a, b, c, d, J;
    double v;
    int line = 0;  // 1-based TBME line of the snt file (readsmsnt's ith)
  };
  std::vector<TB> tb[3];
  int nlines = 0;  // TBME lines of the snt file
};

struct SetupError {
  int code;
  std::string msg;
};

// snt text -> Interaction (readsmsnt semantics, shellmodel_main.jl:293-365)
Interaction read_snt(const std::string& path, int Anum);
// The total angular momentum squared J^2 of the valence particles written as
// an interaction on the same orbits: one-body j(j+1) per orbit and the
// diagonal two-body elements <ab;J|2 j_a.j_b|ab;J> = J(J+1) - j_a(j_a+1) -
// j_b(j_b+1) for every pp, nn (J even when a == b) and pn pair.  Its m-scheme
// matrix on a basis is J^2; the reference builds the same operator as jump
// lists (prep_J / operate_J!, src/ShellModel/shellmodel_main.jl:1439-1650).
Interaction jj_interaction(const Interaction& I);
// "Cr48" / "48Cr" -> A and Z (util_func.jl:1,13-24; shellmodel_main.jl:908-916)
void parse_nucleus(const std::string& nuc, int& A, int& Z);

// Clebsch–Gordan coefficient with doubled arguments (exact, binomial form).
double clebsch_gordan(int tj1, int tm1, int tj2, int tm2, int tJ, int tM);
// Wigner 3j (j1 j2 j3; m1 m2 m3) and 6j {j1 j2 j3; j4 j5 j6} symbols with
// doubled arguments (exact squares, one final rounding), the values of
// WignerSymbols.jl's wigner3j / wigner6j(Float64, ...).
double wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3);
double wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6);

// One m-state of a species, in construct_msps order (shellmodel_main.jl:373-384).
struct MState {
  int orbit;  // 0-based orbit index within the species
  int j2, m2;
};

// m-scheme two-body operator a†b† d c, keyed by one-hot SD bit masks.
struct Op2 {
  uint64_t a, b, c, d;
  double v;
};

// Everything the GPU needs, in flat arrays.
struct Tables {
  // species
  int Lp = 0, Ln = 0;  // number of m-states
  std::vector<MState> msp, msn;
  // blocks (ordered by ascending proton M)
  int nb = 0;
  std::vector<int> np, nn, stride, mp2, mn2;
  std::vector<int64_t> tdims;    // nb+1, unpadded offsets (reference order)
  std::vector<int64_t> off_pad;  // nb+1, padded offsets (rows padded to `stride`)
  int64_t mdim = 0, len_pad = 0;
  std::vector<uint64_t> pbits, nbits;  // per block, descending
  std::vector<int> pstart, nstart;     // nb+1
  std::vector<double> ep, en;          // one-body diagonal per SD
  // m-scheme operators (reference prep_Hamil_T1 / prep_Hamil_pn lists)
  std::vector<Op2> vpp, vnn;
  std::vector<int> delMs;                   // descending, as the reference's Mzs
  std::vector<std::vector<Op2>> vpn;        // per delMs entry (fields a,b,c,d = bit_a,bit_b,bit_c,bit_d)
  // pp / nn pull CSR (rows = SDs of a block, cols local, merged duplicates)
  std::vector<int> pp_ptr, pp_col, nn_ptr, nn_col;
  std::vector<double> pp_val, nn_val;
  // pn: links (output block b <- source block s)
  struct Link {
    int b, s, dm;   // dm = index of the V table
    int nA, nB;
    int64_t vtab_off;   // into vtab
    int64_t nptr_off;   // into npn_ptr: nn[b]+1 row pointers
  };
  std::vector<Link> links;
  std::vector<int> link_begin;  // nb+1
  // proton pull entries per global proton row: src row (local in s), meta = link<<16 | ia<<1 | sign
  std::vector<int> ppn_ptr;
  std::vector<uint32_t> ppn_src, ppn_meta;
  // neutron pull CSR per link: entries n'<<14 | ib<<1 | sign
  std::vector<int64_t> npn_ptr;
  std::vector<uint32_t> npn_ent;
  std::vector<double> vtab;  // V tables [nA x nB] per delMs index (only ΔM >= 0 used)
  std::vector<int64_t> vtab_off_dm;
  std::vector<int> nA_dm, nB_dm;
  std::vector<std::vector<uint64_t>> Aops_dm, Bops_dm;  // per dm: one-hot (a, c) / (b, d) mask pairs, flattened
  // statistics
  int64_t updates = 0;
};

// Full set-up of one problem (enum.cu): the basis and the jump tables are
// enumerated on the device and copied into T; the interaction-dependent
// operator lists are built on the host.  vp, vn valence numbers, mtot2
// doubled M.  Needs a CUDA device.
void build_tables(const Interaction& I, int vp, int vn, int mtot2, Tables& T);

// Host pieces of the set-up (setup.cpp), used by build_tables.
// m-states of a species in construct_msps order (shellmodel_main.jl:373-384).
std::vector<MState> mstates(const std::vector<Orbit>& orb);
// prep_Hamil_T1 / prep_Hamil_pn (:580-730): the m-scheme pp, nn and per-ΔM pn
// operator lists, the per-ΔM V tables and their distinct one-body operators
// (T.msp and T.msn must be set).
void build_operators(const Interaction& I, Tables& T);
// Index of the hermitian conjugate (c,d,a,b) of every operator, or -1.
std::vector<long> conjugate_index(const std::vector<Op2>& ops);
// prep_pn's block links (:1139-1151) and the neutron-pointer offsets of
// every link; Mps = every proton M value of the species (doubled), ascending.
void build_links(Tables& T, const std::vector<int>& Mps);
// Multiply-adds of one H·v (T.updates).
void count_updates(Tables& T);

}  // namespace smgpu
