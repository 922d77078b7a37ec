// CPU ORACLE — test infrastructure only, never the product.
//
// A plain C++17 restatement of NuclearToolkit.jl's valence shell-model path
// (`main_sm` with target_J = [] and truncation_scheme = ""), used by the test
// suite as the parity checker for the GPU library and by bench.py as the timed
// CPU baseline ("port").  Nothing in the product links or calls this file.
//
// Each function names the reference function it restates (paths relative to
// the NuclearToolkit.jl source tree).  Loop orders, summation orders, the
// de-duplication rules and the phase conventions follow the reference so that
// basis, jump tables and H·v agree entry by entry.
//
// Parity pins: the ckpot.snt ⁸Be known-answer energies
// (test/ShellModel_test.jl:8-15) and the ²⁴Mg sd-shell dimension 28,503
// (example/log_sample_script.txt:323) are checked in tests/test_oracle.py.
// Two inputs cannot be pinned: the Julia RNG start vector (replaced by the
// hash-based start vector below, shared with the GPU library) and per-element
// Clebsch–Gordan values (WignerSymbols.jl 2.0.0, not vendored; restated here
// with exact rational arithmetic).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef long long i64;
typedef unsigned long long u64;

// ---------------------------------------------------------------------------
// util_func.jl:13-24 — element symbols by Z.
const char* kElements[] = {
    "n",  "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",
    "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga",
    "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag",
    "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu",
    "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au",
    "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Np", "Pu", "Am",
    "Cm", "Bk", "Cf", "Es", "Fm", "Md", "No", "Lr", "Rf", "Db", "Sg", "Bh", "Hs", "Mt", "Ds", "Rg",
    "Cn", "Nh", "Fl", "Mc", "Lv", "Ts", "Og"};

// util_func.jl:26-38 rm_comment: strip, drop lines starting with '!' or '#'
// (empty lines are kept, as in the reference).
std::vector<std::string> rm_comment(const std::vector<std::string>& lines) {
  std::vector<std::string> out;
  for (auto line : lines) {
    size_t b = line.find_first_not_of(" \t\r\n");
    size_t e = line.find_last_not_of(" \t\r\n");
    line = (b == std::string::npos) ? std::string() : line.substr(b, e - b + 1);
    if (!line.empty() && (line[0] == '!' || line[0] == '#')) continue;
    out.push_back(line);
  }
  return out;
}
// util_func.jl:40-46 rm_nan(split(line," ")): split on single spaces, drop empties.
std::vector<std::string> fields(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  for (char ch : line) {
    if (ch == ' ') {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(ch);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

struct Err {
  std::string msg;
};

// ---------------------------------------------------------------------------
// shellmodel_main.jl:38-53 SMobject (the parts main_sm uses).
struct Snt {
  int lp = 0, ln = 0, cp = 0, cn = 0, massop = 0;
  double Aref = 0, p = 0;
  std::vector<std::array<int, 4>> p_sps, n_sps;  // n,l,j,tz
  std::vector<double> SPEs[2];
  std::vector<std::array<int, 6>> labels[3];  // a,b,c,d,J,line  (pp, nn, pn)
  std::vector<double> TBMEs[3];
  int ntbme = 0;  // TBME lines (length of oTBMEs)
};

int parse_int(const std::string& s) {
  size_t pos = 0;
  int v = std::stoi(s, &pos);
  if (pos != s.size()) throw Err{"bad integer '" + s + "'"};
  return v;
}
double parse_dbl(const std::string& s) { return std::stod(s); }

// shellmodel_main.jl:293-365 readsmsnt
Snt readsmsnt(const std::string& path, int Anum) {
  if (Anum <= 0) throw Err{"invalid nucleus (A<=0)"};
  std::ifstream f(path);
  if (!f) throw Err{"cannot open " + path};
  std::vector<std::string> raw;
  std::string l;
  while (std::getline(f, l)) raw.push_back(l);
  std::vector<std::string> lines = rm_comment(raw);
  auto L = [&](size_t one_based) -> const std::string& {
    if (one_based < 1 || one_based > lines.size()) throw Err{"snt file too short"};
    return lines[one_based - 1];
  };
  Snt s;
  auto h = fields(L(1));
  if (h.size() < 4) throw Err{"bad snt header"};
  s.lp = parse_int(h[0]); s.ln = parse_int(h[1]); s.cp = parse_int(h[2]); s.cn = parse_int(h[3]);
  s.p_sps.assign(s.lp, {0, 0, 0, 0});
  s.n_sps.assign(s.ln, {0, 0, 0, 0});
  for (int i = 1; i <= s.lp; ++i) {
    auto t = fields(L(1 + i));
    int ith = parse_int(t[0]);
    s.p_sps.at(ith - 1) = {parse_int(t[1]), parse_int(t[2]), parse_int(t[3]), parse_int(t[4])};
  }
  for (int i = 1; i <= s.ln; ++i) {
    auto t = fields(L(1 + i + s.ln));  // the reference indexes neutron lines with +ln
    int ith = parse_int(t[0]);
    s.n_sps.at(ith - s.lp - 1) = {parse_int(t[1]), parse_int(t[2]), parse_int(t[3]), parse_int(t[4])};
  }
  auto hs = fields(L(1 + s.ln + s.lp + 1));
  int nsp = parse_int(hs[0]);
  s.SPEs[0].assign(s.lp, 0.0);
  s.SPEs[1].assign(s.ln, 0.0);
  for (int i = 1; i <= nsp; ++i) {
    auto t = fields(L(1 + s.ln + s.lp + 1 + i));
    int j = parse_int(t[0]);
    int idx = (j <= s.lp) ? 0 : 1;
    if (idx == 1) j -= s.lp;
    s.SPEs[idx].at(j - 1) = parse_dbl(t[2]);
  }
  auto ht = fields(L(1 + s.ln + s.lp + 1 + nsp + 1));
  int ntbme = parse_int(ht[0]);
  s.ntbme = ntbme;
  s.massop = parse_int(ht[1]);
  s.Aref = parse_dbl(ht[2]);
  if (ht.size() > 3) s.p = parse_dbl(ht[3]);
  for (int ith = 1; ith <= ntbme; ++ith) {
    auto t = fields(L(1 + s.ln + s.lp + 1 + nsp + 1 + ith));
    int i = parse_int(t[0]), j = parse_int(t[1]), k = parse_int(t[2]), ll = parse_int(t[3]);
    int totJ = parse_int(t[4]);
    double tbme = parse_dbl(t[5]);
    int nth;
    if (i <= s.lp && j <= s.lp) nth = 0;
    else if (i > s.lp && j > s.lp) nth = 1;
    else if (i <= s.lp && j > s.lp) nth = 2;
    else throw Err{"TBME with proton index > neutron index"};
    if (s.massop == 1) tbme *= std::pow((double)Anum / s.Aref, s.p);
    // unique([i,j]) != unique([k,l]): add the hermitian partner first
    std::vector<int> u1 = (i == j) ? std::vector<int>{i} : std::vector<int>{i, j};
    std::vector<int> u2 = (k == ll) ? std::vector<int>{k} : std::vector<int>{k, ll};
    if (u1 != u2) {
      s.labels[nth].push_back({k, ll, i, j, totJ, ith});
      s.TBMEs[nth].push_back(tbme);
    }
    s.labels[nth].push_back({i, j, k, ll, totJ, ith});
    s.TBMEs[nth].push_back(tbme);
  }
  return s;
}

// ---------------------------------------------------------------------------
// Clebsch–Gordan ⟨j1 m1 j2 m2|J M⟩ (doubled arguments), exact Racah sum in
// rationals, as WignerSymbols.jl clebschgordan(Float64, ...) returns it.
typedef __int128 i128;
i128 gcd128(i128 a, i128 b) {
  if (a < 0) a = -a;
  if (b < 0) b = -b;
  while (b) { i128 t = a % b; a = b; b = t; }
  return a;
}
struct Rat {
  i128 n = 0, d = 1;
  void norm() {
    if (d < 0) { d = -d; n = -n; }
    i128 g = gcd128(n, d);
    if (g > 1) { n /= g; d /= g; }
  }
};
Rat rmul(Rat a, Rat b) {
  i128 g1 = gcd128(a.n, b.d), g2 = gcd128(b.n, a.d);
  if (g1 == 0) g1 = 1;
  if (g2 == 0) g2 = 1;
  Rat r;
  r.n = (a.n / g1) * (b.n / g2);
  r.d = (a.d / g2) * (b.d / g1);
  r.norm();
  return r;
}
Rat radd(Rat a, Rat b) {
  i128 g = gcd128(a.d, b.d);
  Rat r;
  r.n = a.n * (b.d / g) + b.n * (a.d / g);
  r.d = (a.d / g) * b.d;
  r.norm();
  return r;
}
i128 fact(int n) {
  i128 r = 1;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}
// CG² as an exact fraction with the sign of CG; false when CG = 0.
bool clebsch_sq(int tj1, int tm1, int tj2, int tm2, int tJ, int tM, Rat& c2, int& sign) {
  if (tm1 + tm2 != tM) return false;
  if (std::abs(tm1) > tj1 || std::abs(tm2) > tj2 || std::abs(tM) > tJ) return false;
  if (((tj1 + tm1) & 1) || ((tj2 + tm2) & 1) || ((tJ + tM) & 1)) return false;
  if (tJ > tj1 + tj2 || tJ < std::abs(tj1 - tj2) || ((tj1 + tj2 + tJ) & 1)) return false;
  int a = (tj1 + tj2 - tJ) / 2, b = (tj1 - tj2 + tJ) / 2, c = (-tj1 + tj2 + tJ) / 2;
  int s = (tj1 + tj2 + tJ) / 2 + 1;
  // A = (2J+1) a! b! c! / s! * (j1+m1)!(j1-m1)!(j2+m2)!(j2-m2)!(J+M)!(J-M)!
  Rat A{tJ + 1, 1};
  A = rmul(A, Rat{fact(a), 1});
  A = rmul(A, Rat{fact(b), 1});
  A = rmul(A, Rat{fact(c), 1});
  A = rmul(A, Rat{1, fact(s)});
  int f6[6] = {(tj1 + tm1) / 2, (tj1 - tm1) / 2, (tj2 + tm2) / 2, (tj2 - tm2) / 2, (tJ + tM) / 2, (tJ - tM) / 2};
  for (int x : f6) A = rmul(A, Rat{fact(x), 1});
  // S = sum_k (-1)^k / [k! (j1+j2-J-k)! (j1-m1-k)! (j2+m2-k)! (J-j2+m1+k)! (J-j1-m2+k)!]
  Rat S{0, 1};
  int e1 = a, e2 = (tj1 - tm1) / 2, e3 = (tj2 + tm2) / 2;
  int e4 = (tJ - tj2 + tm1) / 2, e5 = (tJ - tj1 - tm2) / 2;
  for (int k = 0; k <= 200; ++k) {
    if (e1 - k < 0 || e2 - k < 0 || e3 - k < 0) break;
    if (e4 + k < 0 || e5 + k < 0) continue;
    i128 den = fact(k) * fact(e1 - k) * fact(e2 - k) * fact(e3 - k) * fact(e4 + k) * fact(e5 + k);
    Rat t{(k & 1) ? -1 : 1, den};
    S = radd(S, t);
  }
  if (S.n == 0) return false;
  c2 = rmul(rmul(A, S), S);
  sign = S.n < 0 ? -1 : 1;
  return true;
}
double clebsch(int tj1, int tm1, int tj2, int tm2, int tJ, int tM) {
  Rat c2;
  int sign;
  if (!clebsch_sq(tj1, tm1, tj2, tm2, tJ, tM, c2, sign)) return 0.0;
  double v = std::sqrt((double)c2.n / (double)c2.d);
  return sign < 0 ? -v : v;
}
// WignerSymbols.jl wigner3j(Float64, j1, j2, j3, m1, m2, m3) (doubled
// arguments): (-1)^(j1-j2-m3) <j1 m1 j2 m2|j3 -m3> / sqrt(2 j3 + 1).
double wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3) {
  Rat c2;
  int sign;
  if (!clebsch_sq(tj1, tm1, tj2, tm2, tj3, -tm3, c2, sign)) return 0.0;
  c2 = rmul(c2, Rat{1, (i128)(tj3 + 1)});
  if (((tj1 - tj2 - tm3) / 2) & 1) sign = -sign;
  double v = std::sqrt((double)c2.n / (double)c2.d);
  return sign < 0 ? -v : v;
}
// WignerSymbols.jl wigner6j(Float64, ...) (doubled arguments), Racah's formula
// {a b c; d e f} = Δ(abc)Δ(aef)Δ(dbf)Δ(dec) Σ_t (-1)^t (t+1)! /
// [(t-abc)!(t-aef)!(t-dbf)!(t-dec)!(a+b+d+e-t)!(b+c+e+f-t)!(c+a+f+d-t)!].
double wigner6j(int a, int b, int c, int d, int e, int f) {
  auto tri = [](int x, int y, int z, Rat& out) {
    if (((x + y + z) & 1) || z > x + y || z < std::abs(x - y)) return false;
    out = rmul(Rat{fact((x + y - z) / 2) * fact((x - y + z) / 2), 1},
               Rat{fact((-x + y + z) / 2), fact((x + y + z) / 2 + 1)});
    return true;
  };
  Rat d1, d2, d3, d4;
  if (!tri(a, b, c, d1) || !tri(a, e, f, d2) || !tri(d, b, f, d3) || !tri(d, e, c, d4)) return 0.0;
  int al[4] = {(a + b + c) / 2, (a + e + f) / 2, (d + b + f) / 2, (d + e + c) / 2};
  int be[3] = {(a + b + d + e) / 2, (b + c + e + f) / 2, (c + a + f + d) / 2};
  Rat S{0, 1};
  for (int t = *std::max_element(al, al + 4); t <= *std::min_element(be, be + 3); ++t) {
    i128 den = fact(t - al[0]) * fact(t - al[1]) * fact(t - al[2]) * fact(t - al[3]);
    den *= fact(be[0] - t) * fact(be[1] - t) * fact(be[2] - t);
    S = radd(S, Rat{(t & 1) ? -fact(t + 1) : fact(t + 1), den});
  }
  if (S.n == 0) return 0.0;
  Rat q = rmul(rmul(rmul(d1, d2), rmul(d3, d4)), rmul(S, S));
  double v = std::sqrt((double)q.n / (double)q.d);
  return S.n < 0 ? -v : v;
}

// ---------------------------------------------------------------------------
struct Msps {
  // shellmodel_main.jl:373-384 construct_msps: [n,l,j,tz,mz,orbit(1-based)]
  std::vector<std::array<int, 6>> p, n;
};
Msps construct_msps(const Snt& s) {
  Msps m;
  for (size_t i = 0; i < s.p_sps.size(); ++i) {
    auto o = s.p_sps[i];
    for (int mz = -o[2]; mz <= o[2]; mz += 2) m.p.push_back({o[0], o[1], o[2], o[3], mz, (int)i + 1});
  }
  for (size_t i = 0; i < s.n_sps.size(); ++i) {
    auto o = s.n_sps[i];
    for (int mz = -o[2]; mz <= o[2]; mz += 2) m.n.push_back({o[0], o[1], o[2], o[3], mz, (int)i + 1});
  }
  return m;
}

// shellmodel_main.jl:732-739 bitarr_to_int: m-state k (1-based) is bit L-k.
inline i64 onehot(int L, int k1) { return (i64)1 << (L - k1); }

struct Basis {
  // shellmodel_main.jl:769-848 occ
  std::vector<std::vector<i64>> pbits, nbits;
  std::vector<std::vector<std::vector<double>>> jocc_p, jocc_n;
  std::vector<int> Mps, Mns;  // unique M lists (Mps ascending, Mns descending)
  std::vector<int> blkMp, blkMn;
  std::vector<i64> tdims;
};

void lex_combinations(int L, int k, std::vector<std::vector<int>>& out) {
  std::vector<int> c(k);
  for (int i = 0; i < k; ++i) c[i] = i + 1;
  if (k == 0) { out.push_back(c); return; }
  if (k > L) return;
  while (true) {
    out.push_back(c);
    int i = k - 1;
    while (i >= 0 && c[i] == L - k + i + 1) --i;
    if (i < 0) break;
    ++c[i];
    for (int j = i + 1; j < k; ++j) c[j] = c[j - 1] + 1;
  }
}

Basis occ(const Snt& s, const Msps& m, int vp, int vn, int Mtot) {
  Basis B;
  int lp = (int)m.p.size(), ln = (int)m.n.size();
  std::vector<std::vector<int>> cp, cn;
  lex_combinations(lp, vp, cp);
  lex_combinations(ln, vn, cn);
  std::vector<int> Mp_all, Mn_all;
  auto Mof = [](const std::vector<int>& comb, const std::vector<std::array<int, 6>>& ms) {
    int M = 0;
    for (int k : comb) M += ms[k - 1][4];
    return M;
  };
  for (auto& c : cp) Mp_all.push_back(Mof(c, m.p));
  for (auto& c : cn) Mn_all.push_back(Mof(c, m.n));
  B.Mps = Mp_all;
  B.Mns = Mn_all;
  std::sort(B.Mps.begin(), B.Mps.end());
  B.Mps.erase(std::unique(B.Mps.begin(), B.Mps.end()), B.Mps.end());
  std::sort(B.Mns.begin(), B.Mns.end());
  B.Mns.erase(std::unique(B.Mns.begin(), B.Mns.end()), B.Mns.end());
  std::reverse(B.Mns.begin(), B.Mns.end());
  B.tdims.push_back(0);
  i64 mdim = 0;
  for (int Mp : B.Mps)
    for (int Mn : B.Mns) {
      if (Mp + Mn != Mtot) continue;
      B.blkMp.push_back(Mp);
      B.blkMn.push_back(Mn);
      std::vector<i64> pb, nb;
      std::vector<std::vector<double>> jp, jn;
      i64 nn_count = 0;
      for (size_t j = 0; j < cn.size(); ++j)
        if (Mp + Mn_all[j] == Mtot) ++nn_count;
      for (size_t i = 0; i < cp.size(); ++i) {
        if (Mp_all[i] != Mp) continue;
        i64 bits = 0;
        std::vector<double> occ_j(s.p_sps.size(), 0.0);
        for (int k : cp[i]) { bits += onehot(lp, k); occ_j[m.p[k - 1][5] - 1] += 1.0; }
        pb.push_back(bits);
        jp.push_back(occ_j);
        mdim += nn_count;
      }
      for (size_t j = 0; j < cn.size(); ++j) {
        if (Mn_all[j] != Mn) continue;
        i64 bits = 0;
        std::vector<double> occ_j(s.n_sps.size(), 0.0);
        for (int k : cn[j]) { bits += onehot(ln, k); occ_j[m.n[k - 1][5] - 1] += 1.0; }
        nb.push_back(bits);
        jn.push_back(occ_j);
      }
      B.pbits.push_back(pb);
      B.nbits.push_back(nb);
      B.jocc_p.push_back(jp);
      B.jocc_n.push_back(jn);
      B.tdims.push_back(mdim);
    }
  return B;
}

// shellmodel_main.jl:552-565 possible_mz: m-state indices (1-based) of an orbit.
void possible_mz(const std::array<int, 4>& o, const std::vector<std::array<int, 6>>& ms, int& j,
                 std::vector<int>& mzs, std::vector<int>& idxs) {
  j = o[2];
  mzs.clear();
  idxs.clear();
  for (int mz = -o[2]; mz <= o[2]; mz += 2) {
    mzs.push_back(mz);
    for (size_t k = 0; k < ms.size(); ++k)
      if (ms[k][0] == o[0] && ms[k][1] == o[1] && ms[k][2] == o[2] && ms[k][3] == o[3] && ms[k][4] == mz) {
        idxs.push_back((int)k + 1);
        break;
      }
  }
}

struct Key4 {
  i64 a, b, c, d;
  bool operator==(const Key4& o) const { return a == o.a && b == o.b && c == o.c && d == o.d; }
};
struct Key4Hash {
  size_t operator()(const Key4& k) const {
    u64 h = (u64)k.a * 0x9E3779B97F4A7C15ull;
    h ^= (u64)k.b + 0x7F4A7C15ull + (h << 6) + (h >> 2);
    h ^= (u64)k.c + 0x9E3779B9ull + (h << 6) + (h >> 2);
    h ^= (u64)k.d + 0x85EBCA6Bull + (h << 6) + (h >> 2);
    return (size_t)h;
  }
};
// Insertion-ordered de-duplicating list: the same order and the same
// accumulation order as the reference's linear search (`tl in blist`).
struct DedupList {
  std::vector<Key4> keys;
  std::vector<double> vals;
  std::unordered_map<Key4, size_t, Key4Hash> index;
  void add(const Key4& k, double v) {
    auto it = index.find(k);
    if (it == index.end()) {
      index.emplace(k, keys.size());
      keys.push_back(k);
      vals.push_back(v);
    } else {
      vals[it->second] += v;
    }
  }
};

// shellmodel_main.jl:27-30 T1info
struct T1info {
  int f;  // 1-based
  double coef;
};
typedef std::vector<std::vector<std::vector<T1info>>> Jump2b;  // [block][i] -> list

// shellmodel_main.jl:850-859 TF_connectable
inline bool TF_connectable(i64 Phi, const Key4& v) {
  if (v.c != (v.c & Phi)) return false;
  if (v.d != (v.d & Phi)) return false;
  i64 APhi = (~v.d) & ((~v.c) & Phi);
  if (v.a != (v.a & (~APhi))) return false;
  if (v.b != (v.b & (~APhi))) return false;
  return true;
}
inline int popc(i64 x) { return __builtin_popcountll((u64)x); }
// shellmodel_main.jl:869-885 calc_phase!
inline void calc_phase(i64 Phi, const Key4& v, int& phase, i64& nPhi) {
  int cnt = 0;
  cnt += popc(Phi & (~(v.c - 1)));
  nPhi = (~v.c) & Phi;
  cnt += popc(nPhi & (~(v.d - 1)));
  nPhi = (~v.d) & nPhi;
  cnt += popc(nPhi & (~(v.b - 1)));
  nPhi = v.b | nPhi;
  cnt += popc(nPhi & (~(v.a - 1)));
  nPhi = v.a | nPhi;
  phase = (cnt & 1) ? -1 : 1;
}
// shellmodel_main.jl:861-867 TF_connectable_1
inline bool TF_connectable_1(i64 Phi, i64 a, i64 c) {
  if (c != (c & Phi)) return false;
  if (a != (a & (~((~c) & Phi)))) return false;
  return true;
}
// shellmodel_main.jl:887-897 calc_phase_1! (count starts at 1)
inline void calc_phase_1(i64 Phi, i64 cre, i64 ani, int& phase, i64& nPhi) {
  int cnt = 1;
  cnt += popc(Phi & (~(ani - 1)));
  nPhi = (~ani) & Phi;
  cnt += popc(nPhi & (~(cre - 1)));
  nPhi = cre | nPhi;
  phase = (cnt & 1) ? -1 : 1;
}
// shellmodel_main.jl:1068-1083 bisearch! on a descending list; 1-based index or 0.
inline int bisearch_desc(const std::vector<i64>& v, i64 target) {
  int lo = 1, hi = (int)v.size();
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (v[mid - 1] > target) lo = mid + 1;
    else if (v[mid - 1] < target) hi = mid - 1;
    else return mid;
  }
  return 0;
}
inline int bisearch_desc_int(const std::vector<int>& v, int target) {
  int lo = 1, hi = (int)v.size();
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (v[mid - 1] > target) lo = mid + 1;
    else if (v[mid - 1] < target) hi = mid - 1;
    else return mid;
  }
  return 0;
}

// shellmodel_main.jl:1115-1137 prep_2bjumps
Jump2b prep_2bjumps(const std::vector<std::vector<i64>>& bits, const std::vector<Key4>& bV,
                    const std::vector<double>& V) {
  int nb = (int)bits.size();
  Jump2b J(nb);
  for (int b = 0; b < nb; ++b) J[b].resize(bits[b].size());
#pragma omp parallel for schedule(dynamic)
  for (int b = 0; b < nb; ++b) {
    for (size_t ii = 0; ii < bits[b].size(); ++ii) {
      i64 Phi = bits[b][ii];
      int i1 = (int)ii + 1;
      for (size_t nth = 0; nth < V.size(); ++nth) {
        if (V[nth] == 0.0) continue;
        if (!TF_connectable(Phi, bV[nth])) continue;
        int ph;
        i64 fin;
        calc_phase(Phi, bV[nth], ph, fin);
        int r = bisearch_desc(bits[b], fin);
        if (i1 <= r) {
          double coef = V[nth] * ph * (i1 == r ? 0.5 : 1.0);
          J[b][ii].push_back(T1info{r, coef});
        }
      }
    }
  }
  return J;
}

// shellmodel_main.jl:8-12 ifph
struct Ifph {
  int i, f;  // 1-based
  bool phase;
};

struct Problem {
  Snt snt;
  int Anum = 0, Z = 0, N = 0, vp = 0, vn = 0, Mtot = 0;
  Msps ms;
  Basis B;
  // prep_Hamil_T1 m-scheme lists
  std::vector<Key4> bV1[2];
  std::vector<double> V1[2];
  Jump2b pp, nn;
  // prep_Hamil_pn
  std::vector<int> delMs;
  std::vector<std::vector<Key4>> bVpn;
  std::vector<std::vector<double>> Vpn;
  // prep_pn
  std::vector<std::vector<int>> bis, bfs;  // 1-based block numbers
  // [bi][bfidx][nth] -> list
  std::vector<std::vector<std::vector<std::vector<Ifph>>>> pNiNfs, nNiNfs;
  std::vector<int> block_tasks;  // 1-based, 0 = padding
  i64 mdim = 0;
};

// shellmodel_main.jl:580-649 prep_Hamil_T1 (m-scheme pp/nn lists)
void prep_Hamil_T1(Problem& P) {
  const Snt& s = P.snt;
  const std::vector<std::array<int, 6>>* mst[2] = {&P.ms.p, &P.ms.n};
  const std::vector<std::array<int, 4>>* sps[2] = {&s.p_sps, &s.n_sps};
  int loffs[2] = {0, s.lp};
  for (int vr = 0; vr < 2; ++vr) {
    int Lm = (int)mst[vr]->size();
    DedupList dl;
    int ja, jb, jc, jd;
    std::vector<int> ma_s, mb_s, mc_s, md_s, ma_i, mb_i, mc_i, md_i;
    for (size_t i = 0; i < s.TBMEs[vr].size(); ++i) {
      double ME = s.TBMEs[vr][i];
      auto lab = s.labels[vr][i];
      int a = lab[0], b = lab[1], c = lab[2], d = lab[3], J2 = 2 * lab[4];
      int lo = loffs[vr];
      possible_mz((*sps[vr])[a - lo - 1], *mst[vr], ja, ma_s, ma_i);
      possible_mz((*sps[vr])[b - lo - 1], *mst[vr], jb, mb_s, mb_i);
      possible_mz((*sps[vr])[c - lo - 1], *mst[vr], jc, mc_s, mc_i);
      possible_mz((*sps[vr])[d - lo - 1], *mst[vr], jd, md_s, md_i);
      double nfac = std::sqrt((1.0 + (a == b ? 1.0 : 0.0)) * (1.0 + (c == d ? 1.0 : 0.0)));
      for (size_t ic = 0; ic < mc_s.size(); ++ic)
        for (size_t id = 0; id < md_s.size(); ++id) {
          int mc = mc_s[ic], md = md_s[id];
          if (c == d && mc >= md) continue;
          if (std::abs(mc + md) > J2) continue;
          int Mani = mc + md;
          i64 bit_c = onehot(Lm, mc_i[ic]), bit_d = onehot(Lm, md_i[id]);
          for (size_t ia = 0; ia < ma_s.size(); ++ia)
            for (size_t ib = 0; ib < mb_s.size(); ++ib) {
              int ma = ma_s[ia], mb = mb_s[ib];
              if (a == b && ma >= mb) continue;
              if (ma + mb != Mani) continue;
              i64 bit_a = onehot(Lm, ma_i[ia]), bit_b = onehot(Lm, mb_i[ib]);
              double CG1 = clebsch(ja, ma, jb, mb, J2, Mani);
              double CG2 = clebsch(jc, mc, jd, md, J2, Mani);
              dl.add(Key4{bit_a, bit_b, bit_c, bit_d}, ME * nfac * CG1 * CG2);
            }
        }
    }
    P.bV1[vr] = dl.keys;
    P.V1[vr] = dl.vals;
  }
  P.pp = prep_2bjumps(P.B.pbits, P.bV1[0], P.V1[0]);
  P.nn = prep_2bjumps(P.B.nbits, P.bV1[1], P.V1[1]);
}

// shellmodel_main.jl:658-730 prep_Hamil_pn
void prep_Hamil_pn(Problem& P) {
  const Snt& s = P.snt;
  const auto& mp = P.ms.p;
  const auto& mn = P.ms.n;
  int lpm = (int)mp.size(), lnm = (int)mn.size();
  int loff = (int)s.p_sps.size();
  std::vector<int> Mzs;
  for (int j = 0; j < lpm; ++j)
    for (int i = 0; i < lpm; ++i) Mzs.push_back(mp[i][4] - mp[j][4]);
  std::sort(Mzs.begin(), Mzs.end());
  Mzs.erase(std::unique(Mzs.begin(), Mzs.end()), Mzs.end());
  std::reverse(Mzs.begin(), Mzs.end());
  P.delMs = Mzs;
  std::vector<DedupList> dl(Mzs.size());
  int ja, jb, jc, jd;
  std::vector<int> ma_s, mb_s, mc_s, md_s, ma_i, mb_i, mc_i, md_i;
  for (size_t i = 0; i < s.TBMEs[2].size(); ++i) {
    double ME = s.TBMEs[2][i];
    auto lab = s.labels[2][i];
    int a = lab[0], b = lab[1], c = lab[2], d = lab[3], J2 = 2 * lab[4];
    possible_mz(s.p_sps[a - 1], mp, ja, ma_s, ma_i);
    possible_mz(s.p_sps[c - 1], mp, jc, mc_s, mc_i);
    possible_mz(s.n_sps[b - loff - 1], mn, jb, mb_s, mb_i);
    possible_mz(s.n_sps[d - loff - 1], mn, jd, md_s, md_i);
    for (size_t ic = 0; ic < mc_s.size(); ++ic) {
      int mc = mc_s[ic];
      i64 bit_c = onehot(lpm, mc_i[ic]);
      for (size_t ia = 0; ia < ma_s.size(); ++ia) {
        int ma = ma_s[ia];
        i64 bit_a = onehot(lpm, ma_i[ia]);
        int Mp = ma - mc;
        int idx = bisearch_desc_int(Mzs, Mp) - 1;
        for (size_t id = 0; id < md_s.size(); ++id) {
          int md = md_s[id];
          if (std::abs(mc + md) > J2) continue;
          i64 bit_d = onehot(lnm, md_i[id]);
          double CG1 = clebsch(jc, mc, jd, md, J2, mc + md);
          double tfac = ME * CG1;
          for (size_t ib = 0; ib < mb_s.size(); ++ib) {
            int mb = mb_s[ib];
            if (mb - md + Mp != 0) continue;
            i64 bit_b = onehot(lnm, mb_i[ib]);
            double fac = tfac * clebsch(ja, ma, jb, mb, J2, ma + mb);
            dl[idx].add(Key4{bit_a, bit_b, bit_c, bit_d}, fac);
          }
        }
      }
    }
  }
  P.bVpn.resize(Mzs.size());
  P.Vpn.resize(Mzs.size());
  for (size_t k = 0; k < Mzs.size(); ++k) {
    P.bVpn[k] = dl[k].keys;
    P.Vpn[k] = dl[k].vals;
  }
}

// shellmodel_main.jl:1169-1199 calc_1b_jumps!
void calc_1b_jumps(Problem& P, int bi, int bf, int j, const std::vector<Key4>& bV, const std::vector<double>& V) {
  const auto& pb = P.B.pbits;
  const auto& nb = P.B.nbits;
  std::vector<std::vector<Ifph>> plist(V.size()), nlist(V.size());
  for (size_t nth = 0; nth < V.size(); ++nth) {
    const Key4& k = bV[nth];
    if (V[nth] == 0.0) continue;
    for (size_t ip = 0; ip < pb[bi - 1].size(); ++ip) {
      i64 Phi = pb[bi - 1][ip];
      if (!TF_connectable_1(Phi, k.a, k.c)) continue;
      int ph;
      i64 fin;
      calc_phase_1(Phi, k.a, k.c, ph, fin);
      int r = bisearch_desc(pb[bf - 1], fin);
      if (r == 0) continue;
      plist[nth].push_back(Ifph{(int)ip + 1, r, ph == -1});
    }
    for (size_t in = 0; in < nb[bi - 1].size(); ++in) {
      i64 Phi = nb[bi - 1][in];
      if (!TF_connectable_1(Phi, k.b, k.d)) continue;
      int ph;
      i64 fin;
      calc_phase_1(Phi, k.b, k.d, ph, fin);
      int r = bisearch_desc(nb[bf - 1], fin);
      if (r == 0) continue;
      nlist[nth].push_back(Ifph{(int)in + 1, r, ph == -1});
    }
  }
  P.pNiNfs[bi - 1][j] = std::move(plist);
  P.nNiNfs[bi - 1][j] = std::move(nlist);
}

// shellmodel_main.jl:1139-1167 prep_pn
void prep_pn(Problem& P) {
  int lblock = (int)P.B.pbits.size();
  const auto& Mps = P.B.Mps;
  P.bfs.assign(lblock, {});
  P.bis.assign(lblock, {});
  auto inDel = [&](int dm) { return std::find(P.delMs.begin(), P.delMs.end(), dm) != P.delMs.end(); };
  for (int i = 1; i <= lblock; ++i)
    for (int j = i; j <= lblock; ++j)
      if (inDel(Mps[j - 1] - Mps[i - 1])) {
        P.bfs[i - 1].push_back(j);
        P.bis[j - 1].push_back(i);
      }
  P.pNiNfs.assign(lblock, {});
  P.nNiNfs.assign(lblock, {});
  for (int i = 0; i < lblock; ++i) {
    P.pNiNfs[i].resize(P.bfs[i].size());
    P.nNiNfs[i].resize(P.bfs[i].size());
  }
#pragma omp parallel for schedule(dynamic)
  for (int bi = 1; bi <= lblock; ++bi) {
    for (size_t j = 0; j < P.bfs[bi - 1].size(); ++j) {
      int bf = P.bfs[bi - 1][j];
      int dm = Mps[bf - 1] - Mps[bi - 1];
      if (!inDel(dm)) continue;
      int idx = bisearch_desc_int(P.delMs, dm) - 1;
      calc_1b_jumps(P, bi, bf, (int)j, P.bVpn[idx], P.Vpn[idx]);
    }
  }
}

// shellmodel_main.jl:1231-1263 make_distribute (block order for the threads)
std::vector<int> make_distribute(const std::vector<i64>& tasks_in, int n) {
  int lblock = (int)tasks_in.size();
  std::vector<int> idxs(lblock);
  for (int i = 0; i < lblock; ++i) idxs[i] = i + 1;
  std::stable_sort(idxs.begin(), idxs.end(), [&](int x, int y) { return tasks_in[x - 1] > tasks_in[y - 1]; });
  std::vector<std::vector<int>> tmp(n);
  int imin = 1;
  bool order = true;
  auto total = [&]() { size_t t = 0; for (auto& v : tmp) t += v.size(); return (int)t; };
  while (total() < lblock) {
    int imax = std::min(imin + n - 1, lblock);
    if (order) {
      for (int i = imin; i <= imax; ++i) tmp[i - imin].push_back(idxs[i - 1]);
      order = false;
    } else {
      for (int i = n; i >= 1; --i) {
        int j = imax - (n - i);
        tmp[i - 1].push_back(j < imin ? 0 : idxs[j - 1]);
      }
      order = true;
    }
    imin += n;
  }
  std::vector<int> out;
  for (auto& v : tmp) out.insert(out.end(), v.begin(), v.end());
  return out;
}

int n_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// lanczos_methods.jl:153-248 operate_H! (twf accumulates)
void operate_H(const Problem& P, const double* wf, double* twf) {
  const auto& B = P.B;
  const auto& tasks = P.block_tasks;
  int ntask = (int)tasks.size();
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < ntask; ++t) {
    int bi = tasks[t];
    if (bi == 0) continue;
    i64 idim = B.tdims[bi - 1];  // Julia tdims[bi] (1-based) = start of block bi
    i64 l_Np = (i64)B.pbits[bi - 1].size();
    i64 l_Nn = (i64)B.nbits[bi - 1].size();
    i64 offset = idim - l_Nn;
    // pn, forward: rows of bi <- columns of bf >= bi
    for (size_t bfidx = 0; bfidx < P.bfs[bi - 1].size(); ++bfidx) {
      int bf = P.bfs[bi - 1][bfidx];
      int r = bisearch_desc_int(P.delMs, B.Mps[bf - 1] - B.Mps[bi - 1]) - 1;
      const auto& Vs = P.Vpn[r];
      i64 fdim = B.tdims[bf - 1];
      i64 l_Nn_f = (i64)B.nbits[bf - 1].size();
      const auto& pN = P.pNiNfs[bi - 1][bfidx];
      const auto& nN = P.nNiNfs[bi - 1][bfidx];
      i64 off_f = fdim - l_Nn_f;
      for (size_t nth = 0; nth < Vs.size(); ++nth) {
        double V = Vs[nth];
        for (const Ifph& pj : pN[nth]) {
          i64 tMi = offset + pj.i * l_Nn, tMf = off_f + pj.f * l_Nn_f;
          for (const Ifph& nj : nN[nth]) {
            i64 Mi = tMi + nj.i, Mf = tMf + nj.f;
            twf[Mi - 1] += ((pj.phase != nj.phase) ? -V : V) * wf[Mf - 1];
          }
        }
      }
    }
    // pn, transpose: rows of bi <- columns of lower blocks
    for (size_t j = 0; j + 1 < P.bis[bi - 1].size(); ++j) {
      int tbi = P.bis[bi - 1][j];
      int r = bisearch_desc_int(P.delMs, B.Mps[bi - 1] - B.Mps[tbi - 1]) - 1;
      // bisearch_ord!(bfs[tbi], bi): ascending search
      const auto& bft = P.bfs[tbi - 1];
      int r2 = (int)(std::lower_bound(bft.begin(), bft.end(), bi) - bft.begin());
      i64 fdim = B.tdims[tbi - 1];
      i64 l_Nn_i = (i64)B.nbits[tbi - 1].size();
      const auto& pN = P.pNiNfs[tbi - 1][r2];
      const auto& nN = P.nNiNfs[tbi - 1][r2];
      i64 off_f = fdim - l_Nn_i;
      const auto& Vs = P.Vpn[r];
      for (size_t nth = 0; nth < Vs.size(); ++nth) {
        double V = Vs[nth];
        for (const Ifph& pj : pN[nth]) {
          i64 tMi = off_f + pj.i * l_Nn_i, tMf = offset + pj.f * l_Nn;
          for (const Ifph& nj : nN[nth]) {
            i64 Mi = tMi + nj.i, Mf = tMf + nj.f;
            twf[Mf - 1] += ((pj.phase != nj.phase) ? -V : V) * wf[Mi - 1];
          }
        }
      }
    }
    // pp
    for (i64 Npi = 1; Npi <= l_Np; ++Npi) {
      i64 tMi = offset + Npi * l_Nn;
      for (const T1info& t1 : P.pp[bi - 1][Npi - 1]) {
        i64 tMf = offset + l_Nn * t1.f;
        double fac = t1.coef;
        for (i64 nidx = 1; nidx <= l_Nn; ++nidx) {
          i64 Mi = tMi + nidx, Mf = tMf + nidx;
          twf[Mf - 1] += fac * wf[Mi - 1];
          twf[Mi - 1] += fac * wf[Mf - 1];
        }
      }
    }
    // nn
    for (i64 Nni = 1; Nni <= l_Nn; ++Nni) {
      i64 tMi = offset + Nni;
      for (const T1info& t1 : P.nn[bi - 1][Nni - 1]) {
        i64 tMf = offset + t1.f;
        double fac = t1.coef;
        for (i64 pidx = 1; pidx <= l_Np; ++pidx) {
          i64 Mi = tMi + pidx * l_Nn, Mf = tMf + pidx * l_Nn;
          twf[Mf - 1] += fac * wf[Mi - 1];
          twf[Mi - 1] += fac * wf[Mf - 1];
        }
      }
    }
    // one-body
    const auto& Sp = P.snt.SPEs[0];
    const auto& Sn = P.snt.SPEs[1];
    for (i64 pidx = 1; pidx <= l_Np; ++pidx) {
      const auto& jp = B.jocc_p[bi - 1][pidx - 1];
      double ep = 0.0;
      for (size_t k = 0; k < Sp.size(); ++k) ep += Sp[k] * jp[k];
      i64 tMi = offset + pidx * l_Nn;
      for (i64 nidx = 1; nidx <= l_Nn; ++nidx) {
        const auto& jn = B.jocc_n[bi - 1][nidx - 1];
        double en = 0.0;
        for (size_t k = 0; k < Sn.size(); ++k) en += Sn[k] * jn[k];
        i64 Mi = tMi + nidx;
        twf[Mi - 1] += (ep + en) * wf[Mi - 1];
      }
    }
  }
}

// Number of distinct (row, col) pairs that operate_H! touches: the structural
// non-zeros of H (diagonal included).  Each block's owner emits the pairs of
// its rows in the same loops as operate_H!, then sorts and de-duplicates them.
long long count_nnz(const Problem& P) {
  const auto& B = P.B;
  int nb = (int)B.pbits.size();
  long long total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
  for (int bi = 1; bi <= nb; ++bi) {
    std::vector<u64> pr;
    auto push = [&](i64 row, i64 col) { pr.push_back(((u64)(row - 1) << 32) | (u64)(col - 1)); };
    i64 idim = B.tdims[bi - 1];
    i64 l_Np = (i64)B.pbits[bi - 1].size(), l_Nn = (i64)B.nbits[bi - 1].size();
    i64 offset = idim - l_Nn;
    for (size_t bfidx = 0; bfidx < P.bfs[bi - 1].size(); ++bfidx) {
      int bf = P.bfs[bi - 1][bfidx];
      i64 l_Nn_f = (i64)B.nbits[bf - 1].size(), off_f = B.tdims[bf - 1] - l_Nn_f;
      const auto& pN = P.pNiNfs[bi - 1][bfidx];
      const auto& nN = P.nNiNfs[bi - 1][bfidx];
      for (size_t nth = 0; nth < pN.size(); ++nth)
        for (const Ifph& pj : pN[nth])
          for (const Ifph& nj : nN[nth]) push(offset + pj.i * l_Nn + nj.i, off_f + pj.f * l_Nn_f + nj.f);
    }
    for (size_t j = 0; j + 1 < P.bis[bi - 1].size(); ++j) {
      int tbi = P.bis[bi - 1][j];
      const auto& bft = P.bfs[tbi - 1];
      int r2 = (int)(std::lower_bound(bft.begin(), bft.end(), bi) - bft.begin());
      i64 l_Nn_i = (i64)B.nbits[tbi - 1].size(), off_f = B.tdims[tbi - 1] - l_Nn_i;
      const auto& pN = P.pNiNfs[tbi - 1][r2];
      const auto& nN = P.nNiNfs[tbi - 1][r2];
      for (size_t nth = 0; nth < pN.size(); ++nth)
        for (const Ifph& pj : pN[nth])
          for (const Ifph& nj : nN[nth]) push(offset + pj.f * l_Nn + nj.f, off_f + pj.i * l_Nn_i + nj.i);
    }
    for (i64 Npi = 1; Npi <= l_Np; ++Npi)
      for (const T1info& t1 : P.pp[bi - 1][Npi - 1])
        for (i64 n = 1; n <= l_Nn; ++n) {
          i64 Mi = offset + Npi * l_Nn + n, Mf = offset + t1.f * l_Nn + n;
          push(Mf, Mi);
          push(Mi, Mf);
        }
    for (i64 Nni = 1; Nni <= l_Nn; ++Nni)
      for (const T1info& t1 : P.nn[bi - 1][Nni - 1])
        for (i64 p = 1; p <= l_Np; ++p) {
          i64 Mi = offset + p * l_Nn + Nni, Mf = offset + p * l_Nn + t1.f;
          push(Mf, Mi);
          push(Mi, Mf);
        }
    for (i64 p = 1; p <= l_Np; ++p)
      for (i64 n = 1; n <= l_Nn; ++n) push(offset + p * l_Nn + n, offset + p * l_Nn + n);
    std::sort(pr.begin(), pr.end());
    total += (long long)(std::unique(pr.begin(), pr.end()) - pr.begin());
  }
  return total;
}

// ---------------------------------------------------------------------------
// Dense symmetric eigen-decomposition by cyclic Jacobi rotations (stands in
// for LAPACK eigen/eigvals at lanczos_methods.jl:255,261 and
// shellmodel_main.jl:209).  A is n×n column-major; w ascending; Z columns are
// the eigenvectors (Z may be null).
void sym_eig(int n, const double* A, double* w, double* Z) {
  std::vector<double> a(A, A + (size_t)n * n), v;
  bool want = Z != nullptr;
  if (want) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  }
  auto at = [&](int i, int j) -> double& { return a[(size_t)j * n + i]; };
  double fro = 0;
  for (size_t k = 0; k < a.size(); ++k) fro += a[k] * a[k];
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < j; ++i) off += at(i, j) * at(i, j);
    if (off <= 1e-34 * fro || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = at(p, q);
        if (apq == 0.0) continue;
        double app = at(p, p), aqq = at(q, q);
        if (std::fabs(apq) < 1e-300) { at(p, q) = at(q, p) = 0.0; continue; }
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(1.0 + theta * theta));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = at(k, p), akq = at(k, q);
          at(k, p) = c * akp - s * akq;
          at(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = at(p, k), aqk = at(q, k);
          at(p, k) = c * apk - s * aqk;
          at(q, k) = s * apk + c * aqk;
        }
        at(p, q) = at(q, p) = 0.0;
        if (want)
          for (int k = 0; k < n; ++k) {
            double vkp = v[(size_t)p * n + k], vkq = v[(size_t)q * n + k];
            v[(size_t)p * n + k] = c * vkp - s * vkq;
            v[(size_t)q * n + k] = s * vkp + c * vkq;
          }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return at(x, x) < at(y, y); });
  for (int i = 0; i < n; ++i) w[i] = at(ord[i], ord[i]);
  if (want)
    for (int i = 0; i < n; ++i)
      std::memcpy(Z + (size_t)i * n, v.data() + (size_t)ord[i] * n, sizeof(double) * n);
}

// Start vector: the reference draws randn with Julia's seeded RNG
// (shellmodel_main.jl:939-948), which cannot be reproduced outside Julia.
// Both this oracle and the GPU library use this hash-based draw instead:
// v[i] = u0+u1+u2+u3-2 with u_k = splitmix64(seed + φ·(4i+k+1)) >> 11 · 2^-53.
inline double start_elem(u64 seed, i64 i) {
  double u[4];
  for (int k = 0; k < 4; ++k) {
    u64 z = seed + 0x9E3779B97F4A7C15ull * (u64)(4 * i + k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    u[k] = (double)(z >> 11) * 0x1.0p-53;
  }
  return ((u[0] + u[1]) + (u[2] + u[3])) - 2.0;
}

double dotp(i64 n, const double* x, const double* y) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (i64 i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}
void axpy(i64 n, double a, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < n; ++i) y[i] += a * x[i];
}
void scal(i64 n, double a, double* x) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < n; ++i) x[i] *= a;
}

struct TrlResult {
  std::vector<double> en;
  int elit = 0, n_hv = 0, n_restart = 0;
  bool converged = false;
  std::vector<double> ritz;  // num_ev × mdim
  double t_hv = 0, t_reorth = 0, t_restart = 0;
};

}  // namespace

#include <chrono>
namespace {
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// shellmodel_main.jl:1005-1012 ReORTH: MGS of vt against vks[it..1].
void ReORTH(int it, double* vt, std::vector<std::vector<double>>& vks, i64 n) {
  for (int l = it; l >= 1; --l) {
    double a = dotp(n, vks[l - 1].data(), vt);
    axpy(n, -a, vks[l - 1].data(), vt);
  }
}

// SD pair -> basis index, for the ladder operators below.
struct PairHash {
  size_t operator()(const std::pair<i64, i64>& k) const { return std::hash<i64>()(k.first * 1000003 + k.second); }
};
typedef std::unordered_map<std::pair<i64, i64>, i64, PairHash> BasisIndex;

BasisIndex index_basis(const Problem& P) {
  BasisIndex at;
  const Basis& B = P.B;
  for (size_t b = 0; b < B.pbits.size(); ++b)
    for (size_t ip = 0; ip < B.pbits[b].size(); ++ip)
      for (size_t in = 0; in < B.nbits[b].size(); ++in)
        at[{B.pbits[b][ip], B.nbits[b][in]}] = B.tdims[b] + (i64)ip * (i64)B.nbits[b].size() + (i64)in;
  return at;
}

// out = (J- J+) v on the M basis: the product that operate_J! applies
// (shellmodel_main.jl:1566-1650, jump lists from prep_J :1439-1565),
// restated with the ladder operators J+- = sum sqrt(j(j+1) - m(m+-1)) a+_{m+-1} a_m
// over both species.  Neighbouring m-states of an orbit are adjacent in
// construct_msps order, so every move has fermion sign +1.
void operate_JmJp(const Problem& P, const BasisIndex& at, const double* v, double* out) {
  const Basis& B = P.B;
  const int Lp = (int)P.ms.p.size(), Ln = (int)P.ms.n.size();
  std::unordered_map<std::pair<i64, i64>, double, PairHash> up;
  for (size_t b = 0; b < B.pbits.size(); ++b)
    for (size_t ip = 0; ip < B.pbits[b].size(); ++ip)
      for (size_t in = 0; in < B.nbits[b].size(); ++in) {
        const double c = v[B.tdims[b] + (i64)ip * (i64)B.nbits[b].size() + (i64)in];
        if (c == 0.0) continue;
        for (int sp = 0; sp < 2; ++sp) {
          const auto& ms = sp == 0 ? P.ms.p : P.ms.n;
          const int L = sp == 0 ? Lp : Ln;
          const i64 bits = sp == 0 ? B.pbits[b][ip] : B.nbits[b][in];
          for (int k = 1; k < L; ++k) {
            if (ms[k][5] != ms[k - 1][5]) continue;
            const i64 bk = onehot(L, k), bk1 = onehot(L, k + 1);
            if (!(bits & bk) || (bits & bk1)) continue;
            const double j2 = ms[k - 1][2], m2 = ms[k - 1][4];
            const double f = 0.5 * std::sqrt(j2 * (j2 + 2.0) - m2 * (m2 + 2.0));
            const i64 nb = bits ^ bk ^ bk1;
            up[sp == 0 ? std::make_pair(nb, B.nbits[b][in]) : std::make_pair(B.pbits[b][ip], nb)] += f * c;
          }
        }
      }
  std::fill(out, out + P.mdim, 0.0);
  for (const auto& kv : up) {
    for (int sp = 0; sp < 2; ++sp) {
      const auto& ms = sp == 0 ? P.ms.p : P.ms.n;
      const int L = sp == 0 ? Lp : Ln;
      const i64 bits = sp == 0 ? kv.first.first : kv.first.second;
      for (int k = 1; k < L; ++k) {
        if (ms[k][5] != ms[k - 1][5]) continue;
        const i64 bk = onehot(L, k), bk1 = onehot(L, k + 1);
        if (!(bits & bk1) || (bits & bk)) continue;
        const double j2 = ms[k][2], m2 = ms[k][4];
        const double f = 0.5 * std::sqrt(j2 * (j2 + 2.0) - m2 * (m2 - 2.0));
        const i64 nb = bits ^ bk ^ bk1;
        auto it = at.find(sp == 0 ? std::make_pair(nb, kv.first.second) : std::make_pair(kv.first.first, nb));
        if (it != at.end()) out[it->second] += f * kv.second;
      }
    }
  }
}

// lanczos_methods.jl:132-151 ThickRestart_J (ls = 1): keep the Ritz vector of
// the eigenvalue closest to eval_jj; the arrow element goes to row ls+1 and
// column k as in the reference.
void ThickRestart_J(std::vector<std::vector<double>>& vks, std::vector<double>& Tm, int ldT, int lm, double eval_jj,
                    i64 mdim) {
  auto T = [&](int i, int j) -> double& { return Tm[(size_t)(j - 1) * ldT + (i - 1)]; };
  const int m = lm - 1, ls = 1;
  std::vector<double> sub((size_t)m * m), vals(m), vecs((size_t)m * m);
  for (int j = 1; j <= m; ++j)
    for (int i = 1; i <= m; ++i) sub[(size_t)(j - 1) * m + (i - 1)] = T(i, j);
  sym_eig(m, sub.data(), vals.data(), vecs.data());
  int k = 1;
  for (int i = 2; i <= m; ++i)
    if (std::fabs(vals[i - 1] - eval_jj) < std::fabs(vals[k - 1] - eval_jj)) k = i;
  const double beta = T(lm - 1, lm);
  std::fill(Tm.begin(), Tm.end(), 0.0);
  T(1, 1) = vals[k - 1];
  const double tmp = beta * vecs[(size_t)(k - 1) * m + (lm - 2)];
  T(ls + 1, k) = tmp;
  T(k, ls + 1) = tmp;
  std::vector<double> uk(mdim, 0.0);
  for (int j = 1; j <= m; ++j) axpy(mdim, vecs[(size_t)(k - 1) * m + (j - 1)], vks[j - 1].data(), uk.data());
  const double nrm = 1.0 / std::sqrt(dotp(mdim, uk.data(), uk.data()));
  for (i64 i = 0; i < mdim; ++i) vks[0][i] = uk[i] * nrm;
  vks[1] = vks[lm - 1];
  for (int kk = ls + 2; kk <= (int)vks.size(); ++kk) std::fill(vks[kk - 1].begin(), vks[kk - 1].end(), 0.0);
}

// lanczos_methods.jl:93-131 Jlanczos: Lanczos on J^2 = J-J+ + eval_jj (the
// space has M = J) from Jvs[0] until the lowest Ritz value is within Jtol of
// eval_jj; Jvs[0] returns the projection.
void Jlanczos(const Problem& P, const BasisIndex& at, std::vector<std::vector<double>>& Jvs, double eval_jj,
              double Jtol) {
  const i64 mdim = P.mdim;
  const int lnJ = (int)Jvs.size();
  std::vector<double> Jmat((size_t)lnJ * lnJ, 0.0);
  auto Jm = [&](int i, int j) -> double& { return Jmat[(size_t)(j - 1) * lnJ + (i - 1)]; };
  int eljit = 1, k = 1, inow = k;
  bool JTF = false;
  std::vector<double> w;
  while (!JTF) {
    for (int it = k; it <= lnJ - 1; ++it) {
      inow = it;
      double* vk = Jvs[it - 1].data();
      double* vkp1 = Jvs[it].data();
      operate_JmJp(P, at, vk, vkp1);
      axpy(mdim, eval_jj, vk, vkp1);
      Jm(it, it) = dotp(mdim, vk, vkp1);
      std::vector<double> sub((size_t)it * it);
      for (int j = 1; j <= it; ++j)
        for (int i = 1; i <= it; ++i) sub[(size_t)(j - 1) * it + (i - 1)] = Jm(i, j);
      w.assign(it, 0.0);
      sym_eig(it, sub.data(), w.data(), nullptr);
      if (std::fabs(w[0] - eval_jj) < Jtol) {
        eljit = it;
        JTF = true;
        break;
      }
      ReORTH(it, vkp1, Jvs, mdim);
      const double beta = std::sqrt(dotp(mdim, vkp1, vkp1));
      scal(mdim, 1.0 / beta, vkp1);
      Jm(it + 1, it) = beta;
      Jm(it, it + 1) = beta;
      eljit = it;
    }
    if (!JTF) {
      ThickRestart_J(Jvs, Jmat, lnJ, eljit + 1, eval_jj, mdim);
      k = 2;
    }
  }
  if (inow > k) ThickRestart_J(Jvs, Jmat, lnJ, eljit + 1, eval_jj, mdim);
}

// lanczos_methods.jl:1-91 TRL + 250-258 diagonalize_T! + 260-307 ThickRestart,
// then shellmodel_main.jl:208-224 Ritz vectors.
TrlResult TRL(const Problem& P, int num_ev, int lm, int ls, double tol, int max_restart, const double* v1,
              u64 seed, bool want_vecs, int num_history, int max_hv = 0, double eval_jj = -1.0) {
  i64 mdim = P.mdim;
  num_ev = (int)std::min<i64>(num_ev, mdim);
  TrlResult R;
  std::vector<std::vector<double>> vks(lm, std::vector<double>(mdim, 0.0));
  std::vector<std::vector<double>> uks(ls, std::vector<double>(mdim, 0.0));
  std::vector<double> T((size_t)lm * lm, 0.0);
  auto Tm = [&](int i, int j) -> double& { return T[(size_t)(j - 1) * lm + (i - 1)]; };
  std::vector<std::vector<double>> en(num_history, std::vector<double>(num_ev, 1.0e4));
  if (v1) {
    std::memcpy(vks[0].data(), v1, sizeof(double) * mdim);
  } else {
    for (i64 i = 0; i < mdim; ++i) vks[0][i] = start_elem(seed, i);
  }
  scal(mdim, 1.0 / std::sqrt(dotp(mdim, vks[0].data(), vks[0].data())), vks[0].data());
  // doubleLanczos (target_J): J-projection of every new Krylov vector
  const bool dl = eval_jj >= 0.0;
  const double Jtol = 1.e-7;
  std::vector<std::vector<double>> Jvs;
  BasisIndex bindex;
  if (dl) {
    bindex = index_basis(P);
    Jvs.assign(ls, std::vector<double>(mdim, 0.0));
    Jvs[0] = vks[0];
    Jlanczos(P, bindex, Jvs, eval_jj, Jtol);
    vks[0] = Jvs[0];
    scal(mdim, 1.0 / std::sqrt(dotp(mdim, vks[0].data(), vks[0].data())), vks[0].data());
  }
  bool TF = false;
  int elit = 1, k = 1;
  std::vector<double> wbuf, Zbuf;
  while (!TF) {
    for (int it = k; it <= lm - 1; ++it) {
      double* vk = vks[it - 1].data();
      double* vkp1 = vks[it].data();
      double t0 = now_s();
      operate_H(P, vk, vkp1);
      R.t_hv += now_s() - t0;
      R.n_hv++;
      if (max_hv > 0 && R.n_hv >= max_hv) { TF = false; elit = it; goto sample_end; }
      {
      double talpha = dotp(mdim, vk, vkp1);
      Tm(it, it) = talpha;
      // diagonalize_T!
      for (int ith = num_history - 1; ith >= 1; --ith) en[ith] = en[ith - 1];
      int n = std::min(num_ev, it);
      std::vector<double> sub((size_t)it * it);
      for (int j = 1; j <= it; ++j)
        for (int i = 1; i <= it; ++i) sub[(size_t)(j - 1) * it + (i - 1)] = Tm(i, j);
      wbuf.assign(it, 0.0);
      sym_eig(it, sub.data(), wbuf.data(), nullptr);
      for (int i = 0; i < n; ++i) en[0][i] = wbuf[i];
      bool all_ok = true;
      for (int i = 0; i < num_ev; ++i)
        if (!(en[1][i] - en[0][i] < tol)) all_ok = false;
      if (all_ok) TF = true;
      if (it == mdim) TF = true;
      if (TF) { elit = it; break; }
      t0 = now_s();
      ReORTH(it, vkp1, vks, mdim);
      R.t_reorth += now_s() - t0;
      double tbeta = std::sqrt(dotp(mdim, vkp1, vkp1));
      scal(mdim, 1.0 / tbeta, vkp1);
      Tm(it + 1, it) = tbeta;
      Tm(it, it + 1) = tbeta;
      if (dl) {
        if (tbeta < Jtol) { TF = true; elit = it; break; }
        for (size_t q = 1; q < Jvs.size(); ++q) std::fill(Jvs[q].begin(), Jvs[q].end(), 0.0);
        std::memcpy(Jvs[0].data(), vkp1, sizeof(double) * mdim);
        Jlanczos(P, bindex, Jvs, eval_jj, Jtol);
        std::memcpy(vkp1, Jvs[0].data(), sizeof(double) * mdim);
        ReORTH(it, vkp1, vks, mdim);
        scal(mdim, 1.0 / std::sqrt(dotp(mdim, vkp1, vkp1)), vkp1);
      }
      }
    }
    if (!TF) {
      if (R.n_restart >= max_restart) break;
      R.n_restart++;
      double t_rs0 = now_s();
      // ThickRestart
      int m = lm - 1;
      std::vector<double> sub((size_t)m * m), vals(m), vecs((size_t)m * m);
      for (int j = 1; j <= m; ++j)
        for (int i = 1; i <= m; ++i) sub[(size_t)(j - 1) * m + (i - 1)] = Tm(i, j);
      sym_eig(m, sub.data(), vals.data(), vecs.data());
      auto V = [&](int j, int kk) { return vecs[(size_t)(kk - 1) * m + (j - 1)]; };
      double beta = Tm(lm - 1, lm);
      std::fill(T.begin(), T.end(), 0.0);
      for (int kk = 1; kk <= ls; ++kk) Tm(kk, kk) = vals[kk - 1];
      for (int kk = 1; kk <= ls; ++kk) {
        double tmp = beta * V(lm - 1, kk);
        Tm(ls + 1, kk) = tmp;
        Tm(kk, ls + 1) = tmp;
        std::fill(uks[kk - 1].begin(), uks[kk - 1].end(), 0.0);
        for (int j = 1; j <= lm - 1; ++j) axpy(mdim, V(j, kk), vks[j - 1].data(), uks[kk - 1].data());
      }
      for (int kk = 1; kk <= ls; ++kk) {
        if (kk > 1) ReORTH(kk - 1, uks[kk - 1].data(), uks, mdim);
        double nrm = 1.0 / std::sqrt(dotp(mdim, uks[kk - 1].data(), uks[kk - 1].data()));
        for (i64 i = 0; i < mdim; ++i) vks[kk - 1][i] = uks[kk - 1][i] * nrm;
      }
      vks[ls] = vks[lm - 1];
      ReORTH(ls, vks[ls].data(), vks, mdim);
      for (int kk = ls + 2; kk <= lm; ++kk) std::fill(vks[kk - 1].begin(), vks[kk - 1].end(), 0.0);
      R.t_restart += now_s() - t_rs0;
    }
    k = ls + 1;
  }
sample_end:
  R.converged = TF;
  R.elit = elit;
  R.en = en[0];
  if (want_vecs) {
    int m = elit;
    std::vector<double> sub((size_t)m * m), vals(m), vecs((size_t)m * m);
    for (int j = 1; j <= m; ++j)
      for (int i = 1; i <= m; ++i) sub[(size_t)(j - 1) * m + (i - 1)] = Tm(i, j);
    sym_eig(m, sub.data(), vals.data(), vecs.data());
    R.ritz.assign((size_t)num_ev * mdim, 0.0);
    for (int nth = 0; nth < num_ev; ++nth) {
      double* Rv = R.ritz.data() + (size_t)nth * mdim;
      for (int kk = 0; kk < m; ++kk) axpy(mdim, vecs[(size_t)nth * m + kk], vks[kk].data(), Rv);
      scal(mdim, 1.0 / std::sqrt(dotp(mdim, Rv, Rv)), Rv);
    }
  }
  return R;
}

// ---------------------------------------------------------------------------
// Block Lanczos: TRBL (lanczos_methods.jl:312-423), bl_ReORTH (:425-436),
// bl_QR! (shellmodel_main.jl:1049-1066), add_bl_T! (:1201-1205),
// bl_ThickRestart (lanczos_methods.jl:647-716) and the block Ritz vectors
// (shellmodel_main.jl:208-224).  A block is q rows of mdim; the start block is
// q hash draws (seeds seed..seed+q-1), orthonormalised as initialize_bl_wav
// (:950-965) does and then QR-factorised.
typedef std::vector<std::vector<double>> Block;  // q rows

// bl_QR!: modified Gram-Schmidt over the rows; R upper triangular (q x q, R[j*q+k] = R(j,k))
void bl_QR(Block& Q, std::vector<double>& R, i64 mdim) {
  const int q = (int)Q.size();
  std::fill(R.begin(), R.end(), 0.0);
  for (int j = 0; j < q; ++j) {
    const double t = std::sqrt(dotp(mdim, Q[j].data(), Q[j].data()));
    R[(size_t)j * q + j] = t;
    scal(mdim, 1.0 / t, Q[j].data());
    for (int k = j + 1; k < q; ++k) {
      double r = 0.0;
      for (i64 i = 0; i < mdim; ++i) r += Q[j][i] * Q[k][i];
      R[(size_t)j * q + k] = r;
      axpy(mdim, -r, Q[j].data(), Q[k].data());
    }
  }
}

// HV -= (HV Vt^T) Vt for the blocks vks[it-2] .. vks[0]
void bl_ReORTH(int it, Block& HV, std::vector<Block>& vks, i64 mdim) {
  const int q = (int)HV.size();
  for (int l = it - 1; l >= 1; --l) {
    const Block& Vt = vks[l - 1];
    std::vector<double> R((size_t)q * q);
    for (int i = 0; i < q; ++i)
      for (int j = 0; j < q; ++j) R[(size_t)i * q + j] = dotp(mdim, HV[i].data(), Vt[j].data());
    for (int i = 0; i < q; ++i)
      for (int j = 0; j < q; ++j) axpy(mdim, -R[(size_t)i * q + j], Vt[j].data(), HV[i].data());
  }
}

TrlResult TRBL(const Problem& P, int q, int num_ev, int lm, int ls, double tol, int max_restart, const double* v1,
               u64 seed, bool want_vecs, int num_history) {
  const i64 mdim = P.mdim;
  num_ev = (int)std::min<i64>(num_ev, mdim);
  TrlResult R;
  const int ls_sub = ls / q, itmax = lm / q - 1;
  const int nblk = lm / q;
  std::vector<Block> vks(nblk, Block(q, std::vector<double>(mdim, 0.0)));
  std::vector<Block> uks(ls_sub, Block(q, std::vector<double>(mdim, 0.0)));
  std::vector<double> T((size_t)lm * lm, 0.0);
  auto Tm = [&](int i, int j) -> double& { return T[(size_t)(j - 1) * lm + (i - 1)]; };
  std::vector<std::vector<double>> en(num_history, std::vector<double>(num_ev, 1.0e4));
  std::vector<double> Beta((size_t)q * q, 0.0);
  // start block (initialize_bl_wav + bl_QR!)
  for (int i = 0; i < q; ++i) {
    double* v = vks[0][i].data();
    if (v1) std::memcpy(v, v1 + (size_t)i * mdim, sizeof(double) * mdim);
    else
      for (i64 x = 0; x < mdim; ++x) v[x] = start_elem(seed + (u64)i, x);
    for (int k = i - 1; k >= 0; --k) axpy(mdim, -dotp(mdim, v, vks[0][k].data()), vks[0][k].data(), v);
    scal(mdim, 1.0 / std::sqrt(dotp(mdim, v, v)), v);
  }
  bl_QR(vks[0], Beta, mdim);
  bool TF = false;
  int elit = 1, inow = 1, itmin = 1;
  std::vector<double> wbuf;
  while (!TF) {
    for (int it = itmin; it <= itmax; ++it) {
      inow = it;
      Block& V = vks[it - 1];
      Block& HV = vks[it];
      for (int i = 0; i < q; ++i) {
        std::fill(HV[i].begin(), HV[i].end(), 0.0);
        operate_H(P, V[i].data(), HV[i].data());
      }
      R.n_hv += q;
      std::vector<double> Rm((size_t)q * q);  // Rm[i*q+j] = V_i . HV_j
      for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) Rm[(size_t)i * q + j] = dotp(mdim, V[i].data(), HV[j].data());
      bool sym = true;
      for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j)
          if (Rm[(size_t)i * q + j] != Rm[(size_t)j * q + i]) sym = false;
      if (!sym)
        for (int i = 0; i < q; ++i)
          for (int j = i; j < q; ++j) Rm[(size_t)i * q + j] = Rm[(size_t)j * q + i];
      for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) Tm(q * it - q + 1 + i, q * it - q + 1 + j) = Rm[(size_t)i * q + j];
      // diagonalize_T!(it*q)
      const int kk = it * q;
      for (int ith = num_history - 1; ith >= 1; --ith) en[ith] = en[ith - 1];
      std::vector<double> sub((size_t)kk * kk);
      for (int j = 1; j <= kk; ++j)
        for (int i = 1; i <= kk; ++i) sub[(size_t)(j - 1) * kk + (i - 1)] = Tm(i, j);
      wbuf.assign(kk, 0.0);
      sym_eig(kk, sub.data(), wbuf.data(), nullptr);
      for (int i = 0; i < std::min(num_ev, kk); ++i) en[0][i] = wbuf[i];
      bool all_ok = true;
      for (int i = 0; i < num_ev; ++i)
        if (!(en[1][i] - en[0][i] < tol)) all_ok = false;
      if (all_ok) TF = true;
      // HV -= R V
      for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) axpy(mdim, -Rm[(size_t)i * q + j], V[j].data(), HV[i].data());
      bl_ReORTH(it, HV, vks, mdim);
      bl_QR(HV, Beta, mdim);
      // add_bl_T!: T[block it+1, block it] = Beta, T[block it, block it+1] = Beta^T
      for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) {
          Tm(q * it + 1 + i, q * it - q + 1 + j) = Beta[(size_t)i * q + j];
          Tm(q * it - q + 1 + j, q * it + 1 + i) = Beta[(size_t)i * q + j];
        }
      if (TF) { elit = it; break; }
    }
    if (!TF) {
      if (R.n_restart >= max_restart) break;
      R.n_restart++;
      // bl_ThickRestart
      const int lmq = q * inow, lsq = q * ls_sub;
      std::vector<double> sub((size_t)lmq * lmq), vals(lmq), vecs((size_t)lmq * lmq);
      for (int j = 1; j <= lmq; ++j)
        for (int i = 1; i <= lmq; ++i) sub[(size_t)(j - 1) * lmq + (i - 1)] = Tm(i, j);
      sym_eig(lmq, sub.data(), vals.data(), vecs.data());
      auto VV = [&](int row, int col) { return vecs[(size_t)(col - 1) * lmq + (row - 1)]; };
      std::fill(T.begin(), T.end(), 0.0);
      for (int k = 1; k <= lsq; ++k) Tm(k, k) = vals[k - 1];
      for (int a = 1; a <= q; ++a)
        for (int k = 1; k <= lsq; ++k) {
          double r = 0.0;
          for (int b = 1; b <= q; ++b) r += Beta[(size_t)(a - 1) * q + (b - 1)] * VV(lmq - q + b, k);
          Tm(lsq + a, k) = r;
          Tm(k, lsq + a) = r;
        }
      for (int bi = 1; bi <= ls_sub; ++bi)
        for (int b = 1; b <= q; ++b) {
          std::vector<double>& u = uks[bi - 1][b - 1];
          std::fill(u.begin(), u.end(), 0.0);
          const int k = q * (bi - 1) + b;
          for (int j = 1; j <= inow; ++j)
            for (int bj = 1; bj <= q; ++bj) axpy(mdim, VV(q * (j - 1) + bj, k), vks[j - 1][bj - 1].data(), u.data());
        }
      for (int i = 0; i < ls_sub; ++i) vks[i] = uks[i];
      vks[ls_sub] = vks[inow];
      for (int i = ls_sub + 1; i < nblk; ++i)
        for (auto& r : vks[i]) std::fill(r.begin(), r.end(), 0.0);
      for (int i = 2; i <= ls_sub + 1; ++i) {
        Block& V = vks[i - 1];
        for (int j = i - 1; j >= 1; --j) {
          const Block& Vt = vks[j - 1];
          std::vector<double> Rm((size_t)q * q);
          for (int a = 0; a < q; ++a)
            for (int b = 0; b < q; ++b) Rm[(size_t)a * q + b] = dotp(mdim, V[a].data(), Vt[b].data());
          for (int a = 0; a < q; ++a)
            for (int b = 0; b < q; ++b) axpy(mdim, -Rm[(size_t)a * q + b], Vt[b].data(), V[a].data());
        }
        bl_QR(V, Beta, mdim);
      }
      itmin = ls_sub + 1;
    }
  }
  R.converged = TF;
  R.elit = elit;
  R.en = en[0];
  if (want_vecs) {
    const int m = elit * q;
    std::vector<double> sub((size_t)m * m), vals(m), vecs((size_t)m * m);
    for (int j = 1; j <= m; ++j)
      for (int i = 1; i <= m; ++i) sub[(size_t)(j - 1) * m + (i - 1)] = Tm(i, j);
    sym_eig(m, sub.data(), vals.data(), vecs.data());
    R.ritz.assign((size_t)num_ev * mdim, 0.0);
    for (int nth = 0; nth < num_ev; ++nth) {
      double* Rv = R.ritz.data() + (size_t)nth * mdim;
      for (int k = 1; k <= m; ++k) {
        const int it = (k - 1) / q, b = k - q * it;
        axpy(mdim, vecs[(size_t)nth * m + (k - 1)], vks[it][b - 1].data(), Rv);
      }
      scal(mdim, 1.0 / std::sqrt(dotp(mdim, Rv, Rv)), Rv);
    }
  }
  return R;
}

// shellmodel_main.jl:89-147 main_sm set-up (target_J = [], no truncation).
Problem* build_problem(const std::string& sntf, const std::string& nuc, int nthreads_for_tasks, int mtot_override = -1) {
  Problem* P = new Problem();
  // util_func.jl:1 reg = r"[0-9]+": first run of digits is A
  size_t d0 = nuc.find_first_of("0123456789");
  if (d0 == std::string::npos) throw Err{"no mass number in nucleus name"};
  size_t d1 = nuc.find_first_not_of("0123456789", d0);
  std::string anum = nuc.substr(d0, d1 == std::string::npos ? std::string::npos : d1 - d0);
  P->Anum = std::stoi(anum);
  P->snt = readsmsnt(sntf, P->Anum);
  P->Mtot = (P->Anum % 2 == 0) ? 0 : 1;
  // target_J = [tJ]: Mtot = tJ (shellmodel_main.jl:112-115)
  if (mtot_override >= 0) {
    if (mtot_override % 2 != P->Anum % 2) throw Err{"invalid target J for this nucleus"};
    P->Mtot = mtot_override;
  }
  // replace(target_nuc, string(Anum) => "")
  std::string el = nuc;
  size_t pos = el.find(std::to_string(P->Anum));
  if (pos != std::string::npos) el.erase(pos, std::to_string(P->Anum).size());
  // shellmodel_main.jl:908-916 getZNA
  int Z = 0;
  for (int i = 0; i < (int)(sizeof(kElements) / sizeof(kElements[0])); ++i)
    if (el == kElements[i]) { Z = i; break; }
  P->Z = Z;
  P->N = P->Anum - Z;
  P->vp = Z - P->snt.cp;
  P->vn = P->N - P->snt.cn;
  if (P->vp < 0 || P->vn < 0) throw Err{"negative valence particle number"};
  P->ms = construct_msps(P->snt);
  if (P->vp > (int)P->ms.p.size() || P->vn > (int)P->ms.n.size()) throw Err{"too many valence particles"};
  P->B = occ(P->snt, P->ms, P->vp, P->vn, P->Mtot);
  P->mdim = P->B.tdims.back();
  if (P->mdim == 0) return P;
  prep_Hamil_T1(*P);
  prep_Hamil_pn(*P);
  prep_pn(*P);
  std::vector<i64> tasks;
  for (size_t b = 0; b < P->B.pbits.size(); ++b) tasks.push_back((i64)P->B.pbits[b].size() * (i64)P->B.nbits[b].size());
  P->block_tasks = make_distribute(tasks, std::max(1, nthreads_for_tasks));
  return P;
}


// ===========================================================================
// One-body M1 / E2 operators (src/ShellModel/transit.jl).

// transit.jl:49-60 init_ho_by_mass
void init_ho_by_mass(int A, int hwprm, double& hw, double& bpar) {
  const double nmass[2] = {938.27231, 939.56563};
  const double amass = (nmass[0] + nmass[1]) / 2;
  const double hc = 197.32696;
  if (hwprm == 1) hw = 41.0 * std::pow((double)A, -1.0 / 3.0);
  else hw = 45.0 * std::pow((double)A, -1.0 / 3.0) - 25.0 * std::pow((double)A, -2.0 / 3.0);
  bpar = hc / std::sqrt(hw * amass);
}

// transit.jl:62-80 radius_power.  Julia evaluates the sum in BigInt/BigFloat
// (Combinatorics.doublefactorial); here exact integers up to the two square
// roots, which are taken in long double.
long double jl_binomial(int n, int k) {
  if (k < 0) return 0;
  if (n < 0) return ((k & 1) ? -1 : 1) * jl_binomial(k - n - 1, k);
  if (k > n) return 0;
  long double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}
long double doublefactorial(int n) {
  long double r = 1;
  for (int i = n; i >= 2; i -= 2) r *= i;
  return r;
}
double radius_power(int k, int n1, int l1, int n2, int l2, double bpar) {
  long double s = 0;
  int ll = l1 + l2 + k, ll1 = l2 - l1 + k, ll2 = l1 - l2 + k;
  ll1 = ll1 / 2;
  ll2 = ll2 / 2;
  int imin = std::max(std::max(0, n1 - ll1), n2 - ll2), imax = std::min(n1, n2);
  for (int i = imin; i <= imax; ++i)
    s += jl_binomial(ll1, n1 - i) * jl_binomial(ll2, n2 - i) * (doublefactorial(ll + 2 * i + 1) / doublefactorial(2 * i));
  s *= std::sqrt(doublefactorial(2 * n1) / doublefactorial(2 * n1 + 2 * l1 + 1));
  s *= std::sqrt(doublefactorial(2 * n2) / doublefactorial(2 * n2 + 2 * l2 + 1));
  return (double)s * (1.0 / std::sqrt(std::pow(2.0, k))) * (((n1 - n2) & 1) ? -1.0 : 1.0) * std::pow(bpar, k);
}

inline double pm1(int e) { return (e & 1) ? -1.0 : 1.0; }

// transit.jl:1-15 op_M1 / op_E2 (1-based block and SD numbers)
struct OpD {
  int bi, i, f;
  bool phase;
  double fac;
};
// transit.jl:17-31 op_M1_nd / op_E2_nd
struct OpND {
  int bl, Nl, br, Nr;
  bool phase;
  double fac;
};
struct Obtr {
  std::vector<OpD> d[4];    // pjumps_mu, njumps_mu, pjumps_Q, njumps_Q
  std::vector<OpND> nd[4];
};

// transit.jl:82-245 prep_obtr_diag
void prep_obtr_diag(const Problem& P, double bpar, const double* gfactors, const double* eff_charge, Obtr& O) {
  const double ec_p = eff_charge[0], ec_n = eff_charge[1];
  const double c_mom_mu = std::sqrt(3.0 / (4.0 * M_PI)), c_mom_Q = std::sqrt(5.0 / (16.0 * M_PI));
  const int lblock = (int)P.B.nbits.size();
  for (int sp = 0; sp < 2; ++sp) {
    const auto& sps = sp == 0 ? P.snt.p_sps : P.snt.n_sps;
    const auto& msps = sp == 0 ? P.ms.p : P.ms.n;
    const int L = (int)msps.size();
    const auto& bits = sp == 0 ? P.B.pbits : P.B.nbits;
    const int lsp = (int)sps.size();
    for (int i = 1; i <= lsp; ++i) {
      const int ni = sps[i - 1][0], li = sps[i - 1][1], ji = sps[i - 1][2];
      for (int f = i; f <= lsp; ++f) {
        const int nf = sps[f - 1][0], lf = sps[f - 1][1], jf = sps[f - 1][2];
        const double ex_r2 = radius_power(2, ni, li, nf, lf, bpar);
        const double l6j = wigner6j(2 * lf, 2 * li, 2, ji, jf, 1);
        const double s6j = wigner6j(1, 1, 2, ji, jf, 2 * lf);
        const double Q3j = wigner3j(ji, 4, jf, 1, 0, -1);
        int jc, ja;
        std::vector<int> mc_s, mc_idxs, ma_s, ma_idxs;
        possible_mz(sps[i - 1], msps, jc, mc_s, mc_idxs);
        possible_mz(sps[f - 1], msps, ja, ma_s, ma_idxs);
        for (int mode = 0; mode < 2; ++mode) {  // "M1", "E2"
          if (mode == 0 && (ni != nf || li != lf)) continue;
          for (size_t ic = 0; ic < mc_s.size(); ++ic) {
            const int mc = mc_s[ic];
            const i64 bit_c = onehot(L, mc_idxs[ic]);
            for (size_t ia = 0; ia < ma_s.size(); ++ia) {
              const int ma = ma_s[ia];
              if (ma != mc) continue;
              const i64 bit_a = onehot(L, ma_idxs[ia]);
              const double pfac = std::sqrt((double)((ji + 1) * (jf + 1)));
              double coeff;
              if (sp == 0) {
                if (mode == 0) {
                  const double sign1 = pm1((jf - ma) / 2 + lf + (ji + 3) / 2);
                  const double sign2 = pm1((jf - ma) / 2 + lf + (jf + 3) / 2);
                  const double fac1 = sign1 * l6j * std::sqrt((double)(lf * (lf + 1) * (2 * lf + 1)));
                  const double fac2 = sign2 * s6j * std::sqrt(1.5);
                  const double m3j = pfac * wigner3j(jf, 2, ji, -ma, 0, mc);
                  coeff = m3j * (fac1 * gfactors[0] + fac2 * gfactors[2]) * c_mom_mu;
                } else {
                  const double signQ = pm1(jf + (1 - ma) / 2) * (1 + pm1(li + lf));
                  if (signQ == 0) continue;
                  const double m3j = wigner3j(jf, 4, ji, -ma, 0, mc);
                  coeff = signQ * m3j * Q3j * pfac * ec_p * c_mom_Q * ex_r2;
                }
              } else {
                const double sign1 = pm1((jf - ma) / 2 + lf + (ji + 3) / 2);
                const double sign2 = pm1((jf - ma) / 2 + lf + (jf + 3) / 2);
                if (mode == 0) {
                  const double fac1 = sign1 * pfac * std::sqrt((double)(lf * (lf + 1) * (2 * lf + 1))) * l6j;
                  const double fac2 = sign2 * pfac * std::sqrt(1.5) * s6j;
                  const double m3j = wigner3j(jf, 2, ji, -ma, 0, mc);
                  coeff = m3j * (fac1 * gfactors[1] + fac2 * gfactors[3]) * c_mom_mu;
                } else {
                  const double signQ = pm1(jf + (1 - ma) / 2) * (1 + pm1(li + lf));
                  if (signQ == 0) continue;
                  const double m3j = wigner3j(jf, 4, ji, -ma, 0, mc);
                  coeff = signQ * m3j * Q3j * pfac * ec_n * c_mom_Q * ex_r2;
                  if (coeff == 0.0) continue;
                }
              }
              for (int bi = 1; bi <= lblock; ++bi) {
                const auto& bl = bits[bi - 1];
                for (size_t N = 0; N < bl.size(); ++N) {
                  const i64 Phi = bl[N];
                  if (!TF_connectable_1(Phi, bit_a, bit_c)) continue;
                  int ph;
                  i64 nPhi;
                  calc_phase_1(Phi, bit_a, bit_c, ph, nPhi);
                  const int Nf = bisearch_desc(bl, nPhi);
                  if (Nf == 0) continue;
                  const int Ni = (int)N + 1;
                  O.d[2 * mode + sp].push_back(OpD{bi, Ni, Nf, ph == -1, coeff * (Ni == Nf ? 0.5 : 1.0)});
                }
              }
            }
          }
        }
      }
    }
  }
}

// transit.jl:247-284 op_obtr_diag (twf accumulates)
void op_obtr_diag(const Problem& P, const std::vector<OpD>& p_oprts, const std::vector<OpD>& n_oprts,
                  const double* wf, double* twf) {
  for (const OpD& t : p_oprts) {
    const double coeff = t.phase ? -t.fac : t.fac;
    const i64 idim = P.B.tdims[t.bi - 1];
    const i64 l_Nn = (i64)P.B.nbits[t.bi - 1].size();
    const i64 tMi = idim + (t.i - 1) * l_Nn, tMf = idim + (t.f - 1) * l_Nn;  // 0-based
    for (i64 n = 0; n < l_Nn; ++n) {
      twf[tMf + n] += coeff * wf[tMi + n];
      twf[tMi + n] += coeff * wf[tMf + n];
    }
  }
  for (const OpD& t : n_oprts) {
    const double coeff = t.phase ? -t.fac : t.fac;
    const i64 idim = P.B.tdims[t.bi - 1];
    const i64 l_Nn = (i64)P.B.nbits[t.bi - 1].size(), l_Np = (i64)P.B.pbits[t.bi - 1].size();
    for (i64 p = 0; p < l_Np; ++p) {
      const i64 Mi = idim + p * l_Nn + (t.i - 1), Mf = idim + p * l_Nn + (t.f - 1);
      twf[Mf] += coeff * wf[Mi];
      twf[Mi] += coeff * wf[Mf];
    }
  }
}

// transit.jl:501-531 calc_bifs (1-based [il, ir] pairs)
void calc_bifs(const Problem& L, const Problem& R, std::vector<std::array<int, 2>>& p_bifs,
               std::vector<std::array<int, 2>>& n_bifs) {
  std::vector<std::array<int, 2>> blocks_r, blocks_l;
  for (int Mp : R.B.Mps)
    for (int Mn : R.B.Mns)
      if (Mp + Mn == R.Mtot) blocks_r.push_back({Mp, Mn});
  for (int Mp : L.B.Mps)
    for (int Mn : L.B.Mns)
      if (Mp + Mn == L.Mtot) blocks_l.push_back({Mp, Mn});
  for (size_t ir = 0; ir < blocks_r.size(); ++ir)
    for (size_t il = 0; il < blocks_l.size(); ++il) {
      if (blocks_r[ir][1] == blocks_l[il][1]) p_bifs.push_back({(int)il + 1, (int)ir + 1});
      if (blocks_r[ir][0] == blocks_l[il][0]) n_bifs.push_back({(int)il + 1, (int)ir + 1});
    }
}

// transit.jl:286-445 prep_obtr_nondiag (Mtot_l = jl2, Mtot_r = jr2)
void prep_obtr_nondiag(const Problem& L, const Problem& R, double bpar, const double* gfactors,
                       const double* eff_charge, Obtr& O) {
  const int jl2 = L.Mtot, jr2 = R.Mtot;
  const int omu = (jl2 - jr2) / 2;  // Julia div truncates toward zero
  std::vector<std::array<int, 2>> bifs[2];
  calc_bifs(L, R, bifs[0], bifs[1]);
  const double ec_p = eff_charge[0], ec_n = eff_charge[1];
  const double c_mom_mu = std::sqrt(3.0 / (4.0 * M_PI)), c_mom_Q = std::sqrt(5.0 / (16.0 * M_PI));
  for (int sp = 0; sp < 2; ++sp) {
    const auto& sps = sp == 0 ? L.snt.p_sps : L.snt.n_sps;
    const auto& msps = sp == 0 ? L.ms.p : L.ms.n;
    const int Lm = (int)msps.size();
    const auto& bits_l = sp == 0 ? L.B.pbits : L.B.nbits;
    const auto& bits_r = sp == 0 ? R.B.pbits : R.B.nbits;
    const int lsp = (int)sps.size();
    for (int i = 1; i <= lsp; ++i) {
      const int ni = sps[i - 1][0], li = sps[i - 1][1], ji = sps[i - 1][2];
      for (int f = 1; f <= lsp; ++f) {
        const int nf = sps[f - 1][0], lf = sps[f - 1][1], jf = sps[f - 1][2];
        const double ex_r2 = radius_power(2, ni, li, nf, lf, bpar);
        const double l6j = wigner6j(2 * lf, 2 * li, 2, ji, jf, 1);
        const double s6j = wigner6j(1, 1, 2, ji, jf, 2 * lf);
        const double Q3j = wigner3j(ji, 4, jf, 1, 0, -1);
        int jc, ja;
        std::vector<int> mc_s, mc_idxs, ma_s, ma_idxs;
        possible_mz(sps[i - 1], msps, jc, mc_s, mc_idxs);
        possible_mz(sps[f - 1], msps, ja, ma_s, ma_idxs);
        for (int mode = 0; mode < 2; ++mode) {
          if (mode == 0) {
            if (ni != nf || li != lf) continue;
            if ((jl2 - jr2) / 2 > 1) continue;
          } else if ((jl2 - jr2) / 2 > 2) {
            continue;
          }
          for (size_t ic = 0; ic < mc_s.size(); ++ic) {
            const int mc = mc_s[ic];
            const i64 bit_c = onehot(Lm, mc_idxs[ic]);
            for (size_t ia = 0; ia < ma_s.size(); ++ia) {
              const int ma = ma_s[ia];
              if ((ma - mc) / 2 != omu) continue;
              const i64 bit_a = onehot(Lm, ma_idxs[ia]);
              const double pfac = std::sqrt((double)((ji + 1) * (jf + 1)));
              double coeff;
              const double sign1 = pm1((jf - ma) / 2 + lf + (ji + 3) / 2);
              const double sign2 = pm1((jf - ma) / 2 + lf + (jf + 3) / 2);
              if (mode == 0) {
                if (sp == 0) {
                  const double fac1 = sign1 * l6j * std::sqrt((double)(lf * (lf + 1) * (2 * lf + 1)));
                  const double fac2 = sign2 * s6j * std::sqrt(1.5);
                  const double m3j = pfac * wigner3j(jf, 2, ji, -ma, 2 * omu, mc);
                  coeff = m3j * (fac1 * gfactors[0] + fac2 * gfactors[2]) * c_mom_mu;
                } else {
                  const double fac1 = sign1 * pfac * std::sqrt((double)(lf * (lf + 1) * (2 * lf + 1))) * l6j;
                  const double fac2 = sign2 * pfac * std::sqrt(1.5) * s6j;
                  const double m3j = wigner3j(jf, 2, ji, -ma, 2 * omu, mc);
                  coeff = m3j * (fac1 * gfactors[1] + fac2 * gfactors[3]) * c_mom_mu;
                }
              } else {
                const double signQ = pm1(jf + (1 - ma) / 2) * (1 + pm1(li + lf));
                if (signQ == 0) continue;
                const double m3j = wigner3j(jf, 4, ji, -ma, 2 * omu, mc);
                coeff = signQ * m3j * Q3j * pfac * (sp == 0 ? ec_p : ec_n) * c_mom_Q * ex_r2;
              }
              for (const auto& lr : bifs[sp]) {
                const int bl = lr[0], br = lr[1];
                const auto& rb = bits_r[br - 1];
                for (size_t N = 0; N < rb.size(); ++N) {
                  const i64 Phi = rb[N];
                  if (!TF_connectable_1(Phi, bit_a, bit_c)) continue;
                  int ph;
                  i64 nPhi;
                  calc_phase_1(Phi, bit_a, bit_c, ph, nPhi);
                  const int Nf = bisearch_desc(bits_l[bl - 1], nPhi);
                  if (Nf == 0) continue;
                  O.nd[2 * mode + sp].push_back(OpND{bl, Nf, br, (int)N + 1, ph == -1, coeff});
                }
              }
            }
          }
        }
      }
    }
  }
}

// transit.jl:447-499 op_obtr_nondiag (twf accumulates, left basis)
void op_obtr_nondiag(const Problem& L, const Problem& R, const std::vector<OpND>& p_oprts,
                     const std::vector<OpND>& n_oprts, const double* wf, double* twf) {
  for (const OpND& t : p_oprts) {
    const double coeff = t.phase ? -t.fac : t.fac;
    const auto& nbit_r = R.B.nbits[t.br - 1];
    const auto& nbit_l = L.B.nbits[t.bl - 1];
    const i64 tMi = R.B.tdims[t.br - 1] + (i64)(t.Nr - 1) * (i64)nbit_r.size();
    const i64 tMf = L.B.tdims[t.bl - 1] + (i64)(t.Nl - 1) * (i64)nbit_l.size();
    for (size_t r = 0; r < nbit_r.size(); ++r)
      for (size_t l = 0; l < nbit_l.size(); ++l) {
        if (nbit_r[r] != nbit_l[l]) continue;
        twf[tMf + (i64)l] += coeff * wf[tMi + (i64)r];
      }
  }
  for (const OpND& t : n_oprts) {
    const double coeff = t.phase ? -t.fac : t.fac;
    const auto& pbit_r = R.B.pbits[t.br - 1];
    const auto& pbit_l = L.B.pbits[t.bl - 1];
    const i64 lNr = (i64)R.B.nbits[t.br - 1].size(), lNl = (i64)L.B.nbits[t.bl - 1].size();
    for (size_t r = 0; r < pbit_r.size(); ++r)
      for (size_t l = 0; l < pbit_l.size(); ++l) {
        if (pbit_r[r] != pbit_l[l]) continue;
        const i64 Mi = R.B.tdims[t.br - 1] + (i64)r * lNr + (t.Nr - 1);
        const i64 Mf = L.B.tdims[t.bl - 1] + (i64)l * lNl + (t.Nl - 1);
        twf[Mf] += coeff * wf[Mi];
      }
  }
}


// ===========================================================================
// Eigenvector-continuation transition densities
// (src/ShellModel/eigenvector_continuation.jl).

// shellmodel_main.jl:1297-1299 idx_from_ij (1-based)
i64 idx_from_ij(i64 i, i64 j, i64 Dim) { return (Dim + 1) * (i - 1) - (i * (i - 1)) / 2 + j - i + 1; }

// eigenvector_continuation.jl:1035-1099 calcOBTD: per pair, Σ_M w_i[M] w_j[M] jocc.
void calcOBTD(const Problem& P, const std::vector<const double*>& wfs, std::vector<std::vector<double>>& OBTDs) {
  const int lps = (int)P.snt.p_sps.size(), lns = (int)P.snt.n_sps.size();
  const int Dim = (int)wfs.size();
  for (int i = 1; i <= Dim; ++i)
    for (int j = i; j <= Dim; ++j) {
      std::vector<double>& T = OBTDs[idx_from_ij(i, j, Dim) - 1];
      const double* wi = wfs[i - 1];
      const double* wj = wfs[j - 1];
      for (size_t bi = 0; bi < P.B.pbits.size(); ++bi) {
        const i64 l_Nn = (i64)P.B.nbits[bi].size();
        for (size_t p = 0; p < P.B.jocc_p[bi].size(); ++p)
          for (i64 n = 0; n < l_Nn; ++n) {
            const i64 M = P.B.tdims[bi] + (i64)p * l_Nn + n;
            const double wfprod = wi[M] * wj[M];
            for (int o = 0; o < lps; ++o) T[o] += wfprod * P.B.jocc_p[bi][p][o];
            for (int o = 0; o < lns; ++o) T[lps + o] += wfprod * P.B.jocc_n[bi][n][o];
          }
      }
    }
}

// eigenvector_continuation.jl:1085-1100 T1ifc / T0ifc
struct T1ifc {
  int nth, bi, i, f;
  double fac;
};
struct T0ifc {
  int i, f;
  double fac;
};

// eigenvector_continuation.jl:1101-1304 prepTBTD + :1306-1380 calcTBTD,
// accumulated into TBTDs[pair][line-1].
void calcTBTD(const Problem& P, const std::vector<const double*>& wfs, std::vector<std::vector<double>>& TBTDs,
              int off) {
  const int lblock = (int)P.B.pbits.size();
  const int lp = (int)P.ms.p.size(), ln = (int)P.ms.n.size();
  const int Dim = (int)wfs.size();
  const int loffs[2] = {0, (int)P.snt.p_sps.size()};
  // pp / nn
  std::vector<T1ifc> TBTD1[2];
  for (int vrank = 0; vrank < 2; ++vrank) {
    const int loff = loffs[vrank];
    const auto& sps = vrank == 0 ? P.snt.p_sps : P.snt.n_sps;
    const auto& ms = vrank == 0 ? P.ms.p : P.ms.n;
    const auto& bits = vrank == 0 ? P.B.pbits : P.B.nbits;
    const int L = vrank == 0 ? lp : ln;
    for (size_t nth = 0; nth < P.snt.labels[vrank].size(); ++nth) {
      const auto& lab = P.snt.labels[vrank][nth];
      const int a = lab[0], b = lab[1], c = lab[2], d = lab[3], J2 = 2 * lab[4];
      int ja, jb, jc, jd;
      std::vector<int> ma_s, ma_i, mb_s, mb_i, mc_s, mc_i, md_s, md_i;
      possible_mz(sps[a - loff - 1], ms, ja, ma_s, ma_i);
      possible_mz(sps[b - loff - 1], ms, jb, mb_s, mb_i);
      possible_mz(sps[c - loff - 1], ms, jc, mc_s, mc_i);
      possible_mz(sps[d - loff - 1], ms, jd, md_s, md_i);
      for (size_t ic = 0; ic < mc_s.size(); ++ic)
        for (size_t id = 0; id < md_s.size(); ++id) {
          const int mc = mc_s[ic], md = md_s[id];
          if (c == d && mc >= md) continue;
          if (std::abs(mc + md) > J2) continue;
          const int M_ani = mc + md;
          const i64 bit_c = onehot(L, mc_i[ic]), bit_d = onehot(L, md_i[id]);
          for (size_t ia = 0; ia < ma_s.size(); ++ia)
            for (size_t ib = 0; ib < mb_s.size(); ++ib) {
              const int ma = ma_s[ia], mb = mb_s[ib];
              if (a == b && ma >= mb) continue;
              if (ma + mb != M_ani) continue;
              const i64 bit_a = onehot(L, ma_i[ia]), bit_b = onehot(L, mb_i[ib]);
              const double CG1 = clebsch(ja, ma, jb, mb, J2, M_ani);
              const double CG2 = clebsch(jc, mc, jd, md, J2, M_ani);
              const Key4 bl{bit_a, bit_b, bit_c, bit_d};
              const double coeff = std::sqrt((1.0 + (a == b)) * (1.0 + (c == d))) * CG1 * CG2;
              for (int bi = 1; bi <= lblock; ++bi) {
                const auto& lst = bits[bi - 1];
                for (size_t N = 0; N < lst.size(); ++N) {
                  if (!TF_connectable(lst[N], bl)) continue;
                  int ph;
                  i64 nPhi;
                  calc_phase(lst[N], bl, ph, nPhi);
                  const int Nf = bisearch_desc(lst, nPhi);
                  TBTD1[vrank].push_back(T1ifc{(int)nth, bi, (int)N + 1, Nf, coeff * ph});
                }
              }
            }
        }
    }
  }
  // pn jumps: delMs over proton m-state pairs (descending), blocks bi <= bf
  std::vector<int> delMs;
  for (int j = 0; j < lp; ++j)
    for (int i = 0; i < lp; ++i) delMs.push_back(P.ms.p[i][4] - P.ms.p[j][4]);
  std::sort(delMs.begin(), delMs.end(), std::greater<int>());
  delMs.erase(std::unique(delMs.begin(), delMs.end()), delMs.end());
  auto inDel = [&](int dm) { return std::find(delMs.begin(), delMs.end(), dm) != delMs.end(); };
  std::vector<std::vector<int>> bfs(lblock);
  for (int i = 1; i <= lblock; ++i)
    for (int j = i; j <= lblock; ++j)
      if (inDel(P.B.Mps[j - 1] - P.B.Mps[i - 1])) bfs[i - 1].push_back(j);
  const int nbif = lblock * (lblock + 1) / 2;
  struct PnOp {
    int nth;
    std::vector<std::vector<T0ifc>> pj, nj;  // per bif_idx
  };
  std::vector<PnOp> pnops;
  const auto& lab3 = P.snt.labels[2];
  for (size_t nth = 0; nth < lab3.size(); ++nth) {
    const int a = lab3[nth][0], b = lab3[nth][1], c = lab3[nth][2], d = lab3[nth][3], J2 = 2 * lab3[nth][4];
    const int loff = loffs[1];
    int ja, jb, jc, jd;
    std::vector<int> ma_s, ma_i, mb_s, mb_i, mc_s, mc_i, md_s, md_i;
    possible_mz(P.snt.p_sps[a - 1], P.ms.p, ja, ma_s, ma_i);
    possible_mz(P.snt.p_sps[c - 1], P.ms.p, jc, mc_s, mc_i);
    possible_mz(P.snt.n_sps[b - loff - 1], P.ms.n, jb, mb_s, mb_i);
    possible_mz(P.snt.n_sps[d - loff - 1], P.ms.n, jd, md_s, md_i);
    for (size_t ic = 0; ic < mc_s.size(); ++ic) {
      const int mc = mc_s[ic];
      const i64 bit_c = onehot(lp, mc_i[ic]);
      for (size_t ia = 0; ia < ma_s.size(); ++ia) {
        const int ma = ma_s[ia];
        const i64 bit_a = onehot(lp, ma_i[ia]);
        const int Mp = ma - mc;
        for (size_t id = 0; id < md_s.size(); ++id) {
          const int md = md_s[id];
          if (std::abs(mc + md) > J2) continue;
          const i64 bit_d = onehot(ln, md_i[id]);
          for (size_t ib = 0; ib < mb_s.size(); ++ib) {
            const int mb = mb_s[ib];
            if (mb - md + Mp != 0) continue;
            const i64 bit_b = onehot(ln, mb_i[ib]);
            const double CG1 = clebsch(ja, ma, jb, mb, J2, ma + mb);
            const double CG2 = clebsch(jc, mc, jd, md, J2, mc + md);
            const double fac = CG1 * CG2;
            PnOp op;
            op.nth = (int)nth;
            op.pj.assign(nbif, {});
            op.nj.assign(nbif, {});
            for (int bi = 1; bi <= lblock; ++bi)
              for (int bf : bfs[bi - 1]) {
                const int deltaM = P.B.Mps[bf - 1] - P.B.Mps[bi - 1];
                const double tfac = fac * (bi == bf ? 0.5 : 1.0);
                if (!inDel(deltaM)) continue;
                const int bif = (int)idx_from_ij(bi, bf, lblock) - 1;
                const auto& pb = P.B.pbits[bi - 1];
                for (size_t N = 0; N < pb.size(); ++N) {
                  if (!TF_connectable_1(pb[N], bit_a, bit_c)) continue;
                  int ph;
                  i64 f;
                  calc_phase_1(pb[N], bit_a, bit_c, ph, f);
                  const int Nf = bisearch_desc(P.B.pbits[bf - 1], f);
                  if (Nf == 0) continue;
                  op.pj[bif].push_back(T0ifc{(int)N + 1, Nf, tfac * ph});
                }
                const auto& nb = P.B.nbits[bi - 1];
                for (size_t N = 0; N < nb.size(); ++N) {
                  if (!TF_connectable_1(nb[N], bit_b, bit_d)) continue;
                  int ph;
                  i64 f;
                  calc_phase_1(nb[N], bit_b, bit_d, ph, f);
                  const int Nf = bisearch_desc(P.B.nbits[bf - 1], f);
                  if (Nf == 0) continue;
                  op.nj[bif].push_back(T0ifc{(int)N + 1, Nf, 1.0 * ph});
                }
              }
            pnops.push_back(std::move(op));
          }
        }
      }
    }
  }
  std::vector<std::array<int, 2>> bif_idxs;
  for (int i = 1; i <= lblock; ++i)
    for (int j = i; j <= lblock; ++j) bif_idxs.push_back({i, j});
  // calcTBTD
  for (int i = 1; i <= Dim; ++i)
    for (int j = i; j <= Dim; ++j) {
      const double* w_i = wfs[i - 1];
      const double* w_j = wfs[j - 1];
      std::vector<double>& T = TBTDs[idx_from_ij(i, j, Dim) - 1];
      for (int vrank = 0; vrank < 2; ++vrank)
        for (const T1ifc& t : TBTD1[vrank]) {
          const int vidx = P.snt.labels[vrank][t.nth][5];
          const i64 lN = (i64)P.B.nbits[t.bi - 1].size(), lP = (i64)P.B.pbits[t.bi - 1].size();
          const i64 td = P.B.tdims[t.bi - 1];
          if (vrank == 0) {
            for (i64 n = 0; n < lN; ++n) {
              const i64 Mi = td + (t.i - 1) * lN + n, Mf = td + (t.f - 1) * lN + n;
              T[off + vidx - 1] += t.fac * (w_i[Mf] * w_j[Mi]);
            }
          } else {
            for (i64 p = 0; p < lP; ++p) {
              const i64 Mi = td + p * lN + (t.i - 1), Mf = td + p * lN + (t.f - 1);
              T[off + vidx - 1] += t.fac * (w_i[Mf] * w_j[Mi]);
            }
          }
        }
      for (const PnOp& op : pnops) {
        const int vidx = lab3[op.nth][5];
        for (size_t bidx = 0; bidx < bif_idxs.size(); ++bidx) {
          const int bi = bif_idxs[bidx][0], bf = bif_idxs[bidx][1];
          const i64 idim = P.B.tdims[bi - 1], fdim = P.B.tdims[bf - 1];
          const i64 lNi = (i64)P.B.nbits[bi - 1].size(), lNf = (i64)P.B.nbits[bf - 1].size();
          for (const T0ifc& pj : op.pj[bidx]) {
            const i64 tMi = idim + (pj.i - 1) * lNi, tMf = fdim + (pj.f - 1) * lNf;
            for (const T0ifc& nj : op.nj[bidx]) {
              const i64 Mi = tMi + nj.i - 1, Mf = tMf + nj.f - 1;
              T[off + vidx - 1] += pj.fac * nj.fac * (w_i[Mf] * w_j[Mi]);
              T[off + vidx - 1] += pj.fac * nj.fac * (w_i[Mi] * w_j[Mf]);
            }
          }
        }
      }
    }
}

thread_local std::string g_err;
}  // namespace

// ===========================================================================
// C API used by the test harness (ctypes) and the CPU baseline in bench.py.
extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_threads() { return n_threads(); }

void* orc_create(const char* sntf, const char* nuc) {
  try {
    return build_problem(sntf, nuc, n_threads());
  } catch (const Err& e) {
    g_err = e.msg;
  } catch (const std::exception& e) {
    g_err = e.what();
  }
  return nullptr;
}
// main_sm with target_J = [tJ]: the basis of Mtot = tJ (doubled).
void* orc_create_M(const char* sntf, const char* nuc, int mtot) {
  try {
    return build_problem(sntf, nuc, n_threads(), mtot);
  } catch (const Err& e) {
    g_err = e.msg;
  } catch (const std::exception& e) {
    g_err = e.what();
  }
  return nullptr;
}
void orc_destroy(void* h) { delete (Problem*)h; }

long long orc_mdim(void* h) { return ((Problem*)h)->mdim; }
int orc_nblocks(void* h) { return (int)((Problem*)h)->B.pbits.size(); }
void orc_info(void* h, int* out /* Anum,Z,N,vp,vn,Mtot,lp_m,ln_m */) {
  Problem* P = (Problem*)h;
  out[0] = P->Anum; out[1] = P->Z; out[2] = P->N; out[3] = P->vp; out[4] = P->vn; out[5] = P->Mtot;
  out[6] = (int)P->ms.p.size(); out[7] = (int)P->ms.n.size();
}
void orc_blocks(void* h, long long* tdims, int* np, int* nn, int* Mp, int* Mn) {
  Problem* P = (Problem*)h;
  int nb = (int)P->B.pbits.size();
  for (int b = 0; b <= nb; ++b) tdims[b] = P->B.tdims[b];
  for (int b = 0; b < nb; ++b) {
    np[b] = (int)P->B.pbits[b].size();
    nn[b] = (int)P->B.nbits[b].size();
    Mp[b] = P->B.blkMp[b];
    Mn[b] = P->B.blkMn[b];
  }
}
// Concatenated SD bit strings, blocks in order.
void orc_sds(void* h, long long* pbits, long long* nbits) {
  Problem* P = (Problem*)h;
  size_t kp = 0, kn = 0;
  for (auto& v : P->B.pbits) for (i64 x : v) pbits[kp++] = x;
  for (auto& v : P->B.nbits) for (i64 x : v) nbits[kn++] = x;
}
// pp (which=0) / nn (which=1) 2b-jump tables: entries (block, i, f, coef), 1-based i,f.
long long orc_2b_count(void* h, int which) {
  Problem* P = (Problem*)h;
  const Jump2b& J = which == 0 ? P->pp : P->nn;
  long long c = 0;
  for (auto& b : J) for (auto& l : b) c += (long long)l.size();
  return c;
}
void orc_2b_export(void* h, int which, int* blk, int* i, int* f, double* coef) {
  Problem* P = (Problem*)h;
  const Jump2b& J = which == 0 ? P->pp : P->nn;
  long long c = 0;
  for (size_t b = 0; b < J.size(); ++b)
    for (size_t ii = 0; ii < J[b].size(); ++ii)
      for (auto& t : J[b][ii]) {
        blk[c] = (int)b + 1; i[c] = (int)ii + 1; f[c] = t.f; coef[c] = t.coef; ++c;
      }
}
// pn one-body lists: which=0 proton, 1 neutron; entries (bi, bf, nth, i, f, phase).
long long orc_pn_count(void* h, int which) {
  Problem* P = (Problem*)h;
  auto& L = which == 0 ? P->pNiNfs : P->nNiNfs;
  long long c = 0;
  for (auto& a : L) for (auto& b : a) for (auto& l : b) c += (long long)l.size();
  return c;
}
void orc_pn_export(void* h, int which, int* bi, int* bf, int* nth, int* i, int* f, int* phase) {
  Problem* P = (Problem*)h;
  auto& L = which == 0 ? P->pNiNfs : P->nNiNfs;
  long long c = 0;
  for (size_t b = 0; b < L.size(); ++b)
    for (size_t j = 0; j < L[b].size(); ++j)
      for (size_t n = 0; n < L[b][j].size(); ++n)
        for (auto& e : L[b][j][n]) {
          bi[c] = (int)b + 1; bf[c] = P->bfs[b][j]; nth[c] = (int)n + 1;
          i[c] = e.i; f[c] = e.f; phase[c] = e.phase ? 1 : 0; ++c;
        }
}
// m-scheme pn list per ΔM: delMs (descending) and entries (idx, a,b,c,d bits, V).
int orc_ndelM(void* h) { return (int)((Problem*)h)->delMs.size(); }
long long orc_vpn_count(void* h) {
  Problem* P = (Problem*)h;
  long long c = 0;
  for (auto& v : P->Vpn) c += (long long)v.size();
  return c;
}
void orc_vpn_export(void* h, int* delMs, int* idx, long long* abcd, double* V) {
  Problem* P = (Problem*)h;
  for (size_t k = 0; k < P->delMs.size(); ++k) delMs[k] = P->delMs[k];
  long long c = 0;
  for (size_t k = 0; k < P->Vpn.size(); ++k)
    for (size_t n = 0; n < P->Vpn[k].size(); ++n) {
      idx[c] = (int)k;
      const Key4& q = P->bVpn[k][n];
      abcd[4 * c] = q.a; abcd[4 * c + 1] = q.b; abcd[4 * c + 2] = q.c; abcd[4 * c + 3] = q.d;
      V[c] = P->Vpn[k][n];
      ++c;
    }
}
// m-scheme pp/nn list (prep_Hamil_T1): which 0/1.
long long orc_v1_count(void* h, int which) { return (long long)((Problem*)h)->V1[which].size(); }
void orc_v1_export(void* h, int which, long long* abcd, double* V) {
  Problem* P = (Problem*)h;
  for (size_t n = 0; n < P->V1[which].size(); ++n) {
    const Key4& q = P->bV1[which][n];
    abcd[4 * n] = q.a; abcd[4 * n + 1] = q.b; abcd[4 * n + 2] = q.c; abcd[4 * n + 3] = q.d;
    V[n] = P->V1[which][n];
  }
}
// Diagonal one-body energies per SD (dot(SPEs, jocc)).
void orc_spe_diag(void* h, double* ep, double* en) {
  Problem* P = (Problem*)h;
  size_t kp = 0, kn = 0;
  for (auto& b : P->B.jocc_p)
    for (auto& o : b) { double s = 0; for (size_t k = 0; k < o.size(); ++k) s += P->snt.SPEs[0][k] * o[k]; ep[kp++] = s; }
  for (auto& b : P->B.jocc_n)
    for (auto& o : b) { double s = 0; for (size_t k = 0; k < o.size(); ++k) s += P->snt.SPEs[1][k] * o[k]; en[kn++] = s; }
}

// <v|J^2|v> / <v|v> for one vector in basis order.  The reference evaluates
// J^2 = J-J+ + Jz(Jz+1) with jump lists (prep_J / operate_J!,
// shellmodel_main.jl:1439-1650, Js initialised to M(M+1) at :151); this
// restatement applies the ladder operator directly: <v|J-J+|v> = ||J+ v||^2,
// J+ = sum over species and m-states of sqrt(j(j+1) - m(m+1)) a+_{m+1} a_m.
// The m-states of an orbit are consecutive in construct_msps order, so the
// particle moves to the neighbouring position and the fermion sign is +1.
double orc_jj(void* h, const double* v) {
  Problem* P = (Problem*)h;
  const Basis& B = P->B;
  const int Lp = (int)P->ms.p.size(), Ln = (int)P->ms.n.size();
  struct KeyHash {
    size_t operator()(const std::pair<i64, i64>& k) const {
      return std::hash<i64>()(k.first * 1000003 + k.second);
    }
  };
  std::unordered_map<std::pair<i64, i64>, double, KeyHash> out;
  double vv = 0.0;
  for (size_t b = 0; b < B.pbits.size(); ++b) {
    const auto& pb = B.pbits[b];
    const auto& nb = B.nbits[b];
    for (size_t ip = 0; ip < pb.size(); ++ip)
      for (size_t in = 0; in < nb.size(); ++in) {
        const double c = v[B.tdims[b] + (i64)ip * (i64)nb.size() + (i64)in];
        vv += c * c;
        if (c == 0.0) continue;
        for (int sp = 0; sp < 2; ++sp) {
          const auto& ms = sp == 0 ? P->ms.p : P->ms.n;
          const int L = sp == 0 ? Lp : Ln;
          const i64 bits = sp == 0 ? pb[ip] : nb[in];
          for (int k = 1; k < L; ++k) {
            const auto& a = ms[k - 1];
            const auto& a1 = ms[k];
            if (a1[5] != a[5]) continue;  // k is the top m-state of its orbit
            const i64 bk = onehot(L, k), bk1 = onehot(L, k + 1);
            if (!(bits & bk) || (bits & bk1)) continue;
            const double j2 = a[2], m2 = a[4];
            const double f = 0.5 * std::sqrt(j2 * (j2 + 2.0) - m2 * (m2 + 2.0));
            const i64 nbits = bits ^ bk ^ bk1;
            const std::pair<i64, i64> key = sp == 0 ? std::make_pair(nbits, nb[in]) : std::make_pair(pb[ip], nbits);
            out[key] += f * c;
          }
        }
      }
  }
  double jp = 0.0;
  for (const auto& kv : out) jp += kv.second * kv.second;
  const double M = 0.5 * P->Mtot;
  return (jp + M * (M + 1.0) * vv) / vv;
}

// twf += H wf   (lanczos_methods.jl:153 operate_H! semantics)
void orc_operate_H(void* h, const double* wf, double* twf) { operate_H(*(Problem*)h, wf, twf); }

long long orc_nnz(void* h) { return count_nnz(*(Problem*)h); }

void orc_start_vector(long long mdim, unsigned long long seed, double* v) {
  for (i64 i = 0; i < mdim; ++i) v[i] = start_elem(seed, i);
}

// Block thick-restart Lanczos (TRBL, q vectors per block); v1: NULL or q x mdim.
int orc_trbl(void* h, int q, int num_ev, int lm, int ls, double tol, int max_restart, const double* v1,
             unsigned long long seed, double* evals, double* evecs, int* stats) {
  try {
    TrlResult R = TRBL(*(Problem*)h, q, num_ev, lm, ls, tol, max_restart, v1, seed, evecs != nullptr, 3);
    for (size_t i = 0; i < R.en.size(); ++i) evals[i] = R.en[i];
    if (evecs) std::memcpy(evecs, R.ritz.data(), sizeof(double) * R.ritz.size());
    if (stats) { stats[0] = R.elit; stats[1] = R.n_hv; stats[2] = R.n_restart; stats[3] = R.converged ? 1 : 0; }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Full thick-restart Lanczos.  stats: [elit, n_hv, n_restart, converged]; times: [t_hv, t_reorth, t_total].
int orc_trl(void* h, int num_ev, int lm, int ls, double tol, int max_restart, const double* v1,
            unsigned long long seed, double* evals, double* evecs, int* stats, double* times, double eval_jj) {
  try {
    double t0 = now_s();
    TrlResult R = TRL(*(Problem*)h, num_ev, lm, ls, tol, max_restart, v1, seed, evecs != nullptr, 3, 0, eval_jj);
    for (size_t i = 0; i < R.en.size(); ++i) evals[i] = R.en[i];
    if (evecs) std::memcpy(evecs, R.ritz.data(), sizeof(double) * R.ritz.size());
    if (stats) { stats[0] = R.elit; stats[1] = R.n_hv; stats[2] = R.n_restart; stats[3] = R.converged ? 1 : 0; }
    if (times) { times[0] = R.t_hv; times[1] = R.t_reorth; times[2] = now_s() - t0; }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Timed sample of the TRL loop for the CPU baseline: stops after max_hv
// H·v products.  out: [t_hv, t_reorth, t_restart, t_total, n_hv, n_restart].
int orc_trl_sample(void* h, int num_ev, int lm, int ls, double tol, int max_hv, double* out) {
  try {
    double t0 = now_s();
    TrlResult R = TRL(*(Problem*)h, num_ev, lm, ls, tol, 1000000, nullptr, 1234ull, false, 3, max_hv);
    out[0] = R.t_hv; out[1] = R.t_reorth; out[2] = R.t_restart; out[3] = now_s() - t0;
    out[4] = R.n_hv; out[5] = R.n_restart;
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Dense eigen-solver exposed for tests.
void orc_sym_eig(int n, const double* A, double* w, double* Z) { sym_eig(n, A, w, Z); }
double orc_clebsch(int tj1, int tm1, int tj2, int tm2, int tJ, int tM) { return clebsch(tj1, tm1, tj2, tm2, tJ, tM); }

// <vl_a| O |vr_b> for the M1 (op 0) or E2 (op 1) operator: symmetric = 1 is
// eval_moment's form (prep_obtr_diag / op_obtr_diag, one basis), 0 is
// transit_main's (prep_obtr_nondiag / op_obtr_nondiag).  The oscillator
// length follows main_sm / transit_main (hwprm 2 for 16 <= A <= 40).
int orc_obtr(void* hl, void* hr, int op, int symmetric, const double* gfactors, const double* eff_charge,
             const double* vl, int nl, const double* vr, int nr, double* out) {
  try {
    const Problem& L = *(Problem*)hl;
    const Problem& R = *(Problem*)hr;
    double hw, bpar;
    init_ho_by_mass(L.Anum, (16 <= L.Anum && L.Anum <= 40) ? 2 : 1, hw, bpar);
    Obtr O;
    if (symmetric) prep_obtr_diag(L, bpar, gfactors, eff_charge, O);
    else prep_obtr_nondiag(L, R, bpar, gfactors, eff_charge, O);
    std::vector<double> twf(L.mdim);
    for (int b = 0; b < nr; ++b) {
      std::fill(twf.begin(), twf.end(), 0.0);
      const double* wf = vr + (size_t)b * R.mdim;
      if (symmetric) op_obtr_diag(L, O.d[2 * op], O.d[2 * op + 1], wf, twf.data());
      else op_obtr_nondiag(L, R, O.nd[2 * op], O.nd[2 * op + 1], wf, twf.data());
      for (int a = 0; a < nl; ++a) out[(size_t)a * nr + b] = dotp(L.mdim, vl + (size_t)a * L.mdim, twf.data());
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
double orc_wigner3j(int a, int b, int c, int d, int e, int f) { return wigner3j(a, b, c, d, e, f); }
double orc_wigner6j(int a, int b, int c, int d, int e, int f) { return wigner6j(a, b, c, d, e, f); }
double orc_radius_power(int k, int n1, int l1, int n2, int l2, double bpar) { return radius_power(k, n1, l1, n2, l2, bpar); }

// prepEC mode "TD" (eigenvector_continuation.jl:212-310): Nmat (Dim x Dim)
// and, per pair i <= j in idx_from_ij order, the TD vector [OBTD_p, OBTD_n,
// TBTD per snt line].  ltd() gives its length.
int orc_ec_td_length(void* h) {
  const Problem& P = *(Problem*)h;
  return (int)(P.snt.p_sps.size() + P.snt.n_sps.size()) + P.snt.ntbme;
}
int orc_ec_td(void* h, const double* vecs, int nvec, double* nmat, double* td) {
  try {
    const Problem& P = *(Problem*)h;
    const int ltd = orc_ec_td_length(h);
    std::vector<const double*> wfs(nvec);
    for (int k = 0; k < nvec; ++k) wfs[k] = vecs + (size_t)k * P.mdim;
    for (int j = 0; j < nvec; ++j)
      for (int i = 0; i <= j; ++i) {
        const double tN = dotp(P.mdim, wfs[i], wfs[j]);
        nmat[(size_t)i * nvec + j] = tN;
        nmat[(size_t)j * nvec + i] = tN;
      }
    const int npair = nvec * (nvec + 1) / 2;
    std::vector<std::vector<double>> T(npair, std::vector<double>(ltd, 0.0));
    calcOBTD(P, wfs, T);
    calcTBTD(P, wfs, T, (int)(P.snt.p_sps.size() + P.snt.n_sps.size()));
    for (int p = 0; p < npair; ++p)
      for (int u = 0; u < ltd; ++u) td[(size_t)p * ltd + u] = T[p][u];
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"
