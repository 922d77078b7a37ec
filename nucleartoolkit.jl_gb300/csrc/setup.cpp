// Host-side set-up of a shell-model problem for the GPU kernels.
//
// Restates, for the GPU table layout, what NuclearToolkit.jl does before its
// Lanczos loop (paths relative to the NuclearToolkit.jl source tree):
//   readsmsnt          src/ShellModel/shellmodel_main.jl:293-365
//   construct_msps     :373-384      occ (basis, blocks)  :769-848
//   prep_Hamil_T1      :580-649      prep_2bjumps         :1115-1137
//   prep_Hamil_pn      :658-730      prep_pn/calc_1b_jumps! :1139-1199
// The m-scheme matrix elements are accumulated in the reference's loop and
// insertion order, so every operator value is bit-identical to the
// reference's.  The jump tables are re-organised for the GPU: instead of the
// reference's per-(block pair, V entry) lists they are "pull" tables in which
// every output row of H·v lists the source rows it reads (see hv.cu).
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <unordered_map>

#include "../../include/smgpu.h"

namespace smgpu {

// ---------------------------------------------------------------- parsing
namespace {
std::string trim(const std::string& s) {
  size_t b = s.find_first_not_of(" \t\r\n");
  if (b == std::string::npos) return std::string();
  size_t e = s.find_last_not_of(" \t\r\n");
  return s.substr(b, e - b + 1);
}
// Fields separated by single spaces (empty fields dropped), as
// rm_nan(split(line," ")) in util_func.jl:40-46.
std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && line[i] == ' ') ++i;
    size_t j = i;
    while (j < line.size() && line[j] != ' ') ++j;
    if (j > i) out.push_back(line.substr(i, j - i));
    i = j;
  }
  return out;
}
int to_int(const std::string& s) {
  char* end = nullptr;
  long v = std::strtol(s.c_str(), &end, 10);
  if (end == s.c_str() || *end != '\0') throw SetupError{SMGPU_ERR_PARSE, "not an integer: '" + s + "'"};
  return (int)v;
}
double to_dbl(const std::string& s) {
  char* end = nullptr;
  double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') throw SetupError{SMGPU_ERR_PARSE, "not a number: '" + s + "'"};
  return v;
}
}  // namespace

Interaction read_snt(const std::string& path, int Anum) {
  std::ifstream f(path);
  if (!f) throw SetupError{SMGPU_ERR_IO, "cannot open interaction file " + path};
  // util_func.jl:26-38 rm_comment: lines starting with '!' or '#' go, blank lines stay.
  std::vector<std::string> lines;
  std::string raw;
  while (std::getline(f, raw)) {
    std::string t = trim(raw);
    if (!t.empty() && (t[0] == '!' || t[0] == '#')) continue;
    lines.push_back(t);
  }
  size_t cur = 0;
  auto next = [&](size_t need) {
    if (cur >= lines.size()) throw SetupError{SMGPU_ERR_PARSE, "interaction file ends early"};
    auto t = tokens(lines[cur++]);
    if (t.size() < need) throw SetupError{SMGPU_ERR_PARSE, "too few fields on an snt line"};
    return t;
  };
  Interaction I;
  auto h = next(4);
  I.lp = to_int(h[0]); I.ln = to_int(h[1]); I.cp = to_int(h[2]); I.cn = to_int(h[3]);
  if (I.lp <= 0 || I.ln <= 0 || I.lp > 64 || I.ln > 64) throw SetupError{SMGPU_ERR_PARSE, "bad orbit counts"};
  I.porb.assign(I.lp, Orbit{-1, -1, -1, 0});
  I.norb.assign(I.ln, Orbit{-1, -1, -1, 0});
  for (int k = 0; k < I.lp + I.ln; ++k) {
    auto t = next(5);
    int idx = to_int(t[0]);
    Orbit o{to_int(t[1]), to_int(t[2]), to_int(t[3]), to_int(t[4])};
    if (idx >= 1 && idx <= I.lp) I.porb[idx - 1] = o;
    else if (idx > I.lp && idx <= I.lp + I.ln) I.norb[idx - I.lp - 1] = o;
    else throw SetupError{SMGPU_ERR_PARSE, "orbit index out of range"};
  }
  for (auto& o : I.porb) if (o.j2 < 0) throw SetupError{SMGPU_ERR_PARSE, "missing proton orbit"};
  for (auto& o : I.norb) if (o.j2 < 0) throw SetupError{SMGPU_ERR_PARSE, "missing neutron orbit"};
  // SPE block: only the first column selects the orbit, the third is the value.
  auto hs = next(2);
  int nsp = to_int(hs[0]);
  I.spe_p.assign(I.lp, 0.0);
  I.spe_n.assign(I.ln, 0.0);
  for (int k = 0; k < nsp; ++k) {
    auto t = next(3);
    int j = to_int(t[0]);
    if (j >= 1 && j <= I.lp) I.spe_p[j - 1] = to_dbl(t[2]);
    else if (j > I.lp && j <= I.lp + I.ln) I.spe_n[j - I.lp - 1] = to_dbl(t[2]);
    else throw SetupError{SMGPU_ERR_PARSE, "SPE index out of range"};
  }
  auto ht = next(3);
  int ntbme = to_int(ht[0]);
  int massop = to_int(ht[1]);
  double Aref = to_dbl(ht[2]);
  double pw = ht.size() > 3 ? to_dbl(ht[3]) : 0.0;
  for (int k = 0; k < ntbme; ++k) {
    auto t = next(6);
    int a = to_int(t[0]), b = to_int(t[1]), c = to_int(t[2]), d = to_int(t[3]), J = to_int(t[4]);
    double v = to_dbl(t[5]);
    int kind;
    if (a <= I.lp && b <= I.lp) kind = 0;
    else if (a > I.lp && b > I.lp) kind = 1;
    else if (a <= I.lp && b > I.lp) kind = 2;
    else throw SetupError{SMGPU_ERR_PARSE, "TBME with the proton index after the neutron index"};
    int lim = I.lp + I.ln;
    if (a < 1 || b < 1 || c < 1 || d < 1 || a > lim || b > lim || c > lim || d > lim)
      throw SetupError{SMGPU_ERR_PARSE, "TBME orbit index out of range"};
    if (massop == 1) v *= std::pow((double)Anum / Aref, pw);
    // readsmsnt adds (c,d,a,b) first when unique([a,b]) != unique([c,d]) (:354-357)
    bool same = (a == b) ? (c == d && c == a) : (c != d && a == c && b == d);
    if (!same) I.tb[kind].push_back({c, d, a, b, J, v, k + 1});
    I.tb[kind].push_back({a, b, c, d, J, v, k + 1});
  }
  I.nlines = ntbme;
  return I;
}

Interaction jj_interaction(const Interaction& I) {
  Interaction J;
  J.lp = I.lp;
  J.ln = I.ln;
  J.cp = I.cp;
  J.cn = I.cn;
  J.porb = I.porb;
  J.norb = I.norb;
  auto jj1 = [](int j2) { return 0.25 * j2 * (j2 + 2); };  // j(j+1) with j = j2/2
  for (const Orbit& o : I.porb) J.spe_p.push_back(jj1(o.j2));
  for (const Orbit& o : I.norb) J.spe_n.push_back(jj1(o.j2));
  for (int kind = 0; kind < 2; ++kind) {
    const std::vector<Orbit>& orb = kind == 0 ? I.porb : I.norb;
    const int off = kind == 0 ? 0 : I.lp;
    for (int a = 0; a < (int)orb.size(); ++a)
      for (int b = a; b < (int)orb.size(); ++b)
        for (int Jt = std::abs(orb[a].j2 - orb[b].j2) / 2; Jt <= (orb[a].j2 + orb[b].j2) / 2; ++Jt) {
          if (a == b && Jt % 2 == 1) continue;
          const double v = Jt * (Jt + 1.0) - jj1(orb[a].j2) - jj1(orb[b].j2);
          J.tb[kind].push_back({a + 1 + off, b + 1 + off, a + 1 + off, b + 1 + off, Jt, v});
        }
  }
  for (int a = 0; a < I.lp; ++a)
    for (int b = 0; b < I.ln; ++b)
      for (int Jt = std::abs(I.porb[a].j2 - I.norb[b].j2) / 2; Jt <= (I.porb[a].j2 + I.norb[b].j2) / 2; ++Jt) {
        const double v = Jt * (Jt + 1.0) - jj1(I.porb[a].j2) - jj1(I.norb[b].j2);
        J.tb[2].push_back({a + 1, I.lp + b + 1, a + 1, I.lp + b + 1, Jt, v});
      }
  return J;
}

void parse_nucleus(const std::string& nuc, int& A, int& Z) {
  static const char* el[] = {
      "n",  "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",
      "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As",
      "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn",
      "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho",
      "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po",
      "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md",
      "No", "Lr", "Rf", "Db", "Sg", "Bh", "Hs", "Mt", "Ds", "Rg", "Cn", "Nh", "Fl", "Mc", "Lv", "Ts", "Og"};
  size_t d0 = nuc.find_first_of("0123456789");
  if (d0 == std::string::npos) throw SetupError{SMGPU_ERR_NUCLEUS, "no mass number in '" + nuc + "'"};
  size_t d1 = nuc.find_first_not_of("0123456789", d0);
  std::string digits = nuc.substr(d0, d1 == std::string::npos ? std::string::npos : d1 - d0);
  A = to_int(digits);
  if (A <= 0) throw SetupError{SMGPU_ERR_NUCLEUS, "invalid mass number in '" + nuc + "'"};
  // replace(target_nuc, string(Anum) => ""): remove every occurrence
  std::string s = nuc, a = std::to_string(A);
  for (size_t p; (p = s.find(a)) != std::string::npos;) s.erase(p, a.size());
  Z = -1;
  for (int z = 1; z < (int)(sizeof(el) / sizeof(el[0])); ++z)
    if (s == el[z]) { Z = z; break; }
  if (Z < 0) throw SetupError{SMGPU_ERR_NUCLEUS, "unknown element in '" + nuc + "'"};
}

// ------------------------------------------------------ Clebsch–Gordan
// ⟨j1 m1 j2 m2|J M⟩ = sign(S)·sqrt(S²·C(2j1,n1)C(2j2,n1)(2J+1) /
//   [(j1+j2+J+1)·C(j1+j2+J,n1)·C(2j1,j1-m1)·C(2j2,j2-m2)·C(2J,J-M)])
// with n1 = j1+j2-J, n2 = j1-j2+J, n3 = j2-j1+J and the integer
// S = Σ_k (-1)^k C(n1,k) C(n2,j1-m1-k) C(n3,j2+m2-k) — Racah's sum
// rewritten in binomials.  The square is reduced exactly before the final
// sqrt, so the result is the rounded square root of the rounded quotient.
namespace {
typedef __int128 i128;
i128 binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  i128 r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}
i128 gcd_(i128 a, i128 b) {
  if (a < 0) a = -a;
  if (b < 0) b = -b;
  while (b != 0) { i128 t = a % b; a = b; b = t; }
  return a;
}
}  // namespace

namespace {
double clebsch_gordan_exact(int tj1, int tm1, int tj2, int tm2, int tJ, int tM);
}  // namespace

// Memoised per thread: the m-scheme loops ask for the same few hundred
// coefficients millions of times.
double clebsch_gordan(int tj1, int tm1, int tj2, int tm2, int tJ, int tM) {
  if (tj1 < 0 || tj2 < 0 || tJ < 0 || tj1 > 500 || tj2 > 500 || tJ > 1000 || std::abs(tm1) > 1000 ||
      std::abs(tm2) > 1000 || std::abs(tM) > 2000)
    return clebsch_gordan_exact(tj1, tm1, tj2, tm2, tJ, tM);
  const uint64_t key = ((uint64_t)tj1 << 52) | ((uint64_t)(tm1 + 1024) << 40) | ((uint64_t)tj2 << 31) |
                       ((uint64_t)(tm2 + 1024) << 19) | ((uint64_t)tJ << 9) | (uint64_t)((tM + 2048) & 0x1ff);
  // a direct-mapped cache in front of the map (a shell-model set-up asks for
  // a few thousand distinct coefficients some 10^5 times)
  struct Ent {
    uint64_t key;
    int tM;
    double v;
  };
  constexpr int kCache = 8192;
  thread_local std::vector<Ent> cache(kCache, Ent{~0ull, 0, 0.0});
  Ent& c = cache[(size_t)((key * 0x9E3779B97F4A7C15ull) >> 51) & (kCache - 1)];
  if (c.key == key && c.tM == tM) return c.v;
  thread_local std::unordered_map<uint64_t, std::pair<int, double>> memo;
  auto it = memo.find(key);
  double v;
  if (it != memo.end() && it->second.first == tM) {
    v = it->second.second;
  } else {
    v = clebsch_gordan_exact(tj1, tm1, tj2, tm2, tJ, tM);
    memo[key] = {tM, v};
  }
  c = Ent{key, tM, v};
  return v;
}

namespace {
// ⟨j1 m1 j2 m2|J M⟩² as an exact reduced fraction num/den and its sign;
// false when the coefficient vanishes.
bool cg_square(int tj1, int tm1, int tj2, int tm2, int tJ, int tM, i128& num, i128& den, int& sign) {
  if (tm1 + tm2 != tM) return false;
  if (std::abs(tm1) > tj1 || std::abs(tm2) > tj2 || std::abs(tM) > tJ) return false;
  if (((tj1 + tm1) | (tj2 + tm2) | (tJ + tM)) & 1) return false;
  if (tJ > tj1 + tj2 || tJ < std::abs(tj1 - tj2) || ((tj1 + tj2 + tJ) & 1)) return false;
  int n1 = (tj1 + tj2 - tJ) / 2, n2 = (tj1 - tj2 + tJ) / 2, n3 = (tj2 - tj1 + tJ) / 2;
  int j1mm1 = (tj1 - tm1) / 2, j2pm2 = (tj2 + tm2) / 2;
  i128 S = 0;
  for (int k = 0; k <= n1; ++k) {
    i128 t = binom(n1, k) * binom(n2, j1mm1 - k) * binom(n3, j2pm2 - k);
    S += (k & 1) ? -t : t;
  }
  if (S == 0) return false;
  int s3 = (tj1 + tj2 + tJ) / 2;
  num = S * S;
  den = 1;
  auto mul_num = [&](i128 x) { i128 g = gcd_(x, den); num *= x / g; den /= g; g = gcd_(num, den); num /= g; den /= g; };
  auto mul_den = [&](i128 x) { i128 g = gcd_(x, num); den *= x / g; num /= g; g = gcd_(num, den); num /= g; den /= g; };
  mul_num(binom(tj1, n1));
  mul_num(binom(tj2, n1));
  mul_num(tJ + 1);
  mul_den(s3 + 1);
  mul_den(binom(s3, n1));
  mul_den(binom(tj1, j1mm1));
  mul_den(binom(tj2, (tj2 - tm2) / 2));
  mul_den(binom(tJ, (tJ - tM) / 2));
  sign = S < 0 ? -1 : 1;
  return true;
}

double clebsch_gordan_exact(int tj1, int tm1, int tj2, int tm2, int tJ, int tM) {
  i128 num, den;
  int sign;
  if (!cg_square(tj1, tm1, tj2, tm2, tJ, tM, num, den, sign)) return 0.0;
  double v = std::sqrt((double)num / (double)den);
  return sign < 0 ? -v : v;
}

// Exact fraction with 128-bit parts, reduced after every operation.
struct Frac {
  i128 n = 0, d = 1;
  void reduce() {
    if (d < 0) { d = -d; n = -n; }
    i128 g = gcd_(n, d);
    if (g > 1) { n /= g; d /= g; }
  }
};
Frac fmul(Frac a, Frac b) {
  i128 g1 = gcd_(a.n, b.d), g2 = gcd_(b.n, a.d);
  if (g1 == 0) g1 = 1;
  if (g2 == 0) g2 = 1;
  Frac r{(a.n / g1) * (b.n / g2), (a.d / g2) * (b.d / g1)};
  r.reduce();
  return r;
}
Frac fadd(Frac a, Frac b) {
  i128 g = gcd_(a.d, b.d);
  if (g == 0) g = 1;
  Frac r{a.n * (b.d / g) + b.n * (a.d / g), (a.d / g) * b.d};
  r.reduce();
  return r;
}
i128 factorial(int n) {
  i128 r = 1;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}
// Δ(abc)² = (a+b-c)!(a-b+c)!(-a+b+c)!/(a+b+c+1)! for doubled a, b, c; false
// when the triad is not a triangle with an integer sum.
bool triad(int ta, int tb, int tc, Frac& out) {
  if (((ta + tb + tc) & 1) || tc > ta + tb || tc < std::abs(ta - tb)) return false;
  out = Frac{factorial((ta + tb - tc) / 2) * factorial((ta - tb + tc) / 2), 1};
  out = fmul(out, Frac{factorial((-ta + tb + tc) / 2), factorial((ta + tb + tc) / 2 + 1)});
  return true;
}
}  // namespace

// (j1 j2 j3; m1 m2 m3) = (-1)^(j1-j2-m3) ⟨j1 m1 j2 m2|j3 -m3⟩ / sqrt(2 j3 + 1),
// squared exactly before the one final square root.
double wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3) {
  i128 num, den;
  int sign;
  if (!cg_square(tj1, tm1, tj2, tm2, tj3, -tm3, num, den, sign)) return 0.0;
  Frac q = fmul(Frac{num, den}, Frac{1, (i128)(tj3 + 1)});
  if (((tj1 - tj2 - tm3) / 2) & 1) sign = -sign;
  const double v = std::sqrt((double)q.n / (double)q.d);
  return sign < 0 ? -v : v;
}

// {j1 j2 j3; j4 j5 j6} by Racah's single sum:
//   Δ(j1 j2 j3)Δ(j1 j5 j6)Δ(j4 j2 j6)Δ(j4 j5 j3) Σ_t (-1)^t (t+1)! /
//   [Π_k (t-α_k)! Π_l (β_l-t)!],
// α = the four triad sums, β = j1+j2+j4+j5, j2+j3+j5+j6, j3+j1+j6+j4;
// the square is exact and rounded once.
double wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6) {
  Frac d1, d2, d3, d4;
  if (!triad(tj1, tj2, tj3, d1) || !triad(tj1, tj5, tj6, d2) || !triad(tj4, tj2, tj6, d3) ||
      !triad(tj4, tj5, tj3, d4))
    return 0.0;
  const int a[4] = {(tj1 + tj2 + tj3) / 2, (tj1 + tj5 + tj6) / 2, (tj4 + tj2 + tj6) / 2, (tj4 + tj5 + tj3) / 2};
  const int b[3] = {(tj1 + tj2 + tj4 + tj5) / 2, (tj2 + tj3 + tj5 + tj6) / 2, (tj3 + tj1 + tj6 + tj4) / 2};
  const int tmin = std::max(std::max(a[0], a[1]), std::max(a[2], a[3]));
  const int tmax = std::min(std::min(b[0], b[1]), b[2]);
  Frac S{0, 1};
  for (int t = tmin; t <= tmax; ++t) {
    i128 den = 1;
    for (int k = 0; k < 4; ++k) den *= factorial(t - a[k]);
    for (int l = 0; l < 3; ++l) den *= factorial(b[l] - t);
    S = fadd(S, Frac{(t & 1) ? -factorial(t + 1) : factorial(t + 1), den});
  }
  if (S.n == 0) return 0.0;
  Frac q = fmul(fmul(fmul(d1, d2), fmul(d3, d4)), fmul(S, S));
  const double v = std::sqrt((double)q.n / (double)q.d);
  return S.n < 0 ? -v : v;
}

// ------------------------------------------------------------- helpers
namespace {
struct Key4 {
  uint64_t a, b, c, d;
  bool operator==(const Key4& o) const { return a == o.a && b == o.b && c == o.c && d == o.d; }
};
struct Key4H {
  size_t operator()(const Key4& k) const {
    uint64_t h = k.a * 0x9E3779B97F4A7C15ull ^ (k.b + 0x632BE59BD9B4E019ull);
    h = (h ^ (h >> 29)) * 0xBF58476D1CE4E5B9ull ^ (k.c * 0x94D049BB133111EBull);
    h = (h ^ (h >> 31)) * 0x9E3779B97F4A7C15ull ^ (k.d + 0x2545F4914F6CDD1Dull);
    return (size_t)(h ^ (h >> 32));
  }
};
// Where an operator (one-hot masks a, b, c, d) sits in its list: a dense
// array over the four bit positions when the m-state counts are small (the
// shell-model spaces in practice), a hash map otherwise.  Each key belongs to
// one list, so several lists can share one index.
struct OpIndex {
  int La = 0, Lb = 0;
  bool dense = false;
  std::vector<int32_t> slot;
  std::unordered_map<Key4, int32_t, Key4H> map;
  OpIndex(int la, int lb) : La(la), Lb(lb) {
    const size_t n = (size_t)la * la * lb * lb;
    dense = n <= ((size_t)1 << 22);
    if (dense) slot.assign(n, -1);
  }
  static int pos(uint64_t m) { return __builtin_ctzll(m); }
  // the slot of the key (-1: new; the caller then stores its position)
  int32_t& at(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    if (dense) return slot[(((size_t)pos(a) * Lb + pos(b)) * La + pos(c)) * Lb + pos(d)];
    auto it = map.emplace(Key4{a, b, c, d}, -1).first;
    return it->second;
  }
};

// Operator list with first-insertion order and in-place accumulation: same
// order and sums as the reference's `tl in blist` linear search.
struct OpList {
  std::vector<Op2> ops;
  void add(OpIndex& ix, uint64_t a, uint64_t b, uint64_t c, uint64_t d, double v) {
    int32_t& w = ix.at(a, b, c, d);
    if (w < 0) {
      w = (int32_t)ops.size();
      ops.push_back(Op2{a, b, c, d, v});
    } else {
      ops[w].v += v;
    }
  }
};

std::vector<MState> msps(const std::vector<Orbit>& orb) {
  std::vector<MState> m;
  for (size_t o = 0; o < orb.size(); ++o)
    for (int m2 = -orb[o].j2; m2 <= orb[o].j2; m2 += 2) m.push_back(MState{(int)o, orb[o].j2, m2});
  return m;
}
inline uint64_t bit_of(int L, int k0) { return 1ull << (L - 1 - k0); }
// m-state indices of orbit o (possible_mz, :552-565)
std::vector<int> mstates_of(const std::vector<MState>& ms, int o) {
  std::vector<int> r;
  for (size_t k = 0; k < ms.size(); ++k)
    if (ms[k].orbit == o) r.push_back((int)k);
  return r;
}

// prep_Hamil_T1 (:580-649) for one species.
std::vector<Op2> two_body_ops(const std::vector<Interaction::TB>& tbs, const std::vector<Orbit>& orb,
                              const std::vector<MState>& ms, int loff) {
  int L = (int)ms.size();
  OpList list;
  OpIndex ix(L, L);
  for (const auto& t : tbs) {
    int oa = t.a - 1 - loff, ob = t.b - 1 - loff, oc = t.c - 1 - loff, od = t.d - 1 - loff;
    auto ia = mstates_of(ms, oa), ib = mstates_of(ms, ob), ic = mstates_of(ms, oc), id = mstates_of(ms, od);
    int J2 = 2 * t.J;
    double nfac = std::sqrt((1.0 + (t.a == t.b ? 1.0 : 0.0)) * (1.0 + (t.c == t.d ? 1.0 : 0.0)));
    for (int kc : ic)
      for (int kd : id) {
        int mc = ms[kc].m2, md = ms[kd].m2;
        if (t.c == t.d && mc >= md) continue;
        if (std::abs(mc + md) > J2) continue;
        int Mani = mc + md;
        for (int ka : ia)
          for (int kb : ib) {
            int ma = ms[ka].m2, mb = ms[kb].m2;
            if (t.a == t.b && ma >= mb) continue;
            if (ma + mb != Mani) continue;
            double cg1 = clebsch_gordan(orb[oa].j2, ma, orb[ob].j2, mb, J2, Mani);
            double cg2 = clebsch_gordan(orb[oc].j2, mc, orb[od].j2, md, J2, Mani);
            list.add(ix, bit_of(L, ka), bit_of(L, kb), bit_of(L, kc), bit_of(L, kd), t.v * nfac * cg1 * cg2);
          }
      }
  }
  return list.ops;
}
}  // namespace

// ------------------------------------------------------------ set-up pieces
// (composed by build_tables in enum.cu, which enumerates the basis and builds
// the jump tables on the device)

std::vector<MState> mstates(const std::vector<Orbit>& orb) { return msps(orb); }

std::vector<long> conjugate_index(const std::vector<Op2>& ops) {
  std::unordered_map<Key4, size_t, Key4H> where;
  for (size_t k = 0; k < ops.size(); ++k) where.emplace(Key4{ops[k].a, ops[k].b, ops[k].c, ops[k].d}, k);
  std::vector<long> conj(ops.size());
  for (size_t k = 0; k < ops.size(); ++k) {
    auto it = where.find(Key4{ops[k].c, ops[k].d, ops[k].a, ops[k].b});
    conj[k] = it == where.end() ? -1 : (long)it->second;
  }
  return conj;
}

void build_operators(const Interaction& I, Tables& T) {
  // ---- pp / nn operators (prep_Hamil_T1, :580-649)
  T.vpp = two_body_ops(I.tb[0], I.porb, T.msp, 0);
  T.vnn = two_body_ops(I.tb[1], I.norb, T.msn, I.lp);
  // ---- pn operators (prep_Hamil_pn, :658-730)
  {
    std::vector<int> Mzs;
    for (int j = 0; j < T.Lp; ++j)
      for (int i = 0; i < T.Lp; ++i) Mzs.push_back(T.msp[i].m2 - T.msp[j].m2);
    std::sort(Mzs.begin(), Mzs.end());
    Mzs.erase(std::unique(Mzs.begin(), Mzs.end()), Mzs.end());
    std::reverse(Mzs.begin(), Mzs.end());
    T.delMs = Mzs;
    std::vector<OpList> lists(Mzs.size());
    OpIndex ix(T.Lp, T.Ln);  // a key's ΔM fixes its list
    // m-state lists of every orbit, and the list index of every ΔM value
    std::vector<std::vector<int>> mp_of(I.porb.size()), mn_of(I.norb.size());
    for (size_t o = 0; o < I.porb.size(); ++o) mp_of[o] = mstates_of(T.msp, (int)o);
    for (size_t o = 0; o < I.norb.size(); ++o) mn_of[o] = mstates_of(T.msn, (int)o);
    const int dm0 = Mzs.empty() ? 0 : Mzs.back();
    std::vector<int> dm_idx(Mzs.empty() ? 0 : (size_t)(Mzs.front() - dm0 + 1), (int)Mzs.size());
    for (size_t k = 0; k < Mzs.size(); ++k) dm_idx[Mzs[k] - dm0] = (int)k;
    std::vector<double> cgcd, cgab;
    for (const auto& t : I.tb[2]) {
      int oa = t.a - 1, oc = t.c - 1, ob = t.b - 1 - I.lp, od = t.d - 1 - I.lp;
      const std::vector<int>& ia = mp_of[oa];
      const std::vector<int>& ic = mp_of[oc];
      const std::vector<int>& ib = mn_of[ob];
      const std::vector<int>& id = mn_of[od];
      int J2 = 2 * t.J;
      // the line's Clebsch–Gordan coefficients, once per m-state pair
      cgcd.assign(ic.size() * id.size(), 0.0);
      for (size_t u = 0; u < ic.size(); ++u)
        for (size_t w = 0; w < id.size(); ++w) {
          const int mc = T.msp[ic[u]].m2, md = T.msn[id[w]].m2;
          if (std::abs(mc + md) <= J2) cgcd[u * id.size() + w] = clebsch_gordan(I.porb[oc].j2, mc, I.norb[od].j2, md, J2, mc + md);
        }
      cgab.assign(ia.size() * ib.size(), 0.0);
      for (size_t u = 0; u < ia.size(); ++u)
        for (size_t w = 0; w < ib.size(); ++w) {
          const int ma = T.msp[ia[u]].m2, mb = T.msn[ib[w]].m2;
          cgab[u * ib.size() + w] = clebsch_gordan(I.porb[oa].j2, ma, I.norb[ob].j2, mb, J2, ma + mb);
        }
      for (size_t uc = 0; uc < ic.size(); ++uc) {
        const int kc = ic[uc];
        int mc = T.msp[kc].m2;
        for (size_t ua = 0; ua < ia.size(); ++ua) {
          const int ka = ia[ua];
          int ma = T.msp[ka].m2;
          int Mp = ma - mc;
          int idx = dm_idx[Mp - dm0];
          for (size_t ud = 0; ud < id.size(); ++ud) {
            const int kd = id[ud];
            int md = T.msn[kd].m2;
            if (std::abs(mc + md) > J2) continue;
            double tfac = t.v * cgcd[uc * id.size() + ud];
            for (size_t ub = 0; ub < ib.size(); ++ub) {
              const int kb = ib[ub];
              int mb = T.msn[kb].m2;
              if (mb - md + Mp != 0) continue;
              double fac = tfac * cgab[ua * ib.size() + ub];
              lists[idx].add(ix, bit_of(T.Lp, ka), bit_of(T.Ln, kb), bit_of(T.Lp, kc), bit_of(T.Ln, kd), fac);
            }
          }
        }
      }
    }
    T.vpn.resize(Mzs.size());
    for (size_t k = 0; k < Mzs.size(); ++k) T.vpn[k] = lists[k].ops;
  }
  // ---- V tables: per ΔM, distinct proton operators (a,c) and neutron
  // operators (b,d) among the non-zero entries, in first-appearance order.
  const size_t ndm = T.delMs.size();
  T.vtab_off_dm.assign(ndm + 1, 0);
  T.nA_dm.assign(ndm, 0);
  T.nB_dm.assign(ndm, 0);
  T.Aops_dm.assign(ndm, {});
  T.Bops_dm.assign(ndm, {});
  for (size_t k = 0; k < ndm; ++k) {
    std::unordered_map<uint64_t, int> ai, bi;
    std::vector<std::pair<int, int>> cells;
    for (const Op2& o : T.vpn[k]) {
      if (o.v == 0.0) { cells.push_back({-1, -1}); continue; }
      // one-hot masks identify m-states uniquely
      const uint64_t ka = (uint64_t)(63 - __builtin_clzll(o.a)) * 64 + (uint64_t)(63 - __builtin_clzll(o.c));
      const uint64_t kb = (uint64_t)(63 - __builtin_clzll(o.b)) * 64 + (uint64_t)(63 - __builtin_clzll(o.d));
      auto pa = ai.find(ka);
      if (pa == ai.end()) {
        pa = ai.emplace(ka, T.nA_dm[k]++).first;
        T.Aops_dm[k].push_back(o.a);
        T.Aops_dm[k].push_back(o.c);
      }
      auto pb = bi.find(kb);
      if (pb == bi.end()) {
        pb = bi.emplace(kb, T.nB_dm[k]++).first;
        T.Bops_dm[k].push_back(o.b);
        T.Bops_dm[k].push_back(o.d);
      }
      cells.push_back({pa->second, pb->second});
    }
    T.vtab_off_dm[k + 1] = T.vtab_off_dm[k] + (int64_t)T.nA_dm[k] * T.nB_dm[k];
    if (T.nA_dm[k] >= (1 << 15) || T.nB_dm[k] >= (1 << 13))
      throw SetupError{SMGPU_ERR_LIMIT, "too many distinct one-body operators for one ΔM"};
    T.vtab.resize(T.vtab_off_dm[k + 1], 0.0);
    for (size_t e = 0; e < T.vpn[k].size(); ++e) {
      if (cells[e].first < 0) continue;
      T.vtab[T.vtab_off_dm[k] + (int64_t)cells[e].first * T.nB_dm[k] + cells[e].second] = T.vpn[k][e].v;
    }
  }
}

void build_links(Tables& T, const std::vector<int>& Mps) {
  // prep_pn's bfs/bis (:1139-1151).  The reference indexes its list of all
  // proton M values by block number; that is reproduced here.
  const int nb = T.nb;
  std::vector<std::vector<Tables::Link>> per_b(nb);
  for (int bi = 0; bi < nb; ++bi)
    for (int bf = bi; bf < nb; ++bf) {
      if (bf >= (int)Mps.size()) break;
      int dm = Mps[bf] - Mps[bi];
      auto it = std::find(T.delMs.begin(), T.delMs.end(), dm);
      if (it == T.delMs.end()) continue;
      int k = (int)(it - T.delMs.begin());
      if (T.nA_dm[k] == 0) continue;
      per_b[bi].push_back(Tables::Link{bi, bf, k, T.nA_dm[k], T.nB_dm[k], T.vtab_off_dm[k], 0});
      if (bf != bi) per_b[bf].push_back(Tables::Link{bf, bi, k, T.nA_dm[k], T.nB_dm[k], T.vtab_off_dm[k], 0});
    }
  T.links.clear();
  T.link_begin.assign(nb + 1, 0);
  for (int b = 0; b < nb; ++b) {
    std::sort(per_b[b].begin(), per_b[b].end(), [](const Tables::Link& x, const Tables::Link& y) { return x.s < y.s; });
    for (auto& L : per_b[b]) T.links.push_back(L);
    T.link_begin[b + 1] = (int)T.links.size();
  }
  if (T.links.size() >= (1u << 16)) throw SetupError{SMGPU_ERR_LIMIT, "too many block links"};
  int64_t nptr_total = 0;
  for (auto& L : T.links) {
    L.nptr_off = nptr_total;
    nptr_total += T.nn[L.b] + 1;
  }
}

void count_updates(Tables& T) {
  int64_t upd = 0;
  for (int b = 0; b < T.nb; ++b) {
    upd += (int64_t)T.np[b] * T.nn[b];  // diagonal
    upd += (int64_t)(T.pp_ptr[T.pstart[b + 1]] - T.pp_ptr[T.pstart[b]]) * T.nn[b];
    upd += (int64_t)(T.nn_ptr[T.nstart[b + 1]] - T.nn_ptr[T.nstart[b]]) * T.np[b];
  }
  std::vector<int64_t> link_pcount(T.links.size(), 0);
  for (int64_t k = 0; k < (int64_t)T.ppn_meta.size(); ++k) link_pcount[T.ppn_meta[k] >> 16]++;
  for (size_t li = 0; li < T.links.size(); ++li) {
    const auto& L = T.links[li];
    const int64_t nent = T.npn_ptr[L.nptr_off + T.nn[L.b]] - T.npn_ptr[L.nptr_off];
    // every proton entry of a row meets every neutron entry of the link once
    upd += link_pcount[li] * nent;
  }
  T.updates = upd;
}

}  // namespace smgpu
