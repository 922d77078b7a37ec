// Host construction of the M1 / E2 one-body operators (obtr.h).
#include "obtr.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "../../include/smgpu.h"
#include "sdbits.h"

namespace smgpu {

void ho_parameter(int A, int hwprm, double& hw, double& bpar) {
  const double mp = 938.27231, mn = 939.56563, hc = 197.32696;
  const double amass = 0.5 * (mp + mn);
  if (hwprm == 2) hw = 45.0 * std::pow((double)A, -1.0 / 3.0) - 25.0 * std::pow((double)A, -2.0 / 3.0);
  else hw = 41.0 * std::pow((double)A, -1.0 / 3.0);
  bpar = hc / std::sqrt(hw * amass);
}

namespace {
// Julia's binomial: 0 for k < 0, (-1)^k C(k-n-1, k) for n < 0.
long double binomial(int n, int k) {
  if (k < 0) return 0.0L;
  if (n < 0) {
    const long double b = binomial(k - n - 1, k);
    return (k & 1) ? -b : b;
  }
  if (k > n) return 0.0L;
  long double r = 1.0L;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}
long double dfact(int n) {
  long double r = 1.0L;
  for (int i = n; i > 1; i -= 2) r *= i;
  return r;
}
}  // namespace

double radius_power(int k, int n1, int l1, int n2, int l2, double bpar) {
  const int ll = l1 + l2 + k;
  const int ll1 = (l2 - l1 + k) / 2, ll2 = (l1 - l2 + k) / 2;  // Julia div truncates toward zero, as C does
  const int imin = std::max(std::max(0, n1 - ll1), n2 - ll2), imax = std::min(n1, n2);
  long double s = 0.0L;
  for (int i = imin; i <= imax; ++i)
    s += binomial(ll1, n1 - i) * binomial(ll2, n2 - i) * (dfact(ll + 2 * i + 1) / dfact(2 * i));
  s *= std::sqrt(dfact(2 * n1) / dfact(2 * n1 + 2 * l1 + 1));
  s *= std::sqrt(dfact(2 * n2) / dfact(2 * n2 + 2 * l2 + 1));
  double r = (double)s * (1.0 / std::sqrt(std::pow(2.0, k)));
  if ((n1 - n2) & 1) r = -r;
  return r * std::pow(bpar, k);
}

namespace {
struct Pull {
  int row, col;
  double v;
};

// ⟨f|a†c|i⟩ with calc_phase_1!'s sign (shellmodel_main.jl:861-867,887-897):
// the count starts at 1 and includes the annihilated state itself.
bool apply1_ref(uint64_t phi, uint64_t a, uint64_t c, uint64_t& f, bool& negative) {
  if ((phi & c) != c) return false;
  const uint64_t r = phi & ~c;
  if (r & a) return false;
  const int cnt = 1 + sd_popc(phi & ~(c - 1)) + sd_popc(r & ~(a - 1));
  f = r | a;
  negative = (cnt & 1) != 0;
  return true;
}

void to_csr(std::vector<Pull>& e, int nrows, std::vector<int>& ptr, std::vector<int>& col, std::vector<double>& val) {
  std::stable_sort(e.begin(), e.end(), [](const Pull& x, const Pull& y) {
    return x.row != y.row ? x.row < y.row : x.col < y.col;
  });
  ptr.assign(nrows + 1, 0);
  col.clear();
  val.clear();
  for (size_t k = 0; k < e.size();) {
    size_t m = k;
    double s = 0.0;
    while (m < e.size() && e[m].row == e[k].row && e[m].col == e[k].col) s += e[m++].v;
    col.push_back(e[k].col);
    val.push_back(s);
    ptr[e[k].row + 1]++;
    k = m;
  }
  for (int r = 0; r < nrows; ++r) ptr[r + 1] += ptr[r];
}
}  // namespace

void build_obtr(const Interaction& I, const Tables& L, const Tables& R, int mtot2_l, int mtot2_r, int A, int op,
                bool symmetric, const double gf[4], const double ec[2], ObtrTables& out) {
  if ((mtot2_l - mtot2_r) & 1) throw SetupError{SMGPU_ERR_ARG, "the two bases differ by a half-integer M"};
  if (symmetric && (mtot2_l != mtot2_r || L.pbits != R.pbits || L.nbits != R.nbits))
    throw SetupError{SMGPU_ERR_ARG, "the symmetric (expectation-value) form needs one basis"};
  const int omu = (mtot2_l - mtot2_r) / 2;
  double hw, bpar;
  ho_parameter(A, (16 <= A && A <= 40) ? 2 : 1, hw, bpar);
  const double c_mom_mu = std::sqrt(3.0 / (4.0 * M_PI)), c_mom_Q = std::sqrt(5.0 / (16.0 * M_PI));
  out.psrc.assign(L.nb, -1);
  out.nsrc.assign(L.nb, -1);

  for (int sp = 0; sp < 2; ++sp) {
    const std::vector<Orbit>& orb = sp == 0 ? I.porb : I.norb;
    const std::vector<MState>& ms = sp == 0 ? L.msp : L.msn;
    const int Lm = sp == 0 ? L.Lp : L.Ln;
    const double g_l = gf[sp], g_s = gf[2 + sp], e = ec[sp];
    // calc_bifs (transit.jl:501-531): the proton part joins blocks of equal
    // neutron M, the neutron part blocks of equal proton M.
    std::vector<int>& src = sp == 0 ? out.psrc : out.nsrc;
    for (int bl = 0; bl < L.nb; ++bl) {
      if (symmetric) {
        src[bl] = bl;
        continue;
      }
      for (int br = 0; br < R.nb; ++br)
        if (sp == 0 ? R.mn2[br] == L.mn2[bl] : R.mp2[br] == L.mp2[bl]) src[bl] = br;
    }
    // the kernel indexes the unchanged species by the output block's index
    for (int bl = 0; bl < L.nb; ++bl)
      if (src[bl] >= 0 && (sp == 0 ? R.nn[src[bl]] != L.nn[bl] : R.np[src[bl]] != L.np[bl]))
        throw SetupError{SMGPU_ERR_DEVICE, "blocks of equal M hold different SD lists"};
    const std::vector<uint64_t>& lbits = sp == 0 ? L.pbits : L.nbits;
    const std::vector<uint64_t>& rbits = sp == 0 ? R.pbits : R.nbits;
    const std::vector<int>& lst = sp == 0 ? L.pstart : L.nstart;
    const std::vector<int>& rst = sp == 0 ? R.pstart : R.nstart;
    std::vector<Pull> pulls;

    const int no = (int)orb.size();
    for (int i = 0; i < no; ++i) {
      const int ni = orb[i].n, li = orb[i].l, ji = orb[i].j2;
      for (int f = symmetric ? i : 0; f < no; ++f) {
        const int nf = orb[f].n, lf = orb[f].l, jf = orb[f].j2;
        if (op == OBTR_M1) {
          if (ni != nf || li != lf) continue;  // selection rule
          if (!symmetric && omu > 1) continue;
        } else if (!symmetric && omu > 2) {
          continue;
        }
        const double ex_r2 = op == OBTR_E2 ? radius_power(2, ni, li, nf, lf, bpar) : 0.0;
        const double l6j = wigner6j(2 * lf, 2 * li, 2, ji, jf, 1);
        const double s6j = wigner6j(1, 1, 2, ji, jf, 2 * lf);
        const double Q3j = wigner3j(ji, 4, jf, 1, 0, -1);
        const double pfac = std::sqrt((double)((ji + 1) * (jf + 1)));
        for (int kc = 0; kc < Lm; ++kc) {
          if (ms[kc].orbit != i) continue;
          const int mc = ms[kc].m2;
          for (int ka = 0; ka < Lm; ++ka) {
            if (ms[ka].orbit != f) continue;
            const int ma = ms[ka].m2;
            if ((ma - mc) / 2 != omu) continue;  // M conservation (ΔM = 0 for the symmetric form)
            double coeff;
            if (op == OBTR_M1) {
              const int e1 = (jf - ma) / 2 + lf + (ji + 3) / 2, e2 = (jf - ma) / 2 + lf + (jf + 3) / 2;
              const double fac1 = ((e1 & 1) ? -1.0 : 1.0) * l6j * std::sqrt((double)(lf * (lf + 1) * (2 * lf + 1)));
              const double fac2 = ((e2 & 1) ? -1.0 : 1.0) * s6j * std::sqrt(1.5);
              const double m3j = pfac * wigner3j(jf, 2, ji, -ma, 2 * omu, mc);
              coeff = m3j * (fac1 * g_l + fac2 * g_s) * c_mom_mu;
            } else {
              if ((li + lf) & 1) continue;  // signQ = 0
              const int eq = jf + (1 - ma) / 2;
              const double signQ = (eq & 1) ? -2.0 : 2.0;
              const double m3j = wigner3j(jf, 4, ji, -ma, 2 * omu, mc);
              coeff = signQ * m3j * Q3j * pfac * e * c_mom_Q * ex_r2;
            }
            const uint64_t bit_c = sd_bit(Lm, kc), bit_a = sd_bit(Lm, ka);
            for (int bl = 0; bl < L.nb; ++bl) {
              const int br = src[bl];
              if (br < 0) continue;
              const uint64_t* tl = lbits.data() + lst[bl];
              const int nl = lst[bl + 1] - lst[bl];
              for (int x = rst[br]; x < rst[br + 1]; ++x) {
                uint64_t fsd;
                bool neg;
                if (!apply1_ref(rbits[x], bit_a, bit_c, fsd, neg)) continue;
                const int y = sd_find_desc(tl, nl, fsd);
                if (y < 0) continue;
                const int xi = x - rst[br];
                double c = neg ? -coeff : coeff;
                if (symmetric) {
                  if (xi == y) c *= 0.5;
                  pulls.push_back(Pull{lst[bl] + y, xi, c});
                  pulls.push_back(Pull{lst[bl] + xi, y, c});
                } else {
                  pulls.push_back(Pull{lst[bl] + y, xi, c});
                }
              }
            }
          }
        }
      }
    }
    if (sp == 0) to_csr(pulls, L.pstart[L.nb], out.p_ptr, out.p_col, out.p_val);
    else to_csr(pulls, L.nstart[L.nb], out.n_ptr, out.n_col, out.n_val);
  }
}

}  // namespace smgpu
