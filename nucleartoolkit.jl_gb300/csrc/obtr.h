// One-body electromagnetic operators (M1, E2) between two M-scheme bases of
// one nucleus: the jump lists of prep_obtr_diag / prep_obtr_nondiag
// (src/ShellModel/transit.jl:82-245, 286-445) gathered into pull tables for
// the GPU kernel in obtr.cu.
#pragma once
#include <cstdint>
#include <vector>

#include "setup.h"

namespace smgpu {

enum { OBTR_M1 = 0, OBTR_E2 = 1 };

// init_ho_by_mass (transit.jl:49-60): hw = 41 A^(-1/3) (hwprm 1) or
// 45 A^(-1/3) - 25 A^(-2/3) (hwprm 2); b = ħc / sqrt(hw · m_N).
void ho_parameter(int A, int hwprm, double& hw, double& bpar);
// radius_power (transit.jl:62-80): the HO radial integral <n1 l1| r^k |n2 l2>.
double radius_power(int k, int n1, int l1, int n2, int l2, double bpar);

// Pull form of a one-body operator O from the right basis R to the left basis
// L:  (O v)[bl; p, n] = Σ_e p_val[e] v[psrc[bl]; p_col[e], n]
//                     + Σ_e n_val[e] v[nsrc[bl]; p, n_col[e]],
// rows of the proton (neutron) CSR = the left basis' SDs in pstart (nstart)
// numbering, columns local to the source block.
struct ObtrTables {
  std::vector<int> psrc, nsrc;
  std::vector<int> p_ptr, p_col, n_ptr, n_col;
  std::vector<double> p_val, n_val;
};

// op: OBTR_M1 or OBTR_E2.  symmetric = true builds prep_obtr_diag's operator
// (orbit pairs f >= i, applied with its transpose, halves on i == f; L and R
// must be the same basis); false builds prep_obtr_nondiag's (all orbit pairs,
// ΔM = mtot2_l - mtot2_r).  A selects the oscillator length (hwprm 2 for
// 16 <= A <= 40).  gf = [g_l(p), g_l(n), g_s(p), g_s(n)], ec = [e_p, e_n].
void build_obtr(const Interaction& I, const Tables& L, const Tables& R, int mtot2_l, int mtot2_r, int A, int op,
                bool symmetric, const double gf[4], const double ec[2], ObtrTables& out);

}  // namespace smgpu
