// FP64 combination of the per-point bilinear forms into the current tensor,
// density and tensor divergence.
//
// The reference (src/libgimic/jtensor.F90:148-237) forms, per point,
//   ct(m,b) = 1/2 [ (P_b^T phi).g_m - (D^T(dbop_b phi)).g_m + (D^T phi).d2(m,b) ]
//             + eps_mbc rho r_c / 2
// with dbop = r x R_A (bfeval.f90:168-189) and d2 from d2fdrdb (:191-246).
// Writing R_A = r - s (s = position relative to the function's atom) and
// C_d = D o (R_d,nu - R_d,mu) turns this, exactly, into
//   para = 1/2 [ Z_bm + sum_cd eps_bcd r_c Y_dm + sum_c eps_bmc (r_c rho - X_c) ]
//   dia  = -1/2 sum_c eps_bmc rho r_c
// so that with both parts on the large r_c rho terms cancel before any
// rounding.  The divergence sum_m d/dm ct(m,b) (no reference counterpart) is
//   1/2 [ ZL_b + sum_cd eps_bcd r_c YL_d - 2 sum_mc eps_bmc E_mc ]
// for a symmetric D and antisymmetric dD/dB.
#pragma once
#include "gg_kernels.h"

namespace gg {

__device__ __forceinline__ void combine_point(const double* d, const double r[3], Flags fl, double ct[9],
                                              double* divt) {
  const double rho = d[0];
  const double* X = d + 1;
  const double* E = d + 4;
  const double* Y = d + 13;
  const double* YL = d + 22;
  const double* Z = d + 25;
  const double* ZL = d + 34;
  const bool all = fl.giao && fl.dia && fl.para;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const int e1 = (b + 1) % 3, e2 = (b + 2) % 3;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      // sum_c eps_bmc v_c for a vector v: +v_e2 if m == e1, -v_e1 if m == e2
      const double sgn = m == e1 ? 1.0 : (m == e2 ? -1.0 : 0.0);
      const int c = m == e1 ? e2 : e1;
      double t;
      if (all) {
        t = 0.5 * (Z[3 * b + m] + (r[e1] * Y[3 * e2 + m] - r[e2] * Y[3 * e1 + m]) - sgn * X[c]);
      } else {
        double para = 0.0, dia = 0.0;
        if (fl.para) {
          para = Z[3 * b + m];
          if (fl.giao) para += (r[e1] * Y[3 * e2 + m] - r[e2] * Y[3 * e1 + m]) + sgn * (r[c] * rho - X[c]);
          para *= 0.5;
        }
        if (fl.dia) dia = -0.5 * sgn * rho * r[c];
        t = para + dia;
      }
      ct[m + 3 * b] = t;
    }
    if (divt) divt[b] = all ? 0.5 * (ZL[b] + (r[e1] * YL[e2] - r[e2] * YL[e1]) - 2.0 * (E[3 * e1 + e2] - E[3 * e2 + e1]))
                            : 0.0;
  }
}

}  // namespace gg
