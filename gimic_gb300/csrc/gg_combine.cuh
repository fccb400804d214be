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

// The same with GIAO, diamagnetic and paramagnetic terms all on, in
// double-float arithmetic (about 44 bits; the r_c rho terms cancel
// algebraically above, so no catastrophic cancellation is left): the FP64
// pipe, 1/64 of the fp32 rate, is then needed only for the outputs.  d(i)
// returns bilinear form i (slots as in combine_point) and put(k, v) takes
// output k (ct(m, b) at m + 3 b, then div_b at 9 + b), so that neither the
// inputs nor the outputs are held all at once.
template <typename F, typename G>
__device__ __forceinline__ void combine_point_df(F d, const DFloat r[3], G put) {
  constexpr int X = 1, E = 4, Y = 13, YL = 22, Z = 25, ZL = 34;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const int e1 = (b + 1) % 3, e2 = (b + 2) % 3;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      DFloat t = df_add(d(Z + 3 * b + m), df_sub(df_mul(r[e1], d(Y + 3 * e2 + m)), df_mul(r[e2], d(Y + 3 * e1 + m))));
      if (m == e1) t = df_sub(t, d(X + e2));
      if (m == e2) t = df_add(t, d(X + e1));
      put(m + 3 * b, DFloat{0.5f * t.h, 0.5f * t.l});
    }
    DFloat v = df_add(d(ZL + b), df_sub(df_mul(r[e1], d(YL + e2)), df_mul(r[e2], d(YL + e1))));
    const DFloat w = df_sub(d(E + 3 * e1 + e2), d(E + 3 * e2 + e1));
    v = df_sub(v, DFloat{2.f * w.h, 2.f * w.l});
    put(9 + b, DFloat{0.5f * v.h, 0.5f * v.l});
  }
}

}  // namespace gg
