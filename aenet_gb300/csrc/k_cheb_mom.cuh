// Angular Chebyshev terms in moment form (FP32 path).
//
// The reference sums the angular basis over the pairs of neighbours inside
// the angular cut-off (sfb_angular, src/ext/sfbasis.f90:797-858):
//     G_n = sum_{a<b} w_a w_b T_n(x(u_a . u_b)),   w = fc (x spin product
// for the spin block), u the unit vectors, x(c) = c or (2c - pi)/pi.
// x is linear in c, so T_n(x(c)) = sum_{l<=n} q_nl P_l(c) (a Legendre
// expansion computed on the host), and the addition theorem
//     P_l(u . v) = sum_m Y_lm(u) Y_lm(v)
// with real, unit-normalised harmonics (Y_lm = sqrt(N_lm) Q_l^m(z)
// {1 | Re | Im}(x + i y)^m, Q_l^m = d^m P_l / dz^m, N_l0 = 1,
// N_lm = 2 (l-m)!/(l+m)!) turns the pair sum into
//     G_n = 1/2 sum_l q_nl p_l - 1/2 T_n(x(1)) W,
//     p_l = sum_m M_lm^2,  M_lm = sum_a w_a Y_lm(u_a),  W = sum_a w_a^2
// (the full double sum minus its diagonal).  The cost per atom is linear
// in the number of angular neighbours instead of quadratic, with the same
// values up to rounding.
//
// Adjoint: with g_n = dE/dG_n, B_l = sum_n g_n q_nl and tau = sum_l B_l,
//     dE/dM_lm = B_l M_lm =: D_lm,   dE/dW = -tau/2,
// and per neighbour (C_lm = D_lm of the plain block + s_a D_lm of the spin
// block, F = sum C_lm Y_lm(u_a), P the polynomial extension of F):
//     dE/dR_a = [w_a' F - (tau + tau_s s_a^2) w_a w_a'] u_a
//               + (w_a / d_a) (grad P - (u_a . grad P) u_a).
// grad P comes in closed form: d/dz Q_l^m = Q_l^{m+1} and
// d/dx, d/dy (x + i y)^m = m (x + i y)^{m-1}, i m (x + i y)^{m-1}.
//
// Component order (l-major): k(l, 0) = l^2, k(l, m, cos) = l^2 + 2m - 1,
// k(l, m, sin) = l^2 + 2m.
#pragma once
#include "common.h"

namespace cheb {

struct MomConsts {
  float qmm[AE_MOMA];            // Y_mm / {Re|Im}(x+iy)^m
  float a1[AE_MOMA];             // Q_{m+1}^m = a1 z Q_m^m
  float a[AE_MOMA][AE_MOMA];     // Q_l^m = a z Q_{l-1}^m - b Q_{l-2}^m
  float b[AE_MOMA][AE_MOMA];
  float kap[AE_MOMA][AE_MOMA];   // dQ_l^m/dz = kap Q_l^{m+1} (normalised)
};

__host__ __device__ constexpr double mc_sqrt(double x) {
  if (x <= 0.0) return 0.0;
  double r = x > 1.0 ? x : 1.0;
  for (int k = 0; k < 200; ++k) r = 0.5 * (r + x / r);
  return r;
}
__host__ __device__ constexpr double mc_fact(int n) {
  double r = 1.0;
  for (int k = 2; k <= n; ++k) r *= k;
  return r;
}
__host__ __device__ constexpr double mc_dfact(int n) {
  double r = 1.0;
  for (int k = n; k > 1; k -= 2) r *= k;
  return r;
}
__host__ __device__ constexpr MomConsts mom_consts() {
  MomConsts c{};
  for (int m = 0; m < AE_MOMA; ++m) {
    c.qmm[m] = (float)(m == 0 ? 1.0 : mc_sqrt(2.0 / mc_fact(2 * m)) * mc_dfact(2 * m - 1));
    c.a1[m] = (float)mc_sqrt(2.0 * m + 1.0);
    for (int l = m; l < AE_MOMA; ++l) {
      if (l >= m + 2) {
        c.a[l][m] = (float)((2.0 * l - 1.0) / mc_sqrt((double)(l - m) * (l + m)));
        c.b[l][m] = (float)mc_sqrt((double)(l + m - 1) * (l - m - 1) / ((double)(l - m) * (l + m)));
      }
      c.kap[l][m] = (float)(m == 0 ? mc_sqrt(0.5 * l * (l + 1)) : mc_sqrt((double)(l - m) * (l + m + 1)));
    }
  }
  return c;
}

static __constant__ MomConsts c_mom = mom_consts();

// M0 += w0 Y(u), M1 += w1 Y(u) for all components up to degree L
template <int L, bool MULTI>
__device__ __forceinline__ void mom_accumulate(float x, float y, float z, float w0, float w1,
                                               float (&M0)[(L + 1) * (L + 1)],
                                               float (&M1)[(L + 1) * (L + 1)]) {
  float cm = 1.f, sm = 0.f;
#pragma unroll
  for (int m = 0; m <= L; ++m) {
    if (m > 0) {
      const float cn = fmaf(x, cm, -y * sm);
      sm = fmaf(x, sm, y * cm);
      cm = cn;
    }
    const float c0 = w0 * cm, s0 = w0 * sm, c1 = w1 * cm, s1 = w1 * sm;
    float q1 = 0.f, q2 = 0.f;
#pragma unroll
    for (int l = m; l <= L; ++l) {
      float q;
      if (l == m) q = c_mom.qmm[m];
      else if (l == m + 1) q = c_mom.a1[m] * z * q1;
      else q = fmaf(c_mom.a[l][m] * z, q1, -c_mom.b[l][m] * q2);
      q2 = q1;
      q1 = q;
      const int k = l * l + (m ? 2 * m - 1 : 0);
      if (m == 0) {
        M0[k] = fmaf(q, w0, M0[k]);
        if (MULTI) M1[k] = fmaf(q, w1, M1[k]);
      } else {
        M0[k] = fmaf(q, c0, M0[k]);
        M0[k + 1] = fmaf(q, s0, M0[k + 1]);
        if (MULTI) {
          M1[k] = fmaf(q, c1, M1[k]);
          M1[k + 1] = fmaf(q, s1, M1[k + 1]);
        }
      }
    }
  }
}

// F = sum_k C_k Y_k(u) with C = D0 + s D1, and the gradient (px, py, pz) of
// its polynomial extension at u
template <int L, bool MULTI>
__device__ __forceinline__ void mom_gradient(float x, float y, float z, float s,
                                             const float (&D0)[(L + 1) * (L + 1)],
                                             const float (&D1)[(L + 1) * (L + 1)], float& F,
                                             float& px, float& py, float& pz) {
  float cp[L + 1], sp[L + 1], Ep[L + 1];
  cp[0] = 1.f;
  sp[0] = 0.f;
#pragma unroll
  for (int m = 1; m <= L; ++m) {
    cp[m] = fmaf(x, cp[m - 1], -y * sp[m - 1]);
    sp[m] = fmaf(x, sp[m - 1], y * cp[m - 1]);
  }
  F = px = py = pz = 0.f;
#pragma unroll
  for (int m = 0; m <= L; ++m) {
    float gam = 0.f, del = 0.f, q1 = 0.f, q2 = 0.f;
#pragma unroll
    for (int l = m; l <= L; ++l) {
      float q;
      if (l == m) q = c_mom.qmm[m];
      else if (l == m + 1) q = c_mom.a1[m] * z * q1;
      else q = fmaf(c_mom.a[l][m] * z, q1, -c_mom.b[l][m] * q2);
      q2 = q1;
      q1 = q;
      if (m == 0) {
        const int k = l * l;
        const float C = MULTI ? fmaf(s, D1[k], D0[k]) : D0[k];
        F = fmaf(C, q, F);
        Ep[l] = c_mom.kap[l][0] * C;
      } else {
        const int k = l * l + 2 * m - 1;
        const float Cc = MULTI ? fmaf(s, D1[k], D0[k]) : D0[k];
        const float Cs = MULTI ? fmaf(s, D1[k + 1], D0[k + 1]) : D0[k + 1];
        gam = fmaf(q, Cc, gam);
        del = fmaf(q, Cs, del);
        pz = fmaf(Ep[l], q, pz);   // d/dz of the order m-1 term
        if (l > m) Ep[l] = c_mom.kap[l][m] * fmaf(Cc, cp[m], Cs * sp[m]);
      }
    }
    if (m > 0) {
      F = fmaf(gam, cp[m], fmaf(del, sp[m], F));
      px = fmaf(float(m), fmaf(gam, cp[m - 1], del * sp[m - 1]), px);
      py = fmaf(float(m), fmaf(del, cp[m - 1], -gam * sp[m - 1]), py);
    }
  }
}

}  // namespace cheb
