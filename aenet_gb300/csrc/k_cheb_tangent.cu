// Tangent (Jacobian-vector product) of the Chebyshev descriptor: for
// per-atom directions u (one 3-vector per atom)
//   V_a = sum_i (dG_a/dr_i) u_i = sum_j (dG_a/dR_aj) (u_j - u_a),
// normalised like the descriptor (times 1/s, sfsetup.f90:985-1035, no
// shift).  Used by the force term of the training loss, where u = dL/dF.
// The derivatives are those of sfb_radial / sfb_angular
// (src/ext/sfbasis.f90:762-858) and chebyshev_polynomial_d1
// (src/ext/chebyshev.f90:110-126):
//   radial  dG_n/dR_j = (fc' T_n + fc T_n' 2/Rc) Rhat_j
//   angular dG_n/dR_j = fc_j' fc_k T_n Rhat_j
//                       + w T_n'(x) dx/dcos (Rhat_k - cos Rhat_j)/d_j
// Same group structure as the forward kernel: LPA lanes per atom, radial
// terms over neighbours, angular pairs over the staged neighbours (or, in
// FP32 with the forward's moments, the angular terms in moment form).
#include "k_cheb_impl.cuh"

namespace cheb {

template <typename T, int R, int A, int LPA>
__global__ void __launch_bounds__(128) k_tangent(PotDevice pd, DescBuffers b) {
  using T4 = typename Vec4<T>::type;
  constexpr int GPW = 32 / LPA;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  __shared__ float s_spin[AE_MAXT * AE_MAXT];   // typespin by (central, neighbour) species
  for (int q = threadIdx.x; q < pd.ntypes * AE_MAXT; q += blockDim.x)
    s_spin[q] = pd.sp[q / AE_MAXT].cheb.spin[q % AE_MAXT];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int grp = lane / LPA, sl = lane % LPA;
  const int wglobal = blockIdx.x * (blockDim.x >> 5) + warp;
  if (wglobal * GPW >= b.natoms) return;
  const int gid = wglobal * GPW + grp;
  const bool active = gid < b.natoms;
  const int i = active ? gid : b.natoms - 1;
  // per group: staged angular neighbours (unit vector + d, fc/fc'/spin,
  // direction difference + projection)
  const size_t per = (3 * sizeof(T4) * b.cap_a + 31) & ~size_t(31);
  T4* au = reinterpret_cast<T4*>(smem_raw + per * (warp * GPW + grp));
  T4* af = au + b.cap_a;
  T4* ad = af + b.cap_a;
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const int n = active ? b.nb_cnt[i] : 0;
  const int nloop = warp_max(n);
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  const T4* __restrict__ U = reinterpret_cast<const T4*>(b.U);
  const T4 ui = U[i];
  const T r_Rc = T(ct.r_Rc), a_Rc = T(ct.a_Rc);
  const T two_over_rc = T(2) / r_Rc;
  const int rN = ct.r_N, aN = ct.a_N;
  const bool multi = ct.multi;
  const unsigned gmask = (LPA == 32) ? 0xffffffffu : (((1u << LPA) - 1u) << (grp * LPA));

  T acc[R], accs[R];
#pragma unroll
  for (int q = 0; q < R; ++q) acc[q] = accs[q] = T(0);
  int na = 0;
  // the table row is read one iteration ahead (its load latency overlaps
  // the previous neighbour's work)
  T4 vn;
  int qn = 0;
  if (sl < n) {
    vn = vec[sl];
    qn = jt[sl];
  }
  for (int base = 0; base < nloop; base += LPA) {
    const int j = base + sl;
    const bool valid = j < n;
    T4 v = vn, dlt;
    const int q = qn;
    int t = 0;
    if (j + LPA < n) {
      vn = vec[j + LPA];
      qn = jt[j + LPA];
    }
    if (valid) {
      t = q >> AE_TYPE_SHIFT;
      const T4 uj = U[q & AE_INDEX_MASK];
      dlt.x = uj.x - ui.x;
      dlt.y = uj.y - ui.y;
      dlt.z = uj.z - ui.z;
    } else {
      v.x = v.y = v.z = T(0);
      v.w = T(1e30);
      dlt.x = dlt.y = dlt.z = T(0);
    }
    const T d = v.w;
    const T s = multi ? T(s_spin[ti * AE_MAXT + t]) : T(0);
    const T inv = (d > T(SFB_EPS) && d < T(1e29)) ? div_t(T(1), d) : T(0);
    const T p = (v.x * dlt.x + v.y * dlt.y + v.z * dlt.z) * inv;   // Rhat . delta
    dlt.w = p;
    if (d <= r_Rc && d > T(SFB_EPS)) {
      T fc, dfc;
      cutoff(d, r_Rc, fc, dfc);
      const T x = radial_x(d, r_Rc, two_over_rc);
      const T x2 = x + x;
      T tm1 = T(1), t0 = x, um1 = T(1), u0 = x2;
      acc[0] += dfc * p;
      accs[0] += s * dfc * p;
#pragma unroll
      for (int q = 1; q < R; ++q) {
        if (q < rN) {
          const T dT = T(q) * um1 * two_over_rc;
          const T c = fma(dfc, t0, fc * dT) * p;
          acc[q] += c;
          accs[q] = fma(s, c, accs[q]);
          const T tn = fma(x2, t0, -tm1);
          tm1 = t0;
          t0 = tn;
          const T un = fma(x2, u0, -um1);
          um1 = u0;
          u0 = un;
        }
      }
    }
    const bool inA = d <= a_Rc && d >= T(SFB_EPS);
    const unsigned m = __ballot_sync(0xffffffffu, inA) & gmask;
    if (inA) {
      const int k = na + __popc(m & ((1u << lane) - 1u));
      if (k < b.cap_a) {
        T fc, dfc;
        cutoff(d, a_Rc, fc, dfc);
        T4 u, f;
        u.x = v.x * inv;
        u.y = v.y * inv;
        u.z = v.z * inv;
        u.w = d;
        f.x = fc;
        f.y = dfc;
        f.z = s;
        f.w = T(0);
        au[k] = u;
        af[k] = f;
        ad[k] = dlt;
      }
    }
    na += __popc(m);
  }
  if (na > b.cap_a) {
    if (sl == 0 && active) atomicOr(b.status, AE_ST_NB_OVERFLOW);
    na = b.cap_a;
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    acc[q] = gsum<T, LPA>(acc[q]);
    if (multi) accs[q] = gsum<T, LPA>(accs[q]);
  }
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  T* V = reinterpret_cast<T*>(b.V) + (size_t)i * pd.nsf_pad;
  if (active) {
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if (q % LPA == sl && q < rN) {
        V[ct.r_i1 + q] = acc[q] * T(sizeof(T) == 8 ? pd.scale[nrow + ct.r_i1 + q]
                                                    : pd.scale32[nrow + ct.r_i1 + q]);
        if (multi)
          V[ct.r_i2 + q] = accs[q] * T(sizeof(T) == 8 ? pd.scale[nrow + ct.r_i2 + q]
                                                      : pd.scale32[nrow + ct.r_i2 + q]);
      }
    }
  }

  // angular pairs j < k
  T ang[A], angs[A];
#pragma unroll
  for (int q = 0; q < A; ++q) ang[q] = angs[q] = T(0);
  const int P = na * (na - 1) / 2;
  const int Ploop = warp_max(P);
  PairWalk pw;
  pw.start(sl, na);
  for (int p = sl; p < Ploop; p += LPA) {
    if (p < P) {
      const T4 uj = au[pw.a], uk = au[pw.b];
      const T4 fj = af[pw.a], fk = af[pw.b];
      const T4 dj = ad[pw.a], dk = ad[pw.b];
      const T cosv = uj.x * uk.x + uj.y * uk.y + uj.z * uk.z;
      const T w = fj.x * fk.x;
      const T ss = fj.z * fk.z;
      T x, dxdc;
      angular_arg(cosv, ct.angular_legacy, x, dxdc);
      // d cos along the directions: (Rhat_k . delta_j - cos p_j)/d_j + (j <-> k)
      const T dcos = (uk.x * dj.x + uk.y * dj.y + uk.z * dj.z - cosv * dj.w) / uj.w +
                     (uj.x * dk.x + uj.y * dk.y + uj.z * dk.z - cosv * dk.w) / uk.w;
      const T alpha = fj.y * fk.x * dj.w + fj.x * fk.y * dk.w;
      const T beta = w * dxdc * dcos;
      const T x2 = x + x;
      T tm1 = T(1), t0 = x, um1 = T(1), u0 = x2;
      ang[0] += alpha;
      angs[0] = fma(ss, alpha, angs[0]);
#pragma unroll
      for (int q = 1; q < A; ++q) {
        if (q < aN) {
          const T c = fma(alpha, t0, beta * T(q) * um1);
          ang[q] += c;
          angs[q] = fma(ss, c, angs[q]);
          const T tn = fma(x2, t0, -tm1);
          tm1 = t0;
          t0 = tn;
          const T un = fma(x2, u0, -um1);
          um1 = u0;
          u0 = un;
        }
      }
      pw.advance(na, LPA);
    }
  }
#pragma unroll
  for (int q = 0; q < A; ++q) {
    ang[q] = gsum<T, LPA>(ang[q]);
    if (multi) angs[q] = gsum<T, LPA>(angs[q]);
  }
  if (active) {
#pragma unroll
    for (int q = 0; q < A; ++q) {
      if (q % LPA == sl && q < aN) {
        V[ct.a_i1 + q] = ang[q] * T(sizeof(T) == 8 ? pd.scale[nrow + ct.a_i1 + q]
                                                    : pd.scale32[nrow + ct.a_i1 + q]);
        if (multi)
          V[ct.a_i2 + q] = angs[q] * T(sizeof(T) == 8 ? pd.scale[nrow + ct.a_i2 + q]
                                                      : pd.scale32[nrow + ct.a_i2 + q]);
      }
    }
  }
}

// Moment form of the angular tangent (FP32): with the forward's moments
// M_lm (both blocks) of the atom, dG_n = sum_l q_nl sum_m M_lm dM_lm
// - 1/2 T_n(x(1)) dW, where the neighbours' displacements delta_a give
//   dM_lm = sum_a sigma_a [w_a' p_a Y_lm(u_a) + w_a D_e Y_lm(u_a)],
//   e = (delta_a - p_a u_a)/d_a (tangential part), p_a = u_a . delta_a,
//   dW = sum_a sigma_a^2 2 w_a w_a' p_a   (sigma = 1 or the spin).
// D_e Y_lm from the recurrences: d/dz Q_l^m = kap Q_l^{m+1} and
// d (x + i y)^m = m (x + i y)^{m-1} (e_x + i e_y).  Each lane contracts its
// neighbours' terms with M at once, so only 2 (A + 1) sums cross lanes.
// resident blocks per SM asked of the register allocator (angular degree
// up to 4; the degree-6 instance would spill under the same cap and keeps
// three)
#ifndef AE_TAN_MOM_BLOCKS
#define AE_TAN_MOM_BLOCKS 5
#endif

template <int R, int A, int LPA>
__global__ void __launch_bounds__(128, A <= 5 ? AE_TAN_MOM_BLOCKS : 3) k_tangent_mom(PotDevice pd, DescBuffers b) {
  using T = float;
  using T4 = float4;
  constexpr int L = A - 1;
  constexpr int K = A * A;
  constexpr int GPW = 32 / LPA;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  __shared__ float s_spin[AE_MAXT * AE_MAXT];
  for (int q = threadIdx.x; q < pd.ntypes * AE_MAXT; q += blockDim.x)
    s_spin[q] = pd.sp[q / AE_MAXT].cheb.spin[q % AE_MAXT];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int grp = lane / LPA, sl = lane % LPA;
  const int wglobal = blockIdx.x * (blockDim.x >> 5) + warp;
  if (wglobal * GPW >= b.natoms) return;
  const int gid = wglobal * GPW + grp;
  const bool active = gid < b.natoms;
  const int i = active ? gid : b.natoms - 1;
  const size_t per = (3 * sizeof(T4) * b.cap_a + 31) & ~size_t(31);
  T4* au = reinterpret_cast<T4*>(smem_raw + per * (warp * GPW + grp));
  T4* af = au + b.cap_a;
  T4* ad = af + b.cap_a;
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const int n = active ? b.nb_cnt[i] : 0;
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  if (sl == 0) prefetch_rows(vec, jt, n);
  const int nloop = warp_max(n);
  const T4* __restrict__ U = reinterpret_cast<const T4*>(b.U);
  const T4 ui = U[i];
  const T r_Rc = T(ct.r_Rc), a_Rc = T(ct.a_Rc);
  const T two_over_rc = T(2) / r_Rc;
  const T r_a = T(SFB_PI) / r_Rc, a_a = T(SFB_PI) / a_Rc;
  const bool multi = ct.multi;
  const unsigned gmask = (LPA == 32) ? 0xffffffffu : (((1u << LPA) - 1u) << (grp * LPA));

  // ---- radial terms and angular staging (as k_tangent)
  T acc[R], accs[R];
#pragma unroll
  for (int q = 0; q < R; ++q) acc[q] = accs[q] = T(0);
  int na = 0;
  // the table row is read one iteration ahead (its load latency overlaps
  // the previous neighbour's work)
  T4 vn;
  int qn = 0;
  if (sl < n) {
    vn = vec[sl];
    qn = jt[sl];
  }
  for (int base = 0; base < nloop; base += LPA) {
    const int j = base + sl;
    const bool valid = j < n;
    T4 v = vn, dlt;
    const int q = qn;
    int t = 0;
    if (j + LPA < n) {
      vn = vec[j + LPA];
      qn = jt[j + LPA];
    }
    if (valid) {
      t = q >> AE_TYPE_SHIFT;
      const T4 uj = U[q & AE_INDEX_MASK];
      dlt.x = uj.x - ui.x;
      dlt.y = uj.y - ui.y;
      dlt.z = uj.z - ui.z;
    } else {
      v.x = v.y = v.z = T(0);
      v.w = T(1e30);
      dlt.x = dlt.y = dlt.z = T(0);
    }
    const T d = v.w;
    const T s = multi ? s_spin[ti * AE_MAXT + t] : T(0);
    const T inv = (d > T(SFB_EPS) && d < T(1e29)) ? div_t(T(1), d) : T(0);
    const T p = (v.x * dlt.x + v.y * dlt.y + v.z * dlt.z) * inv;   // Rhat . delta
    dlt.w = p;
    if (d <= r_Rc && d > T(SFB_EPS)) {
      T fc, dfc;
      cutoff_a(d, r_Rc, r_a, fc, dfc);
      const T x = radial_x(d, r_Rc, two_over_rc);
      const T x2 = x + x;
      T tm1 = T(1), t0 = x, um1 = T(1), u0 = x2;
      acc[0] += dfc * p;
      accs[0] += s * dfc * p;
#pragma unroll
      for (int q = 1; q < R; ++q) {
        const T dT = T(q) * um1 * two_over_rc;
        const T c = fmaf(dfc, t0, fc * dT) * p;
        acc[q] += c;
        accs[q] = fmaf(s, c, accs[q]);
        const T tn = fmaf(x2, t0, -tm1);
        tm1 = t0;
        t0 = tn;
        const T un = fmaf(x2, u0, -um1);
        um1 = u0;
        u0 = un;
      }
    }
    const bool inA = d <= a_Rc && d >= T(SFB_EPS);
    const unsigned m = __ballot_sync(0xffffffffu, inA) & gmask;
    if (inA) {
      const int k = na + __popc(m & ((1u << lane) - 1u));
      if (k < b.cap_a) {
        T fc, dfc;
        cutoff_a(d, a_Rc, a_a, fc, dfc);
        au[k] = make_float4(v.x * inv, v.y * inv, v.z * inv, inv);
        af[k] = make_float4(fc, dfc, s, T(0));
        ad[k] = dlt;
      }
    }
    na += __popc(m);
  }
  if (na > b.cap_a) {
    if (sl == 0 && active) atomicOr(b.status, AE_ST_NB_OVERFLOW);
    na = b.cap_a;
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    acc[q] = gsum<T, LPA>(acc[q]);
    if (multi) accs[q] = gsum<T, LPA>(accs[q]);
  }
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  T* V = reinterpret_cast<T*>(b.V) + (size_t)i * pd.nsf_pad;
  if (active) {
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if (q % LPA == sl) {
        V[ct.r_i1 + q] = acc[q] * pd.scale32[nrow + ct.r_i1 + q];
        if (multi) V[ct.r_i2 + q] = accs[q] * pd.scale32[nrow + ct.r_i2 + q];
      }
    }
  }

  // ---- angular terms from the moments
  float Mv[4 * ((2 * K + 3) / 4)];
  const float4* M4 = reinterpret_cast<const float4*>(b.M + (size_t)i * b.mom_pad);
#pragma unroll
  for (int c4 = 0; c4 < (2 * K + 3) / 4; ++c4) {
    const float4 t4 = M4[c4];
    Mv[4 * c4] = t4.x;
    Mv[4 * c4 + 1] = t4.y;
    Mv[4 * c4 + 2] = t4.z;
    Mv[4 * c4 + 3] = t4.w;
  }
  float h0[A], h1[A];   // sum_m M_lm dM_lm of both blocks, per l
#pragma unroll
  for (int l = 0; l < A; ++l) h0[l] = h1[l] = 0.f;
  float dW0 = 0.f, dW1 = 0.f;
  for (int a = sl; a < na; a += LPA) {
    if (!active) break;
    const float4 u = au[a], f = af[a], dl = ad[a];   // unit vector, 1/d; fc, fc', spin; delta, p
    const float pw = dl.w;
    const float ex = (dl.x - pw * u.x) * u.w, ey = (dl.y - pw * u.y) * u.w,
                ez = (dl.z - pw * u.z) * u.w;
    const float wp = f.y * pw, w = f.x, sp = f.z;
    dW0 = fmaf(2.f * w, wp, dW0);
    dW1 = fmaf(2.f * sp * sp * w, wp, dW1);
    // Q_l^m(z) for all l, m
    float Q[A][A];
#pragma unroll
    for (int m = 0; m <= L; ++m) {
      float q1 = 0.f, q2 = 0.f;
#pragma unroll
      for (int l = m; l <= L; ++l) {
        float q;
        if (l == m) q = c_mom.qmm[m];
        else if (l == m + 1) q = c_mom.a1[m] * u.z * q1;
        else q = fmaf(c_mom.a[l][m] * u.z, q1, -c_mom.b[l][m] * q2);
        q2 = q1;
        q1 = q;
        Q[l][m] = q;
      }
    }
    float cm = 1.f, sm = 0.f, dc = 0.f, ds = 0.f;   // (x+iy)^m and its derivative along e
#pragma unroll
    for (int m = 0; m <= L; ++m) {
      if (m > 0) {
        // d (x+iy)^m = m (x+iy)^{m-1} (e_x + i e_y), with (cm, sm) still at m-1
        const float ndc = float(m) * (cm * ex - sm * ey), nds = float(m) * (sm * ex + cm * ey);
        const float cn = fmaf(u.x, cm, -u.y * sm);
        sm = fmaf(u.x, sm, u.y * cm);
        cm = cn;
        dc = ndc;
        ds = nds;
      }
#pragma unroll
      for (int l = m; l <= L; ++l) {
        const float dq = (l > m) ? c_mom.kap[l][m] * Q[l][m + 1] * ez : 0.f;   // D_e Q_l^m
        if (m == 0) {
          const int k = l * l;
          const float g = fmaf(wp, Q[l][0], w * dq);
          h0[l] = fmaf(Mv[k], g, h0[l]);
          h1[l] = fmaf(Mv[K + k], sp * g, h1[l]);
        } else {
          const int k = l * l + 2 * m - 1;
          const float yc = Q[l][m] * cm, ys = Q[l][m] * sm;
          const float gc = fmaf(wp, yc, w * fmaf(dq, cm, Q[l][m] * dc));
          const float gs = fmaf(wp, ys, w * fmaf(dq, sm, Q[l][m] * ds));
          h0[l] = fmaf(Mv[k], gc, fmaf(Mv[k + 1], gs, h0[l]));
          h1[l] = fmaf(Mv[K + k], sp * gc, fmaf(Mv[K + k + 1], sp * gs, h1[l]));
        }
      }
    }
  }
#pragma unroll
  for (int l = 0; l < A; ++l) {
    h0[l] = gsum<T, LPA>(h0[l]);
    h1[l] = gsum<T, LPA>(h1[l]);
  }
  dW0 = gsum<T, LPA>(dW0);
  dW1 = gsum<T, LPA>(dW1);
  if (active) {
    const float* q = pd.qleg + (size_t)ti * AE_MOMA * AE_MOMA;
#pragma unroll
    for (int nn = 0; nn < A; ++nn) {
      if (nn % LPA == sl) {
        float g0 = 0.f, g1 = 0.f, t1 = 0.f;
#pragma unroll
        for (int l = 0; l <= nn; ++l) {
          const float ql = q[nn * AE_MOMA + l];
          g0 = fmaf(ql, h0[l], g0);
          g1 = fmaf(ql, h1[l], g1);
          t1 += ql;
        }
        V[ct.a_i1 + nn] = (g0 - 0.5f * t1 * dW0) * pd.scale32[nrow + ct.a_i1 + nn];
        if (multi) V[ct.a_i2 + nn] = (g1 - 0.5f * t1 * dW1) * pd.scale32[nrow + ct.a_i2 + nn];
      }
    }
  }
}

template <int R, int A>
int launch_tangent_mom(const PotDevice& pd, const DescBuffers& b, cudaStream_t s) {
  constexpr int LPA = 8;
  const int warps = 4;
  const int groups = warps * (32 / LPA);
  const size_t per = (3 * sizeof(float4) * b.cap_a + 31) & ~size_t(31);
  const size_t smem = per * groups;
  if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
  const int blocks = (b.natoms + groups - 1) / groups;
  auto kern = k_tangent_mom<R, A, LPA>;
  if (smem + AE_STATIC_SMEM > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  return (int)cudaGetLastError();
}

template <typename T, int R, int A>
int launch_tangent(const PotDevice& pd, const DescBuffers& b, cudaStream_t s) {
  using T4 = typename Vec4<T>::type;
  constexpr int LPA = 16;
  const int warps = 4;
  const int groups = warps * (32 / LPA);
  const size_t per = (3 * sizeof(T4) * b.cap_a + 31) & ~size_t(31);
  const size_t smem = per * groups;
  if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
  const int blocks = (b.natoms + groups - 1) / groups;
  auto kern = k_tangent<T, R, A, LPA>;
  if (smem + AE_STATIC_SMEM > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  return (int)cudaGetLastError();
}

template <typename T>
int dispatch_tangent(const PotDevice& pd, const DescBuffers& b, cudaStream_t s) {
  int rN = 0, aN = 0;
  const bool same = uniform_sizes(pd, rN, aN);
  // moment form where the forward stored moments of an instantiated size
  if (sizeof(T) == 4 && b.M && pd.qleg && same && (size_t)b.mom_pad >= (size_t)(2 * aN * aN)) {
    if (rN == 11 && aN == 5) return launch_tangent_mom<11, 5>(pd, b, s);
    if (rN == 13 && aN == 7) return launch_tangent_mom<13, 7>(pd, b, s);
    if (rN == 17 && aN == 5) return launch_tangent_mom<17, 5>(pd, b, s);
  }
  if (rN <= 17 && aN <= 9) return launch_tangent<T, 17, 9>(pd, b, s);
  if (rN <= 32 && aN <= 32) return launch_tangent<T, 32, 32>(pd, b, s);
  return (int)cudaErrorInvalidValue;
}

}  // namespace cheb

int ae_launch_chebyshev_tangent(const PotDevice& pd, const DescBuffers& b, int fp64,
                                cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  if (!b.U || !b.V) return (int)cudaErrorInvalidValue;
  return fp64 ? cheb::dispatch_tangent<double>(pd, b, s) : cheb::dispatch_tangent<float>(pd, b, s);
}
