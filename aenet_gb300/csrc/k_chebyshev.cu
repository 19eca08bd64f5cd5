// Chebyshev descriptor (replaces sfb_eval / sfb_radial / sfb_angular of
// src/ext/sfbasis.f90:440-571, 762-858 and chebyshev.f90:41-128) and its
// adjoint (the force chain rule of src/aenet.f90:471-477 without ever
// materialising the descriptor Jacobian).
//
// One warp per central atom.  Radial terms: lanes over neighbours, each
// lane runs the T_n recurrence for its neighbour and accumulates all
// orders in registers, followed by a warp reduction per order.  Angular
// terms: the neighbours inside the angular cut-off are compacted into
// shared memory (unit vector, distance, cut-off value and slope, spin) and
// the pairs j < k are spread over the lanes through a flattened triangular
// index.
//
// Feature layout per atom (sfbasis.f90:114-131):
//   [radial r_N][angular a_N][radial x spin r_N][angular x spin a_N]
// The spin block exists when the setup has more than one species;
// typespin values follow sfbasis.f90:142-147.
//
// The adjoint contracts dE/dG (already multiplied by E_scale and the
// normalisation scale) with the analytic derivatives:
//   radial:  dE/dd_ij = sum_n g_n (fc' T_n + fc T_n')      along R_ij/d_ij
//   angular: E_jk = w A(cos), w = fc_j fc_k, A = sum_n g_n T_n
//            grad_j E_jk = fc_j' fc_k A Rhat_j + w A' (Rhat_k - cos Rhat_j)/d_j
// Forces on neighbours are gathered per neighbour slot in shared memory and
// scattered once per slot; the central atom's force is the negative sum.
#include "common.h"

namespace {

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  using type = float4;
};
template <>
struct Vec4<double> {
  using type = double4_32a;
};

// PI as written in sfbasis.f90:72
constexpr double SFB_PI = 3.14159265358979;
constexpr double SFB_EPS = 1.0e-12;

__device__ __forceinline__ void sincos_t(float x, float* s, float* c) { __sincosf(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, double* s, double* c) { sincos(x, s, c); }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

// fc(d) = 0.5 (cos(pi d / Rc) + 1), fc' = -0.5 (pi/Rc) sin(pi d / Rc), zero
// beyond Rc (sfb_fc / sfb_fc_d1, sfbasis.f90:719-752)
template <typename T>
__device__ __forceinline__ void cutoff(T d, T Rc, T& fc, T& dfc) {
  if (d >= Rc) {
    fc = T(0);
    dfc = T(0);
    return;
  }
  const T a = T(SFB_PI) / Rc;
  T s, c;
  sincos_t(a * d, &s, &c);
  fc = T(0.5) * (c + T(1));
  dfc = T(-0.5) * a * s;
}

template <typename T>
struct WarpSmem {
  typename Vec4<T>::type* au;   // angular neighbours: unit vector, distance
  typename Vec4<T>::type* af;   // fc, fc', spin, slot (as bits)
  T* fbuf;                      // [cap][3] neighbour force accumulators
  T* g;                         // [nsf_pad] dE/dG
};

template <typename T>
__device__ __forceinline__ WarpSmem<T> warp_smem(unsigned char* base, int cap, int nsf_pad,
                                                 int warp, bool adjoint) {
  using T4 = typename Vec4<T>::type;
  size_t per = 2 * sizeof(T4) * cap + (adjoint ? (3 * sizeof(T) * cap + sizeof(T) * nsf_pad) : 0);
  per = (per + 15) & ~size_t(15);
  unsigned char* p = base + per * warp;
  WarpSmem<T> w;
  w.au = reinterpret_cast<T4*>(p);
  w.af = w.au + cap;
  w.fbuf = reinterpret_cast<T*>(w.af + cap);
  w.g = w.fbuf + 3 * cap;
  return w;
}

template <typename T>
__host__ __device__ inline size_t cheb_smem_per_warp(int cap, int nsf_pad, bool adjoint) {
  using T4 = typename Vec4<T>::type;
  size_t per = 2 * sizeof(T4) * cap + (adjoint ? (3 * sizeof(T) * cap + sizeof(T) * nsf_pad) : 0);
  return (per + 15) & ~size_t(15);
}

// Compact the neighbours inside the angular cut-off into shared memory.
// Returns their number.  `slot` records the neighbour-table slot.
template <typename T>
__device__ int stage_angular(const typename Vec4<T>::type* __restrict__ vec,
                             const int* __restrict__ jt, int n, T a_Rc, const ChebTable& ct,
                             WarpSmem<T>& sm, int lane) {
  using T4 = typename Vec4<T>::type;
  int na = 0;
  for (int base = 0; base < n; base += 32) {
    int j = base + lane;
    bool in = false;
    T4 v;
    int t = 0;
    if (j < n) {
      v = vec[j];
      t = jt[j] >> AE_TYPE_SHIFT;
      in = (v.w <= a_Rc) && (v.w >= T(SFB_EPS));
    }
    unsigned m = __ballot_sync(0xffffffffu, in);
    if (in) {
      int k = na + __popc(m & ((1u << lane) - 1u));
      T inv = T(1) / v.w;
      T fc, dfc;
      cutoff(v.w, a_Rc, fc, dfc);
      T4 u;
      u.x = v.x * inv;
      u.y = v.y * inv;
      u.z = v.z * inv;
      u.w = v.w;
      sm.au[k] = u;
      T4 f;
      f.x = fc;
      f.y = dfc;
      f.z = ct.multi ? T(ct.spin[t]) : T(0);
      f.w = T(j);
      sm.af[k] = f;
    }
    na += __popc(m);
  }
  __syncwarp();
  return na;
}

// (G - shift) * scale.  FP64 kernels: in FP64.  FP32 kernels: shift is
// held as hi + lo (FP64 precision); G - hi is exact whenever G and the
// shift are within a factor two of each other (Sterbenz), which is where
// cancellation would otherwise lose digits.
__device__ __forceinline__ double normalise(double g, const PotDevice& pd, size_t k) {
  return (g - pd.shift[k]) * pd.scale[k];
}
__device__ __forceinline__ float normalise(float g, const PotDevice& pd, size_t k) {
  const float2 sh = pd.shift2[k];
  return ((g - sh.x) - sh.y) * pd.scale32[k];
}

__device__ __forceinline__ int gcd_int(int a, int b) {
  while (b) {
    int t = a % b;
    a = b;
    b = t;
  }
  return a;
}

// Walk of the flattened upper triangle a < b < na, 32 pairs apart.
struct PairWalk {
  int a, b;
  __device__ __forceinline__ void start(int p, int na) {
    a = 0;
    int rem = p;
    while (a < na - 1 && rem >= na - 1 - a) {
      rem -= na - 1 - a;
      ++a;
    }
    b = a + 1 + rem;
  }
  __device__ __forceinline__ bool valid(int na) const { return a < na - 1 && b < na; }
  // (a, b) of flattened index q (row-major upper triangle)
  __device__ __forceinline__ void from_index(int q, int na) {
    // a = largest row with start(a) <= q, start(a) = a (2 na - a - 1) / 2
    float fn = (float)(2 * na - 1);
    int aa = (int)((fn - sqrtf(fn * fn - 8.0f * (float)q)) * 0.5f);
    aa = max(0, min(aa, na - 2));
    while (aa > 0 && aa * (2 * na - aa - 1) / 2 > q) --aa;
    while (aa < na - 2 && (aa + 1) * (2 * na - aa - 2) / 2 <= q) ++aa;
    a = aa;
    b = q - aa * (2 * na - aa - 1) / 2 + aa + 1;
  }
  __device__ __forceinline__ void advance(int na) {
    b += 32;
    while (a < na - 1 && b >= na) {
      b = b - na + a + 2;
      ++a;
    }
  }
};

// Angular argument x(cos) and dx/dcos for the current ([-1,1]) and legacy
// ([0,pi]) domains of chebyshev_polynomial.
template <typename T>
__device__ __forceinline__ void angular_arg(T cosv, int legacy, T& x, T& dxdc) {
  if (legacy) {
    x = (T(2) * cosv - T(SFB_PI)) / T(SFB_PI);
    dxdc = T(2) / T(SFB_PI);
  } else {
    x = cosv;
    dxdc = T(1);
  }
}

// ----------------------------------------------------------------------
// forward: G (normalised) per atom
// ----------------------------------------------------------------------
template <typename T, int NR, int NA>
__global__ void __launch_bounds__(128) k_cheb_forward(PotDevice pd, DescBuffers b) {
  using T4 = typename Vec4<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= b.natoms) return;
  WarpSmem<T> sm = warp_smem<T>(smem_raw, b.cap, pd.nsf_pad, warp, false);
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const int n = b.nb_cnt[i];
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  const T r_Rc = T(ct.r_Rc), a_Rc = T(ct.a_Rc);
  const int rN = ct.r_N, aN = ct.a_N;

  // ---- radial
  T acc[NR], accs[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    acc[q] = T(0);
    accs[q] = T(0);
  }
  for (int j = lane; j < n; j += 32) {
    T4 v = vec[j];
    T d = v.w;
    if (d <= r_Rc && d > T(SFB_EPS)) {
      T fc, dfc;
      cutoff(d, r_Rc, fc, dfc);
      T s = ct.multi ? T(ct.spin[jt[j] >> AE_TYPE_SHIFT]) : T(0);
      T x = (T(2) * d - r_Rc) / r_Rc;
      T tm1 = T(1), t0 = x;
      acc[0] += fc;
      accs[0] += s * fc;
#pragma unroll
      for (int q = 1; q < NR; ++q) {
        if (q < rN) {
          acc[q] += fc * t0;
          accs[q] += s * fc * t0;
          T tn = T(2) * x * t0 - tm1;
          tm1 = t0;
          t0 = tn;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    acc[q] = warp_sum(acc[q]);
    if (ct.multi) accs[q] = warp_sum(accs[q]);
  }
  const size_t orow = (size_t)i * pd.nsf_pad;
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  T* G = reinterpret_cast<T*>(b.G) + orow;
  // normalisation (sfsetup.f90:985-1035): lane q writes order q
  {
    T v = T(0), vs = T(0);
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (lane == q) {
        v = acc[q];
        vs = accs[q];
      }
    if (lane < rN) {
      G[ct.r_i1 + lane] = normalise(v, pd, nrow + ct.r_i1 + lane);
      if (ct.multi) G[ct.r_i2 + lane] = normalise(vs, pd, nrow + ct.r_i2 + lane);
    }
  }

  // ---- angular
  const int na = stage_angular<T>(vec, jt, n, a_Rc, ct, sm, lane);
  T ang[NA], angs[NA];
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    ang[q] = T(0);
    angs[q] = T(0);
  }
  PairWalk pw;
  pw.start(lane, na);
  while (pw.valid(na)) {
    T4 uj = sm.au[pw.a], uk = sm.au[pw.b];
    T4 fj = sm.af[pw.a], fk = sm.af[pw.b];
    T cosv = uj.x * uk.x + uj.y * uk.y + uj.z * uk.z;
    T w = fj.x * fk.x;
    T ss = fj.z * fk.z;
    T x, dxdc;
    angular_arg(cosv, ct.angular_legacy, x, dxdc);
    T tm1 = T(1), t0 = x;
    ang[0] += w;
    angs[0] += ss * w;
#pragma unroll
    for (int q = 1; q < NA; ++q) {
      if (q < aN) {
        ang[q] += w * t0;
        angs[q] += ss * w * t0;
        T tn = T(2) * x * t0 - tm1;
        tm1 = t0;
        t0 = tn;
      }
    }
    pw.advance(na);
  }
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    ang[q] = warp_sum(ang[q]);
    if (ct.multi) angs[q] = warp_sum(angs[q]);
  }
  {
    T v = T(0), vs = T(0);
#pragma unroll
    for (int q = 0; q < NA; ++q)
      if (lane == q) {
        v = ang[q];
        vs = angs[q];
      }
    if (lane < aN) {
      G[ct.a_i1 + lane] = normalise(v, pd, nrow + ct.a_i1 + lane);
      if (ct.multi) G[ct.a_i2 + lane] = normalise(vs, pd, nrow + ct.a_i2 + lane);
    }
  }
}

// ----------------------------------------------------------------------
// adjoint: forces (and virial) from dE/dG
// ----------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void atomic_add3(T* F, int atom, T fx, T fy, T fz);

template <>
__device__ __forceinline__ void atomic_add3<float>(float* F, int atom, float fx, float fy,
                                                   float fz) {
  atomicAdd(reinterpret_cast<float4*>(F) + atom, make_float4(fx, fy, fz, 0.f));
}
template <>
__device__ __forceinline__ void atomic_add3<double>(double* F, int atom, double fx, double fy,
                                                    double fz) {
  atomicAdd(F + 4 * atom, fx);
  atomicAdd(F + 4 * atom + 1, fy);
  atomicAdd(F + 4 * atom + 2, fz);
}

template <typename T, int NR, int NA>
__global__ void __launch_bounds__(128) k_cheb_adjoint(PotDevice pd, DescBuffers b) {
  using T4 = typename Vec4<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= b.natoms) return;
  WarpSmem<T> sm = warp_smem<T>(smem_raw, b.cap, pd.nsf_pad, warp, true);
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const int n = b.nb_cnt[i];
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  const T r_Rc = T(ct.r_Rc), a_Rc = T(ct.a_Rc);
  const int rN = ct.r_N, aN = ct.a_N;
  const int sid = b.atom_struct[i];
  const T gs = b.grad_scale ? T(b.grad_scale[sid]) : T(1);

  const T* gsrc = reinterpret_cast<const T*>(b.dEdG) + (size_t)i * pd.nsf_pad;
  for (int k = lane; k < ct.nsf; k += 32) sm.g[k] = gs * gsrc[k];
  __syncwarp();

  // ---- radial: force per neighbour slot
  T fix = T(0), fiy = T(0), fiz = T(0);
  const T dxdd = T(2) / r_Rc;
  for (int j = lane; j < n; j += 32) {
    T4 v = vec[j];
    T d = v.w;
    T c = T(0);
    if (d <= r_Rc && d > T(SFB_EPS)) {
      T fc, dfc;
      cutoff(d, r_Rc, fc, dfc);
      T s = ct.multi ? T(ct.spin[jt[j] >> AE_TYPE_SHIFT]) : T(0);
      T x = (T(2) * d - r_Rc) / r_Rc;
      // T_n and T_n' = n U_{n-1} (chebyshev_polynomial_d1)
      T tm1 = T(1), t0 = x;     // T_{q-1}, T_q
      T um1 = T(1), u0 = T(2) * x;  // U_{q-1}, U_q
      const T* gr = sm.g + ct.r_i1;
      const T* grs = sm.g + ct.r_i2;
      T g0 = gr[0] + (ct.multi ? s * grs[0] : T(0));
      c = g0 * dfc;  // q = 0: T_0 = 1, T_0' = 0
#pragma unroll
      for (int q = 1; q < NR; ++q) {
        if (q < rN) {
          T gq = gr[q] + (ct.multi ? s * grs[q] : T(0));
          T dT = T(q) * um1 * dxdd;
          c += gq * (dfc * t0 + fc * dT);
          T tn = T(2) * x * t0 - tm1;
          tm1 = t0;
          t0 = tn;
          T un = T(2) * x * u0 - um1;
          um1 = u0;
          u0 = un;
        }
      }
    }
    // dE/dR_j = c * R_ij / d ; force on j is minus that
    T inv = (d > T(SFB_EPS)) ? c / d : T(0);
    T gx = inv * v.x, gy = inv * v.y, gz = inv * v.z;
    sm.fbuf[3 * j] = -gx;
    sm.fbuf[3 * j + 1] = -gy;
    sm.fbuf[3 * j + 2] = -gz;
    fix += gx;
    fiy += gy;
    fiz += gz;
  }
  __syncwarp();

  // ---- angular
  const int na = stage_angular<T>(vec, jt, n, a_Rc, ct, sm, lane);
  const T* ga = sm.g + ct.a_i1;
  const T* gas = sm.g + ct.a_i2;
  // Pairs are visited in the order p -> (p * m) mod P with m coprime to P,
  // which scatters the lanes of one step over different rows a, so the
  // shared-memory force accumulations rarely collide.
  const int P = na * (na - 1) / 2;
  int mstep = 1;
  if (P > 64) {
    mstep = (P / 32) | 1;
    while (gcd_int(mstep, P) != 1) mstep += 2;
  }
  for (int p = lane; p < P; p += 32) {
    const int q = (int)(((long long)p * mstep) % P);
    PairWalk pw;
    pw.from_index(q, na);
    T4 uj = sm.au[pw.a], uk = sm.au[pw.b];
    T4 fj = sm.af[pw.a], fk = sm.af[pw.b];
    T cosv = uj.x * uk.x + uj.y * uk.y + uj.z * uk.z;
    T w = fj.x * fk.x;
    T ss = fj.z * fk.z;
    T x, dxdc;
    angular_arg(cosv, ct.angular_legacy, x, dxdc);
    T tm1 = T(1), t0 = x, um1 = T(1), u0 = T(2) * x;
    T A = ga[0] + (ct.multi ? ss * gas[0] : T(0));
    T Bv = T(0);
#pragma unroll
    for (int q = 1; q < NA; ++q) {
      if (q < aN) {
        T gq = ga[q] + (ct.multi ? ss * gas[q] : T(0));
        A += gq * t0;
        Bv += gq * T(q) * um1;
        T tn = T(2) * x * t0 - tm1;
        tm1 = t0;
        t0 = tn;
        T un = T(2) * x * u0 - um1;
        um1 = u0;
        u0 = un;
      }
    }
    Bv *= dxdc;
    const T dEdc = w * Bv;
    const T dEdj = fj.y * fk.x * A;   // d/dd_j of w * A
    const T dEdk = fj.x * fk.y * A;
    const T ij = T(1) / uj.w, ik = T(1) / uk.w;
    // grad_j = dEdj Rhat_j + dEdc (Rhat_k - cos Rhat_j)/d_j
    T gjx = dEdj * uj.x + dEdc * (uk.x - cosv * uj.x) * ij;
    T gjy = dEdj * uj.y + dEdc * (uk.y - cosv * uj.y) * ij;
    T gjz = dEdj * uj.z + dEdc * (uk.z - cosv * uj.z) * ij;
    T gkx = dEdk * uk.x + dEdc * (uj.x - cosv * uk.x) * ik;
    T gky = dEdk * uk.y + dEdc * (uj.y - cosv * uk.y) * ik;
    T gkz = dEdk * uk.z + dEdc * (uj.z - cosv * uk.z) * ik;
    int sj = (int)fj.w, sk = (int)fk.w;
    atomicAdd(&sm.fbuf[3 * sj], -gjx);
    atomicAdd(&sm.fbuf[3 * sj + 1], -gjy);
    atomicAdd(&sm.fbuf[3 * sj + 2], -gjz);
    atomicAdd(&sm.fbuf[3 * sk], -gkx);
    atomicAdd(&sm.fbuf[3 * sk + 1], -gky);
    atomicAdd(&sm.fbuf[3 * sk + 2], -gkz);
    fix += gjx + gkx;
    fiy += gjy + gky;
    fiz += gjz + gkz;
  }
  __syncwarp();

  // ---- scatter neighbour forces, virial W_ab = sum_j R_ij,a f_j,b
  T* F = reinterpret_cast<T*>(b.F);
  T w00 = 0, w01 = 0, w02 = 0, w10 = 0, w11 = 0, w12 = 0, w20 = 0, w21 = 0, w22 = 0;
  for (int j = lane; j < n; j += 32) {
    T fx = sm.fbuf[3 * j], fy = sm.fbuf[3 * j + 1], fz = sm.fbuf[3 * j + 2];
    int atom = jt[j] & AE_INDEX_MASK;
    atomic_add3<T>(F, atom, fx, fy, fz);
    if (b.virial) {
      T4 v = vec[j];
      w00 += v.x * fx; w01 += v.x * fy; w02 += v.x * fz;
      w10 += v.y * fx; w11 += v.y * fy; w12 += v.y * fz;
      w20 += v.z * fx; w21 += v.z * fy; w22 += v.z * fz;
    }
  }
  fix = warp_sum(fix);
  fiy = warp_sum(fiy);
  fiz = warp_sum(fiz);
  if (lane == 0) atomic_add3<T>(F, i, fix, fiy, fiz);
  if (b.virial) {
    T wv[9] = {w00, w01, w02, w10, w11, w12, w20, w21, w22};
#pragma unroll
    for (int q = 0; q < 9; ++q) wv[q] = warp_sum(wv[q]);
    if (lane == 0) {
      double* V = b.virial + 9 * sid;
#pragma unroll
      for (int q = 0; q < 9; ++q) atomicAdd(V + q, (double)wv[q]);
    }
  }
}

template <typename T, int NR, int NA>
int launch_pair(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  const int warps = 4;
  size_t smem = cheb_smem_per_warp<T>(b.cap, pd.nsf_pad, adjoint) * warps;
  int blocks = (b.natoms + warps - 1) / warps;
  if (adjoint) {
    auto kern = k_cheb_adjoint<T, NR, NA>;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  } else {
    auto kern = k_cheb_forward<T, NR, NA>;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  }
  return (int)cudaGetLastError();
}

template <typename T>
int dispatch(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  int rN = 0, aN = 0;
  for (int t = 0; t < pd.ntypes; ++t) {
    rN = max(rN, pd.sp[t].cheb.r_N);
    aN = max(aN, pd.sp[t].cheb.a_N);
  }
  if (rN <= 12 && aN <= 8) return launch_pair<T, 12, 8>(pd, b, adjoint, s);
  if (rN <= 18 && aN <= 10) return launch_pair<T, 18, 10>(pd, b, adjoint, s);
  if (rN <= 24 && aN <= 16) return launch_pair<T, 24, 16>(pd, b, adjoint, s);
  if (rN <= 32 && aN <= 32) return launch_pair<T, 32, 32>(pd, b, adjoint, s);
  return (int)cudaErrorInvalidValue;
}

}  // namespace

int ae_launch_chebyshev_forward(const PotDevice& pd, const DescBuffers& b, int fp64,
                                cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  return fp64 ? dispatch<double>(pd, b, false, s) : dispatch<float>(pd, b, false, s);
}

int ae_launch_chebyshev_adjoint(const PotDevice& pd, const DescBuffers& b, int fp64,
                                cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  return fp64 ? dispatch<double>(pd, b, true, s) : dispatch<float>(pd, b, true, s);
}
