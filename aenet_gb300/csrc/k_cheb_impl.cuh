// Chebyshev descriptor (replaces sfb_eval / sfb_radial / sfb_angular of
// src/ext/sfbasis.f90:440-571, 762-858 and chebyshev.f90:41-128) and its
// adjoint (the force chain rule of src/aenet.f90:471-477, without ever
// materialising the descriptor Jacobian).
//
// One group of LPA lanes (8, 16 or 32) per central atom.  Radial terms:
// lanes over neighbours, each lane runs the T_n recurrence for its
// neighbour and accumulates all orders in registers; a group reduction
// follows.  In the same pass the neighbours inside the angular cut-off are
// compacted into shared memory (unit vector, distance, cut-off value and
// slope, spin, table slot).  Angular terms: the pairs j < k of those are
// spread over the group's lanes in row-major order of the upper triangle.
//
// Feature layout per atom (sfbasis.f90:114-131):
//   [radial R][angular A][radial x spin R][angular x spin A]
// The spin block exists when the setup has more than one species;
// typespin follows sfbasis.f90:142-147.  R and A are compile-time in the
// exact instantiations (no predicated padding); GUARD instantiations take
// them at run time up to their template bounds.
//
// The adjoint contracts dE/dG (already multiplied by E_scale and the
// normalisation scale) with the analytic derivatives:
//   radial:  dE/dd_ij = sum_n g_n (fc' T_n + fc T_n')       along R_ij/d_ij
//   angular: E_jk = w A(cos), w = fc_j fc_k, A = sum_n g_n T_n
//            grad_j E_jk = fc_j' fc_k A Rhat_j + w A' (Rhat_k - cos Rhat_j)/d_j
// In the adjoint every angular pair is evaluated once, on a circulant
// schedule (the owner of staged neighbour a takes partners a + t mod na,
// t = 1 .. na/2): the lanes of a group always touch distinct partners, so
// partner forces accumulate in shared memory without atomics and the
// owner's in registers; each neighbour's force is scattered to global
// memory once; the central atom receives minus the sum.
#pragma once
#include "common.h"
#include "k_cheb_mom.cuh"

namespace cheb {

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

template <typename T, int LPA>
__device__ __forceinline__ T gsum(T v) {
#pragma unroll
  for (int d = LPA / 2; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, d));
  return v;
}

// fc(d) = 0.5 (cos(pi d / Rc) + 1), fc' = -0.5 (pi/Rc) sin(pi d / Rc), zero
// beyond Rc (sfb_fc / sfb_fc_d1, sfbasis.f90:719-752); a = pi/Rc
template <typename T>
__device__ __forceinline__ void cutoff_a(T d, T Rc, T a, T& fc, T& dfc) {
  if (d >= Rc) {
    fc = T(0);
    dfc = T(0);
    return;
  }
  T s, c;
  sincos_t(a * d, &s, &c);
  fc = T(0.5) * (c + T(1));
  dfc = T(-0.5) * a * s;
}
template <typename T>
__device__ __forceinline__ void cutoff(T d, T Rc, T& fc, T& dfc) {
  cutoff_a(d, Rc, T(SFB_PI) / Rc, fc, dfc);
}

// x / y: IEEE division in FP64; in FP32 the hardware reciprocal (~2 ulp,
// far inside the mixed path's error budget)
__device__ __forceinline__ double div_t(double x, double y) { return x / y; }
__device__ __forceinline__ float div_t(float x, float y) { return __fdividef(x, y); }

// radial argument x = (2 d - Rc)/Rc of chebyshev_polynomial(d, 0, Rc)
__device__ __forceinline__ double radial_x(double d, double Rc, double) { return (2.0 * d - Rc) / Rc; }
__device__ __forceinline__ float radial_x(float d, float, float two_over_rc) {
  return fmaf(d, two_over_rc, -1.0f);
}

// angular argument and dx/dcos: current domain [-1, 1] or legacy [0, pi]
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

// (G - shift) * scale (sfsetup.f90:985-1035).  FP32 kernels hold the shift
// as hi + lo floats (FP64 precision); G - hi is exact whenever G and the
// shift are within a factor two of each other (Sterbenz).
__device__ __forceinline__ double normalise(double g, const PotDevice& pd, size_t k) {
  return (g - pd.shift[k]) * pd.scale[k];
}
__device__ __forceinline__ float normalise(float g, const PotDevice& pd, size_t k) {
  const float2 sh = pd.shift2[k];
  return ((g - sh.x) - sh.y) * pd.scale32[k];
}

template <typename T>
struct GroupSmem {
  typename Vec4<T>::type* au;   // angular neighbours: unit vector, distance
  typename Vec4<T>::type* af;   // fc, fc', spin, table slot
  T* fbuf;                      // [cap_a][3] forces on angular neighbours
  T* g;                         // [nsf_pad] dE/dG
};

// the staging area of the forward doubles as the moment reduction scratch
// (`scratch` bytes at least)
template <typename T>
__host__ __device__ inline size_t group_smem_bytes(int cap_a, int nsf_pad, bool adjoint,
                                                   size_t scratch = 0) {
  using T4 = typename Vec4<T>::type;
  size_t stage = 2 * sizeof(T4) * cap_a;
  if (stage < scratch) stage = scratch;
  size_t per = stage + (adjoint ? (3 * sizeof(T) * cap_a + sizeof(T) * nsf_pad) : 0);
  return (per + 31) & ~size_t(31);
}

template <typename T>
__device__ __forceinline__ GroupSmem<T> group_smem(unsigned char* base, int cap_a, int nsf_pad,
                                                   int group, bool adjoint, size_t scratch = 0) {
  using T4 = typename Vec4<T>::type;
  unsigned char* p = base + group_smem_bytes<T>(cap_a, nsf_pad, adjoint, scratch) * group;
  GroupSmem<T> w;
  w.au = reinterpret_cast<T4*>(p);
  w.af = w.au + cap_a;
  w.fbuf = reinterpret_cast<T*>(w.af + cap_a);
  w.g = w.fbuf + 3 * cap_a;
  return w;
}

// moment form: values per lane in the reduction (both blocks' moments, then
// the two weight sums), padded to whole float4
template <int A>
__host__ __device__ constexpr int mom_nv() {
  return 2 * A * A + 2;
}
template <int A>
__host__ __device__ constexpr int mom_nvp() {
  return (mom_nv<A>() + 3) & ~3;
}
template <int A, int LPA>
__host__ __device__ constexpr size_t mom_scratch_bytes() {
  return sizeof(float) * (size_t)(LPA + 1) * mom_nvp<A>();
}

// row-major walk of the upper triangle a < b < na with a fixed stride
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
  __device__ __forceinline__ void advance(int na, int stride) {
    b += stride;
    while (a < na - 1 && b >= na) {
      b = b - na + a + 2;
      ++a;
    }
  }
};

// Bulk prefetch of an atom's neighbour rows into L2 (one instruction per
// row, issued by the group's first lane): the radial rounds then wait on L2
// instead of DRAM.  Rows start 16-byte aligned (the ELL capacity is a
// multiple of 32) and the sizes are rounded up to 16 bytes inside the row.
template <typename T4>
__device__ __forceinline__ void prefetch_rows(const T4* vec, const int* jt, int n) {
  if (n <= 0) return;
  const unsigned bv = (unsigned)(sizeof(T4) * n);
  const unsigned bj = (unsigned)((4 * n + 15) & ~15);
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(__cvta_generic_to_global(vec)),
               "r"(bv)
               : "memory");
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(__cvta_generic_to_global(jt)),
               "r"(bj)
               : "memory");
}

template <typename T>
__device__ __forceinline__ void atomic_add3(T* F, int atom, T fx, T fy, T fz);
template <>
__device__ __forceinline__ void atomic_add3<float>(float* F, int atom, float fx, float fy, float fz) {
  atomicAdd(reinterpret_cast<float4*>(F) + atom, make_float4(fx, fy, fz, 0.f));
}
template <>
__device__ __forceinline__ void atomic_add3<double>(double* F, int atom, double fx, double fy,
                                                    double fz) {
  atomicAdd(F + 4 * atom, fx);
  atomicAdd(F + 4 * atom + 1, fy);
  atomicAdd(F + 4 * atom + 2, fz);
}

// Angular block of the forward in moment form (FP32): the group's lanes
// accumulate moments over the staged neighbours, the partial sums are
// reduced through the (then free) staging area, the moments are stored for
// the adjoint and each output lane assembles its G_n from the power spectra.
template <int A, int LPA>
__device__ __forceinline__ void forward_moments(const PotDevice& pd, const DescBuffers& b,
                                                const GroupSmem<float>& sm, const ChebTable& ct,
                                                int na, int sl, unsigned gmask, bool active, int i,
                                                int ti, bool multi, float* G, size_t nrow) {
  constexpr int L = A - 1;
  constexpr int K = A * A;
  constexpr int NV = mom_nv<A>(), NVP = mom_nvp<A>();
  float M0[K], M1[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    M0[k] = 0.f;
    M1[k] = 0.f;
  }
  float W0 = 0.f, W1 = 0.f;
  for (int a = sl; a < na; a += LPA) {
    const float4 u = sm.au[a], f = sm.af[a];
    const float w1 = f.x * f.z;   // fc x spin (zero for a single species)
    mom_accumulate<L, true>(u.x, u.y, u.z, f.x, w1, M0, M1);
    W0 = fmaf(f.x, f.x, W0);
    W1 = fmaf(w1, w1, W1);
  }
  __syncwarp(gmask);   // the staged neighbours are consumed: reuse the area
  float* scr = reinterpret_cast<float*>(sm.au);
  float4* dst = reinterpret_cast<float4*>(scr + sl * NVP);
#pragma unroll
  for (int c4 = 0; c4 < NVP / 4; ++c4) {
    float v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int c = 4 * c4 + e;
      v[e] = c < K ? M0[c] : (c < 2 * K ? M1[c - K] : (c == 2 * K ? W0 : (c == 2 * K + 1 ? W1 : 0.f)));
    }
    dst[c4] = make_float4(v[0], v[1], v[2], v[3]);
  }
  __syncwarp(gmask);
  float* sq = scr + LPA * NVP;
  float* Mg = b.M + (size_t)i * b.mom_pad;
  for (int c = sl; c < NV; c += LPA) {
    float t = 0.f;
#pragma unroll
    for (int r = 0; r < LPA; ++r) t += scr[r * NVP + c];
    if (c < 2 * K) {
      if (active) Mg[c] = t;
      sq[c] = t * t;
    } else {
      sq[c] = t;
    }
  }
  __syncwarp(gmask);
  if (!active || sl >= A) return;
  float p0[A], p1[A];
#pragma unroll
  for (int l = 0; l < A; ++l) {
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int k = l * l; k < (l + 1) * (l + 1); ++k) {
      s0 += sq[k];
      s1 += sq[K + k];
    }
    p0[l] = s0;
    p1[l] = s1;
  }
  W0 = sq[2 * K];
  W1 = sq[2 * K + 1];
  const float* q = pd.qleg + (size_t)ti * AE_MOMA * AE_MOMA;
#pragma unroll
  for (int n = 0; n < A; ++n) {
    if (n % LPA == sl) {
      float g0 = 0.f, g1 = 0.f, t1 = 0.f;
#pragma unroll
      for (int l = 0; l <= n; ++l) {
        const float ql = q[n * AE_MOMA + l];
        g0 = fmaf(ql, p0[l], g0);
        g1 = fmaf(ql, p1[l], g1);
        t1 += ql;
      }
      G[ct.a_i1 + n] = normalise(0.5f * (g0 - t1 * W0), pd, nrow + ct.a_i1 + n);
      if (multi) G[ct.a_i2 + n] = normalise(0.5f * (g1 - t1 * W1), pd, nrow + ct.a_i2 + n);
    }
  }
}

// Spin weight of the staged angular pair (a, k) with the reference's
// stale s_j (sfbasis.f90:514, 556): the member first in the reference's
// neighbour order contributes s_eff, the other its own spin.  f.z is the
// neighbour's own spin, f.w its slot in the atom's table row.
template <typename T>
__device__ __forceinline__ T ordered_spin(const DescBuffers& b, int i,
                                          const typename Vec4<T>::type& fa,
                                          const typename Vec4<T>::type& fk) {
  const size_t rb = (size_t)i * b.cap;
  const int sa = (int)fa.w, sk = (int)fk.w;
  return b.nb_rank[rb + sa] < b.nb_rank[rb + sk] ? T(b.nb_seff[rb + sa]) * fk.z
                                                 : T(b.nb_seff[rb + sk]) * fa.z;
}

// ----------------------------------------------------------------------
// forward
// ----------------------------------------------------------------------
// resident blocks per SM asked of the register allocator (moment form)
#ifndef AE_MOM_FWD_BLOCKS
#define AE_MOM_FWD_BLOCKS 6
#endif
#ifndef AE_MOM_ADJ_BLOCKS
#define AE_MOM_ADJ_BLOCKS 5
#endif
#ifndef AE_PAIR_ADJ_BLOCKS
#define AE_PAIR_ADJ_BLOCKS 5
#endif

template <typename T, int R, int A, int LPA, bool GUARD, bool MOM>
__global__ void __launch_bounds__(128, MOM ? (A <= 5 ? AE_MOM_FWD_BLOCKS : 3) : 1)
    k_forward(PotDevice pd, DescBuffers b) {
  using T4 = typename Vec4<T>::type;
  constexpr int GPW = 32 / LPA;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  // typespin of (central species, neighbour species): a shared table, as
  // the per-neighbour lookups in the parameter bank would serialise
  __shared__ float s_spin[AE_MAXT * AE_MAXT];
  for (int q = threadIdx.x; q < pd.ntypes * AE_MAXT; q += blockDim.x)
    s_spin[q] = pd.sp[q / AE_MAXT].cheb.spin[q % AE_MAXT];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int grp = lane / LPA, sl = lane % LPA;
  const int wglobal = blockIdx.x * (blockDim.x >> 5) + warp;
  if (wglobal * GPW >= b.natoms) return;   // whole warp idle
  const int gid = wglobal * GPW + grp;
  const bool active = gid < b.natoms;
  const int i = active ? gid : b.natoms - 1;
  GroupSmem<T> sm = group_smem<T>(smem_raw, b.cap_a, pd.nsf_pad, warp * GPW + grp, false,
                                  MOM ? mom_scratch_bytes<A, LPA>() : 0);
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const int n = active ? b.nb_cnt[i] : 0;
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  if (sl == 0) prefetch_rows(vec, jt, n);
  const int nloop = warp_max(n);
  const T r_Rc = T(ct.r_Rc), a_Rc = T(ct.a_Rc);
  const T two_over_rc = T(2) / r_Rc;
  const T r_a = T(SFB_PI) / r_Rc, a_a = T(SFB_PI) / a_Rc;
  const int rN = GUARD ? ct.r_N : R;
  const int aN = GUARD ? ct.a_N : A;
  const bool multi = ct.multi;
  const unsigned gmask = (LPA == 32) ? 0xffffffffu : (((1u << LPA) - 1u) << (grp * LPA));

  // ---- radial terms and angular staging
  T acc[R], accs[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    acc[q] = T(0);
    accs[q] = T(0);
  }
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
    T4 v = vn;
    const int t = valid ? (qn >> AE_TYPE_SHIFT) : 0;
    if (!valid) {
      v.x = v.y = v.z = T(0);
      v.w = T(1e30);
    }
    if (j + LPA < n) {
      vn = vec[j + LPA];
      qn = jt[j + LPA];
    }
    const T d = v.w;
    const T s = multi ? T(s_spin[ti * AE_MAXT + t]) : T(0);
    if (d <= r_Rc && d > T(SFB_EPS)) {
      T fc, dfc;
      cutoff_a(d, r_Rc, r_a, fc, dfc);
      const T x = radial_x(d, r_Rc, two_over_rc);
      const T x2 = x + x;
      const T sfc = s * fc;
      T tm1 = T(1), t0 = x;
      acc[0] += fc;
      accs[0] += sfc;
#pragma unroll
      for (int q = 1; q < R; ++q) {
        if (!GUARD || q < rN) {
          acc[q] = fma(fc, t0, acc[q]);
          accs[q] = fma(sfc, t0, accs[q]);
          const T tn = fma(x2, t0, -tm1);
          tm1 = t0;
          t0 = tn;
        }
      }
    }
    const bool inA = d <= a_Rc && d >= T(SFB_EPS);
    const unsigned m = __ballot_sync(0xffffffffu, inA) & gmask;
    if (inA) {
      const int k = na + __popc(m & ((1u << lane) - 1u));
      if (k < b.cap_a) {
        const T inv = div_t(T(1), d);
        T fc, dfc;
        cutoff_a(d, a_Rc, a_a, fc, dfc);
        T4 u, f;
        u.x = v.x * inv;
        u.y = v.y * inv;
        u.z = v.z * inv;
        u.w = d;
        f.x = fc;
        f.y = dfc;
        f.z = s;
        f.w = T(j);
        sm.au[k] = u;
        sm.af[k] = f;
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
  T* G = reinterpret_cast<T*>(b.G) + (size_t)i * pd.nsf_pad;
  if (active) {
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if (q % LPA == sl && q < rN) {
        G[ct.r_i1 + q] = normalise(acc[q], pd, nrow + ct.r_i1 + q);
        if (multi) G[ct.r_i2 + q] = normalise(accs[q], pd, nrow + ct.r_i2 + q);
      }
    }
  }

  // ---- angular terms
  if constexpr (MOM) {
    forward_moments<A, LPA>(pd, b, sm, ct, na, sl, gmask, active, i, ti, multi, G, nrow);
  } else {
    T ang[A], angs[A];
#pragma unroll
    for (int q = 0; q < A; ++q) {
      ang[q] = T(0);
      angs[q] = T(0);
    }
    // pairs (a, k = a + t mod na), t = 1 .. na/2, as in the adjoint: the
    // owner of a keeps it in registers and every pair is visited once
    const int tmax = na / 2;
    for (int a0 = 0; a0 < na; a0 += LPA) {
      const int a = a0 + sl;
      const bool own = active && a < na;
      T4 uj, fj;
      if (own) {
        uj = sm.au[a];
        fj = sm.af[a];
      } else {
        uj.x = uj.y = uj.z = uj.w = T(0);
        fj.x = fj.y = fj.z = fj.w = T(0);
      }
      for (int t = 1; t <= tmax; ++t) {
        int k = a + t;
        if (k >= na) k -= na;
        if (own && !(2 * t == na && a >= tmax)) {
          const T4 uk = sm.au[k];
          const T4 fk = sm.af[k];
          const T cosv = uj.x * uk.x + uj.y * uk.y + uj.z * uk.z;
          const T w = fj.x * fk.x;
          T sw = fj.z * fk.z * w;
          if constexpr (GUARD) {
            if (b.nb_rank) sw = w * ordered_spin<T>(b, i, fj, fk);
          }
          T x, dxdc;
          angular_arg(cosv, ct.angular_legacy, x, dxdc);
          const T x2 = x + x;
          T tm1 = T(1), t0 = x;
          ang[0] += w;
          angs[0] += sw;
#pragma unroll
          for (int q = 1; q < A; ++q) {
            if (!GUARD || q < aN) {
              ang[q] = fma(w, t0, ang[q]);
              angs[q] = fma(sw, t0, angs[q]);
              const T tn = fma(x2, t0, -tm1);
              tm1 = t0;
              t0 = tn;
            }
          }
        }
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
          G[ct.a_i1 + q] = normalise(ang[q], pd, nrow + ct.a_i1 + q);
          if (multi) G[ct.a_i2 + q] = normalise(angs[q], pd, nrow + ct.a_i2 + q);
        }
      }
    }
  }
}

// ----------------------------------------------------------------------
// adjoint
// ----------------------------------------------------------------------
// FP32 pair form of the exact-size instances: five blocks as well; the
// moment form of degree 6 keeps three (its sums would spill under more)
template <typename T, int R, int A, int LPA, bool GUARD, bool MOM>
__global__ void __launch_bounds__(128, MOM ? (A <= 5 ? AE_MOM_ADJ_BLOCKS : 3)
                                           : (sizeof(T) == 4 && !GUARD ? AE_PAIR_ADJ_BLOCKS : 1))
    k_adjoint(PotDevice pd,
                                                                             DescBuffers b) {
  using T4 = typename Vec4<T>::type;
  constexpr int GPW = 32 / LPA;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  // typespin of (central species, neighbour species): a shared table, as
  // the per-neighbour lookups in the parameter bank would serialise
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
  GroupSmem<T> sm = group_smem<T>(smem_raw, b.cap_a, pd.nsf_pad, warp * GPW + grp, true);
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const int n = active ? b.nb_cnt[i] : 0;
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  if (sl == 0) prefetch_rows(vec, jt, n);
  const int nloop = warp_max(n);
  const T r_Rc = T(ct.r_Rc), a_Rc = T(ct.a_Rc);
  const T two_over_rc = T(2) / r_Rc;
  const T r_a = T(SFB_PI) / r_Rc, a_a = T(SFB_PI) / a_Rc;
  const int rN = GUARD ? ct.r_N : R;
  const int aN = GUARD ? ct.a_N : A;
  const bool multi = ct.multi;
  const unsigned gmask = (LPA == 32) ? 0xffffffffu : (((1u << LPA) - 1u) << (grp * LPA));
  const int sid = b.atom_struct[i];
  const T gs = b.grad_scale ? T(b.grad_scale[sid]) : T(1);
  const bool want_virial = b.virial != nullptr;
  T* F = reinterpret_cast<T*>(b.F);

  const T* gsrc = reinterpret_cast<const T*>(b.dEdG) + (size_t)i * pd.nsf_pad;
  for (int k = sl; k < ct.nsf; k += LPA) sm.g[k] = gs * gsrc[k];
  __syncwarp();
  // radial coefficients in registers
  T gr[R], grs[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    gr[q] = (!GUARD || q < rN) ? sm.g[ct.r_i1 + q] : T(0);
    grs[q] = (multi && (!GUARD || q < rN)) ? sm.g[ct.r_i2 + q] : T(0);
  }

  T fix = T(0), fiy = T(0), fiz = T(0);
  T w00 = 0, w01 = 0, w02 = 0, w10 = 0, w11 = 0, w12 = 0, w20 = 0, w21 = 0, w22 = 0;
  int na = 0;
  // the table row is read one iteration ahead, as in the forward
  T4 vn;
  int qn = 0;
  if (sl < n) {
    vn = vec[sl];
    qn = jt[sl];
  }
  for (int base = 0; base < nloop; base += LPA) {
    const int j = base + sl;
    const bool valid = j < n;
    T4 v = vn;
    int t = 0, jatom = 0;
    if (valid) {
      t = qn >> AE_TYPE_SHIFT;
      jatom = qn & AE_INDEX_MASK;
    } else {
      v.x = v.y = v.z = T(0);
      v.w = T(1e30);
    }
    if (j + LPA < n) {
      vn = vec[j + LPA];
      qn = jt[j + LPA];
    }
    const T d = v.w;
    const T s = multi ? T(s_spin[ti * AE_MAXT + t]) : T(0);
    T c = T(0);
    if (d <= r_Rc && d > T(SFB_EPS)) {
      T fc, dfc;
      cutoff_a(d, r_Rc, r_a, fc, dfc);
      const T x = radial_x(d, r_Rc, two_over_rc);
      const T x2 = x + x;
      // T_q and T_q' = q U_{q-1} (chebyshev_polynomial_d1), times dx/dd
      T tm1 = T(1), t0 = x, um1 = T(1), u0 = x2;
      c = (gr[0] + s * grs[0]) * dfc;
#pragma unroll
      for (int q = 1; q < R; ++q) {
        if (!GUARD || q < rN) {
          const T gq = gr[q] + s * grs[q];
          const T dT = T(q) * um1 * two_over_rc;
          c = fma(gq, fma(dfc, t0, fc * dT), c);
          const T tn = fma(x2, t0, -tm1);
          tm1 = t0;
          t0 = tn;
          const T un = fma(x2, u0, -um1);
          um1 = u0;
          u0 = un;
        }
      }
    }
    // grad_j E = c R_ij / d; the force on j is minus that
    const T inv = (d > T(SFB_EPS) && d < T(1e29)) ? div_t(c, d) : T(0);
    const T gx = inv * v.x, gy = inv * v.y, gz = inv * v.z;
    const bool inA = d <= a_Rc && d >= T(SFB_EPS);
    const unsigned m = __ballot_sync(0xffffffffu, inA) & gmask;
    bool staged = false;
    if (inA) {
      const int k = na + __popc(m & ((1u << lane) - 1u));
      if (k < b.cap_a) {
        const T invd = div_t(T(1), d);
        T fc, dfc;
        cutoff_a(d, a_Rc, a_a, fc, dfc);
        T4 u, f;
        u.x = v.x * invd;
        u.y = v.y * invd;
        u.z = v.z * invd;
        u.w = invd;   // the angular loop needs 1/d only
        f.x = fc;
        f.y = dfc;
        f.z = s;
        f.w = T(j);
        sm.au[k] = u;
        sm.af[k] = f;
        sm.fbuf[3 * k] = -gx;
        sm.fbuf[3 * k + 1] = -gy;
        sm.fbuf[3 * k + 2] = -gz;
        staged = true;
      }
    }
    if (!staged) {
      // staged neighbours hand their force to the central atom at the end
      fix += gx;
      fiy += gy;
      fiz += gz;
    }
    if (valid && !staged && c != T(0)) {
      atomic_add3<T>(F, jatom, -gx, -gy, -gz);
      if (want_virial) {
        w00 -= v.x * gx; w01 -= v.x * gy; w02 -= v.x * gz;
        w10 -= v.y * gx; w11 -= v.y * gy; w12 -= v.y * gz;
        w20 -= v.z * gx; w21 -= v.z * gy; w22 -= v.z * gz;
      }
    }
    na += __popc(m);
  }
  if (na > b.cap_a) {
    if (sl == 0 && active) atomicOr(b.status, AE_ST_NB_OVERFLOW);
    na = b.cap_a;
  }
  __syncwarp();

  // ---- angular terms, one-sided on a circulant schedule: the lane that
  // owns staged neighbour a evaluates the pairs (a, k = a + t mod na) for
  // t = 1 .. na/2 (t = na/2 only from the lower half when na is even), so
  // every pair is evaluated once.  At each step the lanes of a group touch
  // distinct partners k, so the partner's force is added to shared memory
  // without atomics; a's own gradient stays in registers until the end of
  // its round.
  const T* ga = sm.g + ct.a_i1;
  const T* gas = sm.g + ct.a_i2;
  T gav[A], gasv[A];
#pragma unroll
  for (int q = 0; q < A; ++q) {
    gav[q] = (!GUARD || q < aN) ? ga[q] : T(0);
    gasv[q] = (multi && (!GUARD || q < aN)) ? gas[q] : T(0);
  }
  if constexpr (MOM) {
    // moment form: D = B_l M (plain and spin blocks), then one pass over
    // the staged neighbours, each adding its angular gradient to its
    // radial force and scattering the total once
    constexpr int L = A - 1;
    constexpr int K = A * A;
    const float* q = pd.qleg + (size_t)ti * AE_MOMA * AE_MOMA;
    float B0[A], B1[A];
#pragma unroll
    for (int l = 0; l < A; ++l) {
      B0[l] = 0.f;
      B1[l] = 0.f;
    }
#pragma unroll
    for (int nn = 0; nn < A; ++nn) {
#pragma unroll
      for (int l = 0; l <= nn; ++l) {
        const float ql = q[nn * AE_MOMA + l];
        B0[l] = fmaf(gav[nn], ql, B0[l]);
        B1[l] = fmaf(gasv[nn], ql, B1[l]);
      }
    }
    float tau0 = 0.f, tau1 = 0.f;
#pragma unroll
    for (int l = 0; l < A; ++l) {
      tau0 += B0[l];
      tau1 += B1[l];
    }
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
    float D0[K], D1[K];
#pragma unroll
    for (int l = 0; l < A; ++l) {
#pragma unroll
      for (int k = l * l; k < (l + 1) * (l + 1); ++k) {
        D0[k] = B0[l] * Mv[k];
        D1[k] = B1[l] * Mv[K + k];
      }
    }
    for (int a = sl; a < na; a += LPA) {
      if (!active) break;
      const float4 u = sm.au[a], f = sm.af[a];   // unit vector, 1/d; fc, fc', spin, slot
      float Fv, px, py, pz;
      mom_gradient<L, true>(u.x, u.y, u.z, f.z, D0, D1, Fv, px, py, pz);
      const float up = u.x * px + u.y * py + u.z * pz;
      const float wd = f.x * u.w;
      const float cu = f.y * (Fv - (tau0 + tau1 * f.z * f.z) * f.x) - wd * up;
      const int slot = (int)f.w;
      const float fx = sm.fbuf[3 * a] - fmaf(cu, u.x, wd * px);
      const float fy = sm.fbuf[3 * a + 1] - fmaf(cu, u.y, wd * py);
      const float fz = sm.fbuf[3 * a + 2] - fmaf(cu, u.z, wd * pz);
      atomic_add3<T>(F, jt[slot] & AE_INDEX_MASK, fx, fy, fz);
      fix -= fx;
      fiy -= fy;
      fiz -= fz;
      if (want_virial) {
        const T4 v = vec[slot];
        w00 += v.x * fx; w01 += v.x * fy; w02 += v.x * fz;
        w10 += v.y * fx; w11 += v.y * fy; w12 += v.y * fz;
        w20 += v.z * fx; w21 += v.z * fy; w22 += v.z * fz;
      }
    }
  } else {
    const int tmax = na / 2;
    for (int a0 = 0; a0 < na; a0 += LPA) {
      const int a = a0 + sl;
      const bool own = active && a < na;
      T4 ua, fa;
      if (own) {
        ua = sm.au[a];
        fa = sm.af[a];
      } else {
        ua.x = ua.y = ua.z = T(0);
        ua.w = T(1);
        fa.x = fa.y = fa.z = fa.w = T(0);
      }
      const T inva = ua.w;
      T gax = T(0), gay = T(0), gaz = T(0);
      for (int t = 1; t <= tmax; ++t) {
        int k = a + t;
        if (k >= na) k -= na;
        if (own && !(2 * t == na && a >= tmax)) {
          const T4 uk = sm.au[k];
          const T4 fk = sm.af[k];
          const T cosv = ua.x * uk.x + ua.y * uk.y + ua.z * uk.z;
          const T w = fa.x * fk.x;
          T ss = fa.z * fk.z;
          if constexpr (GUARD) {
            if (b.nb_rank) ss = ordered_spin<T>(b, i, fa, fk);
          }
          T x, dxdc;
          angular_arg(cosv, ct.angular_legacy, x, dxdc);
          const T x2 = x + x;
          T tm1 = T(1), t0 = x, um1 = T(1), u0 = x2;
          T Av = fma(ss, gasv[0], gav[0]), Bv = T(0);
#pragma unroll
          for (int q = 1; q < A; ++q) {
            if (!GUARD || q < aN) {
              const T cq = fma(ss, gasv[q], gav[q]);
              Av = fma(cq, t0, Av);
              Bv = fma(cq * T(q), um1, Bv);
              const T tn = fma(x2, t0, -tm1);
              tm1 = t0;
              t0 = tn;
              const T un = fma(x2, u0, -um1);
              um1 = u0;
              u0 = un;
            }
          }
          const T invk = uk.w;
          const T Bc = w * Bv * dxdc;
          const T dEda = fa.y * fk.x * Av, ca = Bc * inva;   // d/dd_a of w A, (dE/dcos)/d_a
          const T dEdk = fa.x * fk.y * Av, ck = Bc * invk;
          const T gx = dEda * ua.x + ca * (uk.x - cosv * ua.x);
          const T gy = dEda * ua.y + ca * (uk.y - cosv * ua.y);
          const T gz = dEda * ua.z + ca * (uk.z - cosv * ua.z);
          const T hx = dEdk * uk.x + ck * (ua.x - cosv * uk.x);
          const T hy = dEdk * uk.y + ck * (ua.y - cosv * uk.y);
          const T hz = dEdk * uk.z + ck * (ua.z - cosv * uk.z);
          gax += gx;
          gay += gy;
          gaz += gz;
          sm.fbuf[3 * k] -= hx;
          sm.fbuf[3 * k + 1] -= hy;
          sm.fbuf[3 * k + 2] -= hz;
        }
        __syncwarp(gmask);
      }
      if (own) {
        sm.fbuf[3 * a] -= gax;
        sm.fbuf[3 * a + 1] -= gay;
        sm.fbuf[3 * a + 2] -= gaz;
      }
      __syncwarp(gmask);
    }
    // forces on the staged neighbours (radial + angular), one scatter each
    for (int a = sl; a < na; a += LPA) {
      if (!active) break;
      const int slot = (int)sm.af[a].w;
      const T fx = sm.fbuf[3 * a], fy = sm.fbuf[3 * a + 1], fz = sm.fbuf[3 * a + 2];
      atomic_add3<T>(F, jt[slot] & AE_INDEX_MASK, fx, fy, fz);
      fix -= fx;   // the central atom takes minus the neighbour's force
      fiy -= fy;
      fiz -= fz;
      if (want_virial) {
        const T4 v = vec[slot];
        w00 += v.x * fx; w01 += v.x * fy; w02 += v.x * fz;
        w10 += v.y * fx; w11 += v.y * fy; w12 += v.y * fz;
        w20 += v.z * fx; w21 += v.z * fy; w22 += v.z * fz;
      }
    }
  }
  fix = gsum<T, LPA>(fix);
  fiy = gsum<T, LPA>(fiy);
  fiz = gsum<T, LPA>(fiz);
  if (active && sl == 0) atomic_add3<T>(F, i, fix, fiy, fiz);
  if (want_virial) {
    T wv[9] = {w00, w01, w02, w10, w11, w12, w20, w21, w22};
#pragma unroll
    for (int q = 0; q < 9; ++q) wv[q] = gsum<T, LPA>(wv[q]);
    if (active && sl == 0) {
      double* V = b.virial + 9 * sid;
#pragma unroll
      for (int q = 0; q < 9; ++q) atomicAdd(V + q, (double)wv[q]);
    }
  }
}

template <typename T, int R, int A, int LPA, bool GUARD, bool MOM>
int launch(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  // four warps per block, fewer when the atoms do not fill them (the
  // per-atom calls: one group, so long rows still fit shared memory)
  const int gpw = 32 / LPA;
  const int warps = b.natoms >= 4 * gpw ? 4 : (b.natoms + gpw - 1) / gpw;
  const int groups = warps * gpw;
  size_t scratch = 0;
  if constexpr (MOM) scratch = adjoint ? 0 : mom_scratch_bytes<A, LPA>();
  size_t smem = group_smem_bytes<T>(b.cap_a, pd.nsf_pad, adjoint, scratch) * groups;
  if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
  const int atoms_per_block = groups;
  const int blocks = (b.natoms + atoms_per_block - 1) / atoms_per_block;
  if (adjoint) {
    auto kern = k_adjoint<T, R, A, LPA, GUARD, MOM>;
    if (smem + AE_STATIC_SMEM > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  } else {
    auto kern = k_forward<T, R, A, LPA, GUARD, MOM>;
    if (smem + AE_STATIC_SMEM > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  }
  return (int)cudaGetLastError();
}

template <typename T, int R, int A, bool MOM>
int launch_lpa(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  switch (b.lpa) {
    case 8: return launch<T, R, A, 8, false, MOM>(pd, b, adjoint, s);
    case 32: return launch<T, R, A, 32, false, MOM>(pd, b, adjoint, s);
    default: return launch<T, R, A, 16, false, MOM>(pd, b, adjoint, s);
  }
}

// common (radial, angular) sizes of every species, or false
inline bool uniform_sizes(const PotDevice& pd, int& rN, int& aN) {
  rN = aN = 0;
  bool same = true;
  for (int t = 0; t < pd.ntypes; ++t) {
    if (t > 0 && (pd.sp[t].cheb.r_N != rN || pd.sp[t].cheb.a_N != aN)) same = false;
    rN = max(rN, pd.sp[t].cheb.r_N);
    aN = max(aN, pd.sp[t].cheb.a_N);
  }
  return same;
}

// FP32 moment form of the angular terms (k_cheb_mom.cu); returns
// AE_MOM_NA when the sizes have no moment instantiation
constexpr int AE_MOM_NA = -1;
int dispatch_moments(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s);

// Exact instantiations for the common (radial, angular) sizes, guarded
// ones for everything else.  FP32 evaluations with a moment buffer take
// the moment form where it is instantiated.
template <typename T>
int dispatch(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  int rN, aN;
  const bool same = uniform_sizes(pd, rN, aN);
  if (b.nb_rank) {
    // ordered spin weights: pair form of the guarded instances
    if (rN <= 24 && aN <= 16) return launch<T, 24, 16, 16, true, false>(pd, b, adjoint, s);
    if (rN <= 32 && aN <= 32) return launch<T, 32, 32, 16, true, false>(pd, b, adjoint, s);
    return (int)cudaErrorInvalidValue;
  }
  if constexpr (sizeof(T) == 4) {
    if (b.M && pd.qleg) {
      const int e = dispatch_moments(pd, b, adjoint, s);
      if (e != AE_MOM_NA) return e;
    }
  }
  if (same) {
    if (rN == 11 && aN == 5) return launch_lpa<T, 11, 5, false>(pd, b, adjoint, s);
    if (rN == 13 && aN == 7) return launch_lpa<T, 13, 7, false>(pd, b, adjoint, s);
    if (rN == 17 && aN == 9) return launch_lpa<T, 17, 9, false>(pd, b, adjoint, s);
    if (rN == 17 && aN == 5) return launch_lpa<T, 17, 5, false>(pd, b, adjoint, s);
  }
  if (rN <= 24 && aN <= 16) return launch<T, 24, 16, 16, true, false>(pd, b, adjoint, s);
  if (rN <= 32 && aN <= 32) return launch<T, 32, 32, 16, true, false>(pd, b, adjoint, s);
  return (int)cudaErrorInvalidValue;
}

}  // namespace cheb
