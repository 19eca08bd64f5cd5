// Behler-Parrinello symmetry functions G1-G5 and their adjoint (replaces
// sf_fingerprint and the G*_update routines of src/ext/symmfunc.f90:311-811).
//
// One warp per central atom.  The neighbours are first staged in shared
// memory grouped by species (buckets), so that every radial list
// (functions of the central species for one neighbour species) and every
// angular list (one unordered pair of neighbour species) sees neighbours,
// or neighbour pairs, of a single kind:
//   radial  : lanes over the neighbours of a bucket, the list's functions
//             accumulated in registers (chunks of 16), warp reduction;
//   angular : lanes over the pairs of a bucket (triangle) or of two buckets
//             (rectangle), same accumulation.
// The tables come from build_behler (capi.cpp): they already encode the
// reference's indexing (functions registered under the global species
// index, evaluated with the central atom's local one) and the feature
// index of every function.
//
// Functions (symmfunc.f90:445-838, PI truncated as there):
//   fc(r)  = 0.5 (cos(pi r/Rc) + 1)                 r < Rc, else 0
//   G1     = fc(r_ij)
//   G2     = exp(-eta (r_ij - Rs)^2) fc(r_ij)
//   G3     = cos(kappa r_ij) fc(r_ij)
//   G4     = 2 [(1 + lambda cos)/2]^zeta e^{-eta(r_ij^2 + r_ik^2 + r_jk^2)} fc_ij fc_ik fc_jk
//   G5     = 2 [(1 + lambda cos)/2]^zeta e^{-eta(r_ij^2 + r_ik^2)} fc_ij fc_ik
// (the factor 2 accounts for k < j, symmfunc.f90:724), cos clamped to
// [-1, 1] (symmfunc.f90:409-411).
//
// Adjoint: two-sided as for the Chebyshev basis -- the lane owning a staged
// neighbour j sweeps every partner k and accumulates only grad_j of the
// pair's terms contracted with dE/dG, so no force is written twice.
#include "common.h"

namespace {

constexpr double SF_PI = 3.14159265358979;   // symmfunc.f90:38
constexpr int FCH = 16;                      // functions per register chunk

template <typename T>
struct V4;
template <>
struct V4<float> {
  using type = float4;
};
template <>
struct V4<double> {
  using type = double4_32a;
};

__device__ __forceinline__ void sincos_t(float x, float* s, float* c) { __sincosf(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float exp_t(float x) { return __expf(x); }
__device__ __forceinline__ double exp_t(double x) { return exp(x); }
__device__ __forceinline__ float pow_t(float a, float b) { return powf(a, b); }
__device__ __forceinline__ double pow_t(double a, double b) { return pow(a, b); }

template <typename T>
struct Fn {
  T Rc, p1, p2, p3;
  int kind, out, izeta;
};

__device__ __forceinline__ Fn<float> load_fn_f(const BehlerFn* f) {
  Fn<float> r;
  r.Rc = f->fRc;
  r.p1 = f->fp1;
  r.p2 = f->fp2;
  r.p3 = f->fp3;
  r.kind = f->kind;
  r.out = f->out;
  r.izeta = f->izeta;
  return r;
}
__device__ __forceinline__ Fn<double> load_fn_d(const BehlerFn* f) {
  Fn<double> r;
  r.Rc = f->Rc;
  r.p1 = f->p1;
  r.p2 = f->p2;
  r.p3 = f->p3;
  r.kind = f->kind;
  r.out = f->out;
  r.izeta = f->izeta;
  return r;
}
template <typename T>
__device__ __forceinline__ Fn<T> load_fn(const BehlerFn* f);
template <>
__device__ __forceinline__ Fn<float> load_fn<float>(const BehlerFn* f) { return load_fn_f(f); }
template <>
__device__ __forceinline__ Fn<double> load_fn<double>(const BehlerFn* f) { return load_fn_d(f); }

// sf_cut (symmfunc.f90:823-838)
template <typename T>
__device__ __forceinline__ void cutfn(T r, T Rc, T& fc, T& dfc) {
  if (r >= Rc) {
    fc = T(0);
    dfc = T(0);
    return;
  }
  const T a = T(SF_PI) / Rc;
  T s, c;
  sincos_t(a * r, &s, &c);
  fc = T(0.5) * (c + T(1));
  dfc = T(-0.5) * a * s;
}

// a^n for a small non-negative integer n (binary exponentiation)
template <typename T>
__device__ __forceinline__ T ipow(T a, int n) {
  T r = T(1);
  while (n) {
    if (n & 1) r *= a;
    a *= a;
    n >>= 1;
  }
  return r;
}

// radial value and d/dr (sf_G1_ij, sf_G2_ij, sf_G3_ij)
template <typename T>
__device__ __forceinline__ void radial_fn(const Fn<T>& f, T r, T& v, T& dv) {
  T fc, dfc;
  cutfn(r, f.Rc, fc, dfc);
  if (f.kind == 2) {
    const T a = r - f.p1;
    const T e = exp_t(-f.p2 * a * a);
    v = e * fc;
    dv = e * (dfc - T(2) * f.p2 * a * fc);
  } else if (f.kind == 3) {
    T s, c;
    sincos_t(f.p1 * r, &s, &c);
    v = c * fc;
    dv = c * dfc - f.p1 * s * fc;
  } else {
    v = fc;
    dv = dfc;
  }
}

// F1 = ((1 + lambda cos)/2)^zeta and dF1/dcos (sf_F1_ijk)
template <typename T>
__device__ __forceinline__ void f1(const Fn<T>& f, T cosv, T& F, T& dF) {
  const T a = T(0.5) * (T(1) + f.p1 * cosv);
  T pz, pz1;
  if (f.izeta > 0) {
    pz1 = ipow(a, f.izeta - 1);
    pz = pz1 * a;
  } else {
    pz = pow_t(a, f.p2);
    pz1 = pow_t(a, f.p2 - T(1));
  }
  F = pz;
  dF = T(0.5) * f.p2 * f.p1 * pz1;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

__device__ __forceinline__ double normalise(double g, const PotDevice& pd, size_t k) {
  return (g - pd.shift[k]) * pd.scale[k];
}
__device__ __forceinline__ float normalise(float g, const PotDevice& pd, size_t k) {
  const float2 sh = pd.shift2[k];
  return ((g - sh.x) - sh.y) * pd.scale32[k];
}

template <typename T>
__host__ __device__ inline size_t behler_smem_per_warp(int cap, int nsf_pad, bool adjoint) {
  using T4 = typename V4<T>::type;
  size_t per = (sizeof(T4) + 4) * (size_t)cap + (adjoint ? sizeof(T) * nsf_pad : 0);
  return (per + 31) & ~size_t(31);
}

// Stage the neighbours inside rc into shared memory grouped by species.
// bstart[s] .. bstart[s+1] is bucket s; returns the number staged.
template <typename T>
__device__ int stage_buckets(const typename V4<T>::type* __restrict__ vec,
                             const int* __restrict__ jt, int n, int nt, T rc,
                             typename V4<T>::type* sR, int* sslot, int* bstart, int lane) {
  using T4 = typename V4<T>::type;
  int cnt = 0;
  for (int s = 0; s < nt; ++s) {
    bstart[s] = cnt;
    for (int base = 0; base < n; base += 32) {
      const int j = base + lane;
      bool in = false;
      T4 v;
      if (j < n) {
        v = vec[j];
        in = ((jt[j] >> AE_TYPE_SHIFT) == s) && v.w < rc && v.w > T(1e-8);
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int k = cnt + __popc(m & ((1u << lane) - 1u));
        sR[k] = v;
        sslot[k] = j;
      }
      cnt += __popc(m);
    }
  }
  bstart[nt] = cnt;
  __syncwarp();
  return cnt;
}

template <typename T>
__device__ __forceinline__ const BehlerTable* table_of(const PotDevice& pd, int t) {
  return reinterpret_cast<const BehlerTable*>(pd.behler_blob + pd.sp[t].behler_off);
}

// ----------------------------------------------------------------------
// forward
// ----------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_behler_forward(PotDevice pd, DescBuffers b) {
  using T4 = typename V4<T>::type;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= b.natoms) return;
  unsigned char* base = smem_raw + behler_smem_per_warp<T>(b.cap, pd.nsf_pad, false) * warp;
  T4* sR = reinterpret_cast<T4*>(base);
  int* sslot = reinterpret_cast<int*>(sR + b.cap);
  const int ti = b.types[i];
  const BehlerTable* tab = table_of<T>(pd, ti);
  const int nt = pd.ntypes;
  const int n = b.nb_cnt[i];
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  int bstart[AE_MAXT + 1];
  stage_buckets<T>(vec, jt, n, nt, T(tab->rc_max), sR, sslot, bstart, lane);
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  T* G = reinterpret_cast<T*>(b.G) + (size_t)i * pd.nsf_pad;
  const int nsf = pd.sp[ti].nsf;
  // features that no function feeds are normalised zeros (symmfunc.f90:367)
  for (int k = lane; k < nsf; k += 32) G[k] = normalise(T(0), pd, nrow + k);
  __syncwarp();

  // ---- radial lists
  for (int s = 0; s < nt; ++s) {
    const int f0 = tab->rad_off[s], f1e = tab->rad_off[s + 1];
    for (int c0 = f0; c0 < f1e; c0 += FCH) {
      const int nf = min(FCH, f1e - c0);
      T acc[FCH];
#pragma unroll
      for (int q = 0; q < FCH; ++q) acc[q] = T(0);
      for (int j = bstart[s] + lane; j < bstart[s + 1]; j += 32) {
        const T r = sR[j].w;
#pragma unroll
        for (int q = 0; q < FCH; ++q) {
          if (q < nf) {
            const Fn<T> f = load_fn<T>(&tab->fn[c0 + q]);
            T v, dv;
            radial_fn(f, r, v, dv);
            acc[q] += v;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < FCH; ++q) {
        if (q < nf) {
          const T v = warp_sum(acc[q]);
          if (lane == q) {
            const int out = tab->fn[c0 + q].out;
            G[out] = normalise(v, pd, nrow + out);
          }
        }
      }
    }
  }

  // ---- angular lists
  for (int a = 0; a < nt; ++a) {
    for (int c = a; c < nt; ++c) {
      const int f0 = tab->ang_off[a * nt + c], f1e = tab->ang_off[a * nt + c + 1];
      if (f0 == f1e) continue;
      const int na = bstart[a + 1] - bstart[a], nc = bstart[c + 1] - bstart[c];
      const int P = (a == c) ? na * (na - 1) / 2 : na * nc;
      for (int c0 = f0; c0 < f1e; c0 += FCH) {
        const int nf = min(FCH, f1e - c0);
        T acc[FCH];
#pragma unroll
        for (int q = 0; q < FCH; ++q) acc[q] = T(0);
        for (int p = lane; p < P; p += 32) {
          int j, k;
          if (a == c) {
            // row-major upper triangle of bucket a: invert start(r) =
            // r (2 na - r - 1) / 2 <= p
            const float fn = (float)(2 * na - 1);
            int rr = (int)((fn - sqrtf(fn * fn - 8.0f * (float)p)) * 0.5f);
            rr = max(0, min(rr, na - 2));
            while (rr > 0 && rr * (2 * na - rr - 1) / 2 > p) --rr;
            while (rr < na - 2 && (rr + 1) * (2 * na - rr - 2) / 2 <= p) ++rr;
            j = bstart[a] + rr;
            k = bstart[a] + p - rr * (2 * na - rr - 1) / 2 + rr + 1;
          } else {
            j = bstart[a] + p / nc;
            k = bstart[c] + p % nc;
          }
          const T4 Rj = sR[j], Rk = sR[k];
          const T dxx = Rk.x - Rj.x, dyy = Rk.y - Rj.y, dzz = Rk.z - Rj.z;
          const T rjk2 = dxx * dxx + dyy * dyy + dzz * dzz;
          const T rjk = sqrt(rjk2);
          T cosv = (Rj.x * Rk.x + Rj.y * Rk.y + Rj.z * Rk.z) / (Rj.w * Rk.w);
          cosv = fmax(T(-1), fmin(T(1), cosv));
          const T rij2 = Rj.w * Rj.w, rik2 = Rk.w * Rk.w;
          T rc_cur = T(-1), fij = T(0), fik = T(0), fjk = T(0), dum;
#pragma unroll
          for (int q = 0; q < FCH; ++q) {
            if (q < nf) {
              const Fn<T> f = load_fn<T>(&tab->fn[c0 + q]);
              if (f.Rc != rc_cur) {
                rc_cur = f.Rc;
                cutfn(Rj.w, rc_cur, fij, dum);
                cutfn(Rk.w, rc_cur, fik, dum);
                cutfn(rjk, rc_cur, fjk, dum);
              }
              T F, dF;
              f1(f, cosv, F, dF);
              if (f.kind == 4)
                acc[q] += T(2) * F * exp_t(-f.p3 * (rij2 + rik2 + rjk2)) * fij * fik * fjk;
              else
                acc[q] += T(2) * F * exp_t(-f.p3 * (rij2 + rik2)) * fij * fik;
            }
          }
        }
#pragma unroll
        for (int q = 0; q < FCH; ++q) {
          if (q < nf) {
            const T v = warp_sum(acc[q]);
            if (lane == q) {
              const int out = tab->fn[c0 + q].out;
              G[out] = normalise(v, pd, nrow + out);
            }
          }
        }
      }
    }
  }
}

// ----------------------------------------------------------------------
// adjoint
// ----------------------------------------------------------------------
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

template <typename T>
__global__ void __launch_bounds__(128) k_behler_adjoint(PotDevice pd, DescBuffers b) {
  using T4 = typename V4<T>::type;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= b.natoms) return;
  unsigned char* base = smem_raw + behler_smem_per_warp<T>(b.cap, pd.nsf_pad, true) * warp;
  T4* sR = reinterpret_cast<T4*>(base);
  int* sslot = reinterpret_cast<int*>(sR + b.cap);
  T* sg = reinterpret_cast<T*>(sslot + b.cap);
  const int ti = b.types[i];
  const BehlerTable* tab = table_of<T>(pd, ti);
  const int nt = pd.ntypes;
  const int n = b.nb_cnt[i];
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  const int sid = b.atom_struct[i];
  const T gs = b.grad_scale ? T(b.grad_scale[sid]) : T(1);
  const T* gsrc = reinterpret_cast<const T*>(b.dEdG) + (size_t)i * pd.nsf_pad;
  const int nsf = pd.sp[ti].nsf;
  for (int k = lane; k < nsf; k += 32) sg[k] = gs * gsrc[k];
  int bstart[AE_MAXT + 1];
  const int nst = stage_buckets<T>(vec, jt, n, nt, T(tab->rc_max), sR, sslot, bstart, lane);
  T* F = reinterpret_cast<T*>(b.F);
  const bool want_virial = b.virial != nullptr;
  T fix = T(0), fiy = T(0), fiz = T(0);
  T w00 = 0, w01 = 0, w02 = 0, w10 = 0, w11 = 0, w12 = 0, w20 = 0, w21 = 0, w22 = 0;

  for (int j0 = 0; j0 < nst; j0 += 32) {
    const int j = j0 + lane;
    const bool own = j < nst;
    int tj = 0;
    for (int s = 0; s < nt; ++s)
      if (j >= bstart[s + 1]) tj = s + 1;
    if (tj >= nt) tj = nt - 1;
    T4 Rj;
    if (own) {
      Rj = sR[j];
    } else {
      Rj.x = Rj.y = Rj.z = T(0);
      Rj.w = T(1);
    }
    const T invj = T(1) / Rj.w;
    const T ux = Rj.x * invj, uy = Rj.y * invj, uz = Rj.z * invj;
    T gx = T(0), gy = T(0), gz = T(0);
    // radial: d/dr_ij of sum_f g_f G_f(r_ij) along Rhat_ij
    if (own) {
      const int f0 = tab->rad_off[tj], f1e = tab->rad_off[tj + 1];
      T c = T(0);
      for (int q = f0; q < f1e; ++q) {
        const Fn<T> f = load_fn<T>(&tab->fn[q]);
        T v, dv;
        radial_fn(f, Rj.w, v, dv);
        c += sg[f.out] * dv;
      }
      gx += c * ux;
      gy += c * uy;
      gz += c * uz;
    }
    // angular, two-sided: grad_j of every pair (j, k)
    for (int k = 0; k < nst; ++k) {
      if (!own || k == j) continue;
      int tk = 0;
      for (int s = 0; s < nt; ++s)
        if (k >= bstart[s + 1]) tk = s + 1;
      const int lo = min(tj, tk), hi = max(tj, tk);
      const int f0 = tab->ang_off[lo * nt + hi], f1e = tab->ang_off[lo * nt + hi + 1];
      if (f0 == f1e) continue;
      const T4 Rk = sR[k];
      const T dxx = Rk.x - Rj.x, dyy = Rk.y - Rj.y, dzz = Rk.z - Rj.z;
      const T rjk2 = dxx * dxx + dyy * dyy + dzz * dzz;
      const T rjk = sqrt(rjk2);
      const T invk = T(1) / Rk.w;
      const T vx = Rk.x * invk, vy = Rk.y * invk, vz = Rk.z * invk;
      T cosv = ux * vx + uy * vy + uz * vz;
      cosv = fmax(T(-1), fmin(T(1), cosv));
      const T rij2 = Rj.w * Rj.w, rik2 = Rk.w * Rk.w;
      T rc_cur = T(-1), fij = 0, dfij = 0, fik = 0, dfik = 0, fjk = 0, dfjk = 0;
      T Sc = T(0), Sij = T(0), Sjk = T(0);
      for (int q = f0; q < f1e; ++q) {
        const Fn<T> f = load_fn<T>(&tab->fn[q]);
        if (f.Rc != rc_cur) {
          rc_cur = f.Rc;
          cutfn(Rj.w, rc_cur, fij, dfij);
          cutfn(Rk.w, rc_cur, fik, dfik);
          cutfn(rjk, rc_cur, fjk, dfjk);
        }
        const T g2 = T(2) * sg[f.out];
        T F1v, dF1v;
        f1(f, cosv, F1v, dF1v);
        if (f.kind == 4) {
          const T E = exp_t(-f.p3 * (rij2 + rik2 + rjk2));
          const T base3 = g2 * E;
          Sc += base3 * dF1v * fij * fik * fjk;
          Sij += base3 * F1v * fik * fjk * (dfij - T(2) * f.p3 * Rj.w * fij);
          Sjk += base3 * F1v * fij * fik * (dfjk - T(2) * f.p3 * rjk * fjk);
        } else {
          const T E = exp_t(-f.p3 * (rij2 + rik2));
          const T base3 = g2 * E;
          Sc += base3 * dF1v * fij * fik;
          Sij += base3 * F1v * fik * (dfij - T(2) * f.p3 * Rj.w * fij);
        }
      }
      // grad_j = Sc (Rhat_k - cos Rhat_j)/r_ij + Sij Rhat_j - Sjk Rhat_jk
      const T cj = Sc * invj;
      const T ijk = rjk > T(1e-8) ? Sjk / rjk : T(0);
      gx += cj * (vx - cosv * ux) + Sij * ux - ijk * dxx;
      gy += cj * (vy - cosv * uy) + Sij * uy - ijk * dyy;
      gz += cj * (vz - cosv * uz) + Sij * uz - ijk * dzz;
    }
    if (own) {
      const int slot = sslot[j];
      atomic_add3<T>(F, jt[slot] & AE_INDEX_MASK, -gx, -gy, -gz);
      if (want_virial) {
        w00 -= Rj.x * gx; w01 -= Rj.x * gy; w02 -= Rj.x * gz;
        w10 -= Rj.y * gx; w11 -= Rj.y * gy; w12 -= Rj.y * gz;
        w20 -= Rj.z * gx; w21 -= Rj.z * gy; w22 -= Rj.z * gz;
      }
      fix += gx;
      fiy += gy;
      fiz += gz;
    }
  }
  fix = warp_sum(fix);
  fiy = warp_sum(fiy);
  fiz = warp_sum(fiz);
  if (lane == 0) atomic_add3<T>(F, i, fix, fiy, fiz);
  if (want_virial) {
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

template <typename T>
int launch(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  const int warps = 4;
  const size_t smem = behler_smem_per_warp<T>(b.cap, pd.nsf_pad, adjoint) * warps;
  if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
  const int blocks = (b.natoms + warps - 1) / warps;
  if (adjoint) {
    if (smem + AE_STATIC_SMEM > 48 * 1024)
      cudaFuncSetAttribute(k_behler_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_behler_adjoint<T><<<blocks, warps * 32, smem, s>>>(pd, b);
  } else {
    if (smem + AE_STATIC_SMEM > 48 * 1024)
      cudaFuncSetAttribute(k_behler_forward<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_behler_forward<T><<<blocks, warps * 32, smem, s>>>(pd, b);
  }
  return (int)cudaGetLastError();
}

// ----------------------------------------------------------------------
// descriptor Jacobians (FP64) for generate.x's PyTorch export: the adjoint's
// two-sided sweep without the contraction with dE/dG -- the lane owning
// staged neighbour j adds dG_f/dR_j of every radial function of its bucket
// and of every angular function of every pair (j, k) to its own slot row
// (G4/G5 carry the factor 2 of symmfunc.f90:724); the central atom's row is
// minus the sum over the neighbours.
// ----------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_behler_jacobian(PotDevice pd, DescBuffers b, int atom0,
                                                         int count, int nsf_max,
                                                         double* __restrict__ Ji,
                                                         double* __restrict__ Jj,
                                                         int* __restrict__ nbl,
                                                         int* __restrict__ nnb) {
  using T = double;
  using T4 = double4_32a;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int r = blockIdx.x * (blockDim.x >> 5) + warp;
  if (r >= count) return;
  const int i = atom0 + r;
  unsigned char* base = smem_raw + behler_smem_per_warp<T>(b.cap, pd.nsf_pad, false) * warp;
  T4* sR = reinterpret_cast<T4*>(base);
  int* sslot = reinterpret_cast<int*>(sR + b.cap);
  const int ti = b.types[i];
  const BehlerTable* tab = table_of<T>(pd, ti);
  const int nt = pd.ntypes;
  const int n = b.nb_cnt[i];
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  const size_t rs = (size_t)nsf_max * 3;
  double* __restrict__ Jrow = Jj + (size_t)r * b.cap * rs;
  if (lane == 0) nnb[r] = n;
  for (int a = lane; a < n; a += 32) {
    for (size_t q = 0; q < rs; ++q) Jrow[(size_t)a * rs + q] = 0.0;
    nbl[(size_t)r * b.cap + a] = jt[a] & AE_INDEX_MASK;
  }
  int bstart[AE_MAXT + 1];
  const int nst = stage_buckets<T>(vec, jt, n, nt, T(tab->rc_max), sR, sslot, bstart, lane);
  __syncwarp();
  for (int j = lane; j < nst; j += 32) {
    int tj = 0;
    for (int s2 = 0; s2 < nt; ++s2)
      if (j >= bstart[s2 + 1]) tj = s2 + 1;
    if (tj >= nt) tj = nt - 1;
    const T4 Rj = sR[j];
    const T invj = T(1) / Rj.w;
    const T ux = Rj.x * invj, uy = Rj.y * invj, uz = Rj.z * invj;
    double* Ja = Jrow + (size_t)sslot[j] * rs;
    // radial functions of bucket tj
    for (int q = tab->rad_off[tj]; q < tab->rad_off[tj + 1]; ++q) {
      const Fn<T> f = load_fn<T>(&tab->fn[q]);
      T v, dv;
      radial_fn(f, Rj.w, v, dv);
      Ja[f.out * 3] += dv * ux;
      Ja[f.out * 3 + 1] += dv * uy;
      Ja[f.out * 3 + 2] += dv * uz;
    }
    // angular functions of every pair (j, k)
    for (int k = 0; k < nst; ++k) {
      if (k == j) continue;
      int tk = 0;
      for (int s2 = 0; s2 < nt; ++s2)
        if (k >= bstart[s2 + 1]) tk = s2 + 1;
      const int lo = min(tj, tk), hi = max(tj, tk);
      const int f0 = tab->ang_off[lo * nt + hi], f1e = tab->ang_off[lo * nt + hi + 1];
      if (f0 == f1e) continue;
      const T4 Rk = sR[k];
      const T dxx = Rk.x - Rj.x, dyy = Rk.y - Rj.y, dzz = Rk.z - Rj.z;
      const T rjk2 = dxx * dxx + dyy * dyy + dzz * dzz;
      const T rjk = sqrt(rjk2);
      const T invk = T(1) / Rk.w;
      const T vx = Rk.x * invk, vy = Rk.y * invk, vz = Rk.z * invk;
      T cosv = ux * vx + uy * vy + uz * vz;
      cosv = fmax(T(-1), fmin(T(1), cosv));
      const T rij2 = Rj.w * Rj.w, rik2 = Rk.w * Rk.w;
      const T ijk = rjk > T(1e-8) ? T(1) / rjk : T(0);
      T rc_cur = T(-1), fij = 0, dfij = 0, fik = 0, dfik = 0, fjk = 0, dfjk = 0;
      for (int q = f0; q < f1e; ++q) {
        const Fn<T> f = load_fn<T>(&tab->fn[q]);
        if (f.Rc != rc_cur) {
          rc_cur = f.Rc;
          cutfn(Rj.w, rc_cur, fij, dfij);
          cutfn(Rk.w, rc_cur, fik, dfik);
          cutfn(rjk, rc_cur, fjk, dfjk);
        }
        T F1v, dF1v;
        f1(f, cosv, F1v, dF1v);
        T Sc, Sij, Sjk = T(0);
        if (f.kind == 4) {
          const T E = T(2) * exp_t(-f.p3 * (rij2 + rik2 + rjk2));
          Sc = E * dF1v * fij * fik * fjk;
          Sij = E * F1v * fik * fjk * (dfij - T(2) * f.p3 * Rj.w * fij);
          Sjk = E * F1v * fij * fik * (dfjk - T(2) * f.p3 * rjk * fjk);
        } else {
          const T E = T(2) * exp_t(-f.p3 * (rij2 + rik2));
          Sc = E * dF1v * fij * fik;
          Sij = E * F1v * fik * (dfij - T(2) * f.p3 * Rj.w * fij);
        }
        // grad_j = Sc (Rhat_k - cos Rhat_j)/r_ij + Sij Rhat_j - Sjk Rhat_jk
        const T cj = Sc * invj;
        Ja[f.out * 3] += cj * (vx - cosv * ux) + Sij * ux - Sjk * ijk * dxx;
        Ja[f.out * 3 + 1] += cj * (vy - cosv * uy) + Sij * uy - Sjk * ijk * dyy;
        Ja[f.out * 3 + 2] += cj * (vz - cosv * uz) + Sij * uz - Sjk * ijk * dzz;
      }
    }
  }
  __syncwarp();
  const int nq = pd.sp[ti].nsf * 3;
  for (int q = lane; q < (int)rs; q += 32) {
    double acc = 0.0;
    if (q < nq)
      for (int a = 0; a < n; ++a) acc -= Jrow[(size_t)a * rs + q];
    Ji[(size_t)r * rs + q] = acc;
  }
}

}  // namespace

int ae_launch_behler_forward(const PotDevice& pd, const DescBuffers& b, int fp64, cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  return fp64 ? launch<double>(pd, b, false, s) : launch<float>(pd, b, false, s);
}

int ae_launch_behler_adjoint(const PotDevice& pd, const DescBuffers& b, int fp64, cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  return fp64 ? launch<double>(pd, b, true, s) : launch<float>(pd, b, true, s);
}

int ae_launch_behler_jacobian(const PotDevice& pd, const DescBuffers& b, int atom0, int count,
                              int nsf_max, double* Ji, double* Jj, int* nbl, int* nnb,
                              cudaStream_t s) {
  if (count <= 0) return 0;
  const int warps = 4;
  const size_t smem = behler_smem_per_warp<double>(b.cap, pd.nsf_pad, false) * warps;
  if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
  if (smem + AE_STATIC_SMEM > 48 * 1024)
    cudaFuncSetAttribute(k_behler_jacobian, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_behler_jacobian<<<(count + warps - 1) / warps, warps * 32, smem, s>>>(pd, b, atom0, count,
                                                                         nsf_max, Ji, Jj, nbl, nnb);
  return (int)cudaGetLastError();
}
