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
//   angular : lanes over the pairs of a bucket (triangle, circulant order)
//             or of two buckets (rectangle), p = lane, lane + 32, ..., so
//             every lane gets the same number of pairs.
// Angular lists that form a product grid (one kind and Rc, lambda = +-1,
// every (lambda, zeta) x eta combination; BehlerGrid) are evaluated per
// pair with one exponential per eta and one power per (lambda, zeta), the
// functions being their products; other lists function by function.
// G4 pairs with r_jk >= Rc contribute nothing (fc(r_jk) = 0) and are
// skipped after the distance test.
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
// Adjoint: one-sided -- each pair (j, k) once, its gradient with respect to
// both neighbours added to per-neighbour accumulators in shared memory;
// the central atom's force and the virial follow from those sums.
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

// Shared memory of one warp: the staged neighbours sR (x, y, z, r), their
// per-neighbour terms sA (1/r, fc, dfc at the table's largest Rc), in the
// adjoint the per-neighbour gradient accumulators sF (x, y, z) and the
// scaled dE/dG row sg, then the table slot of each staged neighbour and a
// queue of QCAP packed pairs (the surviving G4 pairs, see run_pairs).
constexpr int QCAP = 64;
template <typename T>
__host__ __device__ inline size_t behler_smem_per_warp(int cap, int nsf_pad, bool adjoint) {
  using T4 = typename V4<T>::type;
  size_t per = 2 * sizeof(T4) * (size_t)cap + 4 * (size_t)cap + 4 * QCAP +
               (adjoint ? sizeof(T) * (3 * (size_t)cap + nsf_pad) : 0);
  return (per + 31) & ~size_t(31);
}

// Stage the neighbours inside rc into shared memory grouped by species.
// bstart[s] .. bstart[s+1] is bucket s; returns the number staged.  sA
// (optional) receives 1/r, fc(r) and dfc(r) for the cut-off rc.
template <typename T>
__device__ int stage_buckets(const typename V4<T>::type* __restrict__ vec,
                             const int* __restrict__ jt, int n, int nt, T rc,
                             typename V4<T>::type* sR, typename V4<T>::type* sA, int* sslot,
                             int* bstart, int lane) {
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
        if (sA) {
          T4 a;
          a.x = T(1) / v.w;
          cutfn(v.w, rc, a.y, a.z);
          a.w = T(0);
          sA[k] = a;
        }
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
__device__ __forceinline__ const BehlerGrid* grids_of(const BehlerTable* tab) {
  return reinterpret_cast<const BehlerGrid*>(reinterpret_cast<const unsigned char*>(tab) +
                                             tab->grid_off);
}

// ---- pair schedules: lanes take pairs p = lane, lane + 32, ... of a list.
// Unordered pairs of one bucket of m neighbours on a circulant schedule:
// p = q m + r -> (r, (r + q + 1) mod m); with q < (m - 1)/2, plus the pairs
// at distance m/2 from r < m/2 when m is even, every pair occurs once.
// Pairs of bucket A (ma) x bucket C (mc): p = q ma + r -> (r, (q + r) mod mc).
// Each lane keeps (q, r) and r mod mc and advances them by 32 with integer
// adds and compares only (int <-> float conversions are slow on this GPU).
struct PairList {
  int a0, ma, c0, mc, P;
  int s32, mam;     // 32 mod mc, ma mod mc (rectangle)
  bool tri;
};

__device__ __forceinline__ PairList pair_list(const int* bstart, int a, int c) {
  PairList L;
  L.a0 = bstart[a];
  L.ma = bstart[a + 1] - bstart[a];
  L.c0 = bstart[c];
  L.mc = bstart[c + 1] - bstart[c];
  L.tri = a == c;
  L.P = L.tri ? L.ma * (L.ma - 1) / 2 : L.ma * L.mc;
  L.s32 = L.mc > 0 ? 32 % L.mc : 0;
  L.mam = L.mc > 0 ? L.ma % L.mc : 0;
  return L;
}

struct PairWalk {
  int p, q, r, rm;
  __device__ __forceinline__ void init(const PairList& L, int lane) {
    p = lane;
    if (L.P == 0) return;
    q = lane / L.ma;
    r = lane - q * L.ma;
    rm = L.tri ? 0 : r % L.mc;
  }
  __device__ __forceinline__ void get(const PairList& L, int& j, int& k) const {
    if (L.tri) {
      int kk = r + q + 1;
      if (kk >= L.ma) kk -= L.ma;
      j = L.a0 + r;
      k = L.a0 + kk;
    } else {
      int kk = q + rm;
      if (kk >= L.mc) kk -= L.mc;
      j = L.a0 + r;
      k = L.c0 + kk;
    }
  }
  __device__ __forceinline__ void advance(const PairList& L) {
    p += 32;
    r += 32;
    if (!L.tri) {
      rm += L.s32;
      if (rm >= L.mc) rm -= L.mc;
    }
    while (r >= L.ma) {
      r -= L.ma;
      ++q;
      if (!L.tri) {
        rm -= L.mam;
        if (rm < 0) rm += L.mc;
      }
    }
  }
};

// ---- powers of the grid path: F = u^zeta (and dF/du = zeta u^(zeta-1))
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Per-pair terms of the angular factor ((1 + lambda cos)/2)^zeta for
// lambda = +1 and -1.  FP32: u^zeta = 2^(zeta log2 u) (one log per sign,
// one power per (lambda, zeta)); FP64: repeated squaring for integer zeta.
template <typename T>
struct Ang;
template <>
struct Ang<float> {
  float up, um, lp, lm, ip, im;
  __device__ __forceinline__ void init(float c) {
    up = 0.5f + 0.5f * c;
    um = 0.5f - 0.5f * c;
    lp = lg2_approx(up);
    lm = lg2_approx(um);
    ip = up > 0.f ? __frcp_rn(up) : 0.f;
    im = um > 0.f ? __frcp_rn(um) : 0.f;
  }
  __device__ __forceinline__ float F(bool pos, float zeta, int) const {
    return ex2_approx(zeta * (pos ? lp : lm));
  }
  // dF/dcos = zeta lambda u^(zeta - 1) / 2
  __device__ __forceinline__ void FdF(bool pos, float zeta, int iz, float& F, float& dF) const {
    F = ex2_approx(zeta * (pos ? lp : lm));
    const float pz1 = iz == 1 ? 1.f : F * (pos ? ip : im);
    dF = (pos ? 0.5f : -0.5f) * zeta * pz1;
  }
};
template <>
struct Ang<double> {
  double up, um;
  __device__ __forceinline__ void init(double c) {
    up = 0.5 + 0.5 * c;
    um = 0.5 - 0.5 * c;
  }
  __device__ __forceinline__ double F(bool pos, double zeta, int iz) const {
    const double u = pos ? up : um;
    return iz > 0 ? ipow(u, iz) : pow(u, zeta);
  }
  __device__ __forceinline__ void FdF(bool pos, double zeta, int iz, double& F, double& dF) const {
    const double u = pos ? up : um;
    double pz1;
    if (iz > 0) {
      pz1 = ipow(u, iz - 1);
      F = pz1 * u;
    } else {
      F = pow(u, zeta);
      pz1 = pow(u, zeta - 1.0);
    }
    dF = (pos ? 0.5 : -0.5) * zeta * pz1;
  }
};

template <typename T>
__device__ __forceinline__ T gval(const BehlerGrid* g, const double* d, const float* f, int i);
template <>
__device__ __forceinline__ float gval<float>(const BehlerGrid*, const double*, const float* f, int i) {
  return f[i];
}
template <>
__device__ __forceinline__ double gval<double>(const BehlerGrid*, const double* d, const float*, int i) {
  return d[i];
}

// Run body(j, k) over the pairs of a list.  For G4 (kind 4) pairs with
// r_jk >= Rc contribute nothing; they are filtered first and the
// survivors go through a per-warp queue in shared memory, so that every
// call of the body has 32 live pairs (one per lane) instead of the ~45 %
// that a plain strided loop leaves active.  The queue holds j | k << 16
// (staged indices < cap <= 65535).
template <typename T, typename Body>
__device__ __forceinline__ void run_pairs(const PairList& L, const typename V4<T>::type* sR,
                                          bool filter, T Rc2, int* queue, int lane, Body body) {
  using T4 = typename V4<T>::type;
  PairWalk w;
  w.init(L, lane);
  if (!filter) {
    for (; w.p < L.P; w.advance(L)) {
      int j, k;
      w.get(L, j, k);
      body(j, k);
    }
    return;
  }
  const unsigned lt = (1u << lane) - 1u;
  int head = 0;
  for (int p0 = 0; p0 < L.P; p0 += 32, w.advance(L)) {
    int j = 0, k = 0;
    bool ok = false;
    if (w.p < L.P) {
      w.get(L, j, k);
      const T4 Rj = sR[j], Rk = sR[k];
      const T dx = Rk.x - Rj.x, dy = Rk.y - Rj.y, dz = Rk.z - Rj.z;
      ok = dx * dx + dy * dy + dz * dz < Rc2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok) queue[head + __popc(m & lt)] = j | (k << 16);
    head += __popc(m);
    __syncwarp();
    if (head >= 32) {
      head -= 32;
      const int e = queue[head + lane];
      __syncwarp();
      body(e & 0xffff, e >> 16);
    }
  }
  __syncwarp();
  if (lane < head) {
    const int e = queue[lane];
    body(e & 0xffff, e >> 16);
  }
  __syncwarp();
}

constexpr int BL = 8;   // (lambda, zeta) pairs per grid block
constexpr int BE = 2;   // eta values per grid block

// Geometry of one pair (j, k) of staged neighbours for the grid path.
template <typename T>
struct PairGeo {
  typename V4<T>::type Rj, Rk;
  T dx, dy, dz, rjk2, cosv, fcj, dfcj, fck, dfck, S;
  __device__ __forceinline__ void load(const typename V4<T>::type* sR,
                                       const typename V4<T>::type* sA, int j, int k, int kind,
                                       T Rc, bool cached) {
    Rj = sR[j];
    Rk = sR[k];
    dx = Rk.x - Rj.x;
    dy = Rk.y - Rj.y;
    dz = Rk.z - Rj.z;
    rjk2 = dx * dx + dy * dy + dz * dz;
    const typename V4<T>::type Aj = sA[j], Ak = sA[k];
    cosv = (Rj.x * Rk.x + Rj.y * Rk.y + Rj.z * Rk.z) * Aj.x * Ak.x;
    cosv = fmax(T(-1), fmin(T(1), cosv));
    if (cached) {
      fcj = Aj.y;
      dfcj = Aj.z;
      fck = Ak.y;
      dfck = Ak.z;
    } else {
      cutfn(Rj.w, Rc, fcj, dfcj);
      cutfn(Rk.w, Rc, fck, dfck);
    }
    S = Rj.w * Rj.w + Rk.w * Rk.w + (kind == 4 ? rjk2 : T(0));
  }
};

// ----------------------------------------------------------------------
// forward
// ----------------------------------------------------------------------
template <typename T>
__device__ void forward_grid(const BehlerGrid* gr, const PairList& L, const typename V4<T>::type* sR,
                             const typename V4<T>::type* sA, bool cached, int* queue, T* G,
                             const PotDevice& pd, size_t nrow, int lane) {
  const int kind = gr->kind, nl = gr->nl, ne = gr->ne;
  const T Rc = gval<T>(gr, &gr->Rc, &gr->fRc, 0);
  for (int l0 = 0; l0 < nl; l0 += BL)
    for (int e0 = 0; e0 < ne; e0 += BE) {
      T eta[BE], zeta[BL];
      int iz[BL];
      bool pos[BL];
#pragma unroll
      for (int e = 0; e < BE; ++e) eta[e] = e0 + e < ne ? gval<T>(gr, gr->eta, gr->feta, e0 + e) : T(0);
#pragma unroll
      for (int l = 0; l < BL; ++l) {
        const int ll = min(l0 + l, nl - 1);
        zeta[l] = gval<T>(gr, gr->zeta, gr->fzeta, ll);
        iz[l] = gr->izeta[ll];
        pos[l] = gr->flam[ll] > 0.f;
      }
      T acc[BL][BE];
#pragma unroll
      for (int l = 0; l < BL; ++l)
#pragma unroll
        for (int e = 0; e < BE; ++e) acc[l][e] = T(0);
      run_pairs<T>(L, sR, kind == 4, Rc * Rc, queue, lane, [&](int j, int k) {
        PairGeo<T> q;
        q.load(sR, sA, j, k, kind, Rc, cached);
        T FC = T(2) * q.fcj * q.fck;
        if (kind == 4) {
          T fjk, dum;
          cutfn(sqrt(q.rjk2), Rc, fjk, dum);
          FC *= fjk;
        }
        T E[BE];
#pragma unroll
        for (int e = 0; e < BE; ++e) E[e] = exp_t(-eta[e] * q.S) * FC;
        Ang<T> ang;
        ang.init(q.cosv);
#pragma unroll
        for (int l = 0; l < BL; ++l) {
          if (l0 + l < nl) {
            const T F = ang.F(pos[l], zeta[l], iz[l]);
#pragma unroll
            for (int e = 0; e < BE; ++e) acc[l][e] += F * E[e];
          }
        }
      });
#pragma unroll
      for (int l = 0; l < BL; ++l)
#pragma unroll
        for (int e = 0; e < BE; ++e) {
          if (l0 + l < nl && e0 + e < ne) {
            const T v = warp_sum(acc[l][e]);
            if (lane == 0) {
              const int out = gr->out[(l0 + l) * AE_BG_NE + e0 + e];
              G[out] = normalise(v, pd, nrow + out);
            }
          }
        }
    }
}

template <typename T>
__device__ void forward_generic(const BehlerTable* tab, int f0, int f1e, const PairList& L,
                                const typename V4<T>::type* sR, T* G, const PotDevice& pd,
                                size_t nrow, int lane) {
  using T4 = typename V4<T>::type;
  for (int c0 = f0; c0 < f1e; c0 += FCH) {
    const int nf = min(FCH, f1e - c0);
    T acc[FCH];
#pragma unroll
    for (int q = 0; q < FCH; ++q) acc[q] = T(0);
    PairWalk w;
    w.init(L, lane);
    for (; w.p < L.P; w.advance(L)) {
      int j, k;
      w.get(L, j, k);
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

// GRID: every angular list is a BehlerGrid (the generic path is left out,
// which frees its registers)
template <typename T, bool GRID>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 5 : 1) k_behler_forward(PotDevice pd, DescBuffers b) {
  using T4 = typename V4<T>::type;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= b.natoms) return;
  unsigned char* base = smem_raw + behler_smem_per_warp<T>(b.cap, pd.nsf_pad, false) * warp;
  T4* sR = reinterpret_cast<T4*>(base);
  T4* sA = sR + b.cap;
  int* sslot = reinterpret_cast<int*>(sA + b.cap);
  int* queue = sslot + b.cap;
  const int ti = b.types[i];
  const BehlerTable* tab = table_of<T>(pd, ti);
  const int nt = pd.ntypes;
  const int n = b.nb_cnt[i];
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  int bstart[AE_MAXT + 1];
  stage_buckets<T>(vec, jt, n, nt, T(tab->rc_max), sR, sA, sslot, bstart, lane);
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  T* G = reinterpret_cast<T*>(b.G) + (size_t)i * pd.nsf_pad;
  const int nsf = pd.sp[ti].nsf;
  // features that no function feeds are normalised zeros (symmfunc.f90:367)
  for (int k = lane; k < nsf; k += 32) G[k] = normalise(T(0), pd, nrow + k);
  __syncwarp();

  // ---- radial lists: function by function, lanes over the bucket's
  // neighbours (a few per lane), warp sum
  for (int s = 0; s < nt; ++s) {
    const int f0 = tab->rad_off[s], f1e = tab->rad_off[s + 1];
    for (int q = f0; q < f1e; ++q) {
      const Fn<T> f = load_fn<T>(&tab->fn[q]);
      T acc = T(0);
      for (int j = bstart[s] + lane; j < bstart[s + 1]; j += 32) {
        T v, dv;
        radial_fn(f, sR[j].w, v, dv);
        acc += v;
      }
      acc = warp_sum(acc);
      if (lane == 0) G[f.out] = normalise(acc, pd, nrow + f.out);
    }
  }

  // ---- angular lists (one per unordered pair of neighbour species)
  const BehlerGrid* grids = grids_of(tab);
  for (int a = 0; a < nt; ++a) {
    for (int c = a; c < nt; ++c) {
      const int f0 = tab->ang_off[a * nt + c], f1e = tab->ang_off[a * nt + c + 1];
      if (f0 == f1e) continue;
      const PairList L = pair_list(bstart, a, c);
      if (L.P == 0) continue;
      const int gi = tab->grid_of[a * nt + c];
      if (GRID || gi >= 0) {
        const BehlerGrid* gr = grids + gi;
        forward_grid<T>(gr, L, sR, sA, gr->Rc == tab->rc_max, queue, G, pd, nrow, lane);
      } else {
        if constexpr (!GRID) forward_generic<T>(tab, f0, f1e, L, sR, G, pd, nrow, lane);
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

// Gradient of one pair's terms with respect to R_j and R_k from the
// partials of the pair's function sum: Sc (cos theta_jik), Sij (r_ij),
// Sik (r_ik), Sjk (r_jk); added to the staged neighbours' accumulators.
template <typename T>
__device__ __forceinline__ void scatter_pair(const typename V4<T>::type& Rj,
                                             const typename V4<T>::type& Rk, T invj, T invk,
                                             T cosv, T dx, T dy, T dz, T rjk, T Sc, T Sij, T Sik,
                                             T Sjk, T* sF, int j, int k) {
  const T ux = Rj.x * invj, uy = Rj.y * invj, uz = Rj.z * invj;
  const T vx = Rk.x * invk, vy = Rk.y * invk, vz = Rk.z * invk;
  const T cj = Sc * invj, ck = Sc * invk;
  const T ijk = rjk > T(1e-8) ? Sjk / rjk : T(0);
  atomicAdd(sF + 3 * j, cj * (vx - cosv * ux) + Sij * ux - ijk * dx);
  atomicAdd(sF + 3 * j + 1, cj * (vy - cosv * uy) + Sij * uy - ijk * dy);
  atomicAdd(sF + 3 * j + 2, cj * (vz - cosv * uz) + Sij * uz - ijk * dz);
  atomicAdd(sF + 3 * k, ck * (ux - cosv * vx) + Sik * vx + ijk * dx);
  atomicAdd(sF + 3 * k + 1, ck * (uy - cosv * vy) + Sik * vy + ijk * dy);
  atomicAdd(sF + 3 * k + 2, ck * (uz - cosv * vz) + Sik * vz + ijk * dz);
}

template <typename T>
__device__ void adjoint_grid(const BehlerGrid* gr, const PairList& L, const typename V4<T>::type* sR,
                             const typename V4<T>::type* sA, bool cached, const T* sg, T* sF,
                             int* queue, int lane) {
  const int kind = gr->kind, nl = gr->nl, ne = gr->ne;
  const T Rc = gval<T>(gr, &gr->Rc, &gr->fRc, 0);
  for (int l0 = 0; l0 < nl; l0 += BL)
    for (int e0 = 0; e0 < ne; e0 += BE) {
      T eta[BE], zeta[BL], g[BL][BE];
      int iz[BL];
      bool pos[BL];
#pragma unroll
      for (int e = 0; e < BE; ++e) eta[e] = e0 + e < ne ? gval<T>(gr, gr->eta, gr->feta, e0 + e) : T(0);
#pragma unroll
      for (int l = 0; l < BL; ++l) {
        const int ll = min(l0 + l, nl - 1);
        zeta[l] = gval<T>(gr, gr->zeta, gr->fzeta, ll);
        iz[l] = gr->izeta[ll];
        pos[l] = gr->flam[ll] > 0.f;
#pragma unroll
        for (int e = 0; e < BE; ++e)
          g[l][e] = (l0 + l < nl && e0 + e < ne) ? T(2) * sg[gr->out[(l0 + l) * AE_BG_NE + e0 + e]]
                                                 : T(0);
      }
      run_pairs<T>(L, sR, kind == 4, Rc * Rc, queue, lane, [&](int j, int k) {
        PairGeo<T> q;
        q.load(sR, sA, j, k, kind, Rc, cached);
        T rjk = T(0), fjk = T(1), dfjk = T(0);
        if (kind == 4) {
          rjk = sqrt(q.rjk2);
          cutfn(rjk, Rc, fjk, dfjk);
        }
        T Es[BE];
#pragma unroll
        for (int e = 0; e < BE; ++e) Es[e] = exp_t(-eta[e] * q.S);
        Ang<T> ang;
        ang.init(q.cosv);
        T A[BE], B[BE];
#pragma unroll
        for (int e = 0; e < BE; ++e) A[e] = B[e] = T(0);
#pragma unroll
        for (int l = 0; l < BL; ++l) {
          if (l0 + l < nl) {
            T F, dF;
            ang.FdF(pos[l], zeta[l], iz[l], F, dF);
#pragma unroll
            for (int e = 0; e < BE; ++e) {
              A[e] += g[l][e] * F;
              B[e] += g[l][e] * dF;
            }
          }
        }
        T SE = T(0), Seta = T(0), SB = T(0);
#pragma unroll
        for (int e = 0; e < BE; ++e) {
          SE += A[e] * Es[e];
          Seta += A[e] * Es[e] * eta[e];
          SB += B[e] * Es[e];
        }
        const T FC = q.fcj * q.fck * fjk;
        const T t2 = T(2) * FC * Seta;
        const T Sc = SB * FC;
        const T Sij = SE * q.dfcj * q.fck * fjk - t2 * q.Rj.w;
        const T Sik = SE * q.fcj * q.dfck * fjk - t2 * q.Rk.w;
        const T Sjk = kind == 4 ? SE * q.fcj * q.fck * dfjk - t2 * rjk : T(0);
        scatter_pair<T>(q.Rj, q.Rk, sA[j].x, sA[k].x, q.cosv, q.dx, q.dy, q.dz, rjk, Sc, Sij,
                        Sik, Sjk, sF, j, k);
      });
    }
}

template <typename T>
__device__ void adjoint_generic(const BehlerTable* tab, int f0, int f1e, const PairList& L,
                                const typename V4<T>::type* sR, const typename V4<T>::type* sA,
                                const T* sg, T* sF, int lane) {
  using T4 = typename V4<T>::type;
  PairWalk w;
  w.init(L, lane);
  for (; w.p < L.P; w.advance(L)) {
    int j, k;
    w.get(L, j, k);
    const T4 Rj = sR[j], Rk = sR[k];
    const T invj = sA[j].x, invk = sA[k].x;
    const T dx = Rk.x - Rj.x, dy = Rk.y - Rj.y, dz = Rk.z - Rj.z;
    const T rjk2 = dx * dx + dy * dy + dz * dz;
    const T rjk = sqrt(rjk2);
    T cosv = (Rj.x * Rk.x + Rj.y * Rk.y + Rj.z * Rk.z) * invj * invk;
    cosv = fmax(T(-1), fmin(T(1), cosv));
    const T rij2 = Rj.w * Rj.w, rik2 = Rk.w * Rk.w;
    T rc_cur = T(-1), fij = 0, dfij = 0, fik = 0, dfik = 0, fjk = 0, dfjk = 0;
    T Sc = T(0), Sij = T(0), Sik = T(0), Sjk = T(0);
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
        const T base3 = g2 * exp_t(-f.p3 * (rij2 + rik2 + rjk2));
        Sc += base3 * dF1v * fij * fik * fjk;
        Sij += base3 * F1v * fik * fjk * (dfij - T(2) * f.p3 * Rj.w * fij);
        Sik += base3 * F1v * fij * fjk * (dfik - T(2) * f.p3 * Rk.w * fik);
        Sjk += base3 * F1v * fij * fik * (dfjk - T(2) * f.p3 * rjk * fjk);
      } else {
        const T base3 = g2 * exp_t(-f.p3 * (rij2 + rik2));
        Sc += base3 * dF1v * fij * fik;
        Sij += base3 * F1v * fik * (dfij - T(2) * f.p3 * Rj.w * fij);
        Sik += base3 * F1v * fij * (dfik - T(2) * f.p3 * Rk.w * fik);
      }
    }
    scatter_pair<T>(Rj, Rk, invj, invk, cosv, dx, dy, dz, rjk, Sc, Sij, Sik, Sjk, sF, j, k);
  }
}

// One-sided adjoint: every pair (j, k) is evaluated once, by one lane, and
// its gradient goes to both staged neighbours' accumulators in shared
// memory (shared-memory atomics; the pair schedules keep the 32 addresses
// of a step mostly distinct).  The central atom's gradient is minus the
// sum over its neighbours (the energy depends on R_j - R_i only), and the
// atom's virial contribution is -sum_j R_ij (x) dE_i/dR_j.
template <typename T, bool GRID>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 4 : 1) k_behler_adjoint(PotDevice pd, DescBuffers b) {
  using T4 = typename V4<T>::type;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= b.natoms) return;
  unsigned char* base = smem_raw + behler_smem_per_warp<T>(b.cap, pd.nsf_pad, true) * warp;
  T4* sR = reinterpret_cast<T4*>(base);
  T4* sA = sR + b.cap;
  T* sF = reinterpret_cast<T*>(sA + b.cap);
  T* sg = sF + 3 * b.cap;
  int* sslot = reinterpret_cast<int*>(sg + pd.nsf_pad);
  int* queue = sslot + b.cap;
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
  const int nst = stage_buckets<T>(vec, jt, n, nt, T(tab->rc_max), sR, sA, sslot, bstart, lane);

  // radial terms: d/dr_ij of sum_f g_f G_f(r_ij) along Rhat_ij (initialises
  // each staged neighbour's accumulator)
  for (int j = lane; j < nst; j += 32) {
    int tj = 0;
    for (int s = 0; s < nt; ++s)
      if (j >= bstart[s + 1]) tj = s + 1;
    const T4 Rj = sR[j];
    const T inv = sA[j].x;
    const int f0 = tab->rad_off[tj], f1e = tab->rad_off[tj + 1];
    T c = T(0);
    for (int q = f0; q < f1e; ++q) {
      const Fn<T> f = load_fn<T>(&tab->fn[q]);
      T v, dv;
      radial_fn(f, Rj.w, v, dv);
      c += sg[f.out] * dv;
    }
    sF[3 * j] = c * Rj.x * inv;
    sF[3 * j + 1] = c * Rj.y * inv;
    sF[3 * j + 2] = c * Rj.z * inv;
  }
  __syncwarp();

  // angular terms, each pair once
  const BehlerGrid* grids = grids_of(tab);
  for (int a = 0; a < nt; ++a) {
    for (int c = a; c < nt; ++c) {
      const int f0 = tab->ang_off[a * nt + c], f1e = tab->ang_off[a * nt + c + 1];
      if (f0 == f1e) continue;
      const PairList L = pair_list(bstart, a, c);
      if (L.P == 0) continue;
      const int gi = tab->grid_of[a * nt + c];
      if (GRID || gi >= 0) {
        const BehlerGrid* gr = grids + gi;
        adjoint_grid<T>(gr, L, sR, sA, gr->Rc == tab->rc_max, sg, sF, queue, lane);
      } else {
        if constexpr (!GRID) adjoint_generic<T>(tab, f0, f1e, L, sR, sA, sg, sF, lane);
      }
    }
  }
  __syncwarp();

  // forces: F_j -= dE_i/dR_j, F_i += sum_j dE_i/dR_j; virial
  T* F = reinterpret_cast<T*>(b.F);
  const bool want_virial = b.virial != nullptr;
  T fix = T(0), fiy = T(0), fiz = T(0);
  T w00 = 0, w01 = 0, w02 = 0, w10 = 0, w11 = 0, w12 = 0, w20 = 0, w21 = 0, w22 = 0;
  for (int j = lane; j < nst; j += 32) {
    const T gx = sF[3 * j], gy = sF[3 * j + 1], gz = sF[3 * j + 2];
    atomic_add3<T>(F, jt[sslot[j]] & AE_INDEX_MASK, -gx, -gy, -gz);
    if (want_virial) {
      const T4 Rj = sR[j];
      w00 -= Rj.x * gx; w01 -= Rj.x * gy; w02 -= Rj.x * gz;
      w10 -= Rj.y * gx; w11 -= Rj.y * gy; w12 -= Rj.y * gz;
      w20 -= Rj.z * gx; w21 -= Rj.z * gy; w22 -= Rj.z * gz;
    }
    fix += gx;
    fiy += gy;
    fiz += gz;
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
  auto kern = adjoint ? (pd.behler_grid_only ? k_behler_adjoint<T, true> : k_behler_adjoint<T, false>)
                      : (pd.behler_grid_only ? k_behler_forward<T, true> : k_behler_forward<T, false>);
  if (smem + AE_STATIC_SMEM > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<blocks, warps * 32, smem, s>>>(pd, b);
  return (int)cudaGetLastError();
}

// ----------------------------------------------------------------------
// descriptor Jacobians (FP64) for generate.x's PyTorch export: a
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
  int* sslot = reinterpret_cast<int*>(sR + 2 * b.cap);
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
  const int nst = stage_buckets<T>(vec, jt, n, nt, T(tab->rc_max), sR, nullptr, sslot, bstart,
                                   lane);
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
