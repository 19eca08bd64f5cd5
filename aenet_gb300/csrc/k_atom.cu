// One atom per call for FP64 Chebyshev potentials: the libaenet per-atom
// entry points (aenet_atomic_energy / aenet_atomic_energy_and_forces,
// src/aenet.f90:359-486) evaluate one central atom with the caller's
// neighbour list.  A warp per atom leaves an SM's FP64 pipe waiting on the
// dependent chains of one lane group, so here one block of AT_THREADS
// threads takes the whole call in one launch, phase after phase:
//
//   stage    thread per neighbour: radial argument and cut-off, angular
//            cut-off and unit vector (the per-neighbour values of sfb_eval,
//            src/ext/sfbasis.f90:488-512); angular neighbours compacted in
//            list order;
//   forward  warp 0 over the neighbours (radial T_n, chebyshev.f90:41-128),
//            the other warps over the pairs j < k of angular neighbours;
//            the per-thread sums are reduced column by column through
//            shared memory, four lanes per feature;
//   network  eight lanes per node, forward and back (ff_eval / ff_deriv,
//            src/ext/feedforward.f90:586-757);
//   adjoint  thread per neighbour (radial) and per pair (angular); the
//            pair gradients of each round are gathered per neighbour in a
//            fixed order; the central atom takes minus the sum of the
//            neighbour forces (aenet.f90:471-477).
//
// Every sum runs in a fixed order, so repeated calls give identical bits.
// The call's inputs are read from, and its outputs written to, mapped
// pinned host memory: a call is one launch and one stream synchronisation.
#include "common.h"
#include "activate.cuh"
#include "k_cheb_impl.cuh"

namespace {

using cheb::angular_arg;
using cheb::cutoff_a;
using cheb::PairWalk;
using cheb::radial_x;
using cheb::SFB_EPS;
using cheb::SFB_PI;

constexpr int AT_THREADS = 256;
constexpr int AT_WARPS = AT_THREADS / 32;
constexpr int AT_RAD = 32;                    // radial threads (warp 0)
constexpr int AT_ANG = AT_THREADS - AT_RAD;   // pair threads (warps 1 ..)
constexpr int AT_LPN = 8;                     // lanes per network node
constexpr int AT_LPF = 4;                     // lanes per feature sum
constexpr int AT_NSTRIDE = AE_MAXNODES + 1;

template <int RB, int AB>
__host__ __device__ constexpr size_t at_red_elems() {
  return (2 * RB * AT_RAD + 2 * AB * AT_ANG) > 6 * AT_THREADS ? (2 * RB * AT_RAD + 2 * AB * AT_ANG)
                                                              : 6 * AT_THREADS;
}

// shared memory of a call with n neighbours
template <int RB, int AB>
__host__ __device__ size_t at_smem_bytes(int n, int nsf_pad) {
  return 4 * sizeof(double4_32a) * (size_t)n + 6 * sizeof(double) * (size_t)n +
         sizeof(double) * (at_red_elems<RB, AB>() + 2 * (size_t)nsf_pad +
                           2 * (size_t)AE_MAXLAYERS * AT_NSTRIDE) +
         64;
}

__device__ __forceinline__ int tri_index(int a, int b, int na) {
  // row-major index of pair (a, b), a < b, in the upper triangle
  return a * (2 * na - a - 1) / 2 + (b - a - 1);
}

template <int RB, int AB>
__global__ void __launch_bounds__(AT_THREADS, 1)
    k_atom(PotDevice pd, const unsigned char* __restrict__ in, unsigned char* __restrict__ out) {
  extern __shared__ __align__(32) unsigned char smem_raw[];
  __shared__ int s_wcnt[AT_WARPS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const AtomCallHeader hd = *reinterpret_cast<const AtomCallHeader*>(in);
  const int n = hd.n, ti = hd.ti;
  const double4_32a* __restrict__ vin = reinterpret_cast<const double4_32a*>(in + AE_ATOM_IN_VEC);
  const int* __restrict__ tin =
      reinterpret_cast<const int*>(in + AE_ATOM_IN_VEC + sizeof(double4_32a) * (size_t)n);
  const SpeciesTable& sp = pd.sp[ti];
  const ChebTable& ct = sp.cheb;
  const double r_Rc = ct.r_Rc, a_Rc = ct.a_Rc;
  const double two_over_rc = 2.0 / r_Rc;
  const double r_a = SFB_PI / r_Rc, a_a = SFB_PI / a_Rc;
  const int rN = ct.r_N, aN = ct.a_N;
  const bool multi = ct.multi;
  const int legacy = ct.angular_legacy;

  double4_32a* sv = reinterpret_cast<double4_32a*>(smem_raw);   // R_ij, d
  double4_32a* sr = sv + n;                                      // x, fc, fc', spin
  double4_32a* au = sr + n;                                      // unit vector, 1/d
  double4_32a* af = au + n;                                      // fc, fc', spin, slot
  double* sF = reinterpret_cast<double*>(af + n);                // forces on neighbours
  double* aF = sF + 3 * (size_t)n;                               // angular gradients
  double* red = aF + 3 * (size_t)n;
  double* G = red + at_red_elems<RB, AB>();
  double* D = G + pd.nsf_pad;
  double* act = D + pd.nsf_pad;
  double* der = act + AE_MAXLAYERS * AT_NSTRIDE;

  // ---- stage
  int na = 0;
  for (int c0 = 0; c0 < n; c0 += AT_THREADS) {
    const int j = c0 + tid;
    bool inA = false;
    double4_32a v;
    v.x = v.y = v.z = v.w = 0.0;
    double s = 0.0;
    if (j < n) {
      v = vin[j];
      const int t = tin[j];
      sv[j] = v;
      const double d = v.w;
      s = multi ? (double)ct.spin[t] : 0.0;
      double4_32a r;
      r.x = r.y = r.z = 0.0;
      r.w = s;
      if (d <= r_Rc && d > SFB_EPS) {
        cutoff_a(d, r_Rc, r_a, r.y, r.z);
        r.x = radial_x(d, r_Rc, two_over_rc);
      }
      sr[j] = r;
      inA = d <= a_Rc && d >= SFB_EPS;
    }
    const unsigned m = __ballot_sync(0xffffffffu, inA);
    if (lane == 0) s_wcnt[warp] = __popc(m);
    __syncthreads();
    int off = na, tot = 0;
    for (int w = 0; w < AT_WARPS; ++w) {
      if (w < warp) off += s_wcnt[w];
      tot += s_wcnt[w];
    }
    if (inA) {
      const int k = off + __popc(m & ((1u << lane) - 1u));
      const double d = v.w, invd = 1.0 / d;
      double4_32a u, f;
      u.x = v.x * invd;
      u.y = v.y * invd;
      u.z = v.z * invd;
      u.w = invd;
      cutoff_a(d, a_Rc, a_a, f.x, f.y);
      f.z = s;
      f.w = (double)j;
      au[k] = u;
      af[k] = f;
    }
    na += tot;
    __syncthreads();   // s_wcnt is rewritten by the next chunk
  }
  const int np = na * (na - 1) / 2;

  // ---- forward: per-thread sums into shared-memory columns
  double* red_r = red;                       // [2 RB][AT_RAD]
  double* red_a = red + 2 * RB * AT_RAD;     // [2 AB][AT_ANG]
  if (warp == 0) {
    double acc[RB], accs[RB];
#pragma unroll
    for (int q = 0; q < RB; ++q) acc[q] = accs[q] = 0.0;
    for (int j = lane; j < n; j += AT_RAD) {
      const double d = sv[j].w;
      if (d <= r_Rc && d > SFB_EPS) {
        const double4_32a r = sr[j];
        const double fc = r.y, x = r.x, x2 = x + x, sfc = r.w * fc;
        double tm1 = 1.0, t0 = x;
        acc[0] += fc;
        accs[0] += sfc;
#pragma unroll
        for (int q = 1; q < RB; ++q) {
          if (q < rN) {
            acc[q] = fma(fc, t0, acc[q]);
            accs[q] = fma(sfc, t0, accs[q]);
            const double tn = fma(x2, t0, -tm1);
            tm1 = t0;
            t0 = tn;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      red_r[q * AT_RAD + lane] = acc[q];
      red_r[(RB + q) * AT_RAD + lane] = accs[q];
    }
  } else {
    const int p0 = tid - AT_RAD;
    double ang[AB], angs[AB];
#pragma unroll
    for (int q = 0; q < AB; ++q) ang[q] = angs[q] = 0.0;
    if (p0 < np) {
      PairWalk pw;
      pw.start(p0, na);
      for (int p = p0; p < np; p += AT_ANG) {
        const double4_32a ua = au[pw.a], ub = au[pw.b], fa = af[pw.a], fb = af[pw.b];
        const double cosv = ua.x * ub.x + ua.y * ub.y + ua.z * ub.z;
        const double w = fa.x * fb.x;
        const double sw = fa.z * fb.z * w;
        double x, dxdc;
        angular_arg(cosv, legacy, x, dxdc);
        const double x2 = x + x;
        double tm1 = 1.0, t0 = x;
        ang[0] += w;
        angs[0] += sw;
#pragma unroll
        for (int q = 1; q < AB; ++q) {
          if (q < aN) {
            ang[q] = fma(w, t0, ang[q]);
            angs[q] = fma(sw, t0, angs[q]);
            const double tn = fma(x2, t0, -tm1);
            tm1 = t0;
            t0 = tn;
          }
        }
        pw.advance(na, AT_ANG);
      }
    }
#pragma unroll
    for (int q = 0; q < AB; ++q) {
      red_a[q * AT_ANG + p0] = ang[q];
      red_a[(AB + q) * AT_ANG + p0] = angs[q];
    }
  }
  __syncthreads();
  {
    // feature f: radial, radial x spin, angular, angular x spin
    const int nfr = multi ? 2 * rN : rN, nfa = multi ? 2 * aN : aN;
    const int ncol_r = min(n, AT_RAD), ncol_a = min(np, AT_ANG);
    const size_t nrow = (size_t)ti * pd.nsf_pad;
    for (int f0 = 0; f0 < nfr + nfa; f0 += AT_THREADS / AT_LPF) {
      const int f = f0 + tid / AT_LPF, sub = tid % AT_LPF;
      double sum = 0.0;
      int gk = -1;
      if (f < nfr) {
        const int q = f < rN ? f : f - rN;
        const double* col = red_r + (f < rN ? q : RB + q) * AT_RAD;
        for (int c = sub; c < ncol_r; c += AT_LPF) sum += col[c];
        gk = (f < rN ? ct.r_i1 : ct.r_i2) + q;
      } else if (f < nfr + nfa) {
        const int fa = f - nfr;
        const int q = fa < aN ? fa : fa - aN;
        const double* col = red_a + (fa < aN ? q : AB + q) * AT_ANG;
        for (int c = sub; c < ncol_a; c += AT_LPF) sum += col[c];
        gk = (fa < aN ? ct.a_i1 : ct.a_i2) + q;
      }
      sum += __shfl_xor_sync(0xffffffffu, sum, 2);
      sum += __shfl_xor_sync(0xffffffffu, sum, 1);
      if (gk >= 0 && sub == 0) G[gk] = (sum - pd.shift[nrow + gk]) * pd.scale[nrow + gk];
    }
  }
  __syncthreads();

  // ---- network: energy and dE/dG
  const NetTable& net = sp.net;
  const int L = net.nlayers;
  const double* __restrict__ W = pd.w64;
  for (int l = 0; l < L - 1; ++l) {
    const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
    const double* Wl = W + net.w_off[l];
    const int pitch = net.pitch[l];
    const double* hin = (l == 0) ? G : act + l * AT_NSTRIDE;
    double* hout = act + (l + 1) * AT_NSTRIDE;
    double* dout = der + (l + 1) * AT_NSTRIDE;
    const int fa = net.f_a[l + 1];
    for (int ob = 0; ob < nout; ob += AT_THREADS / AT_LPN) {
      const int o = ob + tid / AT_LPN, sub = tid % AT_LPN;
      double part = 0.0;
      if (o < nout) {
        const double* row = Wl + (size_t)o * pitch;
        for (int k = sub; k < nin; k += AT_LPN) part = fma(row[k], hin[k], part);
      }
      part += __shfl_xor_sync(0xffffffffu, part, 4);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      if (o < nout && sub == 0) {
        double y, dy;
        activate<double>(fa, part + Wl[(size_t)o * pitch + nin], y, dy);
        hout[o] = y;
        dout[o] = dy;
      }
    }
    __syncthreads();
  }
  const double y = act[(L - 1) * AT_NSTRIDE];
  // back: delta_l = (W_l^T delta_{l+1}) f'_l, from the output node down
  const double* delta = der + (L - 1) * AT_NSTRIDE;
  for (int l = L - 2; l >= 0; --l) {
    const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
    const double* Wl = W + net.w_off[l];
    const int pitch = net.pitch[l];
    double* dl = (l == 0) ? D : der + l * AT_NSTRIDE;
    for (int kb = 0; kb < nin; kb += AT_THREADS / AT_LPN) {
      const int k = kb + tid / AT_LPN, sub = tid % AT_LPN;
      double part = 0.0;
      if (k < nin)
        for (int o = sub; o < nout; o += AT_LPN) part = fma(Wl[(size_t)o * pitch + k], delta[o], part);
      part += __shfl_xor_sync(0xffffffffu, part, 4);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      if (k < nin && sub == 0) dl[k] = (l > 0) ? part * dl[k] : part;
    }
    __syncthreads();
    delta = dl;
  }
  // dE/dG of the raw descriptor: times E_scale and the normalisation scale
  {
    const size_t nrow = (size_t)ti * pd.nsf_pad;
    for (int k = tid; k < sp.nsf; k += AT_THREADS) D[k] = sp.E_scale * D[k] * pd.scale[nrow + k];
  }
  double* Eo = reinterpret_cast<double*>(out);
  if (tid == 0) {
    Eo[0] = sp.E_scale * y + sp.E_shift + sp.E_atom;
    *reinterpret_cast<unsigned*>(out + 8) = 0u;
  }
  if (!hd.forces) return;
  __syncthreads();

  // ---- adjoint, radial: the force on each neighbour, -c R_ij / d
  {
    double gr[RB], grs[RB];
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      gr[q] = q < rN ? D[ct.r_i1 + q] : 0.0;
      grs[q] = (multi && q < rN) ? D[ct.r_i2 + q] : 0.0;
    }
    for (int j = tid; j < n; j += AT_THREADS) {
      const double4_32a v = sv[j];
      const double d = v.w;
      double c = 0.0;
      if (d <= r_Rc && d > SFB_EPS) {
        const double4_32a r = sr[j];
        const double fc = r.y, dfc = r.z, s = r.w, x = r.x, x2 = x + x;
        double tm1 = 1.0, t0 = x, um1 = 1.0, u0 = x2;
        c = (gr[0] + s * grs[0]) * dfc;
#pragma unroll
        for (int q = 1; q < RB; ++q) {
          if (q < rN) {
            const double gq = gr[q] + s * grs[q];
            const double dT = (double)q * um1 * two_over_rc;
            c = fma(gq, fma(dfc, t0, fc * dT), c);
            const double tn = fma(x2, t0, -tm1);
            tm1 = t0;
            t0 = tn;
            const double un = fma(x2, u0, -um1);
            um1 = u0;
            u0 = un;
          }
        }
      }
      const double inv = (d > SFB_EPS && d < 1e29) ? c / d : 0.0;
      sF[3 * j] = -(inv * v.x);
      sF[3 * j + 1] = -(inv * v.y);
      sF[3 * j + 2] = -(inv * v.z);
    }
    for (int a = tid; a < na; a += AT_THREADS) aF[3 * a] = aF[3 * a + 1] = aF[3 * a + 2] = 0.0;
  }

  // ---- adjoint, angular: rounds of AT_THREADS pairs, gradients of both
  // partners into a pair buffer, then gathered per angular neighbour
  {
    double gav[AB], gasv[AB];
#pragma unroll
    for (int q = 0; q < AB; ++q) {
      gav[q] = q < aN ? D[ct.a_i1 + q] : 0.0;
      gasv[q] = (multi && q < aN) ? D[ct.a_i2 + q] : 0.0;
    }
    double* pbuf = red;   // [AT_THREADS][6]: gradient on a, on k
    PairWalk pw;
    if (tid < np) pw.start(tid, na);
    for (int P0 = 0; P0 < np; P0 += AT_THREADS) {
      __syncthreads();   // the previous round's gather is done with pbuf
      const int p = P0 + tid;
      double g6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      if (p < np) {
        const double4_32a ua = au[pw.a], uk = au[pw.b], fa = af[pw.a], fk = af[pw.b];
        const double cosv = ua.x * uk.x + ua.y * uk.y + ua.z * uk.z;
        const double w = fa.x * fk.x;
        const double ss = fa.z * fk.z;
        double x, dxdc;
        angular_arg(cosv, legacy, x, dxdc);
        const double x2 = x + x;
        double tm1 = 1.0, t0 = x, um1 = 1.0, u0 = x2;
        double Av = fma(ss, gasv[0], gav[0]), Bv = 0.0;
#pragma unroll
        for (int q = 1; q < AB; ++q) {
          if (q < aN) {
            const double cq = fma(ss, gasv[q], gav[q]);
            Av = fma(cq, t0, Av);
            Bv = fma(cq * (double)q, um1, Bv);
            const double tn = fma(x2, t0, -tm1);
            tm1 = t0;
            t0 = tn;
            const double un = fma(x2, u0, -um1);
            um1 = u0;
            u0 = un;
          }
        }
        const double inva = ua.w, invk = uk.w;
        const double Bc = w * Bv * dxdc;
        const double dEda = fa.y * fk.x * Av, ca = Bc * inva;
        const double dEdk = fa.x * fk.y * Av, ck = Bc * invk;
        g6[0] = dEda * ua.x + ca * (uk.x - cosv * ua.x);
        g6[1] = dEda * ua.y + ca * (uk.y - cosv * ua.y);
        g6[2] = dEda * ua.z + ca * (uk.z - cosv * ua.z);
        g6[3] = dEdk * uk.x + ck * (ua.x - cosv * uk.x);
        g6[4] = dEdk * uk.y + ck * (ua.y - cosv * uk.y);
        g6[5] = dEdk * uk.z + ck * (ua.z - cosv * uk.z);
        pw.advance(na, AT_THREADS);
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) pbuf[6 * tid + c] = g6[c];
      __syncthreads();
      const int P1 = min(np, P0 + AT_THREADS);
      for (int a = tid; a < na; a += AT_THREADS) {
        double gx = aF[3 * a], gy = aF[3 * a + 1], gz = aF[3 * a + 2];
        // pairs (c, a), c < a: the gradient on their second partner
        for (int c = 0; c < a; ++c) {
          const int q = tri_index(c, a, na);
          if (q >= P0 && q < P1) {
            const double* e = pbuf + 6 * (q - P0) + 3;
            gx += e[0];
            gy += e[1];
            gz += e[2];
          }
        }
        // pairs (a, b), b > a: consecutive indices, the first partner's
        const int qa = tri_index(a, a + 1, na);
        const int lo = max(qa, P0), hi = min(qa + (na - 1 - a), P1);
        for (int q = lo; q < hi; ++q) {
          const double* e = pbuf + 6 * (q - P0);
          gx += e[0];
          gy += e[1];
          gz += e[2];
        }
        aF[3 * a] = gx;
        aF[3 * a + 1] = gy;
        aF[3 * a + 2] = gz;
      }
    }
  }
  __syncthreads();
  for (int a = tid; a < na; a += AT_THREADS) {
    const int slot = (int)af[a].w;
    sF[3 * slot] -= aF[3 * a];
    sF[3 * slot + 1] -= aF[3 * a + 1];
    sF[3 * slot + 2] -= aF[3 * a + 2];
  }
  __syncthreads();

  // ---- outputs: row 0 the central atom (minus the neighbours' sum), then
  // the neighbours in list order
  double* Fo = reinterpret_cast<double*>(out + AE_ATOM_OUT_F);
  if (warp < 3) {
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += sF[3 * j + warp];
#pragma unroll
    for (int dd = 16; dd > 0; dd >>= 1) s += __shfl_xor_sync(0xffffffffu, s, dd);
    if (lane == 0) Fo[warp] = -s;
  }
  for (int q = tid; q < 3 * n; q += AT_THREADS) Fo[3 + q] = sF[q];
}

template <int RB, int AB>
int launch_atom(const PotDevice& pd, int n, const void* in, void* out, cudaStream_t s) {
  const size_t smem = at_smem_bytes<RB, AB>(n, pd.nsf_pad);
  if (smem > 200 * 1024) return AE_ATOM_NA;
  auto kern = k_atom<RB, AB>;
  // the opt-in limit is raised once, to the largest row's size (callers
  // hold the library lock)
  static size_t opted = 48 * 1024 - AE_STATIC_SMEM;
  if (smem > opted) {
    const cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return (int)e;
    opted = 200 * 1024;
  }
  kern<<<1, AT_THREADS, smem, s>>>(pd, static_cast<const unsigned char*>(in),
                                   static_cast<unsigned char*>(out));
  return (int)cudaGetLastError();
}

}  // namespace

int ae_launch_atom(const PotDevice& pd, int n, const void* in, void* out, cudaStream_t s) {
  if (n < 0 || n > AE_ATOM_NMAX) return AE_ATOM_NA;
  int rN = 0, aN = 0;
  for (int t = 0; t < pd.ntypes; ++t) {
    if (pd.sp[t].sftype != AE_SF_CHEBYSHEV) return AE_ATOM_NA;
    rN = max(rN, pd.sp[t].cheb.r_N);
    aN = max(aN, pd.sp[t].cheb.a_N);
    for (int l = 1; l < pd.sp[t].net.nlayers; ++l)
      if (pd.sp[t].net.nnodes[l] > AE_MAXNODES) return AE_ATOM_NA;
  }
  if (rN <= 17 && aN <= 9) return launch_atom<17, 9>(pd, n, in, out, s);
  if (rN <= 24 && aN <= 16) return launch_atom<24, 16>(pd, n, in, out, s);
  return AE_ATOM_NA;
}
