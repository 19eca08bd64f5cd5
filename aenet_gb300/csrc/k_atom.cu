// One atom per call for FP64 Chebyshev potentials: the libaenet per-atom
// entry points (aenet_atomic_energy / aenet_atomic_energy_and_forces,
// src/aenet.f90:359-486) evaluate one central atom with the caller's
// neighbour list.  A warp per atom leaves an SM's FP64 pipe waiting on the
// dependent chains of one lane group, so the whole call is one launch of
// either one block of AT_THREADS threads (k_atom) or a cluster of AC_CTAS
// such blocks on as many SMs (k_atom_cluster), phase after phase:
//
//   stage    thread per neighbour: radial argument and cut-off, angular
//            cut-off and unit vector (the per-neighbour values of sfb_eval,
//            src/ext/sfbasis.f90:488-512); angular neighbours compacted in
//            list order;
//   forward  warps 0-2 over the neighbours (radial T_n, chebyshev.f90:41-128),
//            the other warps over the pairs j < k of angular neighbours;
//            the per-thread sums are reduced column by column through
//            shared memory, four lanes per feature;
//   network  eight lanes per node for the sums, one lane per node for the
//            activations, forward and back (ff_eval / ff_deriv,
//            src/ext/feedforward.f90:586-757);
//   adjoint  thread per neighbour (radial, warps 0-2) and per pair
//            (angular, warps 3-7, at the same time); the
//            pair gradients of each round are gathered per neighbour in a
//            fixed order; the central atom takes minus the sum of the
//            neighbour forces (aenet.f90:471-477).
//
// In the cluster each block stages a contiguous slice of the rows and takes
// a contiguous slice of the pair index space; the blocks exchange their
// angular records, their partial descriptor sums and their partial pair
// gradients through distributed shared memory between cluster barriers,
// and every block runs the (small) network itself.  Every sum runs in a
// fixed order, so repeated calls give identical bits.  The call's row is
// read from, and its outputs written to, mapped pinned host memory (the
// row length, species and forces flag come as launch arguments): a call is
// one launch and one stream synchronisation.
#include <cooperative_groups.h>

#include "common.h"
#include "activate.cuh"
#include "k_cheb_impl.cuh"

namespace cg = cooperative_groups;

namespace {

using cheb::angular_arg;
using cheb::cutoff_a;
using cheb::PairWalk;
using cheb::radial_x;
using cheb::SFB_EPS;
using cheb::SFB_PI;

constexpr int AT_THREADS = 256;
constexpr int AT_WARPS = AT_THREADS / 32;
// FP64 runs at 2 lanes per clock per SM, so every phase spreads its FP64
// work over as many warps as it can: radial terms on warps 0-2, pairs on
// warps 3-7 (forward and adjoint at the same time), radial and angular
// cut-offs of a row on two threads, activations on one warp
constexpr int AT_RAD = 96;                    // radial threads (warps 0-2)
constexpr int AT_ANG = AT_THREADS - AT_RAD;   // pair threads (warps 3-7)
constexpr int AT_HALF = AT_THREADS / 2;       // rows per staging pass
constexpr int AT_LPN = 8;                     // lanes per network node
constexpr int AT_LPF = 4;                     // lanes per feature sum
constexpr int AT_NSTRIDE = AE_MAXNODES + 1;
constexpr int AC_CTAS = 8;                    // blocks of the cluster form
constexpr int AT_WMAX = 4096;                 // network weights staged in shared memory
                                              // (doubles; larger networks read L2)

template <int RB, int AB>
__host__ __device__ constexpr size_t at_red_elems() {
  return (2 * RB * AT_RAD + 2 * AB * AT_ANG) > 6 * AT_THREADS ? (2 * RB * AT_RAD + 2 * AB * AT_ANG)
                                                              : 6 * AT_THREADS;
}

// shared memory of a call with n neighbours: rows (sv, sr), angular list
// (au, af), in the cluster form also the block's own angular records and
// the row -> angular index map; forces, angular gradients, reduction and
// network scratch
template <int RB, int AB>
__host__ __device__ size_t at_smem_bytes(int n, int nsf_pad, bool cluster, int wcount) {
  return (cluster ? 6 : 4) * sizeof(double4_32a) * (size_t)n + 6 * sizeof(double) * (size_t)n +
         (cluster ? 4 * (size_t)n : 0) +
         sizeof(double) * (at_red_elems<RB, AB>() + 3 * (size_t)nsf_pad +
                           2 * (size_t)AE_MAXLAYERS * AT_NSTRIDE + 4 + (size_t)wcount) +
         64;
}

// first and one-past-last weight of species t's network in the weight array
__host__ __device__ inline void net_range(const NetTable& net, int& w0, int& w1) {
  const int L = net.nlayers;
  w0 = net.w_off[0];
  w1 = net.w_off[L - 2] + net.pitch[L - 2] * net.nnodes[L - 1];
}

__device__ __forceinline__ int tri_index(int a, int b, int na) {
  // row-major index of pair (a, b), a < b, in the upper triangle
  return a * (2 * na - a - 1) / 2 + (b - a - 1);
}

// per-call constants of the central atom's basis
struct AtomCtx {
  double r_Rc, a_Rc, two_over_rc, r_a, a_a;
  int rN, aN, legacy;
  bool multi;
  __device__ void init(const ChebTable& ct) {
    r_Rc = ct.r_Rc;
    a_Rc = ct.a_Rc;
    two_over_rc = 2.0 / r_Rc;
    r_a = SFB_PI / r_Rc;
    a_a = SFB_PI / a_Rc;
    rN = ct.r_N;
    aN = ct.a_N;
    legacy = ct.angular_legacy;
    multi = ct.multi;
  }
};

// Rows [j0, j1) of the call: sv/sr at j - j0, the angular ones compacted in
// row order into au/af (slot = the row's index j), amap[j - j0] = the
// compacted index or -1 (when amap is given).  AT_HALF rows per pass: the
// first half of the block computes their radial records, the second half
// their angular ones.  Block-wide; returns the number of angular rows.
__device__ int stage_rows(const AtomCtx& c, const ChebTable& ct, const double4_32a* vin,
                          const int* tin, int j0, int j1, double4_32a* sv, double4_32a* sr,
                          double4_32a* au, double4_32a* af, int* amap, int* s_wcnt) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool ang_half = tid >= AT_HALF;
  const int h = ang_half ? tid - AT_HALF : tid;
  int na = 0;
  for (int c0 = j0; c0 < j1; c0 += AT_HALF) {
    const int j = c0 + h;
    bool inA = false;
    double4_32a v;
    v.x = v.y = v.z = v.w = 0.0;
    double s = 0.0;
    if (j < j1) {
      v = vin[j];
      const int t = tin[j];
      s = c.multi ? (double)ct.spin[t] : 0.0;
      const double d = v.w;
      if (!ang_half) {
        sv[j - j0] = v;
        double4_32a r;
        r.x = r.y = r.z = 0.0;
        r.w = s;
        if (d <= c.r_Rc && d > SFB_EPS) {
          cutoff_a(d, c.r_Rc, c.r_a, r.y, r.z);
          r.x = radial_x(d, c.r_Rc, c.two_over_rc);
        }
        sr[j - j0] = r;
      } else {
        inA = d <= c.a_Rc && d >= SFB_EPS;
      }
    }
    // compaction over the angular half's warps
    const unsigned m = __ballot_sync(0xffffffffu, inA);
    if (ang_half && lane == 0) s_wcnt[warp - AT_HALF / 32] = __popc(m);
    __syncthreads();
    int off = na, tot = 0;
    for (int w = 0; w < AT_HALF / 32; ++w) {
      if (w < warp - AT_HALF / 32) off += s_wcnt[w];
      tot += s_wcnt[w];
    }
    const int k = off + __popc(m & ((1u << lane) - 1u));
    if (inA) {
      const double d = v.w, invd = 1.0 / d;
      double4_32a u, f;
      u.x = v.x * invd;
      u.y = v.y * invd;
      u.z = v.z * invd;
      u.w = invd;
      cutoff_a(d, c.a_Rc, c.a_a, f.x, f.y);
      f.z = s;
      f.w = (double)j;
      au[k] = u;
      af[k] = f;
    }
    if (ang_half && amap && j < j1) amap[j - j0] = inA ? k : -1;
    na += tot;
    __syncthreads();   // s_wcnt is rewritten by the next pass
  }
  return na;
}

// Raw descriptor sums of rows [0, nl) of sv/sr (radial, warp 0) and of the
// pairs [p_lo, p_hi) of the angular list (warps 1 ..), written to
// fsum[feature index].  Block-wide.
template <int RB, int AB>
__device__ void forward_sums(const AtomCtx& c, const ChebTable& ct, const double4_32a* sv,
                             const double4_32a* sr, int nl, const double4_32a* au,
                             const double4_32a* af, int na, int p_lo, int p_hi, double* red,
                             double* fsum) {
  const int tid = threadIdx.x;
  double* red_r = red;                       // [2 RB][AT_RAD]
  double* red_a = red + 2 * RB * AT_RAD;     // [2 AB][AT_ANG]
  const int rN = c.rN, aN = c.aN;
  if (tid < AT_RAD) {
    double acc[RB], accs[RB];
#pragma unroll
    for (int q = 0; q < RB; ++q) acc[q] = accs[q] = 0.0;
    for (int j = tid; j < nl; j += AT_RAD) {
      const double d = sv[j].w;
      if (d <= c.r_Rc && d > SFB_EPS) {
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
      red_r[q * AT_RAD + tid] = acc[q];
      red_r[(RB + q) * AT_RAD + tid] = accs[q];
    }
  } else {
    const int p0 = tid - AT_RAD;
    double ang[AB], angs[AB];
#pragma unroll
    for (int q = 0; q < AB; ++q) ang[q] = angs[q] = 0.0;
    if (p_lo + p0 < p_hi) {
      PairWalk pw;
      pw.start(p_lo + p0, na);
      for (int p = p_lo + p0; p < p_hi; p += AT_ANG) {
        const double4_32a ua = au[pw.a], ub = au[pw.b], fa = af[pw.a], fb = af[pw.b];
        const double cosv = ua.x * ub.x + ua.y * ub.y + ua.z * ub.z;
        const double w = fa.x * fb.x;
        const double sw = fa.z * fb.z * w;
        double x, dxdc;
        angular_arg(cosv, c.legacy, x, dxdc);
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
  // feature f: radial, radial x spin, angular, angular x spin
  const int nfr = c.multi ? 2 * rN : rN, nfa = c.multi ? 2 * aN : aN;
  const int ncol_r = min(nl, AT_RAD), ncol_a = max(0, min(p_hi - p_lo, AT_ANG));
  for (int f0 = 0; f0 < nfr + nfa; f0 += AT_THREADS / AT_LPF) {
    const int f = f0 + tid / AT_LPF, sub = tid % AT_LPF;
    double sum = 0.0;
    int gk = -1;
    if (f < nfr) {
      const int q = f < rN ? f : f - rN;
      const double* col = red_r + (f < rN ? q : RB + q) * AT_RAD;
      for (int k = sub; k < ncol_r; k += AT_LPF) sum += col[k];
      gk = (f < rN ? ct.r_i1 : ct.r_i2) + q;
    } else if (f < nfr + nfa) {
      const int fa = f - nfr;
      const int q = fa < aN ? fa : fa - aN;
      const double* col = red_a + (fa < aN ? q : AB + q) * AT_ANG;
      for (int k = sub; k < ncol_a; k += AT_LPF) sum += col[k];
      gk = (fa < aN ? ct.a_i1 : ct.a_i2) + q;
    }
    sum += __shfl_xor_sync(0xffffffffu, sum, 2);
    sum += __shfl_xor_sync(0xffffffffu, sum, 1);
    if (gk >= 0 && sub == 0) fsum[gk] = sum;
  }
  __syncthreads();
}

// Network of species ti on the normalised descriptor G: returns the output
// node y and leaves dE/dG of the raw descriptor (times E_scale and the
// normalisation scale) in D.  Block-wide.
__device__ double atom_network(const PotDevice& pd, const SpeciesTable& sp, int ti,
                               const double* G, double* D, double* act, double* der,
                               const double* wsm) {
  const int tid = threadIdx.x;
  const NetTable& net = sp.net;
  const int L = net.nlayers;
  // the species' weights: staged in shared memory (wsm, from its first
  // weight on) or read from the global table
  int w0, w1;
  net_range(net, w0, w1);
  auto layer = [&](int l) { return wsm ? wsm + (net.w_off[l] - w0) : pd.w64 + net.w_off[l]; };
  for (int l = 0; l < L - 1; ++l) {
    const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
    const double* Wl = layer(l);
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
      if (o < nout && sub == 0) hout[o] = part + Wl[(size_t)o * pitch + nin];
    }
    __syncthreads();
    // the activations on the first warp(s), one node per lane
    for (int o = tid; o < nout; o += AT_THREADS) {
      double y, dy;
      activate<double>(fa, hout[o], y, dy);
      hout[o] = y;
      dout[o] = dy;
    }
    __syncthreads();
  }
  const double y = act[(L - 1) * AT_NSTRIDE];
  // back: delta_l = (W_l^T delta_{l+1}) f'_l, from the output node down
  const double* delta = der + (L - 1) * AT_NSTRIDE;
  for (int l = L - 2; l >= 0; --l) {
    const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
    const double* Wl = layer(l);
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
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  for (int k = tid; k < sp.nsf; k += AT_THREADS) D[k] = sp.E_scale * D[k] * pd.scale[nrow + k];
  __syncthreads();
  return y;
}

// The adjoint: radial part of the force on rows [0, nl) (-c R_ij / d into
// sF) on warps 0-2 while warps 3-7 take the gradients of the pairs
// [p_lo, p_hi) on both partners, in rounds of AT_ANG pairs through pbuf,
// gathered per angular neighbour in a fixed order into aF[3 a] (zeroed
// here).  Block-wide.
template <int RB, int AB>
__device__ void adjoint_rows_pairs(const AtomCtx& c, const ChebTable& ct, const double* D,
                                   const double4_32a* sv, const double4_32a* sr, int nl,
                                   double* sF, const double4_32a* au, const double4_32a* af,
                                   int na, int p_lo, int p_hi, double* pbuf, double* aF) {
  const int tid = threadIdx.x, rN = c.rN, aN = c.aN;
  for (int a = tid; a < na; a += AT_THREADS) aF[3 * a] = aF[3 * a + 1] = aF[3 * a + 2] = 0.0;
  __syncthreads();
  if (tid < AT_RAD) {
    double gr[RB], grs[RB];
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      gr[q] = q < rN ? D[ct.r_i1 + q] : 0.0;
      grs[q] = (c.multi && q < rN) ? D[ct.r_i2 + q] : 0.0;
    }
    for (int j = tid; j < nl; j += AT_RAD) {
      const double4_32a v = sv[j];
      const double d = v.w;
      double cc = 0.0;
      if (d <= c.r_Rc && d > SFB_EPS) {
        const double4_32a r = sr[j];
        const double fc = r.y, dfc = r.z, s = r.w, x = r.x, x2 = x + x;
        double tm1 = 1.0, t0 = x, um1 = 1.0, u0 = x2;
        cc = (gr[0] + s * grs[0]) * dfc;
#pragma unroll
        for (int q = 1; q < RB; ++q) {
          if (q < rN) {
            const double gq = gr[q] + s * grs[q];
            const double dT = (double)q * um1 * c.two_over_rc;
            cc = fma(gq, fma(dfc, t0, fc * dT), cc);
            const double tn = fma(x2, t0, -tm1);
            tm1 = t0;
            t0 = tn;
            const double un = fma(x2, u0, -um1);
            um1 = u0;
            u0 = un;
          }
        }
      }
      const double inv = (d > SFB_EPS && d < 1e29) ? cc / d : 0.0;
      sF[3 * j] = -(inv * v.x);
      sF[3 * j + 1] = -(inv * v.y);
      sF[3 * j + 2] = -(inv * v.z);
    }
  }
  const int pt = tid - AT_RAD;   // pair thread
  double gav[AB], gasv[AB];
#pragma unroll
  for (int q = 0; q < AB; ++q) {
    gav[q] = q < aN ? D[ct.a_i1 + q] : 0.0;
    gasv[q] = (c.multi && q < aN) ? D[ct.a_i2 + q] : 0.0;
  }
  PairWalk pw;
  if (pt >= 0 && p_lo + pt < p_hi) pw.start(p_lo + pt, na);
  for (int P0 = p_lo; P0 < p_hi; P0 += AT_ANG) {
    const int p = P0 + pt;
    if (pt >= 0) {
      double g6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      if (p < p_hi) {
        const double4_32a ua = au[pw.a], uk = au[pw.b], fa = af[pw.a], fk = af[pw.b];
        const double cosv = ua.x * uk.x + ua.y * uk.y + ua.z * uk.z;
        const double w = fa.x * fk.x;
        const double ss = fa.z * fk.z;
        double x, dxdc;
        angular_arg(cosv, c.legacy, x, dxdc);
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
        pw.advance(na, AT_ANG);
      }
#pragma unroll
      for (int q = 0; q < 6; ++q) pbuf[6 * pt + q] = g6[q];
    }
    __syncthreads();
    const int P1 = min(p_hi, P0 + AT_ANG);
    for (int a = tid; a < na; a += AT_THREADS) {
      double gx = aF[3 * a], gy = aF[3 * a + 1], gz = aF[3 * a + 2];
      // pairs (c, a), c < a: the gradient on their second partner
      for (int cc = 0; cc < a; ++cc) {
        const int q = tri_index(cc, a, na);
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
    __syncthreads();   // pbuf is rewritten by the next round
  }
  __syncthreads();
}

// The species' network weights into shared memory (when there is room for
// them): issued at the start of the call, so that their loads overlap the
// row reads; the block's later barriers order them before the network.
__device__ __forceinline__ void stage_weights(const NetTable& net, const double* W, double* wsm) {
  if (!wsm) return;
  int w0, w1;
  net_range(net, w0, w1);
  for (int q = threadIdx.x; q < w1 - w0; q += AT_THREADS) wsm[q] = W[w0 + q];
}

// shared-memory carve-up of a call
struct AtomSmem {
  double4_32a *sv, *sr, *au, *af, *lau, *laf;
  double *sF, *aF, *red, *fsum, *G, *D, *act, *der, *cen, *wsm;
  int* amap;
  template <int RB, int AB>
  __device__ void carve(unsigned char* base, int n, int nsf_pad, bool cluster, int wcount) {
    double4_32a* p = reinterpret_cast<double4_32a*>(base);
    sv = p;
    sr = sv + n;
    au = sr + n;
    af = au + n;
    lau = cluster ? af + n : nullptr;
    laf = cluster ? lau + n : nullptr;
    double* q = reinterpret_cast<double*>(af + (cluster ? 3 : 1) * (size_t)n);
    sF = q;
    aF = sF + 3 * (size_t)n;
    red = aF + 3 * (size_t)n;
    fsum = red + at_red_elems<RB, AB>();
    G = fsum + nsf_pad;
    D = G + nsf_pad;
    act = D + nsf_pad;
    der = act + AE_MAXLAYERS * AT_NSTRIDE;
    cen = der + AE_MAXLAYERS * AT_NSTRIDE;
    wsm = wcount > 0 ? cen + 4 : nullptr;
    amap = cluster ? reinterpret_cast<int*>(cen + 4 + wcount) : nullptr;
  }
};

template <int RB, int AB>
__global__ void __launch_bounds__(AT_THREADS, 1)
    k_atom(PotDevice pd, AtomCallHeader hd, int wcount, const unsigned char* __restrict__ in,
           unsigned char* __restrict__ out) {
  extern __shared__ __align__(32) unsigned char smem_raw[];
  __shared__ int s_wcnt[AT_WARPS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = hd.n, ti = hd.ti;
  const double4_32a* __restrict__ vin = reinterpret_cast<const double4_32a*>(in + AE_ATOM_IN_VEC);
  const int* __restrict__ tin =
      reinterpret_cast<const int*>(in + AE_ATOM_IN_VEC + sizeof(double4_32a) * (size_t)n);
  const SpeciesTable& sp = pd.sp[ti];
  const ChebTable& ct = sp.cheb;
  AtomCtx c;
  c.init(ct);
  AtomSmem sm{};
  sm.carve<RB, AB>(smem_raw, n, pd.nsf_pad, false, wcount);
  stage_weights(sp.net, pd.w64, sm.wsm);

  const int na = stage_rows(c, ct, vin, tin, 0, n, sm.sv, sm.sr, sm.au, sm.af, nullptr, s_wcnt);
  const int np = na * (na - 1) / 2;
  forward_sums<RB, AB>(c, ct, sm.sv, sm.sr, n, sm.au, sm.af, na, 0, np, sm.red, sm.fsum);
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  for (int k = tid; k < sp.nsf; k += AT_THREADS)
    sm.G[k] = (sm.fsum[k] - pd.shift[nrow + k]) * pd.scale[nrow + k];
  __syncthreads();
  const double y = atom_network(pd, sp, ti, sm.G, sm.D, sm.act, sm.der, sm.wsm);
  if (tid == 0) {
    *reinterpret_cast<double*>(out) = sp.E_scale * y + sp.E_shift + sp.E_atom;
    *reinterpret_cast<unsigned*>(out + 8) = 0u;
  }
  if (!hd.forces) return;

  adjoint_rows_pairs<RB, AB>(c, ct, sm.D, sm.sv, sm.sr, n, sm.sF, sm.au, sm.af, na, 0, np, sm.red,
                             sm.aF);
  for (int a = tid; a < na; a += AT_THREADS) {
    const int slot = (int)sm.af[a].w;
    sm.sF[3 * slot] -= sm.aF[3 * a];
    sm.sF[3 * slot + 1] -= sm.aF[3 * a + 1];
    sm.sF[3 * slot + 2] -= sm.aF[3 * a + 2];
  }
  __syncthreads();

  // outputs: row 0 the central atom (minus the neighbours' sum), then the
  // neighbours in list order
  double* Fo = reinterpret_cast<double*>(out + AE_ATOM_OUT_F);
  if (warp < 3) {
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += sm.sF[3 * j + warp];
#pragma unroll
    for (int dd = 16; dd > 0; dd >>= 1) s += __shfl_xor_sync(0xffffffffu, s, dd);
    if (lane == 0) Fo[warp] = -s;
  }
  for (int q = tid; q < 3 * n; q += AT_THREADS) Fo[3 + q] = sm.sF[q];
}

template <int RB, int AB>
__global__ void __cluster_dims__(AC_CTAS, 1, 1) __launch_bounds__(AT_THREADS, 1)
    k_atom_cluster(PotDevice pd, AtomCallHeader hd, int wcount,
                   const unsigned char* __restrict__ in, unsigned char* __restrict__ out) {
  extern __shared__ __align__(32) unsigned char smem_raw[];
  __shared__ int s_wcnt[AT_WARPS];
  __shared__ int s_na;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = hd.n, ti = hd.ti;
  const double4_32a* __restrict__ vin = reinterpret_cast<const double4_32a*>(in + AE_ATOM_IN_VEC);
  const int* __restrict__ tin =
      reinterpret_cast<const int*>(in + AE_ATOM_IN_VEC + sizeof(double4_32a) * (size_t)n);
  const SpeciesTable& sp = pd.sp[ti];
  const ChebTable& ct = sp.cheb;
  AtomCtx c;
  c.init(ct);
  AtomSmem sm{};
  sm.carve<RB, AB>(smem_raw, n, pd.nsf_pad, true, wcount);
  stage_weights(sp.net, pd.w64, sm.wsm);
  // this block's rows
  const int j0 = (int)((long long)n * rank / AC_CTAS);
  const int j1 = (int)((long long)n * (rank + 1) / AC_CTAS);
  const int nl = j1 - j0;

  const int nal = stage_rows(c, ct, vin, tin, j0, j1, sm.sv, sm.sr, sm.lau, sm.laf, sm.amap, s_wcnt);
  if (tid == 0) s_na = nal;
  cl.sync();
  // every block's angular records, in row order
  int na = 0, myoff = 0;
  for (int r = 0; r < AC_CTAS; ++r) {
    const int nr = *cl.map_shared_rank(&s_na, r);
    const double4_32a* ru = cl.map_shared_rank(sm.lau, r);
    const double4_32a* rf = cl.map_shared_rank(sm.laf, r);
    for (int k = tid; k < nr; k += AT_THREADS) {
      sm.au[na + k] = ru[k];
      sm.af[na + k] = rf[k];
    }
    if (r == rank) myoff = na;
    na += nr;
  }
  for (int jl = tid; jl < nl; jl += AT_THREADS)
    if (sm.amap[jl] >= 0) sm.amap[jl] += myoff;
  __syncthreads();
  const int np = na * (na - 1) / 2;
  const int p_lo = (int)((long long)np * rank / AC_CTAS);
  const int p_hi = (int)((long long)np * (rank + 1) / AC_CTAS);
  forward_sums<RB, AB>(c, ct, sm.sv, sm.sr, nl, sm.au, sm.af, na, p_lo, p_hi, sm.red, sm.fsum);
  cl.sync();
  // the descriptor: every block's partial sums, in block order
  const size_t nrow = (size_t)ti * pd.nsf_pad;
  for (int k = tid; k < sp.nsf; k += AT_THREADS) {
    double s = 0.0;
    for (int r = 0; r < AC_CTAS; ++r) s += cl.map_shared_rank(sm.fsum, r)[k];
    sm.G[k] = (s - pd.shift[nrow + k]) * pd.scale[nrow + k];
  }
  cl.sync();   // no block reads another's partial sums after this
  const double y = atom_network(pd, sp, ti, sm.G, sm.D, sm.act, sm.der, sm.wsm);
  if (rank == 0 && tid == 0) {
    *reinterpret_cast<double*>(out) = sp.E_scale * y + sp.E_shift + sp.E_atom;
    *reinterpret_cast<unsigned*>(out + 8) = 0u;
  }
  if (!hd.forces) return;

  adjoint_rows_pairs<RB, AB>(c, ct, sm.D, sm.sv, sm.sr, nl, sm.sF, sm.au, sm.af, na, p_lo, p_hi,
                             sm.red, sm.aF);
  cl.sync();
  // this block's rows: radial part minus every block's angular gradients
  double* Fo = reinterpret_cast<double*>(out + AE_ATOM_OUT_F);
  for (int jl = tid; jl < nl; jl += AT_THREADS) {
    double fx = sm.sF[3 * jl], fy = sm.sF[3 * jl + 1], fz = sm.sF[3 * jl + 2];
    const int a = sm.amap[jl];
    if (a >= 0) {
      for (int r = 0; r < AC_CTAS; ++r) {
        const double* g = cl.map_shared_rank(sm.aF, r) + 3 * a;
        fx -= g[0];
        fy -= g[1];
        fz -= g[2];
      }
    }
    sm.sF[3 * jl] = fx;
    sm.sF[3 * jl + 1] = fy;
    sm.sF[3 * jl + 2] = fz;
    Fo[3 * (1 + j0 + jl)] = fx;
    Fo[3 * (1 + j0 + jl) + 1] = fy;
    Fo[3 * (1 + j0 + jl) + 2] = fz;
  }
  __syncthreads();
  if (warp < 3) {
    double s = 0.0;
    for (int j = lane; j < nl; j += 32) s += sm.sF[3 * j + warp];
#pragma unroll
    for (int dd = 16; dd > 0; dd >>= 1) s += __shfl_xor_sync(0xffffffffu, s, dd);
    if (lane == 0) sm.cen[warp] = s;
  }
  cl.sync();
  // the central atom: minus the sum of every block's rows
  if (rank == 0 && tid < 3) {
    double s = 0.0;
    for (int r = 0; r < AC_CTAS; ++r) s += cl.map_shared_rank(sm.cen, r)[tid];
    Fo[tid] = -s;
  }
  cl.sync();   // block 0 has read the others' sums before they exit
}

template <int RB, int AB>
int launch_atom(const PotDevice& pd, const AtomCallHeader& hd, const void* in, void* out,
                bool cluster, cudaStream_t s) {
  // room for the largest species' weights, unless some network exceeds
  // AT_WMAX (then every call reads them from L2)
  int wcount = 0;
  for (int t = 0; t < pd.ntypes; ++t) {
    int w0, w1;
    net_range(pd.sp[t].net, w0, w1);
    wcount = max(wcount, w1 - w0);
  }
  if (wcount > AT_WMAX) wcount = 0;
  size_t smem = at_smem_bytes<RB, AB>(hd.n, pd.nsf_pad, cluster, wcount);
  if (smem > 200 * 1024 && wcount > 0) {
    wcount = 0;
    smem = at_smem_bytes<RB, AB>(hd.n, pd.nsf_pad, cluster, 0);
  }
  if (smem > 200 * 1024) return AE_ATOM_NA;
  const unsigned char* pin = static_cast<const unsigned char*>(in);
  unsigned char* pout = static_cast<unsigned char*>(out);
  // the opt-in limit is raised once per kernel (callers hold the library
  // lock)
  if (cluster) {
    static bool opted = false;
    if (!opted) {
      const cudaError_t e = cudaFuncSetAttribute(
          k_atom_cluster<RB, AB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      if (e != cudaSuccess) return (int)e;
      opted = true;
    }
    k_atom_cluster<RB, AB><<<AC_CTAS, AT_THREADS, smem, s>>>(pd, hd, wcount, pin, pout);
  } else {
    static bool opted = false;
    if (!opted) {
      const cudaError_t e = cudaFuncSetAttribute(
          k_atom<RB, AB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      if (e != cudaSuccess) return (int)e;
      opted = true;
    }
    k_atom<RB, AB><<<1, AT_THREADS, smem, s>>>(pd, hd, wcount, pin, pout);
  }
  return (int)cudaGetLastError();
}

}  // namespace

int ae_launch_atom(const PotDevice& pd, const AtomCallHeader& hd, const void* in, void* out,
                   int cluster, cudaStream_t s) {
  if (hd.n < 0 || hd.n > AE_ATOM_NMAX) return AE_ATOM_NA;
  int rN = 0, aN = 0;
  for (int t = 0; t < pd.ntypes; ++t) {
    if (pd.sp[t].sftype != AE_SF_CHEBYSHEV) return AE_ATOM_NA;
    rN = max(rN, pd.sp[t].cheb.r_N);
    aN = max(aN, pd.sp[t].cheb.a_N);
    for (int l = 1; l < pd.sp[t].net.nlayers; ++l)
      if (pd.sp[t].net.nnodes[l] > AE_MAXNODES) return AE_ATOM_NA;
  }
  if (rN <= 17 && aN <= 9) return launch_atom<17, 9>(pd, hd, in, out, cluster != 0, s);
  if (rN <= 24 && aN <= 16) return launch_atom<24, 16>(pd, hd, in, out, cluster != 0, s);
  return AE_ATOM_NA;
}
