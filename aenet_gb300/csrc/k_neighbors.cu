// Periodic cell-list neighbour search (replaces lcl_init / lcl_nblist /
// lcl_nbdist_cart of src/ext/lclist.f90).
//
// Neighbour set: every (atom j, lattice image T) with
//     |L(s_j + T) - L s_i|^2 <= (Rc + 1e-3)^2        (lclist.f90:572, 621-653)
// on wrapped lattice coordinates s (lclist.f90:953-987), excluding j = i at
// T = 0 and including the periodic images of the atom itself
// (lclist.f90:589-616).  The predicate is decided with the same unfused
// FP64 operations as the reference expression; an FP32 pass filters the
// candidates and hands only distances within a narrow band around the
// cut-off to the FP64 test.
//
// Kernels:
//   k_wrap_bin     one thread per atom: lattice coordinates
//                  (geometry.f90:697-712), wrap, Cartesian of the wrapped
//                  coordinates, cell, rank inside the cell (atomic count)
//   k_scan_*       exclusive prefix sum of the cell counts (CSR offsets)
//   k_scatter      atoms and their FP32 positions in cell order
//   k_neighbors    one warp per atom.  The stencil of cells around the
//                  atom's cell is walked as units (row d0, d1; image t2 along
//                  the third axis): each unit is one contiguous run of cells
//                  and therefore one contiguous range of atoms.  For
//                  orthogonal cells each row is cut to the part of the
//                  cut-off sphere it can reach from the atom.  The ranges of
//                  32 units are flattened into one candidate index space
//                  processed 32 candidates at a time; accepted neighbours are
//                  compacted with ballots into the atom's ELL row.
//   k_neighbors_struct  one block per structure for batches of small
//                  structures: wrap and bin, cell counts, scan and scatter
//                  in shared memory, then the same per-atom search (the
//                  global cell lists and the kernels above are skipped).
#include "common.h"

namespace {

constexpr double TWO_PI = 6.283185307179586;  // 2 * 3.141592653589793

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

// wrap into [0, 1) as the loops of lclist.f90:953-987 do: for |s| >= 1
// every step of the repeated +-1.0 is exact and for s in [-1, 0) both forms
// round s + 1 once, so s - floor(s) gives the same value.
__device__ __forceinline__ double wrap_coordinate(double s, unsigned* status) {
  if (!isfinite(s)) {
    atomicOr(status, AE_ST_BAD_COORD);
    return 0.0;
  }
  double f = floor(s);
  double w = da(s, -f);
  if (w >= 1.0) w = da(w, -1.0);
  if (w < 0.0) w = da(w, 1.0);
  return w;
}

// Lattice coordinates of atom i (geometry.f90:697-712), wrapped, the
// Cartesian position of the wrapped coordinates and the atom's cell: the
// per-atom arrays s_wrap, r_wrap, r_f32 (species in w) and cell_of are
// written (and the checked 0-based species when nb.types0_out is set);
// returns the cell's index inside its structure.
__device__ __forceinline__ int wrap_bin_atom(int i, const StructGeom* g, const double* __restrict__ pos,
                                             const int* __restrict__ types, const NbBuffers& nb) {
  double r[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
  double s[3], rw[3];
  const int nc[3] = {g->nc[0], g->nc[1], g->nc[2]};
  if (g->pbc) {
    for (int v = 0; v < 3; ++v) {
      double t;
      if (g->frac_mode == 2) {
        t = r[v];
      } else {
        // (B r) summed in column order (geometry.f90:708)
        t = dm(g->B[3 * v], r[0]);
        t = da(t, dm(g->B[3 * v + 1], r[1]));
        t = da(t, dm(g->B[3 * v + 2], r[2]));
        if (g->frac_mode == 0) t = __ddiv_rn(t, TWO_PI);
      }
      s[v] = wrap_coordinate(t, nb.status);
    }
    for (int c = 0; c < 3; ++c) {
      double t = dm(g->L[c], s[0]);
      t = da(t, dm(g->L[3 + c], s[1]));
      t = da(t, dm(g->L[6 + c], s[2]));
      rw[c] = t;
    }
  } else {
    for (int v = 0; v < 3; ++v) {
      if (!isfinite(r[v])) {
        atomicOr(nb.status, AE_ST_BAD_COORD);
        r[v] = g->origin[v];
      }
      s[v] = (r[v] - g->origin[v]) / g->box[v];
      rw[v] = r[v];
    }
  }
  int cc[3];
  for (int v = 0; v < 3; ++v) {
    double x = floor(s[v] * (double)nc[v]);
    cc[v] = x < 0.0 ? 0 : (x >= (double)(nc[v] - 1) ? nc[v] - 1 : (int)x);
  }
  int t = types[i];
  if (nb.types0_out) {
    // the caller's 1-based type id, checked and stored 0-based
    t -= 1;
    if (t < 0 || t >= nb.ntypes) {
      atomicOr(nb.status, AE_ST_BAD_TYPE);
      t = 0;
    }
    nb.types0_out[i] = t;
  }
  for (int v = 0; v < 3; ++v) {
    nb.s_wrap[3 * i + v] = s[v];
    nb.r_wrap[3 * i + v] = rw[v];
  }
  nb.r_f32[i] = make_float4((float)rw[0], (float)rw[1], (float)rw[2], __int_as_float(t));
  nb.cell_of[i] = cc[0] | (cc[1] << 10) | (cc[2] << 20);
  return (cc[0] * nc[1] + cc[1]) * nc[2] + cc[2];
}

// one thread per atom; the rank inside the cell from an atomic count
__global__ void k_wrap_bin(int natoms, const double* __restrict__ pos,
                           const int* __restrict__ types, NbBuffers nb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  const StructGeom* g = nb.geom + nb.atom_struct[i];
  const int lin = wrap_bin_atom(i, g, pos, types, nb);
  nb.slot_of[i] = atomicAdd(&nb.cell_count[g->cell_off + lin], 1);
}

// ---- exclusive scan of the cell counts (three phases, 1024 per block)
constexpr int SCAN_B = 1024;

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int u = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += u;
  }
  return v;
}

// block-wide exclusive scan of one value per thread (blockDim.x == 1024)
__device__ __forceinline__ int block_excl_scan(int v, int* warp_tot, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = warp_incl_scan(v, lane);
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int wv = warp_tot[lane];
    int wi = warp_incl_scan(wv, lane);
    warp_tot[lane] = wi - wv;
    if (lane == 31) warp_tot[32] = wi;
  }
  __syncthreads();
  total = warp_tot[32];
  int r = warp_tot[warp] + incl - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(SCAN_B) k_scan_blocks(int n, const int* __restrict__ in,
                                                       int* __restrict__ out,
                                                       int* __restrict__ bsum) {
  __shared__ int wt[33];
  const int e = blockIdx.x * SCAN_B + threadIdx.x;
  const int v = e < n ? in[e] : 0;
  int total;
  const int ex = block_excl_scan(v, wt, total);
  if (e < n) out[e] = ex;
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_B) k_scan_sums(int nb, int* __restrict__ bsum,
                                                     int* __restrict__ out_total) {
  __shared__ int wt[33];
  int carry = 0;
  for (int base = 0; base < nb; base += SCAN_B) {
    const int e = base + threadIdx.x;
    const int v = e < nb ? bsum[e] : 0;
    int total;
    const int ex = block_excl_scan(v, wt, total);
    if (e < nb) bsum[e] = ex + carry;
    carry += total;
  }
  if (threadIdx.x == 0) *out_total = carry;
}

__global__ void k_scan_add(int n, int* __restrict__ out, const int* __restrict__ bsum) {
  const int e = blockIdx.x * SCAN_B + threadIdx.x;
  if (e < n) out[e] += bsum[blockIdx.x];
}

__global__ void k_scatter(int natoms, NbBuffers nb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  const StructGeom* g = nb.geom + nb.atom_struct[i];
  const int packed = nb.cell_of[i];
  const int c0 = packed & 1023, c1 = (packed >> 10) & 1023, c2 = (packed >> 20) & 1023;
  const int lin = (c0 * g->nc[1] + c1) * g->nc[2] + c2;
  const int p = nb.cell_start[g->cell_off + lin] + nb.slot_of[i];
  nb.cell_atoms[p] = i;
  nb.cell_pos[p] = nb.r_f32[i];
}

__device__ __forceinline__ int sext10i(int v) { return (v ^ 512) - 512; }

// floor(a / n) for |a| < 2^20 with a reciprocal: (a + 1/2) / n is at least
// 1/(2n) away from an integer, far more than the error of the product (the
// reciprocal itself may be the ~2 ulp hardware approximation)
__device__ __forceinline__ int floor_div_r(int a, float inv_n) {
  return (int)floorf(((float)a + 0.5f) * inv_n);
}

// |R| of an accepted FP32 pair from the squared length (one reciprocal
// square root; zero length stays zero)
__device__ __forceinline__ float pair_length(float dd2) {
  return dd2 > 0.f ? dd2 * rsqrtf(dd2) : 0.f;
}

template <typename T4>
struct VecOut;
template <>
struct VecOut<float4> {
  static constexpr bool fp64 = false;
};
template <>
struct VecOut<double4_32a> {
  static constexpr bool fp64 = true;
};

// The reference's FP64 predicate |L (s_j + T) - L s_i|^2 <= (Rc + 1e-3)^2,
// unfused as lclist.f90 evaluates it, for FP32 distances too close to the
// cut-off to decide (out of line: rarely taken, so the search loop keeps
// its registers).
__device__ __noinline__ bool band_fp64(const NbBuffers& nb, const StructGeom* g, int pbc,
                                       bool self_img, int img, int i, int j, double rc2) {
  const int oT0 = sext10i(img & 1023), oT1 = sext10i((img >> 10) & 1023),
            oT2 = sext10i((img >> 20) & 1023);
  double e2;
  if (pbc) {
    double cart[3];
    if (self_img) {
      for (int c = 0; c < 3; ++c) {
        double t = dm(g->L[c], (double)oT0);
        t = da(t, dm(g->L[3 + c], (double)oT1));
        t = da(t, dm(g->L[6 + c], (double)oT2));
        cart[c] = t;
      }
    } else {
      const double* sj = nb.s_wrap + 3 * j;
      double u0 = da(sj[0], (double)oT0), u1 = da(sj[1], (double)oT1),
             u2 = da(sj[2], (double)oT2);
      for (int c = 0; c < 3; ++c) {
        double t = dm(g->L[c], u0);
        t = da(t, dm(g->L[3 + c], u1));
        t = da(t, dm(g->L[6 + c], u2));
        cart[c] = da(t, -nb.r_wrap[3 * i + c]);
      }
    }
    e2 = da(da(dm(cart[0], cart[0]), dm(cart[1], cart[1])), dm(cart[2], cart[2]));
  } else {
    double c0d = da(nb.r_wrap[3 * j], -nb.r_wrap[3 * i]);
    double c1d = da(nb.r_wrap[3 * j + 1], -nb.r_wrap[3 * i + 1]);
    double c2d = da(nb.r_wrap[3 * j + 2], -nb.r_wrap[3 * i + 2]);
    e2 = da(da(dm(c0d, c0d), dm(c1d, c1d)), dm(c2d, c2d));
  }
  return e2 <= rc2;
}

// stencil units per lane in one round of the search (a round holds
// 32 NB_UPL units; the stencils of the batch workloads need at most 125)
constexpr int NB_UPL = 1;
#ifndef NB_STRUCT_BLOCKS
#define NB_STRUCT_BLOCKS 4
#endif
// the half-stencil variant runs faster with three blocks per SM (its
// registers then hold the search state without spilling)
#ifndef NB_STRUCT_HALF_BLOCKS
#define NB_STRUCT_HALF_BLOCKS 3
#endif

// Where a search reads the cell lists: the global arrays, or one
// structure's copy in shared memory (cell-ordered entries p at p - base).
struct CellSrc {
  const int* cstart;     // cell_start of the structure's cells
  const float4* cpos;    // cell-ordered positions (species bits in w)
  const int* catoms;     // cell-ordered atom indices
  int base;
};

// The neighbour row of atom i (one warp): the stencil walked as units,
// candidates flattened 32 at a time, FP32 filter + FP64 band predicate,
// accepted pairs compacted with ballots into the atom's ELL row.
template <typename T4>
__device__ __forceinline__ void search_atom(int i, const NbBuffers& nb, const StructGeom* g,
                                            const CellSrc& src, int* su_base_w, float4* su_sh_w,
                                            int* su_first_w, int lane) {
  const int pbc = g->pbc;
  const int nc0 = g->nc[0], nc1 = g->nc[1], nc2 = g->nc[2];
  const int k0 = g->kr[0], k1 = g->kr[1], k2 = g->kr[2];
  const int w1 = 2 * k1 + 1;
  const int packed = nb.cell_of[i];
  const int c0 = packed & 1023, c1 = (packed >> 10) & 1023, c2 = (packed >> 20) & 1023;
  // images along the third axis reachable from this cell
  const int t2lo = pbc ? floor_div_r(c2 - k2, g->inv_nc[2]) : 0;
  const int t2hi = pbc ? floor_div_r(c2 + k2, g->inv_nc[2]) : 0;
  const int nt2 = t2hi - t2lo + 1;
  const int nunits = (2 * k0 + 1) * w1 * nt2;
  const float4 ri = nb.r_f32[i];
  const float rc2_lo = g->rc2_lo, rc2_hi = g->rc2_hi;
  const double rc2 = g->rc2;
  const int cap = nb.cap;
  const size_t row = (size_t)i * cap;
  const int* __restrict__ cstart = src.cstart;
  // lattice coordinates of the atom (pruning in orthogonal cells; the cut
  // is widened slightly so that rounding can only keep extra candidates)
  const float sf0 = (float)nb.s_wrap[3 * i], sf1 = (float)nb.s_wrap[3 * i + 1],
              sf2 = (float)nb.s_wrap[3 * i + 2];
  const float rcf = g->rcf * 1.0001f + 1e-4f;
  int cnt = 0;

  // u / nt2 and r / w1 by multiplication with 2^16 / n rounded up: exact
  // for the unit counts of a stencil (u * n < 2^16)
  const int m_nt2 = (65536 + nt2 - 1) / nt2, m_w1 = (65536 + w1 - 1) / w1;
  const float inc0 = g->inv_nc[0], inc1 = g->inv_nc[1];
  // geometry in registers: the table stores below may alias g as far as
  // the compiler knows, which would otherwise reload these every unit
  const int ortho = g->ortho;
  const float hf0 = g->hf[0], hf1 = g->hf[1], ihf2 = g->inv_hf[2];
  const float* __restrict__ Lf = g->Lf;
  for (int ubase = 0; ubase < nunits; ubase += 32 * NB_UPL) {
    // ---- this lane's units ubase + NB_UPL lane + k: cells [zlo, zhi] of
    // row (d0, d1), image t2; consecutive candidate ranges per lane
    int lens[NB_UPL], starts[NB_UPL];
    int mylen = 0;
    __syncwarp();   // the previous round's readers are done
#pragma unroll
    for (int kk = 0; kk < NB_UPL; ++kk) {
      const int u = ubase + NB_UPL * lane + kk;
      int len = 0, beg = 0, T0 = 0, T1 = 0, T2 = 0;
      float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
      if (u < nunits) {
        const int rr = (u * m_nt2) >> 16;
        const int it2 = u - rr * nt2;
        const int q0 = (rr * m_w1) >> 16;
        const int d1 = rr - q0 * w1 - k1;
        const int d0 = q0 - k0;
        int a0 = c0 + d0, a1 = c1 + d1;
        bool ok = true;
        int zlo = c2 - k2, zhi = c2 + k2;   // unwrapped cell indices
        if (ortho) {
          const float x0 = (float)a0 * inc0, x1 = (float)(a0 + 1) * inc0;
          const float y0 = (float)a1 * inc1, y1 = (float)(a1 + 1) * inc1;
          const float gx = fmaxf(0.f, fmaxf(x0 - sf0, sf0 - x1)) * hf0;
          const float gy = fmaxf(0.f, fmaxf(y0 - sf1, sf1 - y1)) * hf1;
          const float rem = rcf * rcf - gx * gx - gy * gy;
          if (rem < 0.f) {
            ok = false;
          } else {
            const float hz = sqrtf(rem) * ihf2 * 1.0001f + 1e-6f;
            zlo = max(zlo, __float2int_rd((sf2 - hz) * nc2));
            zhi = min(zhi, __float2int_rd((sf2 + hz) * nc2));
          }
        }
        if (pbc) {
          // images of the row's cell: a0, a1 lie within k of the home cell
          while (a0 < 0) {
            a0 += nc0;
            --T0;
          }
          while (a0 >= nc0) {
            a0 -= nc0;
            ++T0;
          }
          while (a1 < 0) {
            a1 += nc1;
            --T1;
          }
          while (a1 >= nc1) {
            a1 -= nc1;
            ++T1;
          }
          T2 = t2lo + it2;
          zlo = max(zlo, T2 * nc2);
          zhi = min(zhi, T2 * nc2 + nc2 - 1);
        } else {
          ok = ok && it2 == 0 && a0 >= 0 && a0 < nc0 && a1 >= 0 && a1 < nc1;
          zlo = max(zlo, 0);
          zhi = min(zhi, nc2 - 1);
        }
        if (ok && zlo <= zhi) {
          const int base = (a0 * nc1 + a1) * nc2 - T2 * nc2;
          beg = cstart[base + zlo];
          len = cstart[base + zhi + 1] - beg;
          const float f0 = (float)T0, f1 = (float)T1, f2 = (float)T2;
          sh0 = f0 * Lf[0] + f1 * Lf[3] + f2 * Lf[6];
          sh1 = f0 * Lf[1] + f1 * Lf[4] + f2 * Lf[7];
          sh2 = f0 * Lf[2] + f1 * Lf[5] + f2 * Lf[8];
        }
      }
      lens[kk] = len;
      starts[kk] = mylen;   // offset inside this lane's range for now
      mylen += len;
      su_base_w[NB_UPL * lane + kk] = beg - starts[kk];   // minus the lane's start below
      su_sh_w[NB_UPL * lane + kk] = make_float4(
          sh0, sh1, sh2, __int_as_float((T0 & 1023) | ((T1 & 1023) << 10) | ((T2 & 1023) << 20)));
    }
    int incl = mylen;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int w = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += w;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int lstart = incl - mylen;
#pragma unroll
    for (int kk = 0; kk < NB_UPL; ++kk) {
      starts[kk] += lstart;
      su_base_w[NB_UPL * lane + kk] -= lstart;   // cell_atoms index = base + q
    }
    __syncwarp();
    int carry = 0;
    for (int qb = 0; qb < total; qb += 32) {
      const int q = qb + lane;
      // units starting inside this batch mark their offsets
      unsigned mine = 0u;
      __syncwarp();   // the previous batch's readers are done
#pragma unroll
      for (int kk = 0; kk < NB_UPL; ++kk) {
        if (lens[kk] > 0 && starts[kk] >= qb && starts[kk] < qb + 32) {
          su_first_w[starts[kk] - qb] = NB_UPL * lane + kk;
          mine |= 1u << (starts[kk] - qb);
        }
      }
      const unsigned marks = __reduce_or_sync(0xffffffffu, mine);
      __syncwarp();
      const unsigned upto = marks & (0xffffffffu >> (31 - lane));
      const int own = upto ? su_first_w[31 - __clz(upto)] : carry;
      carry = __shfl_sync(0xffffffffu, own, 31);
      const float4 osh = su_sh_w[own];
      const int img = __float_as_int(osh.w);   // packed image; zero for T = 0
      const float osh0 = osh.x, osh1 = osh.y, osh2 = osh.z;
      bool accept = false;
      int j = -1, tj = 0;
      float dx = 0.f, dy = 0.f, dz = 0.f, dd2 = 0.f;
      if (q < total) {
        const int p = su_base_w[own] + q;
        const float4 rj = src.cpos[p - src.base];
        j = src.catoms[p - src.base];
        tj = __float_as_int(rj.w);
        const bool self_img = (j == i);
        const bool zeroT = img == 0;
        if (!(self_img && zeroT)) {
          dx = (rj.x - ri.x) + osh0;
          dy = (rj.y - ri.y) + osh1;
          dz = (rj.z - ri.z) + osh2;
          dd2 = dx * dx + dy * dy + dz * dz;
          if (dd2 < rc2_lo) {
            accept = true;
          } else if (dd2 <= rc2_hi) {
            // exact FP64 predicate, evaluated as the reference does
            accept = band_fp64(nb, g, pbc, self_img, img, i, j, rc2);
          }
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, accept);
      if (accept) {
        const int k = cnt + __popc(mask & ((1u << lane) - 1u));
        if (k < cap) {
          nb.nb_jt[row + k] = j | (tj << AE_TYPE_SHIFT);
          if (nb.nb_img) nb.nb_img[row + k] = img;
          if (VecOut<T4>::fp64) {
            // R_ij = L (s_j + T) - L s_i in FP64 (the vectors the reference's
            // descriptor sees)
            const int oT0 = sext10i(img & 1023), oT1 = sext10i((img >> 10) & 1023),
                      oT2 = sext10i((img >> 20) & 1023);
            double R[3];
            if (pbc) {
              const double* sj = nb.s_wrap + 3 * j;
              double u0 = da(sj[0], (double)oT0), u1 = da(sj[1], (double)oT1),
                     u2 = da(sj[2], (double)oT2);
              for (int c = 0; c < 3; ++c) {
                double t = dm(g->L[c], u0);
                t = da(t, dm(g->L[3 + c], u1));
                t = da(t, dm(g->L[6 + c], u2));
                R[c] = da(t, -nb.r_wrap[3 * i + c]);
              }
            } else {
              for (int c = 0; c < 3; ++c) R[c] = da(nb.r_wrap[3 * j + c], -nb.r_wrap[3 * i + c]);
            }
            double dist = sqrt(da(da(dm(R[0], R[0]), dm(R[1], R[1])), dm(R[2], R[2])));
            reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] =
                make_double4_32a(R[0], R[1], R[2], dist);
          } else {
            reinterpret_cast<float4*>(nb.nb_vec)[row + k] =
                make_float4(dx, dy, dz, pair_length(dd2));
          }
        }
      }
      cnt += __popc(mask);
    }
  }
  if (lane == 0) {
    nb.nb_cnt[i] = min(cnt, cap);
    if (cnt > cap) atomicOr(nb.status, AE_ST_NB_OVERFLOW);
  }
}

template <typename T4>
__global__ void __launch_bounds__(256, 4) k_neighbors(int natoms, NbBuffers nb) {
  __shared__ int su_base[8][32 * NB_UPL];      // per warp: cell_atoms offset of each unit
  __shared__ float4 su_sh[8][32 * NB_UPL];     // image shift and packed image of each unit
  __shared__ int su_first[8][32];              // unit starting at each offset of a batch
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= natoms) return;
  const StructGeom* g = nb.geom + nb.atom_struct[i];
  const CellSrc src{nb.cell_start + g->cell_off, nb.cell_pos, nb.cell_atoms, 0};
  search_atom<T4>(i, nb, g, src, su_base[warp], su_sh[warp], su_first[warp], lane);
}

// The cell lists of one structure in shared memory (block-wide): atoms
// wrapped and binned (wrap_bin_atom), counted per cell with shared-memory
// atomics, the counts scanned (scs[c] = first entry of cell c, scs[ncell] =
// n) and the atoms scattered into cell order (spos, satoms).
__device__ __forceinline__ void struct_cells(const StructGeom* g, const double* __restrict__ pos,
                                             const int* __restrict__ types, const NbBuffers& nb,
                                             float4* spos, int* satoms, int* scs, int* sbin,
                                             int* s_wt) {
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int n = g->natoms, a0 = g->atom_off;
  const int ncell = g->nc[0] * g->nc[1] * g->nc[2];
  for (int q = threadIdx.x; q <= ncell; q += blockDim.x) scs[q] = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int lin = wrap_bin_atom(a0 + q, g, pos, types, nb);
    sbin[q] = lin | (atomicAdd(&scs[lin], 1) << 16);
  }
  __syncthreads();
  // exclusive scan of the counts, a block's width at a time
  int carry = 0;
  for (int base = 0; base < ncell; base += blockDim.x) {
    const int c = base + threadIdx.x;
    const int v = c < ncell ? scs[c] : 0;
    int incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += u;
    }
    if (lane == 31) s_wt[warp] = incl;
    __syncthreads();
    int before = carry, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (w < warp) before += s_wt[w];
      total += s_wt[w];
    }
    if (c < ncell) scs[c] = before + incl - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) scs[ncell] = n;
  __syncthreads();
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int w = sbin[q];
    const int p = scs[w & 0xffff] + (w >> 16);
    spos[p] = nb.r_f32[a0 + q];
    satoms[p] = a0 + q;
  }
  __syncthreads();
}

// One block per structure (structures in the order nb.struct_order, largest
// first), its cell lists built in shared memory: the structure's atoms are
// wrapped and binned (wrap_bin_atom), counted per cell with shared-memory
// atomics, the counts scanned and the atoms scattered into cell order
// (positions, atom indices and cell offsets of the structure only), then
// the block's warps take its atoms one by one with the same search.  The
// global cell lists are not used.
template <typename T4>
__global__ void __launch_bounds__(256, NB_STRUCT_BLOCKS)
    k_neighbors_struct(const double* __restrict__ pos, const int* __restrict__ types,
                       NbBuffers nb) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  __shared__ int su_base[8][32 * NB_UPL];
  __shared__ float4 su_sh[8][32 * NB_UPL];
  __shared__ int su_first[8][32];
  __shared__ int s_wt[9];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const StructGeom* g = nb.geom + nb.struct_order[blockIdx.x];
  const int n = g->natoms, a0 = g->atom_off;
  float4* spos = reinterpret_cast<float4*>(sm_raw);
  int* satoms = reinterpret_cast<int*>(spos + nb.smem_atoms);
  int* scs = satoms + nb.smem_atoms;      // [ncell + 1]: counts, then offsets
  int* sbin = scs + nb.smem_cells + 1;    // per atom: cell | rank << 16
  struct_cells(g, pos, types, nb, spos, satoms, scs, sbin, s_wt);
  const CellSrc src{scs, spos, satoms, 0};
  for (int a = warp; a < n; a += (blockDim.x >> 5))
    search_atom<T4>(a0 + a, nb, g, src, su_base[warp], su_sh[warp], su_first[warp], lane);
}

// ---- cell-batched search: one warp per home cell, lane h = home atom h.
// Candidates (the same stencil units as above, pruned for the whole home
// cell in orthogonal cells) are staged 32 at a time in shared memory and
// every lane tests each of them against its own home atom, appending
// accepted pairs to its own row: no ballots or shuffles in the inner loop,
// and the unit mapping and candidate loads are shared by the cell's atoms.
// Acceptance is the same FP32 filter + FP64 band test.
constexpr int NBC_WARPS = 8;

template <typename T4>
__global__ void __launch_bounds__(256) k_neighbors_cell(int ncells, NbBuffers nb) {
  __shared__ float4 s_pos[NBC_WARPS][32];     // candidate position, species bits in w
  __shared__ float4 s_shift[NBC_WARPS][32];   // image shift, packed image in w
  __shared__ int s_j[NBC_WARPS][32];
  __shared__ int su_base[NBC_WARPS][32];
  __shared__ float4 su_sh[NBC_WARPS][32];
  __shared__ int su_first[NBC_WARPS][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gc = blockIdx.x * NBC_WARPS + warp;
  if (gc >= ncells) return;
  const int hb = nb.cell_start[gc], he = nb.cell_start[gc + 1];
  if (hb >= he) return;
  int lo = 0, hi = nb.nstruc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (nb.geom[mid].cell_off <= gc) lo = mid; else hi = mid - 1;
  }
  const StructGeom* g = nb.geom + lo;
  const int pbc = g->pbc;
  const int nc0 = g->nc[0], nc1 = g->nc[1], nc2 = g->nc[2];
  const int k0 = g->kr[0], k1 = g->kr[1], k2 = g->kr[2];
  const int w1 = 2 * k1 + 1;
  const int lin = gc - g->cell_off;
  const int c2 = lin % nc2, c1 = (lin / nc2) % nc1, c0 = lin / (nc1 * nc2);
  const int t2lo = pbc ? floor_div_r(c2 - k2, g->inv_nc[2]) : 0;
  const int t2hi = pbc ? floor_div_r(c2 + k2, g->inv_nc[2]) : 0;
  const int nt2 = t2hi - t2lo + 1;
  const int nunits = (2 * k0 + 1) * w1 * nt2;
  const float rc2_lo = g->rc2_lo, rc2_hi = g->rc2_hi;
  const double rc2 = g->rc2;
  const int cap = nb.cap;
  const int* __restrict__ cstart = nb.cell_start + g->cell_off;
  const float rcf = g->rcf * 1.0001f + 1e-4f;
  const float inv_nt2 = __fdividef(1.0f, (float)nt2), inv_w1 = __fdividef(1.0f, (float)w1);

  for (int hbase = hb; hbase < he; hbase += 32) {
    const bool home = hbase + lane < he;
    const int ih = home ? nb.cell_atoms[hbase + lane] : -1;
    const float4 rh = home ? nb.cell_pos[hbase + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    const size_t row = (size_t)(home ? ih : 0) * cap;
    int cnt = 0;
    for (int ubase = 0; ubase < nunits; ubase += 32) {
      const int u = ubase + lane;
      int len = 0, beg = 0, T0 = 0, T1 = 0, T2 = 0;
      float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
      if (u < nunits) {
        const int rr = floor_div_r(u, inv_nt2);
        const int it2 = u - rr * nt2;
        const int q0 = floor_div_r(rr, inv_w1);
        const int d1 = rr - q0 * w1 - k1;
        const int d0 = q0 - k0;
        int a0 = c0 + d0, a1 = c1 + d1;
        bool ok = true;
        int zlo = c2 - k2, zhi = c2 + k2;
        if (g->ortho) {
          // gap between the home cell and row (a0, a1), whole cells apart
          const float gx = (float)max(0, abs(d0) - 1) * g->hf[0] * g->inv_nc[0];
          const float gy = (float)max(0, abs(d1) - 1) * g->hf[1] * g->inv_nc[1];
          const float rem = rcf * rcf - gx * gx - gy * gy;
          if (rem < 0.f) {
            ok = false;
          } else {
            const int hz = 1 + (int)floorf(sqrtf(rem) * g->inv_hf[2] * nc2 * 1.0001f + 1e-4f);
            zlo = max(zlo, c2 - hz);
            zhi = min(zhi, c2 + hz);
          }
        }
        if (pbc) {
          T0 = floor_div_r(a0, g->inv_nc[0]);
          a0 -= T0 * nc0;
          T1 = floor_div_r(a1, g->inv_nc[1]);
          a1 -= T1 * nc1;
          T2 = t2lo + it2;
          zlo = max(zlo, T2 * nc2);
          zhi = min(zhi, T2 * nc2 + nc2 - 1);
        } else {
          ok = ok && it2 == 0 && a0 >= 0 && a0 < nc0 && a1 >= 0 && a1 < nc1;
          zlo = max(zlo, 0);
          zhi = min(zhi, nc2 - 1);
        }
        if (ok && zlo <= zhi) {
          const int base = (a0 * nc1 + a1) * nc2 - T2 * nc2;
          beg = cstart[base + zlo];
          len = cstart[base + zhi + 1] - beg;
          const float f0 = (float)T0, f1 = (float)T1, f2 = (float)T2;
          sh0 = f0 * g->Lf[0] + f1 * g->Lf[3] + f2 * g->Lf[6];
          sh1 = f0 * g->Lf[1] + f1 * g->Lf[4] + f2 * g->Lf[7];
          sh2 = f0 * g->Lf[2] + f1 * g->Lf[5] + f2 * g->Lf[8];
        }
      }
      int incl = len;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int w = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += w;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      // unit table of this round (see k_neighbors)
      const int start = incl - len;
      __syncwarp();
      su_base[warp][lane] = beg - start;
      su_sh[warp][lane] = make_float4(sh0, sh1, sh2,
                                      __int_as_float((T0 & 1023) | ((T1 & 1023) << 10) |
                                                     ((T2 & 1023) << 20)));
      __syncwarp();
      int carry = 0;
      for (int qb = 0; qb < total; qb += 32) {
        // ---- stage 32 candidates
        const int q = qb + lane;
        const bool starts = len > 0 && start >= qb && start < qb + 32;
        __syncwarp();   // readers of the previous batch are done
        if (starts) su_first[warp][start - qb] = lane;
        const unsigned marks = __reduce_or_sync(0xffffffffu, starts ? (1u << (start - qb)) : 0u);
        __syncwarp();
        const unsigned upto = marks & (0xffffffffu >> (31 - lane));
        const int own = upto ? su_first[warp][31 - __clz(upto)] : carry;
        carry = __shfl_sync(0xffffffffu, own, 31);
        if (q < total) {
          const int p = su_base[warp][own] + q;
          s_pos[warp][lane] = nb.cell_pos[p];
          s_j[warp][lane] = nb.cell_atoms[p];
          s_shift[warp][lane] = su_sh[warp][own];
        }
        __syncwarp();
        // ---- test them against this lane's home atom
        const int nq = min(32, total - qb);
        if (home) {
          for (int c = 0; c < nq; ++c) {
            const float4 rj = s_pos[warp][c];
            const float4 sh = s_shift[warp][c];
            const int j = s_j[warp][c];
            const int img = __float_as_int(sh.w);
            if (j == ih && img == 0) continue;   // the atom itself
            const float dx = (rj.x - rh.x) + sh.x;
            const float dy = (rj.y - rh.y) + sh.y;
            const float dz = (rj.z - rh.z) + sh.z;
            const float dd2 = dx * dx + dy * dy + dz * dz;
            if (dd2 > rc2_hi) continue;
            const int t0 = sext10i(img & 1023), t1 = sext10i((img >> 10) & 1023),
                      t2 = sext10i((img >> 20) & 1023);
            if (dd2 >= rc2_lo) {
              // exact FP64 predicate, evaluated as the reference does
              double e2;
              if (pbc) {
                double cart[3];
                if (j == ih) {
                  for (int cc = 0; cc < 3; ++cc) {
                    double t = dm(g->L[cc], (double)t0);
                    t = da(t, dm(g->L[3 + cc], (double)t1));
                    t = da(t, dm(g->L[6 + cc], (double)t2));
                    cart[cc] = t;
                  }
                } else {
                  const double* sj = nb.s_wrap + 3 * j;
                  const double u0 = da(sj[0], (double)t0), u1 = da(sj[1], (double)t1),
                               u2 = da(sj[2], (double)t2);
                  for (int cc = 0; cc < 3; ++cc) {
                    double t = dm(g->L[cc], u0);
                    t = da(t, dm(g->L[3 + cc], u1));
                    t = da(t, dm(g->L[6 + cc], u2));
                    cart[cc] = da(t, -nb.r_wrap[3 * ih + cc]);
                  }
                }
                e2 = da(da(dm(cart[0], cart[0]), dm(cart[1], cart[1])), dm(cart[2], cart[2]));
              } else {
                const double c0d = da(nb.r_wrap[3 * j], -nb.r_wrap[3 * ih]);
                const double c1d = da(nb.r_wrap[3 * j + 1], -nb.r_wrap[3 * ih + 1]);
                const double c2d = da(nb.r_wrap[3 * j + 2], -nb.r_wrap[3 * ih + 2]);
                e2 = da(da(dm(c0d, c0d), dm(c1d, c1d)), dm(c2d, c2d));
              }
              if (!(e2 <= rc2)) continue;
            }
            if (cnt < cap) {
              nb.nb_jt[row + cnt] = j | (__float_as_int(rj.w) << AE_TYPE_SHIFT);
              if (nb.nb_img) nb.nb_img[row + cnt] = img;
              if (VecOut<T4>::fp64) {
                double R[3];
                if (pbc) {
                  const double* sj = nb.s_wrap + 3 * j;
                  const double u0 = da(sj[0], (double)t0), u1 = da(sj[1], (double)t1),
                               u2 = da(sj[2], (double)t2);
                  for (int cc = 0; cc < 3; ++cc) {
                    double t = dm(g->L[cc], u0);
                    t = da(t, dm(g->L[3 + cc], u1));
                    t = da(t, dm(g->L[6 + cc], u2));
                    R[cc] = da(t, -nb.r_wrap[3 * ih + cc]);
                  }
                } else {
                  for (int cc = 0; cc < 3; ++cc)
                    R[cc] = da(nb.r_wrap[3 * j + cc], -nb.r_wrap[3 * ih + cc]);
                }
                const double dist = sqrt(da(da(dm(R[0], R[0]), dm(R[1], R[1])), dm(R[2], R[2])));
                reinterpret_cast<double4_32a*>(nb.nb_vec)[row + cnt] =
                    make_double4_32a(R[0], R[1], R[2], dist);
              } else {
                reinterpret_cast<float4*>(nb.nb_vec)[row + cnt] =
                    make_float4(dx, dy, dz, sqrtf(dd2));
              }
            }
            ++cnt;
          }
        }
        __syncwarp();
      }
    }
    if (home) {
      nb.nb_cnt[ih] = min(cnt, cap);
      if (cnt > cap) atomicOr(nb.status, AE_ST_NB_OVERFLOW);
    }
  }
}

// ---- candidate-streaming search: one warp per home cell, lane = candidate.
// The stencil units of the home cell (pruned for the whole cell in
// orthogonal cells, as above) are flattened into batches of 32 candidates
// held one per lane; every batch is tested against each home atom of the
// cell in turn (home positions broadcast from shared memory), accepted
// pairs compacted by ballot into the home atom's row.  The unit mapping and
// the candidate loads are shared by all atoms of the cell, and all lanes
// stay busy however few atoms a cell holds.  Same FP32 filter + FP64 band
// test as the other kernels.
constexpr int NBS_WARPS = 8;

// the reference's FP64 predicate for a pair in the band around the cut-off
__device__ __forceinline__ bool band_accept(const StructGeom* g, const NbBuffers& nb, int pbc,
                                            int ih, int j, int t0, int t1, int t2, double rc2) {
  double e2;
  if (pbc) {
    double cart[3];
    if (j == ih) {
      for (int cc = 0; cc < 3; ++cc) {
        double t = dm(g->L[cc], (double)t0);
        t = da(t, dm(g->L[3 + cc], (double)t1));
        t = da(t, dm(g->L[6 + cc], (double)t2));
        cart[cc] = t;
      }
    } else {
      const double* sj = nb.s_wrap + 3 * j;
      const double u0 = da(sj[0], (double)t0), u1 = da(sj[1], (double)t1),
                   u2 = da(sj[2], (double)t2);
      for (int cc = 0; cc < 3; ++cc) {
        double t = dm(g->L[cc], u0);
        t = da(t, dm(g->L[3 + cc], u1));
        t = da(t, dm(g->L[6 + cc], u2));
        cart[cc] = da(t, -nb.r_wrap[3 * ih + cc]);
      }
    }
    e2 = da(da(dm(cart[0], cart[0]), dm(cart[1], cart[1])), dm(cart[2], cart[2]));
  } else {
    const double c0d = da(nb.r_wrap[3 * j], -nb.r_wrap[3 * ih]);
    const double c1d = da(nb.r_wrap[3 * j + 1], -nb.r_wrap[3 * ih + 1]);
    const double c2d = da(nb.r_wrap[3 * j + 2], -nb.r_wrap[3 * ih + 2]);
    e2 = da(da(dm(c0d, c0d), dm(c1d, c1d)), dm(c2d, c2d));
  }
  return e2 <= rc2;
}

// R_ij = L (s_j + T) - L s_i in FP64 and its length
__device__ __forceinline__ double4_32a fp64_pair_vector(const StructGeom* g, const NbBuffers& nb,
                                                        int pbc, int ih, int j, int t0, int t1,
                                                        int t2) {
  double R[3];
  if (pbc) {
    const double* sj = nb.s_wrap + 3 * j;
    const double u0 = da(sj[0], (double)t0), u1 = da(sj[1], (double)t1),
                 u2 = da(sj[2], (double)t2);
    for (int cc = 0; cc < 3; ++cc) {
      double t = dm(g->L[cc], u0);
      t = da(t, dm(g->L[3 + cc], u1));
      t = da(t, dm(g->L[6 + cc], u2));
      R[cc] = da(t, -nb.r_wrap[3 * ih + cc]);
    }
  } else {
    for (int cc = 0; cc < 3; ++cc) R[cc] = da(nb.r_wrap[3 * j + cc], -nb.r_wrap[3 * ih + cc]);
  }
  const double dist = sqrt(da(da(dm(R[0], R[0]), dm(R[1], R[1])), dm(R[2], R[2])));
  return make_double4_32a(R[0], R[1], R[2], dist);
}

template <typename T4>
__global__ void __launch_bounds__(32 * NBS_WARPS) k_neighbors_stream(int ncells, NbBuffers nb) {
  __shared__ int su_base[NBS_WARPS][32];
  __shared__ float4 su_sh[NBS_WARPS][32];
  __shared__ int su_first[NBS_WARPS][32];
  __shared__ float4 sh_pos[NBS_WARPS][32];   // home atoms: position, species bits in w
  __shared__ int sh_i[NBS_WARPS][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gc = blockIdx.x * NBS_WARPS + warp;
  if (gc >= ncells) return;
  const int hb = nb.cell_start[gc], he = nb.cell_start[gc + 1];
  if (hb >= he) return;
  // the structure of the cell is that of any of its atoms
  const StructGeom* g = nb.geom + nb.atom_struct[nb.cell_atoms[hb]];
  const int pbc = g->pbc;
  const int nc0 = g->nc[0], nc1 = g->nc[1], nc2 = g->nc[2];
  const int k0 = g->kr[0], k1 = g->kr[1], k2 = g->kr[2];
  const int w1 = 2 * k1 + 1;
  const int lin = gc - g->cell_off;
  const int c2 = lin % nc2, c1 = (lin / nc2) % nc1, c0 = lin / (nc1 * nc2);
  const int t2lo = pbc ? floor_div_r(c2 - k2, g->inv_nc[2]) : 0;
  const int t2hi = pbc ? floor_div_r(c2 + k2, g->inv_nc[2]) : 0;
  const int nt2 = t2hi - t2lo + 1;
  const int nunits = (2 * k0 + 1) * w1 * nt2;
  const float rc2_lo = g->rc2_lo, rc2_hi = g->rc2_hi;
  const double rc2 = g->rc2;
  const int cap = nb.cap;
  const int* __restrict__ cstart = nb.cell_start + g->cell_off;
  const float rcf = g->rcf * 1.0001f + 1e-4f;
  const float inv_nt2 = __fdividef(1.0f, (float)nt2), inv_w1 = __fdividef(1.0f, (float)w1);
  const int ortho = g->ortho;
  const float cw0 = g->hf[0] * g->inv_nc[0], cw1 = g->hf[1] * g->inv_nc[1];
  const float zsc = g->inv_hf[2] * nc2 * 1.0001f;
  const float inc0 = g->inv_nc[0], inc1 = g->inv_nc[1];
  const float* __restrict__ Lf = g->Lf;

  for (int hbase = hb; hbase < he; hbase += 32) {
    const int nh = min(32, he - hbase);
    __syncwarp();
    if (lane < nh) {
      sh_pos[warp][lane] = nb.cell_pos[hbase + lane];
      sh_i[warp][lane] = nb.cell_atoms[hbase + lane];
    }
    __syncwarp();
    int cnt = 0;   // lane h: neighbours of home atom h found so far
    for (int ubase = 0; ubase < nunits; ubase += 32) {
      const int u = ubase + lane;
      int len = 0, beg = 0, T0 = 0, T1 = 0, T2 = 0;
      float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
      if (u < nunits) {
        const int rr = floor_div_r(u, inv_nt2);
        const int it2 = u - rr * nt2;
        const int q0 = floor_div_r(rr, inv_w1);
        const int d1 = rr - q0 * w1 - k1;
        const int d0 = q0 - k0;
        int a0 = c0 + d0, a1 = c1 + d1;
        bool ok = true;
        int zlo = c2 - k2, zhi = c2 + k2;
        if (ortho) {
          // gap between the home cell and row (a0, a1), whole cells apart
          const float gx = (float)max(0, abs(d0) - 1) * cw0;
          const float gy = (float)max(0, abs(d1) - 1) * cw1;
          const float rem = rcf * rcf - gx * gx - gy * gy;
          if (rem < 0.f) {
            ok = false;
          } else {
            const int hz = 1 + (int)floorf(sqrtf(rem) * zsc + 1e-4f);
            zlo = max(zlo, c2 - hz);
            zhi = min(zhi, c2 + hz);
          }
        }
        if (pbc) {
          T0 = floor_div_r(a0, inc0);
          a0 -= T0 * nc0;
          T1 = floor_div_r(a1, inc1);
          a1 -= T1 * nc1;
          T2 = t2lo + it2;
          zlo = max(zlo, T2 * nc2);
          zhi = min(zhi, T2 * nc2 + nc2 - 1);
        } else {
          ok = ok && it2 == 0 && a0 >= 0 && a0 < nc0 && a1 >= 0 && a1 < nc1;
          zlo = max(zlo, 0);
          zhi = min(zhi, nc2 - 1);
        }
        if (ok && zlo <= zhi) {
          const int base = (a0 * nc1 + a1) * nc2 - T2 * nc2;
          beg = cstart[base + zlo];
          len = cstart[base + zhi + 1] - beg;
          const float f0 = (float)T0, f1 = (float)T1, f2 = (float)T2;
          sh0 = f0 * Lf[0] + f1 * Lf[3] + f2 * Lf[6];
          sh1 = f0 * Lf[1] + f1 * Lf[4] + f2 * Lf[7];
          sh2 = f0 * Lf[2] + f1 * Lf[5] + f2 * Lf[8];
        }
      }
      int incl = len;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int w = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += w;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      const int start = incl - len;
      __syncwarp();
      su_base[warp][lane] = beg - start;
      su_sh[warp][lane] = make_float4(sh0, sh1, sh2,
                                      __int_as_float((T0 & 1023) | ((T1 & 1023) << 10) |
                                                     ((T2 & 1023) << 20)));
      __syncwarp();
      int carry = 0;
      for (int qb = 0; qb < total; qb += 32) {
        // ---- this lane's candidate (unit lookup as in k_neighbors)
        const int q = qb + lane;
        const bool starts = len > 0 && start >= qb && start < qb + 32;
        __syncwarp();
        if (starts) su_first[warp][start - qb] = lane;
        const unsigned marks = __reduce_or_sync(0xffffffffu, starts ? (1u << (start - qb)) : 0u);
        __syncwarp();
        const unsigned upto = marks & (0xffffffffu >> (31 - lane));
        const int own = upto ? su_first[warp][31 - __clz(upto)] : carry;
        carry = __shfl_sync(0xffffffffu, own, 31);
        const bool valid = q < total;
        float4 cp = make_float4(0.f, 0.f, 0.f, 0.f);
        int cj = -1;
        const float4 cs = su_sh[warp][own];
        if (valid) {
          const int p = su_base[warp][own] + q;
          cp = nb.cell_pos[p];
          cj = nb.cell_atoms[p];
        }
        const int img = __float_as_int(cs.w);
        const int jt = cj | (__float_as_int(cp.w) << AE_TYPE_SHIFT);
        // ---- against every home atom of the cell
        for (int h = 0; h < nh; ++h) {
          const float4 rh = sh_pos[warp][h];
          const int ih = sh_i[warp][h];
          bool acc = false, band = false;
          float dx = 0.f, dy = 0.f, dz = 0.f, dd2 = 0.f;
          if (valid && !(cj == ih && img == 0)) {
            dx = (cp.x - rh.x) + cs.x;
            dy = (cp.y - rh.y) + cs.y;
            dz = (cp.z - rh.z) + cs.z;
            dd2 = dx * dx + dy * dy + dz * dz;
            acc = dd2 < rc2_lo;
            band = !acc && dd2 <= rc2_hi;
          }
          if (__any_sync(0xffffffffu, band)) {
            if (band)
              acc = band_accept(g, nb, pbc, ih, cj, sext10i(img & 1023), sext10i((img >> 10) & 1023),
                                sext10i((img >> 20) & 1023), rc2);
          }
          const unsigned m = __ballot_sync(0xffffffffu, acc);
          if (m == 0u) continue;
          const int k = __shfl_sync(0xffffffffu, cnt, h) + __popc(m & ((1u << lane) - 1u));
          if (acc && k < cap) {
            const size_t row = (size_t)ih * cap;
            nb.nb_jt[row + k] = jt;
            if (nb.nb_img) nb.nb_img[row + k] = img;
            if (VecOut<T4>::fp64) {
              reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] = fp64_pair_vector(
                  g, nb, pbc, ih, cj, sext10i(img & 1023), sext10i((img >> 10) & 1023),
                  sext10i((img >> 20) & 1023));
            } else {
              reinterpret_cast<float4*>(nb.nb_vec)[row + k] =
                  make_float4(dx, dy, dz, pair_length(dd2));
            }
          }
          if (lane == h) cnt += __popc(m);
        }
      }
    }
    if (lane < nh) {
      nb.nb_cnt[sh_i[warp][lane]] = min(cnt, cap);
      if (cnt > cap) atomicOr(nb.status, AE_ST_NB_OVERFLOW);
    }
  }
}

// ---- half-stencil search: every pair once.  One warp per atom as in
// k_neighbors, but only over the stencil units whose unwrapped cell offset
// D = (d0, d1, dz) is lexicographically positive (d0 > 0; d0 = 0 and
// d1 > 0; d0 = d1 = 0 and dz >= 0), and within the atom's own cell at T = 0
// only partners j > i.  The offset of a pair seen from j is -D, so each
// unordered pair (i, j, T) is met exactly once; the finder writes it to
// both rows, (j, T) into row i and (i, -T) into row j, each side accepted
// by its own FP64 predicate in the band.  Slots come from atomic counters
// (nb_cnt zeroed before, clamped after): rows hold the same sets as the
// full search in an order that depends on timing.
constexpr int AE_HOME_UNIT = 1 << 30;   // unit flag beside the packed image

template <typename T4>
__global__ void __launch_bounds__(256, 4) k_neighbors_half(int natoms, NbBuffers nb) {
  __shared__ int su_base[8][32 * NB_UPL];
  __shared__ float4 su_sh[8][32 * NB_UPL];
  __shared__ int su_first[8][32];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= natoms) return;
  const StructGeom* g = nb.geom + nb.atom_struct[i];
  const int pbc = g->pbc;
  const int nc0 = g->nc[0], nc1 = g->nc[1], nc2 = g->nc[2];
  const int k0 = g->kr[0], k1 = g->kr[1], k2 = g->kr[2];
  const int w1 = 2 * k1 + 1;
  const int packed = nb.cell_of[i];
  const int c0 = packed & 1023, c1 = (packed >> 10) & 1023, c2 = (packed >> 20) & 1023;
  const int t2lo = pbc ? floor_div_r(c2 - k2, g->inv_nc[2]) : 0;
  const int t2hi = pbc ? floor_div_r(c2 + k2, g->inv_nc[2]) : 0;
  const int nt2 = t2hi - t2lo + 1;
  // rows (0, 0..k1) then (1..k0, -k1..k1); the (0, 0) row from dz = 0 up
  const int nrows = (k1 + 1) + k0 * w1;
  const int nunits = nrows * nt2;
  const float4 ri = nb.r_f32[i];
  const int iti = i | (__float_as_int(ri.w) << AE_TYPE_SHIFT);
  const float rc2_lo = g->rc2_lo, rc2_hi = g->rc2_hi;
  const double rc2 = g->rc2;
  const int cap = nb.cap;
  const int* __restrict__ cstart = nb.cell_start + g->cell_off;
  const int home_end = cstart[(c0 * nc1 + c1) * nc2 + c2 + 1];
  const float sf0 = (float)nb.s_wrap[3 * i], sf1 = (float)nb.s_wrap[3 * i + 1],
              sf2 = (float)nb.s_wrap[3 * i + 2];
  const float rcf = g->rcf * 1.0001f + 1e-4f;
  const float inv_nt2 = __fdividef(1.0f, (float)nt2), inv_w1 = __fdividef(1.0f, (float)w1);
  const float inc0 = g->inv_nc[0], inc1 = g->inv_nc[1];
  const int ortho = g->ortho;
  const float hf0 = g->hf[0], hf1 = g->hf[1], ihf2 = g->inv_hf[2];
  const float* __restrict__ Lf = g->Lf;
  int* __restrict__ cnt = nb.nb_cnt;
  const unsigned lt = (1u << lane) - 1u;

  for (int ubase = 0; ubase < nunits; ubase += 32) {
    const int u = ubase + lane;
    int len = 0, beg = 0, T0 = 0, T1 = 0, T2 = 0, home = 0;
    float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
    if (u < nunits) {
      const int rr = floor_div_r(u, inv_nt2);
      const int it2 = u - rr * nt2;
      int d0, d1;
      if (rr <= k1) {
        d0 = 0;
        d1 = rr;
      } else {
        const int r2 = rr - (k1 + 1);
        const int q0 = floor_div_r(r2, inv_w1);
        d0 = 1 + q0;
        d1 = r2 - q0 * w1 - k1;
      }
      int a0 = c0 + d0, a1 = c1 + d1;
      bool ok = true;
      int zlo = (d0 == 0 && d1 == 0) ? c2 : c2 - k2, zhi = c2 + k2;
      if (ortho) {
        const float x0 = (float)a0 * inc0, x1 = (float)(a0 + 1) * inc0;
        const float y0 = (float)a1 * inc1, y1 = (float)(a1 + 1) * inc1;
        const float gx = fmaxf(0.f, fmaxf(x0 - sf0, sf0 - x1)) * hf0;
        const float gy = fmaxf(0.f, fmaxf(y0 - sf1, sf1 - y1)) * hf1;
        const float rem = rcf * rcf - gx * gx - gy * gy;
        if (rem < 0.f) {
          ok = false;
        } else {
          const float hz = sqrtf(rem) * ihf2 * 1.0001f + 1e-6f;
          zlo = max(zlo, (int)floorf((sf2 - hz) * nc2));
          zhi = min(zhi, (int)floorf((sf2 + hz) * nc2));
        }
      }
      if (pbc) {
        T0 = floor_div_r(a0, inc0);
        a0 -= T0 * nc0;
        T1 = floor_div_r(a1, inc1);
        a1 -= T1 * nc1;
        T2 = t2lo + it2;
        zlo = max(zlo, T2 * nc2);
        zhi = min(zhi, T2 * nc2 + nc2 - 1);
      } else {
        ok = ok && it2 == 0 && a0 >= 0 && a0 < nc0 && a1 >= 0 && a1 < nc1;
        zlo = max(zlo, 0);
        zhi = min(zhi, nc2 - 1);
      }
      if (ok && zlo <= zhi) {
        const int base = (a0 * nc1 + a1) * nc2 - T2 * nc2;
        beg = cstart[base + zlo];
        len = cstart[base + zhi + 1] - beg;
        // the home cell (T = 0) leads the (0, 0) row of image 0
        home = (d0 == 0 && d1 == 0 && zlo == c2) ? AE_HOME_UNIT : 0;
        const float f0 = (float)T0, f1 = (float)T1, f2 = (float)T2;
        sh0 = f0 * Lf[0] + f1 * Lf[3] + f2 * Lf[6];
        sh1 = f0 * Lf[1] + f1 * Lf[4] + f2 * Lf[7];
        sh2 = f0 * Lf[2] + f1 * Lf[5] + f2 * Lf[8];
      }
    }
    int incl = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int w = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += w;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int start = incl - len;
    __syncwarp();
    su_base[warp][lane] = beg - start;
    su_sh[warp][lane] = make_float4(
        sh0, sh1, sh2,
        __int_as_float((T0 & 1023) | ((T1 & 1023) << 10) | ((T2 & 1023) << 20) | home));
    __syncwarp();
    int carry = 0;
    for (int qb = 0; qb < total; qb += 32) {
      const int q = qb + lane;
      const bool starts = len > 0 && start >= qb && start < qb + 32;
      __syncwarp();
      if (starts) su_first[warp][start - qb] = lane;
      const unsigned marks = __reduce_or_sync(0xffffffffu, starts ? (1u << (start - qb)) : 0u);
      __syncwarp();
      const unsigned upto = marks & (0xffffffffu >> (31 - lane));
      const int own = upto ? su_first[warp][31 - __clz(upto)] : carry;
      carry = __shfl_sync(0xffffffffu, own, 31);
      const float4 osh = su_sh[warp][own];
      const int tag = __float_as_int(osh.w);
      const int img = tag & ~AE_HOME_UNIT;
      bool acc_i = false, acc_j = false;
      int j = 0, tj = 0;
      float dx = 0.f, dy = 0.f, dz = 0.f, dd2 = 0.f;
      if (q < total) {
        const int p = su_base[warp][own] + q;
        const float4 rj = nb.cell_pos[p];
        j = nb.cell_atoms[p];
        tj = __float_as_int(rj.w);
        // in the atom's own cell only partners after it
        if (!(tag & AE_HOME_UNIT) || p >= home_end || j > i) {
          dx = (rj.x - ri.x) + osh.x;
          dy = (rj.y - ri.y) + osh.y;
          dz = (rj.z - ri.z) + osh.z;
          dd2 = dx * dx + dy * dy + dz * dz;
          if (dd2 < rc2_lo) {
            acc_i = acc_j = true;
          } else if (dd2 <= rc2_hi) {
            const int t0 = sext10i(img & 1023), t1 = sext10i((img >> 10) & 1023),
                      t2 = sext10i((img >> 20) & 1023);
            acc_i = band_accept(g, nb, pbc, i, j, t0, t1, t2, rc2);
            acc_j = band_accept(g, nb, pbc, j, i, -t0, -t1, -t2, rc2);
          }
        }
      }
      // row i: one counter update per batch
      const unsigned mask = __ballot_sync(0xffffffffu, acc_i);
      int base_i = 0;
      if (mask) {
        if (lane == 0) base_i = atomicAdd(cnt + i, __popc(mask));
        base_i = __shfl_sync(0xffffffffu, base_i, 0);
      }
      const int nimg = ((-sext10i(img & 1023)) & 1023) |
                       (((-sext10i((img >> 10) & 1023)) & 1023) << 10) |
                       (((-sext10i((img >> 20) & 1023)) & 1023) << 20);
      if (acc_i) {
        const int k = base_i + __popc(mask & lt);
        if (k < cap) {
          const size_t row = (size_t)i * cap;
          nb.nb_jt[row + k] = j | (tj << AE_TYPE_SHIFT);
          if (nb.nb_img) nb.nb_img[row + k] = img;
          if (VecOut<T4>::fp64) {
            reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] = fp64_pair_vector(
                g, nb, pbc, i, j, sext10i(img & 1023), sext10i((img >> 10) & 1023),
                sext10i((img >> 20) & 1023));
          } else {
            reinterpret_cast<float4*>(nb.nb_vec)[row + k] =
                make_float4(dx, dy, dz, pair_length(dd2));
          }
        }
      }
      // row j: the mirrored pair
      if (acc_j) {
        const int k = atomicAdd(cnt + j, 1);
        if (k < cap) {
          const size_t row = (size_t)j * cap;
          nb.nb_jt[row + k] = iti;
          if (nb.nb_img) nb.nb_img[row + k] = nimg;
          if (VecOut<T4>::fp64) {
            reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] = fp64_pair_vector(
                g, nb, pbc, j, i, -sext10i(img & 1023), -sext10i((img >> 10) & 1023),
                -sext10i((img >> 20) & 1023));
          } else {
            reinterpret_cast<float4*>(nb.nb_vec)[row + k] =
                make_float4(-dx, -dy, -dz, pair_length(dd2));
          }
        }
      }
    }
  }
}

// ---- half stencil per structure: the shared-memory cell lists of
// k_neighbors_struct walked as k_neighbors_half walks the global ones (each
// unordered pair met once and written to both rows), the rows' counters in
// shared memory.  Same sets as the full search; the order inside a row
// depends on timing.
template <typename T4>
__device__ __forceinline__ void search_atom_half(int i, int a0, const NbBuffers& nb,
                                                 const StructGeom* g, const float4* spos,
                                                 const int* satoms, const int* scs, int* scnt,
                                                 int* su_base_w, float4* su_sh_w,
                                                 int* su_first_w, int lane) {
  const int pbc = g->pbc;
  const int nc0 = g->nc[0], nc1 = g->nc[1], nc2 = g->nc[2];
  const int k0 = g->kr[0], k1 = g->kr[1], k2 = g->kr[2];
  const int w1 = 2 * k1 + 1;
  const int packed = nb.cell_of[i];
  const int c0 = packed & 1023, c1 = (packed >> 10) & 1023, c2 = (packed >> 20) & 1023;
  const int t2lo = pbc ? floor_div_r(c2 - k2, g->inv_nc[2]) : 0;
  const int t2hi = pbc ? floor_div_r(c2 + k2, g->inv_nc[2]) : 0;
  const int nt2 = t2hi - t2lo + 1;
  // rows (0, 0..k1) then (1..k0, -k1..k1); the (0, 0) row from dz = 0 up
  const int nrows = (k1 + 1) + k0 * w1;
  const int nunits = nrows * nt2;
  const float4 ri = nb.r_f32[i];
  const int iti = i | (__float_as_int(ri.w) << AE_TYPE_SHIFT);
  const float rc2_lo = g->rc2_lo, rc2_hi = g->rc2_hi;
  const double rc2 = g->rc2;
  const int cap = nb.cap;
  const int* __restrict__ cstart = scs;
  const int home_end = cstart[(c0 * nc1 + c1) * nc2 + c2 + 1];
  const float sf0 = (float)nb.s_wrap[3 * i], sf1 = (float)nb.s_wrap[3 * i + 1],
              sf2 = (float)nb.s_wrap[3 * i + 2];
  const float rcf = g->rcf * 1.0001f + 1e-4f;
  const float inv_nt2 = __fdividef(1.0f, (float)nt2), inv_w1 = __fdividef(1.0f, (float)w1);
  const float inc0 = g->inv_nc[0], inc1 = g->inv_nc[1];
  const int ortho = g->ortho;
  const float hf0 = g->hf[0], hf1 = g->hf[1], ihf2 = g->inv_hf[2];
  const float* __restrict__ Lf = g->Lf;
  const unsigned lt = (1u << lane) - 1u;

  for (int ubase = 0; ubase < nunits; ubase += 32) {
    const int u = ubase + lane;
    int len = 0, beg = 0, T0 = 0, T1 = 0, T2 = 0, home = 0;
    float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
    if (u < nunits) {
      const int rr = floor_div_r(u, inv_nt2);
      const int it2 = u - rr * nt2;
      int d0, d1;
      if (rr <= k1) {
        d0 = 0;
        d1 = rr;
      } else {
        const int r2 = rr - (k1 + 1);
        const int q0 = floor_div_r(r2, inv_w1);
        d0 = 1 + q0;
        d1 = r2 - q0 * w1 - k1;
      }
      int a0 = c0 + d0, a1 = c1 + d1;
      bool ok = true;
      int zlo = (d0 == 0 && d1 == 0) ? c2 : c2 - k2, zhi = c2 + k2;
      if (ortho) {
        const float x0 = (float)a0 * inc0, x1 = (float)(a0 + 1) * inc0;
        const float y0 = (float)a1 * inc1, y1 = (float)(a1 + 1) * inc1;
        const float gx = fmaxf(0.f, fmaxf(x0 - sf0, sf0 - x1)) * hf0;
        const float gy = fmaxf(0.f, fmaxf(y0 - sf1, sf1 - y1)) * hf1;
        const float rem = rcf * rcf - gx * gx - gy * gy;
        if (rem < 0.f) {
          ok = false;
        } else {
          const float hz = sqrtf(rem) * ihf2 * 1.0001f + 1e-6f;
          zlo = max(zlo, (int)floorf((sf2 - hz) * nc2));
          zhi = min(zhi, (int)floorf((sf2 + hz) * nc2));
        }
      }
      if (pbc) {
        T0 = floor_div_r(a0, inc0);
        a0 -= T0 * nc0;
        T1 = floor_div_r(a1, inc1);
        a1 -= T1 * nc1;
        T2 = t2lo + it2;
        zlo = max(zlo, T2 * nc2);
        zhi = min(zhi, T2 * nc2 + nc2 - 1);
      } else {
        ok = ok && it2 == 0 && a0 >= 0 && a0 < nc0 && a1 >= 0 && a1 < nc1;
        zlo = max(zlo, 0);
        zhi = min(zhi, nc2 - 1);
      }
      if (ok && zlo <= zhi) {
        const int base = (a0 * nc1 + a1) * nc2 - T2 * nc2;
        beg = cstart[base + zlo];
        len = cstart[base + zhi + 1] - beg;
        // the home cell (T = 0) leads the (0, 0) row of image 0
        home = (d0 == 0 && d1 == 0 && zlo == c2) ? AE_HOME_UNIT : 0;
        const float f0 = (float)T0, f1 = (float)T1, f2 = (float)T2;
        sh0 = f0 * Lf[0] + f1 * Lf[3] + f2 * Lf[6];
        sh1 = f0 * Lf[1] + f1 * Lf[4] + f2 * Lf[7];
        sh2 = f0 * Lf[2] + f1 * Lf[5] + f2 * Lf[8];
      }
    }
    int incl = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int w = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += w;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int start = incl - len;
    __syncwarp();
    su_base_w[lane] = beg - start;
    su_sh_w[lane] = make_float4(
        sh0, sh1, sh2,
        __int_as_float((T0 & 1023) | ((T1 & 1023) << 10) | ((T2 & 1023) << 20) | home));
    __syncwarp();
    int carry = 0;
    for (int qb = 0; qb < total; qb += 32) {
      const int q = qb + lane;
      const bool starts = len > 0 && start >= qb && start < qb + 32;
      __syncwarp();
      if (starts) su_first_w[start - qb] = lane;
      const unsigned marks = __reduce_or_sync(0xffffffffu, starts ? (1u << (start - qb)) : 0u);
      __syncwarp();
      const unsigned upto = marks & (0xffffffffu >> (31 - lane));
      const int own = upto ? su_first_w[31 - __clz(upto)] : carry;
      carry = __shfl_sync(0xffffffffu, own, 31);
      const float4 osh = su_sh_w[own];
      const int tag = __float_as_int(osh.w);
      const int img = tag & ~AE_HOME_UNIT;
      bool acc_i = false, acc_j = false;
      int j = 0, tj = 0;
      float dx = 0.f, dy = 0.f, dz = 0.f, dd2 = 0.f;
      if (q < total) {
        const int p = su_base_w[own] + q;
        const float4 rj = spos[p];
        j = satoms[p];
        tj = __float_as_int(rj.w);
        // in the atom's own cell only partners after it
        if (!(tag & AE_HOME_UNIT) || p >= home_end || j > i) {
          dx = (rj.x - ri.x) + osh.x;
          dy = (rj.y - ri.y) + osh.y;
          dz = (rj.z - ri.z) + osh.z;
          dd2 = dx * dx + dy * dy + dz * dz;
          if (dd2 < rc2_lo) {
            acc_i = acc_j = true;
          } else if (dd2 <= rc2_hi) {
            const int t0 = sext10i(img & 1023), t1 = sext10i((img >> 10) & 1023),
                      t2 = sext10i((img >> 20) & 1023);
            acc_i = band_accept(g, nb, pbc, i, j, t0, t1, t2, rc2);
            acc_j = band_accept(g, nb, pbc, j, i, -t0, -t1, -t2, rc2);
          }
        }
      }
      // row i: one counter update per batch
      const unsigned mask = __ballot_sync(0xffffffffu, acc_i);
      int base_i = 0;
      if (mask) {
        if (lane == 0) base_i = atomicAdd(scnt + (i - a0), __popc(mask));
        base_i = __shfl_sync(0xffffffffu, base_i, 0);
      }
      const int nimg = ((-sext10i(img & 1023)) & 1023) |
                       (((-sext10i((img >> 10) & 1023)) & 1023) << 10) |
                       (((-sext10i((img >> 20) & 1023)) & 1023) << 20);
      if (acc_i) {
        const int k = base_i + __popc(mask & lt);
        if (k < cap) {
          const size_t row = (size_t)i * cap;
          nb.nb_jt[row + k] = j | (tj << AE_TYPE_SHIFT);
          if (nb.nb_img) nb.nb_img[row + k] = img;
          if (VecOut<T4>::fp64) {
            reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] = fp64_pair_vector(
                g, nb, pbc, i, j, sext10i(img & 1023), sext10i((img >> 10) & 1023),
                sext10i((img >> 20) & 1023));
          } else {
            reinterpret_cast<float4*>(nb.nb_vec)[row + k] =
                make_float4(dx, dy, dz, pair_length(dd2));
          }
        }
      }
      // row j: the mirrored pair
      if (acc_j) {
        const int k = atomicAdd(scnt + (j - a0), 1);
        if (k < cap) {
          const size_t row = (size_t)j * cap;
          nb.nb_jt[row + k] = iti;
          if (nb.nb_img) nb.nb_img[row + k] = nimg;
          if (VecOut<T4>::fp64) {
            reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] = fp64_pair_vector(
                g, nb, pbc, j, i, -sext10i(img & 1023), -sext10i((img >> 10) & 1023),
                -sext10i((img >> 20) & 1023));
          } else {
            reinterpret_cast<float4*>(nb.nb_vec)[row + k] =
                make_float4(-dx, -dy, -dz, pair_length(dd2));
          }
        }
      }
    }
  }
}

template <typename T4>
__global__ void __launch_bounds__(256, NB_STRUCT_HALF_BLOCKS)
    k_neighbors_struct_half(const double* __restrict__ pos, const int* __restrict__ types,
                            NbBuffers nb) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  __shared__ int su_base[8][32];
  __shared__ float4 su_sh[8][32];
  __shared__ int su_first[8][32];
  __shared__ int s_wt[9];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const StructGeom* g = nb.geom + nb.struct_order[blockIdx.x];
  const int n = g->natoms, a0 = g->atom_off;
  float4* spos = reinterpret_cast<float4*>(sm_raw);
  int* satoms = reinterpret_cast<int*>(spos + nb.smem_atoms);
  int* scs = satoms + nb.smem_atoms;
  int* sbin = scs + nb.smem_cells + 1;
  int* scnt = sbin + nb.smem_atoms;       // row counters
  for (int q = threadIdx.x; q < n; q += blockDim.x) scnt[q] = 0;
  struct_cells(g, pos, types, nb, spos, satoms, scs, sbin, s_wt);
  for (int a = warp; a < n; a += (blockDim.x >> 5))
    search_atom_half<T4>(a0 + a, a0, nb, g, spos, satoms, scs, scnt, su_base[warp], su_sh[warp],
                         su_first[warp], lane);
  __syncthreads();
  const int cap = nb.cap;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int c = scnt[q];
    nb.nb_cnt[a0 + q] = min(c, cap);
    if (c > cap) atomicOr(nb.status, AE_ST_NB_OVERFLOW);
  }
}

// counts of the half-stencil search: clamp to the capacity, flag overflow
__global__ void k_clamp_counts(int natoms, int cap, int* __restrict__ cnt, unsigned* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  const int c = cnt[i];
  if (c > cap) {
    cnt[i] = cap;
    atomicOr(status, AE_ST_NB_OVERFLOW);
  }
}

// ---- caller's neighbour list (CSR over local atoms, indices into local +
// ghost atoms) -> ELL table.  R_ij = x_j - x_i in FP64; pairs beyond
// (Rc + 1e-3) are dropped; species from the caller's type ids.
template <typename T4>
__global__ void k_ell_from_csr(int nlocal, int nall, const double* __restrict__ x,
                               const int* __restrict__ types1, int ntypes,
                               const int* __restrict__ offs, const int* __restrict__ nbr,
                               double rc2, int cap, int* __restrict__ nb_cnt,
                               int* __restrict__ nb_jt, void* nb_vec, unsigned* status) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= nlocal) return;
  const double xi0 = x[3 * i], xi1 = x[3 * i + 1], xi2 = x[3 * i + 2];
  const int b0 = offs[i], b1 = offs[i + 1];
  const size_t row = (size_t)i * cap;
  int cnt = 0;
  for (int base = b0; base < b1; base += 32) {
    const int q = base + lane;
    bool accept = false;
    int j = 0, tj = 0;
    double R0 = 0, R1 = 0, R2 = 0, d2 = 0;
    if (q < b1) {
      j = nbr[q];
      if (j >= 0 && j < nall && j != i) {
        R0 = da(x[3 * j], -xi0);
        R1 = da(x[3 * j + 1], -xi1);
        R2 = da(x[3 * j + 2], -xi2);
        d2 = da(da(dm(R0, R0), dm(R1, R1)), dm(R2, R2));
        tj = types1[j] - 1;
        if (tj < 0 || tj >= ntypes) {
          atomicOr(status, AE_ST_BAD_TYPE);
          tj = 0;
        }
        accept = d2 <= rc2;
      } else if (j < 0 || j >= nall) {
        atomicOr(status, AE_ST_BAD_TYPE);
      }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, accept);
    if (accept) {
      const int k = cnt + __popc(mask & ((1u << lane) - 1u));
      if (k < cap) {
        nb_jt[row + k] = j | (tj << AE_TYPE_SHIFT);
        const double d = sqrt(d2);
        if (VecOut<T4>::fp64)
          reinterpret_cast<double4_32a*>(nb_vec)[row + k] = make_double4_32a(R0, R1, R2, d);
        else
          reinterpret_cast<float4*>(nb_vec)[row + k] =
              make_float4((float)R0, (float)R1, (float)R2, (float)d);
      }
    }
    cnt += __popc(mask);
  }
  if (lane == 0) {
    nb_cnt[i] = min(cnt, cap);
    if (cnt > cap) atomicOr(status, AE_ST_NB_OVERFLOW);
  }
}

}  // namespace

int ae_launch_ell_from_csr(int nlocal, int nall, const double* x, const int* types1, int ntypes,
                           const int* offs, const int* nbr, double rc2, int cap, int* nb_cnt,
                           int* nb_jt, void* nb_vec, int fp64, unsigned* status, cudaStream_t s) {
  if (nlocal <= 0) return 0;
  const int blocks = (int)(((size_t)nlocal * 32 + 255) / 256);
  if (fp64)
    k_ell_from_csr<double4_32a><<<blocks, 256, 0, s>>>(nlocal, nall, x, types1, ntypes, offs, nbr,
                                                       rc2, cap, nb_cnt, nb_jt, nb_vec, status);
  else
    k_ell_from_csr<float4><<<blocks, 256, 0, s>>>(nlocal, nall, x, types1, ntypes, offs, nbr, rc2,
                                                  cap, nb_cnt, nb_jt, nb_vec, status);
  return (int)cudaGetLastError();
}

int ae_launch_neighbors(int natoms, const double* pos, const int* types, const NbBuffers& nb,
                        int fp64, cudaStream_t s) {
  if (natoms <= 0) return 0;
  if (nb.cell_kernel == 5 && nb.struct_order) {
    // half stencil, cell lists and row counters inside the search blocks
    if (nb.ev_search) cudaEventRecord(nb.ev_search, s);
    const size_t smem = 28 * (size_t)nb.smem_atoms + 4 * ((size_t)nb.smem_cells + 1);
    if (fp64) {
      auto kern = k_neighbors_struct_half<double4_32a>;
      if (smem + 24576 > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<nb.nstruc, 256, smem, s>>>(pos, types, nb);
    } else {
      auto kern = k_neighbors_struct_half<float4>;
      if (smem + 24576 > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<nb.nstruc, 256, smem, s>>>(pos, types, nb);
    }
    return (int)cudaGetLastError();
  }
  if (nb.cell_kernel == 4 && nb.struct_order) {
    // cell lists built inside the search blocks
    if (nb.ev_search) cudaEventRecord(nb.ev_search, s);
    const size_t smem = 24 * (size_t)nb.smem_atoms + 4 * ((size_t)nb.smem_cells + 1);
    if (fp64) {
      auto kern = k_neighbors_struct<double4_32a>;
      if (smem + 24576 > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<nb.nstruc, 256, smem, s>>>(pos, types, nb);
    } else {
      auto kern = k_neighbors_struct<float4>;
      if (smem + 24576 > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<nb.nstruc, 256, smem, s>>>(pos, types, nb);
    }
    return (int)cudaGetLastError();
  }
  const int nc = nb.ncells_total;
  cudaError_t e = cudaMemsetAsync(nb.cell_count, 0, sizeof(int) * (size_t)nc, s);
  if (e != cudaSuccess) return (int)e;
  k_wrap_bin<<<(natoms + 255) / 256, 256, 0, s>>>(natoms, pos, types, nb);
  // CSR offsets: cell_start[c] = sum of the counts before c, cell_start[nc] = natoms
  const int nblk = (nc + SCAN_B - 1) / SCAN_B;
  k_scan_blocks<<<nblk, SCAN_B, 0, s>>>(nc, nb.cell_count, nb.cell_start, nb.scan_tmp);
  k_scan_sums<<<1, SCAN_B, 0, s>>>(nblk, nb.scan_tmp, nb.cell_start + nc);
  k_scan_add<<<nblk, SCAN_B, 0, s>>>(nc, nb.cell_start, nb.scan_tmp);
  k_scatter<<<(natoms + 255) / 256, 256, 0, s>>>(natoms, nb);
  if (nb.ev_search) cudaEventRecord(nb.ev_search, s);
  if (nb.cell_kernel == 3) {
    e = cudaMemsetAsync(nb.nb_cnt, 0, sizeof(int) * (size_t)natoms, s);
    if (e != cudaSuccess) return (int)e;
    const int blocks = (natoms + 7) / 8;
    if (fp64)
      k_neighbors_half<double4_32a><<<blocks, 256, 0, s>>>(natoms, nb);
    else
      k_neighbors_half<float4><<<blocks, 256, 0, s>>>(natoms, nb);
    k_clamp_counts<<<(natoms + 255) / 256, 256, 0, s>>>(natoms, nb.cap, nb.nb_cnt, nb.status);
    return (int)cudaGetLastError();
  }
  if (nb.cell_kernel == 2) {
    const int blocks = (nc + NBS_WARPS - 1) / NBS_WARPS;
    if (fp64)
      k_neighbors_stream<double4_32a><<<blocks, 32 * NBS_WARPS, 0, s>>>(nc, nb);
    else
      k_neighbors_stream<float4><<<blocks, 32 * NBS_WARPS, 0, s>>>(nc, nb);
    return (int)cudaGetLastError();
  }
  if (nb.cell_kernel == 1) {
    const int blocks = (nc + NBC_WARPS - 1) / NBC_WARPS;
    if (fp64)
      k_neighbors_cell<double4_32a><<<blocks, 32 * NBC_WARPS, 0, s>>>(nc, nb);
    else
      k_neighbors_cell<float4><<<blocks, 32 * NBC_WARPS, 0, s>>>(nc, nb);
    return (int)cudaGetLastError();
  }
  const int blocks = (natoms + 7) / 8;
  if (fp64)
    k_neighbors<double4_32a><<<blocks, 256, 0, s>>>(natoms, nb);
  else
    k_neighbors<float4><<<blocks, 256, 0, s>>>(natoms, nb);
  return (int)cudaGetLastError();
}
