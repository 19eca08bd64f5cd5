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
//   k_wrap_bin    one thread per atom: lattice coordinates
//                 (geometry.f90:697-712), wrap, Cartesian of the wrapped
//                 coordinates, append to a fixed-capacity cell slot list
//   k_neighbors   one warp per atom: enumerate the stencil of cells around
//                 the atom's cell (each offset is a distinct (cell, image)
//                 pair), flatten their atoms into one candidate index space
//                 processed 32 at a time, filter, compact with ballots into
//                 the atom's ELL row.
#include "common.h"

namespace {

constexpr double TWO_PI = 6.283185307179586;  // 2 * 3.141592653589793

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

// s = (B r) / (2 pi) then wrapped into [0, 1): the matmul of
// geometry.f90:708 summed in column order, the loops of lclist.f90:953-987
// (s - floor(s) gives the same value as repeated +-1.0, see the note in
// wrap_coordinate).
__device__ __forceinline__ double wrap_coordinate(double s, unsigned* status) {
  if (!isfinite(s)) {
    atomicOr(status, AE_ST_BAD_COORD);
    return 0.0;
  }
  // For |s| >= 1 every step of the reference's repeated +-1.0 is exact, and
  // for s in [-1, 0) both forms round s + 1 once; so they agree bitwise.
  double f = floor(s);
  double w = da(s, -f);
  if (w >= 1.0) w = da(w, -1.0);
  if (w < 0.0) w = da(w, 1.0);
  return w;
}

__global__ void k_wrap_bin(int natoms, const double* __restrict__ pos,
                           const int* __restrict__ types, NbBuffers nb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  const StructGeom* g = nb.geom + nb.atom_struct[i];
  double r[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
  double s[3], rw[3];
  int nc[3] = {g->nc[0], g->nc[1], g->nc[2]};
  if (g->pbc) {
    for (int v = 0; v < 3; ++v) {
      double t;
      if (g->frac_mode == 2) {
        t = r[v];
      } else {
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
    int c = x < 0.0 ? 0 : (x >= (double)(nc[v] - 1) ? nc[v] - 1 : (int)x);
    cc[v] = c;
  }
  int lin = (cc[0] * nc[1] + cc[1]) * nc[2] + cc[2];
  int slot = atomicAdd(&nb.cell_count[g->cell_off + lin], 1);
  if (slot < g->cell_cap)
    nb.cell_atoms[g->slot_off + lin * g->cell_cap + slot] = i;
  else
    atomicOr(nb.status, AE_ST_CELL_OVERFLOW);
  int t = types[i];
  for (int v = 0; v < 3; ++v) {
    nb.s_wrap[3 * i + v] = s[v];
    nb.r_wrap[3 * i + v] = rw[v];
  }
  nb.r_f32[i] = make_float4((float)rw[0], (float)rw[1], (float)rw[2], __int_as_float(t));
  nb.cell_of[i] = cc[0] | (cc[1] << 10) | (cc[2] << 20);
}

__device__ __forceinline__ int floor_div(int a, int n) {
  int q = a / n;
  return (a % n != 0 && (a < 0)) ? q - 1 : q;
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

template <typename T4>
__global__ void __launch_bounds__(256) k_neighbors(int natoms, NbBuffers nb) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= natoms) return;
  const StructGeom* g = nb.geom + nb.atom_struct[i];
  const int pbc = g->pbc;
  const int nc0 = g->nc[0], nc1 = g->nc[1], nc2 = g->nc[2];
  const int k0 = g->kr[0], k1 = g->kr[1], k2 = g->kr[2];
  const int w0 = 2 * k0 + 1, w1 = 2 * k1 + 1, w2 = 2 * k2 + 1;
  const int noff = w0 * w1 * w2;
  const int packed = nb.cell_of[i];
  const int c0 = packed & 1023, c1 = (packed >> 10) & 1023, c2 = (packed >> 20) & 1023;
  const float4 ri = nb.r_f32[i];
  const float rc2_lo = g->rc2_lo, rc2_hi = g->rc2_hi;
  const double rc2 = g->rc2;
  const int cap = nb.cap;
  const size_t row = (size_t)i * cap;
  int cnt = 0;

  for (int obase = 0; obase < noff; obase += 32) {
    // ---- this lane's stencil offset: target cell, image, atom count
    int o = obase + lane;
    int cnt_o = 0, slot0 = 0, T0 = 0, T1 = 0, T2 = 0;
    float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
    if (o < noff) {
      int d2 = o % w2 - k2;
      int d1 = (o / w2) % w1 - k1;
      int d0 = o / (w2 * w1) - k0;
      int a0 = c0 + d0, a1 = c1 + d1, a2 = c2 + d2;
      bool ok = true;
      if (pbc) {
        T0 = floor_div(a0, nc0); a0 -= T0 * nc0;
        T1 = floor_div(a1, nc1); a1 -= T1 * nc1;
        T2 = floor_div(a2, nc2); a2 -= T2 * nc2;
      } else {
        ok = a0 >= 0 && a0 < nc0 && a1 >= 0 && a1 < nc1 && a2 >= 0 && a2 < nc2;
      }
      if (ok) {
        int lin = (a0 * nc1 + a1) * nc2 + a2;
        cnt_o = min(nb.cell_count[g->cell_off + lin], g->cell_cap);
        slot0 = g->slot_off + lin * g->cell_cap;
        float f0 = (float)T0, f1 = (float)T1, f2 = (float)T2;
        sh0 = f0 * g->Lf[0] + f1 * g->Lf[3] + f2 * g->Lf[6];
        sh1 = f0 * g->Lf[1] + f1 * g->Lf[4] + f2 * g->Lf[7];
        sh2 = f0 * g->Lf[2] + f1 * g->Lf[5] + f2 * g->Lf[8];
      }
    }
    // inclusive prefix of counts over the 32 offsets of this chunk
    int incl = cnt_o;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    for (int qb = 0; qb < total; qb += 32) {
      const int q = qb + lane;
      // owner offset: first lane whose inclusive prefix exceeds q
      int lo = 0, hi = 31;
#pragma unroll
      for (int step = 0; step < 5; ++step) {
        int mid = (lo + hi) >> 1;
        int pv = __shfl_sync(0xffffffffu, incl, mid);
        if (pv > q) hi = mid; else lo = mid + 1;
      }
      const int own = lo;
      const int own_incl = __shfl_sync(0xffffffffu, incl, own);
      const int own_cnt = __shfl_sync(0xffffffffu, cnt_o, own);
      const int own_slot = __shfl_sync(0xffffffffu, slot0, own);
      const int oT0 = __shfl_sync(0xffffffffu, T0, own);
      const int oT1 = __shfl_sync(0xffffffffu, T1, own);
      const int oT2 = __shfl_sync(0xffffffffu, T2, own);
      const float osh0 = __shfl_sync(0xffffffffu, sh0, own);
      const float osh1 = __shfl_sync(0xffffffffu, sh1, own);
      const float osh2 = __shfl_sync(0xffffffffu, sh2, own);
      bool accept = false;
      int j = -1;
      float dx = 0.f, dy = 0.f, dz = 0.f, dd2 = 0.f;
      if (q < total) {
        j = nb.cell_atoms[own_slot + (q - (own_incl - own_cnt))];
        const bool self_img = (j == i);
        const bool zeroT = (oT0 == 0 && oT1 == 0 && oT2 == 0);
        if (!(self_img && zeroT)) {
          const float4 rj = nb.r_f32[j];
          dx = (rj.x - ri.x) + osh0;
          dy = (rj.y - ri.y) + osh1;
          dz = (rj.z - ri.z) + osh2;
          dd2 = dx * dx + dy * dy + dz * dz;
          if (dd2 < rc2_lo) {
            accept = true;
          } else if (dd2 <= rc2_hi) {
            // exact FP64 predicate, evaluated as the reference does
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
            accept = (e2 <= rc2);
          }
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, accept);
      if (accept) {
        const int k = cnt + __popc(mask & ((1u << lane) - 1u));
        if (k < cap) {
          const int tj = __float_as_int(nb.r_f32[j].w);
          nb.nb_jt[row + k] = j | (tj << AE_TYPE_SHIFT);
          if (nb.nb_img)
            nb.nb_img[row + k] = (oT0 & 1023) | ((oT1 & 1023) << 10) | ((oT2 & 1023) << 20);
          if (VecOut<T4>::fp64) {
            // R_ij = L (s_j + T) - L s_i in FP64 (the coordinates the
            // descriptor of the reference sees)
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
            reinterpret_cast<double4_32a*>(nb.nb_vec)[row + k] = make_double4_32a(R[0], R[1], R[2], dist);
          } else {
            reinterpret_cast<float4*>(nb.nb_vec)[row + k] = make_float4(dx, dy, dz, sqrtf(dd2));
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

}  // namespace

int ae_launch_neighbors(int natoms, const double* pos, const int* types,
                        const NbBuffers& nb, int fp64, cudaStream_t s) {
  if (natoms <= 0) return 0;
  cudaError_t e = cudaMemsetAsync(nb.cell_count, 0, sizeof(int) * (size_t)nb.ncells_total, s);
  if (e != cudaSuccess) return (int)e;
  k_wrap_bin<<<(natoms + 255) / 256, 256, 0, s>>>(natoms, pos, types, nb);
  int blocks = (natoms + 7) / 8;
  if (fp64)
    k_neighbors<double4_32a><<<blocks, 256, 0, s>>>(natoms, nb);
  else
    k_neighbors<float4><<<blocks, 256, 0, s>>>(natoms, nb);
  return (int)cudaGetLastError();
}
