// Loss and weight gradients for training (replaces eval_next_structure /
// eval_net of src/train.f90:799-916 with ff_wderiv of
// src/ext/feedforward.f90:763-860, and the gradient accumulation
// Dw_sum += dE * Dw of src/optimize.f90:698-734).
//
// Two losses:
//   energy (the reference's):  SSE = sum_s dE_s^2 / 2,
//       dE_s = (E_target,s - E_s) / (E_scale N_s)   (normalised units,
//       train.f90:872), gradient sum_s dE_s Dw_s with
//       Dw_s = -sum_{i in s} dy_i/dw / N_s          (train.f90:858-861);
//   energy + force:  L = w_E sum_s (E_s - E_t,s)^2 / N_s^2
//                      + w_F sum_i |F_i - F_t,i|^2.
// The force term needs the derivative of F = -dE/dr with respect to the
// weights.  With u_i = dL/dF_i and the descriptor tangent
//   v_a = sum_i (dG_a/dr_i) u_i          (normalised descriptor)
// it is  dL_F/dw = -sum_a E_scale d/dw [ (dy_a/dG) . v_a ],  a
// forward-over-reverse pass through each atom's network: the forward pass
// carries the primal z, a and the tangent zdot = W adot, and the reverse
// pass propagates the adjoints of both.  Per atom, for the scalar
//   phi_a = kappa (cE_s y_a + cF ydot_a)
// the weight gradient of layer l is  zbar_{l+1} (x) a_l + zdotbar_{l+1} (x) adot_l,
// accumulated over the atoms of one species in a tile in shared memory.
//
// Order-fixed reduction: atoms are partitioned by species with a stable
// counting sort, every block owns a fixed range of them and writes its
// partial gradient to its own row; a final kernel sums the rows in block
// order in FP64.  No atomics touch the gradient (the forces and cell lists
// upstream do use atomics, so reruns agree to rounding, not bit for bit).
#include "common.h"
#include "k_cheb_impl.cuh"

namespace {

using cheb::Vec4;

// ----------------------------------------------------------------------
// stable partition of the atoms by species
// ----------------------------------------------------------------------
constexpr int PART_B = 1024;

__global__ void k_part_count(int n, const int* __restrict__ types, int* __restrict__ bcnt) {
  __shared__ int c[AE_MAXT];
  if (threadIdx.x < AE_MAXT) c[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * PART_B + threadIdx.x;
  if (i < n) atomicAdd(&c[types[i]], 1);
  __syncthreads();
  if (threadIdx.x < AE_MAXT) bcnt[blockIdx.x * AE_MAXT + threadIdx.x] = c[threadIdx.x];
}

// species-major exclusive scan of the block counts: warp t scans the
// column of species t; the species totals are prefixed first
__global__ void k_part_scan(int nblk, int ntypes, const int* __restrict__ bcnt, int* __restrict__ boff,
                            int* __restrict__ spec_off) {
  __shared__ int tot[AE_MAXT];
  const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
  if (t < ntypes) {
    int s = 0;
    for (int b = lane; b < nblk; b += 32) s += bcnt[b * AE_MAXT + t];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if (lane == 0) tot[t] = s;
  }
  __syncthreads();
  if (t < ntypes) {
    int run = 0;
    for (int u = 0; u < t; ++u) run += tot[u];
    if (lane == 0) spec_off[t] = run;
    if (t == ntypes - 1 && lane == 0) spec_off[ntypes] = run + tot[t];
    for (int b0 = 0; b0 < nblk; b0 += 32) {
      const int b = b0 + lane;
      const int c = b < nblk ? bcnt[b * AE_MAXT + t] : 0;
      int x = c;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
      }
      if (b < nblk) boff[b * AE_MAXT + t] = run + x - c;
      run += __shfl_sync(0xffffffffu, x, 31);
    }
  }
}

__global__ void k_part_scatter(int n, int ntypes, const int* __restrict__ types,
                               const int* __restrict__ boff, int* __restrict__ order) {
  __shared__ int wc[PART_B / 32][AE_MAXT];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * PART_B + threadIdx.x;
  const int t = i < n ? types[i] : -1;
  unsigned mine = 0;
  for (int q = 0; q < ntypes; ++q) {
    const unsigned m = __ballot_sync(0xffffffffu, t == q);
    if (q == t) mine = m;
    if (lane == 0) wc[warp][q] = __popc(m);
  }
  __syncthreads();
  if (threadIdx.x < ntypes) {
    const int q = threadIdx.x;
    int run = 0;
    for (int w = 0; w < PART_B / 32; ++w) {
      const int c = wc[w][q];
      wc[w][q] = run;
      run += c;
    }
  }
  __syncthreads();
  if (t >= 0) {
    const int rank = wc[warp][t] + __popc(mine & ((1u << lane) - 1u));
    order[boff[blockIdx.x * AE_MAXT + t] + rank] = i;
  }
}

// ----------------------------------------------------------------------
// loss, structure coefficients cE_s and force residuals u_i
// ----------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// one warp per structure
template <typename T>
__global__ void k_loss(int nstruc, const StructGeom* __restrict__ geom,
                       const double* __restrict__ E_struct, const double* __restrict__ E_tgt,
                       const void* __restrict__ Facc, const double* __restrict__ F_tgt, int mode,
                       double wE, double wF, double E_scale, double* __restrict__ cE,
                       void* __restrict__ U, double* __restrict__ loss_s) {
  using T4 = typename Vec4<T>::type;
  const int lane = threadIdx.x & 31;
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= nstruc) return;
  const int n = geom[s].natoms, off = geom[s].atom_off;
  const double dn = (double)n;
  double lossE, ce;
  if (mode == 0) {
    const double dE = (E_tgt[s] - E_struct[s]) / (E_scale * dn);
    lossE = 0.5 * dE * dE;
    ce = -dE / dn;
  } else {
    const double r = E_struct[s] - E_tgt[s];
    lossE = wE * r * r / (dn * dn);
    ce = 2.0 * wE * r / (dn * dn);
  }
  double acc = 0.0, comp = 0.0;
  if (mode == 1 && F_tgt) {
    const T4* F = reinterpret_cast<const T4*>(Facc);
    T4* Uo = reinterpret_cast<T4*>(U);
    for (int a = lane; a < n; a += 32) {
      const T4 f = F[off + a];
      const double* ft = F_tgt + 3 * (size_t)(off + a);
      const double rx = (double)f.x - ft[0], ry = (double)f.y - ft[1], rz = (double)f.z - ft[2];
      double t, e;
      two_sum(acc, wF * (rx * rx + ry * ry + rz * rz), t, e);
      acc = t;
      comp += e;
      T4 u;
      u.x = T(2.0 * wF * rx);
      u.y = T(2.0 * wF * ry);
      u.z = T(2.0 * wF * rz);
      u.w = T(0);
      Uo[off + a] = u;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const double ao = __shfl_xor_sync(0xffffffffu, acc, d);
    const double co = __shfl_xor_sync(0xffffffffu, comp, d);
    double t, e;
    two_sum(acc, ao, t, e);
    acc = t;
    comp = comp + co + e;
  }
  if (lane == 0) {
    cE[s] = ce;
    loss_s[s] = lossE + (acc + comp);
  }
}

// deterministic sum of the structure losses (one block)
__global__ void k_loss_sum(int nstruc, const double* __restrict__ loss_s, double* __restrict__ out) {
  __shared__ double sh[1024], sc[1024];
  double s = 0.0, c = 0.0;
  for (int q = threadIdx.x; q < nstruc; q += blockDim.x) {
    double t, e;
    two_sum(s, loss_s[q], t, e);
    s = t;
    c += e;
  }
  sh[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      double t, e;
      two_sum(sh[threadIdx.x], sh[threadIdx.x + h], t, e);
      sh[threadIdx.x] = t;
      sc[threadIdx.x] += sc[threadIdx.x + h] + e;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0] + sc[0];
}

// ----------------------------------------------------------------------
// networks: forward-over-reverse with weight-gradient accumulation
// ----------------------------------------------------------------------
__device__ __forceinline__ float tanh_t(float x) { return tanhf(x); }
__device__ __forceinline__ double tanh_t(double x) { return tanh(x); }
__device__ __forceinline__ float exp_t(float x) { return expf(x); }
__device__ __forceinline__ double exp_t(double x) { return exp(x); }

// ff_activate (feedforward.f90:932-969) with the second derivative
template <typename T>
__device__ __forceinline__ void activate2(int t, T x, T& y, T& d1, T& d2) {
  const T a = T(1.7159), b = T(0.666666666666667), c = T(0.1);
  switch (t) {
    case 0: y = x; d1 = T(1); d2 = T(0); break;
    case 1: y = tanh_t(x); d1 = T(1) - y * y; d2 = T(-2) * y * d1; break;
    case 2: y = T(1) / (T(1) + exp_t(-x)); d1 = y * (T(1) - y); d2 = d1 * (T(1) - T(2) * y); break;
    case 3: {
      const T tb = tanh_t(b * x);
      const T s = T(1) - tb * tb;
      y = a * tb; d1 = a * b * s; d2 = T(-2) * a * b * b * tb * s;
    } break;
    case 4: {
      const T tb = tanh_t(b * x);
      const T s = T(1) - tb * tb;
      y = a * tb + c * x; d1 = a * b * s + c; d2 = T(-2) * a * b * b * tb * s;
    } break;
    default: y = d1 = d2 = T(0);
  }
}

template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

struct WgradArgs {
  int ntypes;
  const int* order;        // atoms grouped by species
  const int* spec_off;     // [ntypes + 1]
  const void* G;           // [N][nsf_pad] normalised descriptors (T)
  const void* V;           // [N][nsf_pad] normalised descriptor tangents (T) or null
  const int* atom_struct;
  const double* cE;        // per structure coefficient of y
  double cF;               // coefficient of ydot
  int physical;            // multiply both by the species' E_scale
  double* partial;         // [ntypes][gridDim.x][wcap]
  int wcap;                // row length of partial (>= every species' layout size)
  int tile;                // atoms per tile
};

// shared-memory layout of one block (elements of T)
struct WgLayout {
  int wsz;                        // species weights in device layout
  int row;                        // tile row length per atom
  int scratch;                    // per warp
  int xo[AE_MAXLAYERS], zo[AE_MAXLAYERS], xdo[AE_MAXLAYERS], zdo[AE_MAXLAYERS];
  int so[AE_MAXLAYERS];           // scratch offsets of layer l nodes (f', f'', zdot)
};

__host__ __device__ inline WgLayout wg_layout(const NetTable& net, bool tang) {
  WgLayout w{};
  const int L = net.nlayers;
  w.wsz = net.w_off[L - 2] - net.w_off[0] + net.pitch[L - 2] * net.nnodes[L - 1];
  int r = 0;
  for (int l = 0; l + 1 < L; ++l) {
    w.xo[l] = r; r += net.nnodes[l];
    w.zo[l] = r; r += net.nnodes[l + 1];
    if (tang) {
      w.xdo[l] = r; r += net.nnodes[l];
      w.zdo[l] = r; r += net.nnodes[l + 1];
    }
  }
  w.row = r | 1;   // odd: rows of different atoms fall in different banks
  int s = 0;
  for (int l = 1; l < L; ++l) {
    w.so[l] = s;
    s += 3 * net.nnodes[l];
  }
  w.scratch = s;
  return w;
}

template <typename T>
__host__ __device__ inline size_t wg_smem_bytes(const WgLayout& w, int tile, int warps) {
  return sizeof(T) * ((size_t)2 * w.wsz + (size_t)tile * w.row + (size_t)warps * w.scratch);
}

template <typename T> __device__ __forceinline__ const T* wsrc(const PotDevice& pd);
template <> __device__ __forceinline__ const float* wsrc<float>(const PotDevice& pd) { return pd.w32; }
template <> __device__ __forceinline__ const double* wsrc<double>(const PotDevice& pd) { return pd.w64; }

template <typename T, bool TANG>
__global__ void __launch_bounds__(256) k_mlp_wgrad(PotDevice pd, WgradArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = blockIdx.y;
  const NetTable& net = pd.sp[t].net;
  const int L = net.nlayers;
  __shared__ WgLayout lay;   // indexed by layer at run time: keep it out of registers
  if (threadIdx.x == 0) lay = wg_layout(net, TANG);
  __syncthreads();
  T* sW = reinterpret_cast<T*>(smem_raw);
  T* sdW = sW + lay.wsz;
  T* tileb = sdW + lay.wsz;
  T* scr0 = tileb + (size_t)A.tile * lay.row;
  const int warps = blockDim.x >> 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* scr = scr0 + (size_t)warp * lay.scratch;
  const int wbeg = net.w_off[0];
  const T* Wg = wsrc<T>(pd) + wbeg;
  for (int q = threadIdx.x; q < lay.wsz; q += blockDim.x) {
    sW[q] = Wg[q];
    sdW[q] = T(0);
  }
  const int beg = A.spec_off[t], nt = A.spec_off[t + 1] - beg;
  const int per = (nt + gridDim.x - 1) / gridDim.x;
  const int a0 = min(nt, blockIdx.x * per), a1 = min(nt, a0 + per);
  const T kappa = A.physical ? T(pd.sp[t].E_scale) : T(1);
  const int nsf_pad = pd.nsf_pad;
  __syncthreads();

  for (int tb = a0; tb < a1; tb += A.tile) {
    const int tn = min(A.tile, a1 - tb);
    // ---- per atom: forward (primal + tangent) and reverse pass
    for (int r = warp; r < tn; r += warps) {
      const int i = A.order[beg + tb + r];
      T* row = tileb + (size_t)r * lay.row;
      const T* Gi = reinterpret_cast<const T*>(A.G) + (size_t)i * nsf_pad;
      const int n0 = net.nnodes[0];
      for (int k = lane; k < n0; k += 32) {
        row[lay.xo[0] + k] = Gi[k];
        if (TANG) row[lay.xdo[0] + k] = reinterpret_cast<const T*>(A.V)[(size_t)i * nsf_pad + k];
      }
      __syncwarp();
      T zL = T(0), d1L = T(0), d2L = T(0), zdL = T(0);
      for (int l = 0; l + 1 < L; ++l) {
        const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
        const T* Wl = sW + (net.w_off[l] - wbeg);
        const int pitch = net.pitch[l];
        const T* hin = row + lay.xo[l];
        const T* hdin = TANG ? row + lay.xdo[l] : nullptr;
        const int fa = net.f_a[l + 1];
        if (l + 2 == L) {
          // output node (a single energy)
          T part = T(0), partd = T(0);
          for (int k = lane; k < nin; k += 32) {
            part += Wl[k] * hin[k];
            if (TANG) partd += Wl[k] * hdin[k];
          }
          part = wsum(part) + Wl[nin];
          if (TANG) partd = wsum(partd);
          T y;
          activate2<T>(fa, part, y, d1L, d2L);
          zL = part;
          zdL = partd;
        } else {
          for (int o = lane; o < nout; o += 32) {
            const T* wr = Wl + o * pitch;
            T z = wr[nin], zd = T(0);
            for (int k = 0; k < nin; ++k) {
              z += wr[k] * hin[k];
              if (TANG) zd += wr[k] * hdin[k];
            }
            T y, d1, d2;
            activate2<T>(fa, z, y, d1, d2);
            row[lay.xo[l + 1] + o] = y;
            T* s = scr + lay.so[l + 1];
            s[o] = d1;
            if (TANG) {
              row[lay.xdo[l + 1] + o] = d1 * zd;
              s[nout + o] = d2;
              s[2 * nout + o] = zd;
            }
          }
        }
        __syncwarp();
      }
      (void)zL;
      // reverse: output layer
      const int sidx = A.atom_struct[i];
      const T ce = kappa * T(A.cE[sidx]);
      const T cf = kappa * T(A.cF);
      if (lane == 0) {
        row[lay.zo[L - 2]] = TANG ? ce * d1L + cf * d2L * zdL : ce * d1L;
        if (TANG) row[lay.zdo[L - 2]] = cf * d1L;
      }
      __syncwarp();
      for (int l = L - 2; l >= 1; --l) {
        // adjoints of the n_l nodes of hidden layer l from layer l -> l+1
        const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
        const T* Wl = sW + (net.w_off[l] - wbeg);
        const int pitch = net.pitch[l];
        const T* zb = row + lay.zo[l];
        const T* zdb = TANG ? row + lay.zdo[l] : nullptr;
        const T* s = scr + lay.so[l];
        for (int k = lane; k < nin; k += 32) {
          T ab = T(0), adb = T(0);
          for (int o = 0; o < nout; ++o) {
            const T w = Wl[o * pitch + k];
            ab += w * zb[o];
            if (TANG) adb += w * zdb[o];
          }
          if (TANG) {
            row[lay.zo[l - 1] + k] = s[k] * ab + s[nin + k] * s[2 * nin + k] * adb;
            row[lay.zdo[l - 1] + k] = s[k] * adb;
          } else {
            row[lay.zo[l - 1] + k] = s[k] * ab;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    // ---- weight gradients of the tile: dW_l[o][k] += sum_r zbar[o] x[k] (+ tangents)
    for (int l = 0; l + 1 < L; ++l) {
      const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
      const int pitch = net.pitch[l];
      T* dWl = sdW + (net.w_off[l] - wbeg);
      const int total = nout * (nin + 1);
      for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int o = e / (nin + 1), k = e - o * (nin + 1);
        T acc = T(0);
        if (k < nin) {
          for (int r = 0; r < tn; ++r) {
            const T* row = tileb + (size_t)r * lay.row;
            acc += row[lay.zo[l] + o] * row[lay.xo[l] + k];
            if (TANG) acc += row[lay.zdo[l] + o] * row[lay.xdo[l] + k];
          }
        } else {
          for (int r = 0; r < tn; ++r) acc += tileb[(size_t)r * lay.row + lay.zo[l] + o];
        }
        dWl[o * pitch + k] += acc;
      }
    }
    __syncthreads();
  }
  double* out = A.partial + ((size_t)t * gridDim.x + blockIdx.x) * A.wcap;
  for (int q = threadIdx.x; q < A.wcap; q += blockDim.x) out[q] = q < lay.wsz ? (double)sdW[q] : 0.0;
}

// ---- tile form of the same pass: WT_TN atoms at a time, every layer as
// register-blocked products over the tile.  Activations, tangents and node
// adjoints are held feature-major ([feature][atom], rows WT_P apart) so
// that four atoms of one feature are one vector load; each layer input
// carries a row of ones (and its tangent a row of zeros), which makes the
// bias an ordinary column.  Per layer l (nin -> nout):
//   forward   z = W_l [X_l; 1], zd = W_l [Xd_l; 0]   (threads: 4 atoms x 2 nodes)
//   reverse   dW_l += ZB_l [X_l; 1]^T + ZDB_l [Xd_l; 0]^T  (4 nodes x 4 inputs)
//             ZB_{l-1} = f' (W_l^T ZB_l) + f'' zd (W_l^T ZDB_l),
//             ZDB_{l-1} = f' (W_l^T ZDB_l)                 (4 atoms x 2 inputs)
// The node adjoints of a hidden layer overwrite its f' and f'' zd rows,
// which no other thread reads by then.  Padding atoms of the last tile
// have zero inputs and zero coefficients, so they add nothing.
constexpr int WT_TN = 32;           // atoms per tile
constexpr int WT_P = WT_TN + 4;     // row pitch: 16-byte rows, successive rows 4 banks apart
constexpr int WT_THREADS = 128;
static_assert(WT_THREADS == 4 * WT_TN, "the output node takes four threads per atom");
constexpr int WT_PF = 8;            // inputs per thread and array held for the next tile

struct WtLayout {
  int L;
  int x[AE_MAXLAYERS];    // first row of [X_l; 1]            (nin_l + 1 rows)
  int xd[AE_MAXLAYERS];   // first row of [Xd_l; 0]           (nin_l + 1 rows, tangents)
  int s1[AE_MAXLAYERS];   // f' of the nodes of X_l, l >= 1   (nin_l rows) -> ZB_{l-1}
  int s2[AE_MAXLAYERS];   // f'' zd of those nodes            (nin_l rows) -> ZDB_{l-1}
  int out;                // output node: ZB, ZDB; energy coefficient per atom
  int rows;
  int wr[AE_MAXLAYERS];   // W_l row-major [nout][pr], bias at column nin
  int pr[AE_MAXLAYERS];
  int wt[AE_MAXLAYERS];   // W_l transposed [nin + 1][pt]
  int pt[AE_MAXLAYERS];
  int wend;               // end of both weight copies (elements)
  int wsz;                // gradient in the device weight layout
};

__host__ __device__ inline WtLayout wt_layout(const NetTable& net, bool tang) {
  WtLayout w{};
  const int L = net.nlayers;
  w.L = L;
  int r = 0;
  for (int l = 0; l + 1 < L; ++l) {
    const int n = net.nnodes[l];
    w.x[l] = r;
    r += n + 1;
    w.xd[l] = r;
    if (tang) r += n + 1;
    if (l >= 1) {
      w.s1[l] = r;
      r += n;
      w.s2[l] = r;
      if (tang) r += n;
    }
  }
  w.out = r;
  r += 3;
  w.rows = r;
  int e = r * WT_P;   // even: vector loads of weight pairs stay aligned
  for (int l = 0; l + 1 < L; ++l) {
    const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
    w.pr[l] = (nin + 2) & ~1;
    w.pt[l] = (nout + 1) & ~1;
    w.wr[l] = e;
    e += nout * w.pr[l];
    w.wt[l] = e;
    e += (nin + 1) * w.pt[l];
  }
  w.wend = e;
  w.wsz = net.w_off[L - 2] - net.w_off[0] + net.pitch[L - 2] * net.nnodes[L - 1];
  return w;
}

template <typename T>
__host__ __device__ inline size_t wt_smem_bytes(const WtLayout& w) {
  return sizeof(T) * ((size_t)w.wend + w.wsz);
}

__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ void ld2(const float* p, float (&v)[2]) {
  const float2 q = *reinterpret_cast<const float2*>(p);
  v[0] = q.x; v[1] = q.y;
}
__device__ __forceinline__ void ld2(const double* p, double (&v)[2]) {
  const double2 q = *reinterpret_cast<const double2*>(p);
  v[0] = q.x; v[1] = q.y;
}

template <typename T, bool TANG>
__global__ void __launch_bounds__(WT_THREADS, 3) k_mlp_wgrad_tile(PotDevice pd, WgradArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = blockIdx.y;
  const NetTable& net = pd.sp[t].net;
  __shared__ WtLayout lay;   // indexed by layer at run time: keep it out of registers
  if (threadIdx.x == 0) lay = wt_layout(net, TANG);
  __syncthreads();
  const int L = lay.L;
  const int tid = threadIdx.x;
  T* S = reinterpret_cast<T*>(smem_raw);
  T* sdW = S + lay.wend;
  const int wbeg = net.w_off[0];
  const T* Wg = wsrc<T>(pd) + wbeg;
  for (int q = tid; q < lay.wend + lay.wsz; q += WT_THREADS) S[q] = T(0);
  __syncthreads();
  for (int l = 0; l + 1 < L; ++l) {
    const int nin = net.nnodes[l], nout = net.nnodes[l + 1], pitch = net.pitch[l];
    const T* Wl = Wg + (net.w_off[l] - wbeg);
    for (int q = tid; q < nout * (nin + 1); q += WT_THREADS) {
      const int o = q / (nin + 1), k = q - o * (nin + 1);
      const T v = Wl[o * pitch + k];
      S[lay.wr[l] + o * lay.pr[l] + k] = v;
      S[lay.wt[l] + k * lay.pt[l] + o] = v;
    }
    for (int r = tid; r < WT_P; r += WT_THREADS) S[(lay.x[l] + nin) * WT_P + r] = T(1);
  }
  const int beg = A.spec_off[t], nt = A.spec_off[t + 1] - beg;
  const int per = (nt + gridDim.x - 1) / gridDim.x;
  const int a0 = min(nt, blockIdx.x * per), a1 = min(nt, a0 + per);
  const T kappa = A.physical ? T(pd.sp[t].E_scale) : T(1);
  const int nsf_pad = pd.nsf_pad;
  const int n0 = net.nnodes[0];
  T* ZBo = S + lay.out * WT_P;
  T* ZDBo = ZBo + WT_P;
  T* CE = ZDBo + WT_P;
  const T* Gin = reinterpret_cast<const T*>(A.G);
  const T* Vin = reinterpret_cast<const T*>(A.V);
  // inputs of a tile (zero rows past its atoms) and the energy coefficients;
  // with few enough features the next tile's are loaded into registers
  // while the current tile is processed
  const bool pf = WT_TN * n0 <= WT_PF * WT_THREADS;
  T pg[WT_PF], pv[WT_PF], pce = T(0);
  auto fetch = [&](int tb1) {
    const int tn1 = min(WT_TN, a1 - tb1);
#pragma unroll
    for (int j = 0; j < WT_PF; ++j) {
      const int q = tid + j * WT_THREADS, r = q / n0, k = q - r * n0;
      pg[j] = pv[j] = T(0);
      if (q < WT_TN * n0 && r < tn1) {
        const size_t i = (size_t)A.order[beg + tb1 + r];
        pg[j] = Gin[i * nsf_pad + k];
        if (TANG) pv[j] = Vin[i * nsf_pad + k];
      }
    }
    if (tid < WT_TN) pce = tid < tn1 ? kappa * T(A.cE[A.atom_struct[A.order[beg + tb1 + tid]]]) : T(0);
  };
  if (pf && a0 < a1) fetch(a0);
  __syncthreads();

  for (int tb = a0; tb < a1; tb += WT_TN) {
    const int tn = min(WT_TN, a1 - tb);
    if (pf) {
#pragma unroll
      for (int j = 0; j < WT_PF; ++j) {
        const int q = tid + j * WT_THREADS, r = q / n0, k = q - r * n0;
        if (q < WT_TN * n0) {
          S[(lay.x[0] + k) * WT_P + r] = pg[j];
          if (TANG) S[(lay.xd[0] + k) * WT_P + r] = pv[j];
        }
      }
      if (tid < WT_TN) CE[tid] = pce;
      if (tb + WT_TN < a1) fetch(tb + WT_TN);
    } else {
      for (int q = tid; q < WT_TN * n0; q += WT_THREADS) {
        const int r = q / n0, k = q - r * n0;
        T g = T(0), v = T(0);
        if (r < tn) {
          const size_t i = (size_t)A.order[beg + tb + r];
          g = Gin[i * nsf_pad + k];
          if (TANG) v = Vin[i * nsf_pad + k];
        }
        S[(lay.x[0] + k) * WT_P + r] = g;
        if (TANG) S[(lay.xd[0] + k) * WT_P + r] = v;
      }
      if (tid < WT_TN)
        CE[tid] = tid < tn ? kappa * T(A.cE[A.atom_struct[A.order[beg + tb + tid]]]) : T(0);
    }
    __syncthreads();

    // ---- forward through the hidden layers
    for (int l = 0; l + 2 < L; ++l) {
      const int nin = net.nnodes[l], nout = net.nnodes[l + 1], fa = net.f_a[l + 1];
      const int items = (WT_TN / 4) * ((nout + 1) / 2);
      for (int it = tid; it < items; it += WT_THREADS) {
        const int r0 = 4 * (it % (WT_TN / 4)), o0 = 2 * (it / (WT_TN / 4));
        T z[2][4], zd[2][4];
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e) z[j][e] = zd[j][e] = T(0);
        const T* X = S + lay.x[l] * WT_P + r0;
        const T* Xd = S + lay.xd[l] * WT_P + r0;
        const T* Wt = S + lay.wt[l] + o0;
        for (int k = 0; k <= nin; ++k) {
          T x[4], w[2];
          ld4(X + k * WT_P, x);
          ld2(Wt + k * lay.pt[l], w);
#pragma unroll
          for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) z[j][e] = fma(w[j], x[e], z[j][e]);
          if (TANG) {
            T xd[4];
            ld4(Xd + k * WT_P, xd);
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
              for (int e = 0; e < 4; ++e) zd[j][e] = fma(w[j], xd[e], zd[j][e]);
          }
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int o = o0 + j;
          if (o >= nout) break;
          T y[4], d1[4], d2[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) activate2<T>(fa, z[j][e], y[e], d1[e], d2[e]);
          st4(S + (lay.x[l + 1] + o) * WT_P + r0, y);
          st4(S + (lay.s1[l + 1] + o) * WT_P + r0, d1);
          if (TANG) {
            T a[4], b[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              a[e] = d1[e] * zd[j][e];
              b[e] = d2[e] * zd[j][e];
            }
            st4(S + (lay.xd[l + 1] + o) * WT_P + r0, a);
            st4(S + (lay.s2[l + 1] + o) * WT_P + r0, b);
          }
        }
      }
      __syncthreads();
    }

    // ---- output node and its adjoints: four threads per atom
    {
      const int l = L - 2, nin = net.nnodes[l];
      const int r = tid >> 2, part = tid & 3;
      const T* X = S + lay.x[l] * WT_P + r;
      const T* Xd = S + lay.xd[l] * WT_P + r;
      const T* Wr = S + lay.wr[l];
      T z = T(0), zd = T(0);
      for (int k = part; k <= nin; k += 4) {
        z = fma(Wr[k], X[k * WT_P], z);
        if (TANG) zd = fma(Wr[k], Xd[k * WT_P], zd);
      }
#pragma unroll
      for (int d = 1; d < 4; d <<= 1) {
        z += __shfl_xor_sync(0xffffffffu, z, d);
        if (TANG) zd += __shfl_xor_sync(0xffffffffu, zd, d);
      }
      if (part == 0) {
        T y, d1, d2;
        activate2<T>(net.f_a[L - 1], z, y, d1, d2);
        const T ce = CE[r];
        const T cf = r < tn ? kappa * T(A.cF) : T(0);
        ZBo[r] = TANG ? ce * d1 + cf * d2 * zd : ce * d1;
        if (TANG) ZDBo[r] = cf * d1;
      }
      __syncthreads();
    }

    // ---- reverse: weight gradients of layer l, then the adjoints of its inputs
    for (int l = L - 2; l >= 0; --l) {
      const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
      const T* ZB = l == L - 2 ? ZBo : S + lay.s1[l + 1] * WT_P;
      const T* ZDB = l == L - 2 ? ZDBo : S + lay.s2[l + 1] * WT_P;
      const T* X = S + lay.x[l] * WT_P;
      const T* Xd = S + lay.xd[l] * WT_P;
      {
        // 4 nodes x 4 inputs per thread; the inputs of one thread are kn
        // apart so that neighbouring lanes read neighbouring rows (banks)
        const int kn = (nin + 1 + 3) / 4;
        const int items = ((nout + 3) / 4) * kn;
        T* dWl = sdW + (net.w_off[l] - wbeg);
        for (int it = tid; it < items; it += WT_THREADS) {
          const int o0 = 4 * (it / kn), k0 = it % kn;
          int orow[4], krow[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            orow[j] = min(o0 + j, nout - 1) * WT_P;
            krow[j] = min(k0 + j * kn, nin) * WT_P;
          }
          T acc[4][4];
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[j][c] = T(0);
#pragma unroll 2
          for (int r = 0; r < WT_TN; r += 4) {
            T x[4][4];
#pragma unroll
            for (int c = 0; c < 4; ++c) ld4(X + krow[c] + r, x[c]);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              T zb[4];
              ld4(ZB + orow[j] + r, zb);
#pragma unroll
              for (int c = 0; c < 4; ++c)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[j][c] = fma(zb[e], x[c][e], acc[j][c]);
            }
            if (TANG) {
#pragma unroll
              for (int c = 0; c < 4; ++c) ld4(Xd + krow[c] + r, x[c]);
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                T zb[4];
                ld4(ZDB + orow[j] + r, zb);
#pragma unroll
                for (int c = 0; c < 4; ++c)
#pragma unroll
                  for (int e = 0; e < 4; ++e) acc[j][c] = fma(zb[e], x[c][e], acc[j][c]);
              }
            }
          }
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < 4; ++c)
              if (o0 + j < nout && k0 + c * kn <= nin)
                dWl[(o0 + j) * net.pitch[l] + k0 + c * kn] += acc[j][c];
        }
      }
      if (l >= 1) {
        // adjoints of the nodes of X_l, written over their f' / f'' zd rows
        const int items = (WT_TN / 4) * ((nin + 1) / 2);
        for (int it = tid; it < items; it += WT_THREADS) {
          const int r0 = 4 * (it % (WT_TN / 4)), k0 = 2 * (it / (WT_TN / 4));
          T ab[2][4], adb[2][4];
#pragma unroll
          for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) ab[j][e] = adb[j][e] = T(0);
          const T* Wr = S + lay.wr[l] + k0;
          for (int o = 0; o < nout; ++o) {
            T zb[4], w[2];
            ld4(ZB + o * WT_P + r0, zb);
            ld2(Wr + o * lay.pr[l], w);
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
              for (int e = 0; e < 4; ++e) ab[j][e] = fma(w[j], zb[e], ab[j][e]);
            if (TANG) {
              ld4(ZDB + o * WT_P + r0, zb);
#pragma unroll
              for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) adb[j][e] = fma(w[j], zb[e], adb[j][e]);
            }
          }
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int k = k0 + j;
            if (k >= nin) break;
            T* s1 = S + (lay.s1[l] + k) * WT_P + r0;
            T* s2 = S + (lay.s2[l] + k) * WT_P + r0;
            T d1[4], v[4];
            ld4(s1, d1);
            if (TANG) {
              T d2z[4];
              ld4(s2, d2z);
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                v[e] = d1[e] * ab[j][e] + d2z[e] * adb[j][e];
                d2z[e] = d1[e] * adb[j][e];
              }
              st4(s2, d2z);
            } else {
#pragma unroll
              for (int e = 0; e < 4; ++e) v[e] = d1[e] * ab[j][e];
            }
            st4(s1, v);
          }
        }
      }
      __syncthreads();
    }
  }
  double* out = A.partial + ((size_t)t * gridDim.x + blockIdx.x) * A.wcap;
  for (int q = tid; q < A.wcap; q += WT_THREADS) out[q] = q < lay.wsz ? (double)sdW[q] : 0.0;
}

// sum the block partials (in block order) and write the gradient in the
// reference's W order: per species, per layer, column-major (nout, nin+1)
// with the bias in the last column (feedforward.f90:55-89)
__global__ void k_wgrad_reduce(PotDevice pd, int nblk, int wcap, const double* __restrict__ partial,
                               double* __restrict__ grad) {
  const int t = blockIdx.y;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const NetTable& net = pd.sp[t].net;
  const int L = net.nlayers;
  const int wbeg = net.w_off[0];
  const int wsz = net.w_off[L - 2] - wbeg + net.pitch[L - 2] * net.nnodes[L - 1];
  if (q >= wsz) return;
  // species offset in the flat reference vector
  size_t ref = 0;
  for (int u = 0; u < t; ++u) {
    const NetTable& nu = pd.sp[u].net;
    for (int l = 0; l + 1 < nu.nlayers; ++l) ref += (size_t)(nu.nnodes[l] + 1) * nu.nnodes[l + 1];
  }
  int l = 0;
  while (l + 2 < L && q >= net.w_off[l + 1] - wbeg) {
    ref += (size_t)(net.nnodes[l] + 1) * net.nnodes[l + 1];
    ++l;
  }
  const int rel = q - (net.w_off[l] - wbeg);
  const int o = rel / net.pitch[l], k = rel - o * net.pitch[l];
  const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
  if (k > nin || o >= nout) return;   // row padding
  double s = 0.0;
  const double* p = partial + (size_t)t * nblk * wcap + q;
  for (int b = 0; b < nblk; ++b) s += p[(size_t)b * wcap];
  grad[ref + o + (size_t)k * nout] = s;
}

}  // namespace

// ----------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------
int ae_part_scratch_ints(int natoms) { return 2 * AE_MAXT * ((natoms + PART_B - 1) / PART_B) + AE_MAXT + 1; }

int ae_launch_partition(int natoms, int ntypes, const int* types0, int* scratch, int* order,
                        int* spec_off, cudaStream_t s) {
  const int nblk = (natoms + PART_B - 1) / PART_B;
  if (nblk == 0) {
    cudaMemsetAsync(spec_off, 0, sizeof(int) * (ntypes + 1), s);
    return (int)cudaGetLastError();
  }
  int* bcnt = scratch;
  int* boff = scratch + AE_MAXT * nblk;
  k_part_count<<<nblk, PART_B, 0, s>>>(natoms, types0, bcnt);
  k_part_scan<<<1, 32 * AE_MAXT, 0, s>>>(nblk, ntypes, bcnt, boff, spec_off);
  k_part_scatter<<<nblk, PART_B, 0, s>>>(natoms, ntypes, types0, boff, order);
  return (int)cudaGetLastError();
}

int ae_launch_loss(int nstruc, const StructGeom* geom, const double* E_struct, const double* E_tgt,
                   const void* Facc, const double* F_tgt, int mode, double wE, double wF,
                   double E_scale, double* cE, void* U, double* loss_s, double* loss, int fp64,
                   cudaStream_t s) {
  const int blocks = (nstruc * 32 + 255) / 256;
  if (nstruc > 0) {
    if (fp64)
      k_loss<double><<<blocks, 256, 0, s>>>(nstruc, geom, E_struct, E_tgt, Facc, F_tgt, mode, wE, wF,
                                            E_scale, cE, U, loss_s);
    else
      k_loss<float><<<blocks, 256, 0, s>>>(nstruc, geom, E_struct, E_tgt, Facc, F_tgt, mode, wE, wF,
                                           E_scale, cE, U, loss_s);
  }
  k_loss_sum<<<1, 1024, 0, s>>>(nstruc, loss_s, loss);
  return (int)cudaGetLastError();
}

// size of the per-block gradient rows (elements) for the loaded networks
int ae_wgrad_wcap(const PotDevice& pd) {
  int w = 0;
  for (int t = 0; t < pd.ntypes; ++t) w = max(w, wg_layout(pd.sp[t].net, false).wsz);
  return (w + 31) & ~31;
}

// blocks per species: about three resident blocks (the shared-memory limit
// of the kernel) on every SM over all species, at least 96
int ae_wgrad_nblk(int ntypes) {
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return max(96, (3 * nsm + ntypes - 1) / max(1, ntypes));
}

int ae_launch_mlp_wgrad(const PotDevice& pd, const int* order, const int* spec_off, const void* G,
                        const void* V, const int* atom_struct, const double* cE, double cF,
                        int physical, double* partial, double* grad, int fp64, cudaStream_t s) {
  const int warps = 8, nblk = ae_wgrad_nblk(pd.ntypes);
  const bool tang = V != nullptr;
  WgradArgs A{};
  A.ntypes = pd.ntypes;
  A.order = order;
  A.spec_off = spec_off;
  A.G = G;
  A.V = V;
  A.atom_struct = atom_struct;
  A.cE = cE;
  A.cF = cF;
  A.physical = physical;
  A.partial = partial;
  A.wcap = ae_wgrad_wcap(pd);
  for (int t = 0; t < pd.ntypes; ++t)
    if (pd.sp[t].net.nnodes[pd.sp[t].net.nlayers - 1] != 1 || pd.sp[t].net.nlayers < 2)
      return (int)cudaErrorInvalidValue;
  dim3 grid(nblk, pd.ntypes);
  dim3 rgrid((A.wcap + 255) / 256, pd.ntypes);
  // tile kernel when its shared memory fits every species
  size_t tneed = 0;
  for (int t = 0; t < pd.ntypes; ++t) {
    const WtLayout w = wt_layout(pd.sp[t].net, tang);
    const size_t b = fp64 ? wt_smem_bytes<double>(w) : wt_smem_bytes<float>(w);
    tneed = tneed > b ? tneed : b;
  }
  if (tneed + AE_STATIC_SMEM <= 200 * 1024) {
    auto go_tile = [&](auto kern) {
      if (tneed + AE_STATIC_SMEM > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tneed);
      kern<<<grid, WT_THREADS, tneed, s>>>(pd, A);
    };
    if (fp64) {
      if (tang) go_tile(k_mlp_wgrad_tile<double, true>);
      else go_tile(k_mlp_wgrad_tile<double, false>);
    } else {
      if (tang) go_tile(k_mlp_wgrad_tile<float, true>);
      else go_tile(k_mlp_wgrad_tile<float, false>);
    }
    k_wgrad_reduce<<<rgrid, 256, 0, s>>>(pd, nblk, A.wcap, partial, grad);
    return (int)cudaGetLastError();
  }
  // otherwise one warp per atom: the largest tile whose shared memory fits
  size_t need = 0;
  int tile = 32;
  for (; tile >= 4; tile /= 2) {
    need = 0;
    for (int t = 0; t < pd.ntypes; ++t) {
      WgLayout w = wg_layout(pd.sp[t].net, tang);
      size_t b = fp64 ? wg_smem_bytes<double>(w, tile, warps) : wg_smem_bytes<float>(w, tile, warps);
      need = need > b ? need : b;
    }
    if (need <= 200 * 1024) break;
  }
  if (tile < 4) return (int)cudaErrorInvalidValue;
  A.tile = tile;
  auto go = [&](auto kern) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need);
    kern<<<grid, warps * 32, need, s>>>(pd, A);
  };
  if (fp64) {
    if (tang) go(k_mlp_wgrad<double, true>);
    else go(k_mlp_wgrad<double, false>);
  } else {
    if (tang) go(k_mlp_wgrad<float, true>);
    else go(k_mlp_wgrad<float, false>);
  }
  k_wgrad_reduce<<<rgrid, 256, 0, s>>>(pd, nblk, A.wcap, partial, grad);
  return (int)cudaGetLastError();
}
