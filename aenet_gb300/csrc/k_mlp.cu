// Per-species feed-forward networks: energy and dE/dG (replaces ff_eval /
// ff_deriv of src/ext/feedforward.f90:586-757 and the energy assembly of
// src/aenet.f90:464-469), plus the per-structure energy reduction and the
// force output conversion.
//
// Weights of every species are staged once per block in shared memory;
// blocks are persistent (grid-stride over atoms), one warp per atom, lane o
// computing node o of a layer.  Rows of a layer's weight matrix are stored
// W[o][k] with the bias in column n_in and an odd row pitch, so that both
// the forward pass (lanes over rows) and the backward pass (lanes over
// columns) read shared memory without bank conflicts.
//
// dE/dG is written already multiplied by E_scale and by the descriptor
// normalisation scale 1/s (sfsetup.f90:1010-1031): the adjoint kernels
// contract it with the derivatives of the raw descriptor.
#include "common.h"
#include "activate.cuh"

namespace {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

template <typename T>
__device__ __forceinline__ T nscale(const PotDevice& pd, size_t k);
template <>
__device__ __forceinline__ float nscale<float>(const PotDevice& pd, size_t k) { return pd.scale32[k]; }
template <>
__device__ __forceinline__ double nscale<double>(const PotDevice& pd, size_t k) { return pd.scale[k]; }

__host__ __device__ constexpr int mlp_warp_elems() {
  return 2 * (AE_MAXNSF + 1) + 2 * AE_MAXLAYERS * (AE_MAXNODES + 1) + 1;
}

template <typename T>
__global__ void __launch_bounds__(256) k_mlp(PotDevice pd, DescBuffers b, const T* __restrict__ W,
                                             int wtotal) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sW = reinterpret_cast<T*>(smem_raw);
  const int warps = blockDim.x >> 5;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  for (int q = threadIdx.x; q < wtotal; q += blockDim.x) sW[q] = W[q];
  // per warp: input features and their gradient (up to AE_MAXNSF), then
  // activations and derivatives of layers 1 .. L-1 (up to AE_MAXNODES)
  const int stride = AE_MAXNODES + 1;
  T* xin = sW + ((wtotal + 1) & ~1) + (size_t)warp * mlp_warp_elems();
  T* gin = xin + (AE_MAXNSF + 1);
  T* act = gin + (AE_MAXNSF + 1);
  T* der = act + AE_MAXLAYERS * stride;
  __syncthreads();

  for (int i = blockIdx.x * warps + warp; i < b.natoms; i += gridDim.x * warps) {
    const int ti = b.types[i];
    const SpeciesTable& sp = pd.sp[ti];
    const NetTable& net = sp.net;
    const int nsf = sp.nsf;
    const T* G = reinterpret_cast<const T*>(b.G) + (size_t)i * pd.nsf_pad;
    for (int k = lane; k < nsf; k += 32) xin[k] = G[k];
    __syncwarp();
    T y = T(0);
    const int L = net.nlayers;
    for (int l = 0; l < L - 1; ++l) {
      const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
      const T* Wl = sW + net.w_off[l];
      const int pitch = net.pitch[l];
      const T* hin = (l == 0) ? xin : act + l * stride;
      T* hout = act + (l + 1) * stride;
      T* dout = der + (l + 1) * stride;
      if (nout == 1) {
        T part = T(0);
        for (int k = lane; k < nin; k += 32) part += Wl[k] * hin[k];
        part = warp_sum(part) + Wl[nin];
        T yy, dy;
        activate<T>(net.f_a[l + 1], part, yy, dy);
        if (lane == 0) {
          hout[0] = yy;
          dout[0] = dy;
        }
        y = yy;
      } else {
        for (int o = lane; o < nout; o += 32) {
          const T* row = Wl + o * pitch;
          T z = row[nin];
          for (int k = 0; k < nin; ++k) z += row[k] * hin[k];
          T yy, dy;
          activate<T>(net.f_a[l + 1], z, yy, dy);
          hout[o] = yy;
          dout[o] = dy;
        }
      }
      __syncwarp();
    }
    // backward: delta of the output node (dE/dy = 1 times f'(z_out)), then
    // delta_l = (W_l^T delta_{l+1}) * f'_l down to the inputs
    const T* delta_cur = der + (L - 1) * stride;
    for (int l = L - 2; l >= 0; --l) {
      const int nin = net.nnodes[l], nout = net.nnodes[l + 1];
      const T* Wl = sW + net.w_off[l];
      const int pitch = net.pitch[l];
      T* dl = (l == 0) ? gin : der + l * stride;
      for (int k = lane; k < nin; k += 32) {
        T s = T(0);
        for (int o = 0; o < nout; ++o) s += Wl[o * pitch + k] * delta_cur[o];
        dl[k] = (l > 0) ? s * dl[k] : s;
      }
      __syncwarp();
      delta_cur = dl;
    }
    // delta_cur = dE/dG (normalised inputs)
    T* out = reinterpret_cast<T*>(b.dEdG) + (size_t)i * pd.nsf_pad;
    const T es = T(sp.E_scale);
    for (int k = lane; k < nsf; k += 32)
      out[k] = es * delta_cur[k] * nscale<T>(pd, (size_t)ti * pd.nsf_pad + k);
    if (lane == 0) b.E_atom[i] = sp.E_scale * (double)y + sp.E_shift + sp.E_atom;
    __syncwarp();
  }
}

// Per-structure energy with Neumaier-compensated FP64 summation: one warp
// per structure, each lane sums a strided subset, then the (sum,
// compensation) pairs are combined by a butterfly of two-sums.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__global__ void k_energy_reduce(int nstruc, const StructGeom* geom, const double* __restrict__ E_atom,
                                double* __restrict__ E_struct) {
  const int lane = threadIdx.x & 31;
  const int sidx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (sidx >= nstruc) return;
  const StructGeom& g = geom[sidx];
  double s = 0.0, c = 0.0;
  for (int a = lane; a < g.natoms; a += 32) {
    double t, e;
    two_sum(s, E_atom[g.atom_off + a], t, e);
    s = t;
    c += e;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    double so = __shfl_xor_sync(0xffffffffu, s, d);
    double co = __shfl_xor_sync(0xffffffffu, c, d);
    double t, e;
    two_sum(s, so, t, e);
    s = t;
    c = c + co + e;
  }
  if (lane == 0) E_struct[sidx] = s + c;
}

// chunk c of the structure whose chunk range contains it
__global__ void k_energy_chunks(int nstruc, int nchunks, const StructGeom* __restrict__ geom,
                                const int* __restrict__ chunk_struct,
                                const double* __restrict__ E_atom, double2* __restrict__ part,
                                double* __restrict__ E_struct) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= nchunks) return;
  const int sidx = chunk_struct[c];
  const StructGeom& g = geom[sidx];
  const int a0 = (c - g.chunk_off) * AE_ECHUNK;
  const int a1 = min(g.natoms, a0 + AE_ECHUNK);
  // pairwise order (a lane's run, then a tree over the lanes): the rounding
  // error stays within (AE_ECHUNK/32 + 5) ulp of sum |E_i|
  double s = 0.0;
  for (int a = a0 + lane; a < a1; a += 32) s += E_atom[g.atom_off + a];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if (lane == 0) {
    part[c] = make_double2(s, 0.0);
    if (g.natoms <= AE_ECHUNK) E_struct[sidx] = s;   // single chunk: final already
  }
}

// one warp per structure over its chunks
__global__ void k_energy_struct(int nstruc, int nchunks, const StructGeom* __restrict__ geom,
                                const double2* __restrict__ part, double* __restrict__ E_struct) {
  const int lane = threadIdx.x & 31;
  const int sidx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (sidx >= nstruc) return;
  const int c0 = geom[sidx].chunk_off;
  const int c1 = sidx + 1 < nstruc ? geom[sidx + 1].chunk_off : nchunks;
  if (c1 - c0 == 1) return;   // written by k_energy_chunks
  if (c1 == c0) {
    if (lane == 0) E_struct[sidx] = 0.0;
    return;
  }
  double s = 0.0;
  for (int c = c0 + lane; c < c1; c += 32) s += part[c].x;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if (lane == 0) E_struct[sidx] = s;
}

template <typename T>
__global__ void k_forces_out(int natoms, const T* __restrict__ Facc, double* __restrict__ F,
                             double f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  F[3 * i] = f * (double)Facc[4 * i];
  F[3 * i + 1] = f * (double)Facc[4 * i + 1];
  F[3 * i + 2] = f * (double)Facc[4 * i + 2];
}

__global__ void k_types(int natoms, const int* __restrict__ t1, int* __restrict__ t0, int ntypes,
                        unsigned* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  int t = t1[i] - 1;
  if (t < 0 || t >= ntypes) {
    atomicOr(status, AE_ST_BAD_TYPE);
    t = 0;
  }
  t0[i] = t;
}

// FP32 FMA throughput probe: independent FMA chains per thread, enough
// blocks to fill every SM.  Used only to measure the denominator of the
// FP32 roofline of the descriptor kernels.
__global__ void k_fma_peak(float* out, int iters, float seed) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.999999f, c = 1e-7f;
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 12345.678f) out[blockIdx.x] = r;
}

}  // namespace

int ae_fma_peak(double* tflops, cudaStream_t s) {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  float* out = nullptr;
  if (cudaMalloc(&out, 4096 * sizeof(float)) != cudaSuccess) return 1;
  const int blocks = nsm * 8, threads = 256, iters = 4096;
  k_fma_peak<<<blocks, threads, 0, s>>>(out, 16, 1.f);   // warm-up
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, s);
    k_fma_peak<<<blocks, threads, 0, s>>>(out, iters, 1.f);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return (int)cudaGetLastError();
}

int ae_launch_types(int natoms, const int* types1, int* types0, int ntypes, unsigned* status,
                    cudaStream_t s) {
  if (natoms <= 0) return 0;
  k_types<<<(natoms + 255) / 256, 256, 0, s>>>(natoms, types1, types0, ntypes, status);
  return (int)cudaGetLastError();
}

int ae_launch_mlp(const PotDevice& pd, const DescBuffers& b, int fp64, cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  int wtotal = 0;
  for (int t = 0; t < pd.ntypes; ++t) wtotal = max(wtotal, pd.sp[t].net.wtotal);
  const int warps = 8;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t tsz = fp64 ? sizeof(double) : sizeof(float);
  size_t smem = tsz * (((size_t)wtotal + 1) & ~(size_t)1) + tsz * (size_t)warps * mlp_warp_elems();
  int blocks = (b.natoms + warps - 1) / warps;
  int maxb = nsm * 4;
  if (blocks > maxb) blocks = maxb;
  if (fp64) {
    if (smem + AE_STATIC_SMEM > 48 * 1024)
      cudaFuncSetAttribute(k_mlp<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mlp<double><<<blocks, warps * 32, smem, s>>>(pd, b, pd.w64, wtotal);
  } else {
    if (smem + AE_STATIC_SMEM > 48 * 1024)
      cudaFuncSetAttribute(k_mlp<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mlp<float><<<blocks, warps * 32, smem, s>>>(pd, b, pd.w32, wtotal);
  }
  return (int)cudaGetLastError();
}

int ae_launch_energy_reduce_chunked(int nstruc, int nchunks, const StructGeom* geom,
                                    const int* chunk_struct, const double* E_atom, double2* part,
                                    double* E_struct, int one_chunk_each, cudaStream_t s) {
  if (nstruc <= 0) return 0;
  if (nchunks > 0)
    k_energy_chunks<<<(nchunks + 7) / 8, 256, 0, s>>>(nstruc, nchunks, geom, chunk_struct, E_atom,
                                                      part, E_struct);
  if (!one_chunk_each)
    k_energy_struct<<<(nstruc + 7) / 8, 256, 0, s>>>(nstruc, nchunks, geom, part, E_struct);
  return (int)cudaGetLastError();
}

int ae_launch_energy_reduce(int nstruc, const StructGeom* geom, const double* E_atom,
                            double* E_struct, cudaStream_t s) {
  if (nstruc <= 0) return 0;
  k_energy_reduce<<<(nstruc + 7) / 8, 256, 0, s>>>(nstruc, geom, E_atom, E_struct);
  return (int)cudaGetLastError();
}

int ae_launch_forces_out(int natoms, const void* Facc, int fp64, double* F, double sign,
                         cudaStream_t s) {
  if (natoms <= 0) return 0;
  if (fp64)
    k_forces_out<double><<<(natoms + 255) / 256, 256, 0, s>>>(natoms, (const double*)Facc, F, sign);
  else
    k_forces_out<float><<<(natoms + 255) / 256, 256, 0, s>>>(natoms, (const float*)Facc, F, sign);
  return (int)cudaGetLastError();
}
