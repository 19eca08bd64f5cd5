// Molecular dynamics on the GPU: velocity Verlet with a Verlet skin
// (the integrator ASE's VelocityVerlet applies in python3/scripts/aenet-md.py:72-97,
// with the forces of the ANN potential).
//
// Units: positions A, velocities A/fs, forces eV/A, masses amu, time fs;
// acceleration = F / m * ACC, ACC = 1 / (amu A^2 fs^-2 in eV).
//
// Skin: the neighbour table is built with the cut-off Rc + skin and keeps
// the lattice image T of every pair (relative to the wrapped coordinates
// of that build).  Between builds the pair vectors are refreshed from the
// current positions,
//     R_ij = (r_j + S_j) - (r_i + S_i) + T L,    S = r_wrapped - r at the build,
// and the descriptor kernels skip pairs beyond their cut-offs.  The table
// is rebuilt when an atom has moved more than skin/2 since the build.
#include "common.h"

namespace {

__global__ void k_kick_drift(int n, double* __restrict__ pos, double* __restrict__ vel,
                             const double* __restrict__ F, const double* __restrict__ invm,
                             double half_dt_acc, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = half_dt_acc * invm[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double v = vel[3 * i + c] + a * F[3 * i + c];
    vel[3 * i + c] = v;
    pos[3 * i + c] += dt * v;
  }
}

__global__ void k_kick(int n, double* __restrict__ vel, const double* __restrict__ F,
                       const double* __restrict__ invm, double half_dt_acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = half_dt_acc * invm[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) vel[3 * i + c] += a * F[3 * i + c];
}

// flag = 1 when any atom moved more than sqrt(lim2) since the last build
__global__ void k_displacement(int n, const double* __restrict__ pos, const double* __restrict__ rb,
                               double lim2, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool far = false;
  if (i < n) {
    const double dx = pos[3 * i] - rb[3 * i], dy = pos[3 * i + 1] - rb[3 * i + 1],
                 dz = pos[3 * i + 2] - rb[3 * i + 2];
    far = !(dx * dx + dy * dy + dz * dz <= lim2);   // NaN counts as far
  }
  if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicExch(flag, 1);
}

__global__ void k_after_build(int n, const double* __restrict__ pos, const double* __restrict__ r_wrap,
                              double* __restrict__ S, double* __restrict__ rb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    S[3 * i + c] = r_wrap[3 * i + c] - pos[3 * i + c];
    rb[3 * i + c] = pos[3 * i + c];
  }
}

__device__ __forceinline__ int sext10(int v) { return (v ^ 512) - 512; }

template <typename T4>
__device__ __forceinline__ void store_vec(void* base, size_t k, double x, double y, double z, double d);
template <>
__device__ __forceinline__ void store_vec<float4>(void* base, size_t k, double x, double y, double z,
                                                  double d) {
  reinterpret_cast<float4*>(base)[k] = make_float4((float)x, (float)y, (float)z, (float)d);
}
template <>
__device__ __forceinline__ void store_vec<double4_32a>(void* base, size_t k, double x, double y,
                                                       double z, double d) {
  reinterpret_cast<double4_32a*>(base)[k] = make_double4_32a(x, y, z, d);
}

// one warp per atom, lanes over its table slots
template <typename T4>
__global__ void k_refresh(int n, const StructGeom* __restrict__ geom, const int* __restrict__ atom_struct,
                          const double* __restrict__ pos, const double* __restrict__ S, int cap,
                          const int* __restrict__ nb_cnt, const int* __restrict__ nb_jt,
                          const int* __restrict__ nb_img, void* nb_vec) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const StructGeom& g = geom[atom_struct[i]];
  const double pi0 = pos[3 * i] + S[3 * i], pi1 = pos[3 * i + 1] + S[3 * i + 1],
               pi2 = pos[3 * i + 2] + S[3 * i + 2];
  const int cnt = nb_cnt[i];
  const size_t row = (size_t)i * cap;
  for (int k = lane; k < cnt; k += 32) {
    const int j = nb_jt[row + k] & AE_INDEX_MASK;
    const int im = nb_img[row + k];
    const double t0 = sext10(im & 1023), t1 = sext10((im >> 10) & 1023), t2 = sext10((im >> 20) & 1023);
    double R[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double pj = pos[3 * j + c] + S[3 * j + c];
      const double pi = c == 0 ? pi0 : (c == 1 ? pi1 : pi2);
      R[c] = (pj - pi) + (g.pbc ? t0 * g.L[c] + t1 * g.L[3 + c] + t2 * g.L[6 + c] : 0.0);
    }
    const double d = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
    store_vec<T4>(nb_vec, row + k, R[0], R[1], R[2], d);
  }
}

// FP32 refresh of the mixed path: positions in the frame of the last build
// rounded to float once per step, vectors formed as the neighbour search
// forms them, (p_j - p_i) + T L in FP32
__global__ void k_shifted_f32(int n, const double* __restrict__ pos, const double* __restrict__ S,
                              float4* __restrict__ p32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p32[i] = make_float4((float)(pos[3 * i] + S[3 * i]), (float)(pos[3 * i + 1] + S[3 * i + 1]),
                       (float)(pos[3 * i + 2] + S[3 * i + 2]), 0.f);
}

__global__ void k_refresh_f32(int n, const StructGeom* __restrict__ geom,
                              const int* __restrict__ atom_struct, const float4* __restrict__ p32,
                              int cap, const int* __restrict__ nb_cnt, const int* __restrict__ nb_jt,
                              const int* __restrict__ nb_img, float4* __restrict__ nb_vec) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const StructGeom& g = geom[atom_struct[i]];
  const float4 pi = p32[i];
  const int cnt = nb_cnt[i];
  const size_t row = (size_t)i * cap;
  for (int k = lane; k < cnt; k += 32) {
    const int j = nb_jt[row + k] & AE_INDEX_MASK;
    const int im = nb_img[row + k];
    const float f0 = (float)sext10(im & 1023), f1 = (float)sext10((im >> 10) & 1023),
                f2 = (float)sext10((im >> 20) & 1023);
    const float4 pj = p32[j];
    float sh0 = 0.f, sh1 = 0.f, sh2 = 0.f;
    if (g.pbc) {
      sh0 = f0 * g.Lf[0] + f1 * g.Lf[3] + f2 * g.Lf[6];
      sh1 = f0 * g.Lf[1] + f1 * g.Lf[4] + f2 * g.Lf[7];
      sh2 = f0 * g.Lf[2] + f1 * g.Lf[5] + f2 * g.Lf[8];
    }
    const float dx = (pj.x - pi.x) + sh0, dy = (pj.y - pi.y) + sh1, dz = (pj.z - pi.z) + sh2;
    nb_vec[row + k] = make_float4(dx, dy, dz, sqrtf(dx * dx + dy * dy + dz * dz));
  }
}

// kinetic energy: per-block partial sums (fixed order), then one block
__global__ void k_ekin_part(int n, const double* __restrict__ vel, const double* __restrict__ invm,
                            double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v2 = vel[3 * i] * vel[3 * i] + vel[3 * i + 1] * vel[3 * i + 1] +
                      vel[3 * i + 2] * vel[3 * i + 2];
    s += v2 / invm[i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_ekin_sum(int nb, const double* __restrict__ part, double half_mass_unit,
                           double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) s += part[q];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = half_mass_unit * sh[0];
}

}  // namespace

int ae_md_kick_drift(int n, double* pos, double* vel, const double* F, const double* invm,
                     double half_dt_acc, double dt, cudaStream_t s) {
  if (n > 0) k_kick_drift<<<(n + 255) / 256, 256, 0, s>>>(n, pos, vel, F, invm, half_dt_acc, dt);
  return (int)cudaGetLastError();
}

int ae_md_kick(int n, double* vel, const double* F, const double* invm, double half_dt_acc,
               cudaStream_t s) {
  if (n > 0) k_kick<<<(n + 255) / 256, 256, 0, s>>>(n, vel, F, invm, half_dt_acc);
  return (int)cudaGetLastError();
}

int ae_md_displacement(int n, const double* pos, const double* rb, double lim2, int* flag,
                       cudaStream_t s) {
  if (cudaMemsetAsync(flag, 0, sizeof(int), s)) return (int)cudaErrorUnknown;
  if (n > 0) k_displacement<<<(n + 255) / 256, 256, 0, s>>>(n, pos, rb, lim2, flag);
  return (int)cudaGetLastError();
}

int ae_md_after_build(int n, const double* pos, const double* r_wrap, double* S, double* rb,
                      cudaStream_t s) {
  if (n > 0) k_after_build<<<(n + 255) / 256, 256, 0, s>>>(n, pos, r_wrap, S, rb);
  return (int)cudaGetLastError();
}

int ae_md_refresh(int n, const StructGeom* geom, const int* atom_struct, const double* pos,
                  const double* S, int cap, const int* nb_cnt, const int* nb_jt, const int* nb_img,
                  void* nb_vec, int fp64, cudaStream_t s) {
  if (n <= 0) return 0;
  const int blocks = (int)(((size_t)n * 32 + 255) / 256);
  if (fp64)
    k_refresh<double4_32a><<<blocks, 256, 0, s>>>(n, geom, atom_struct, pos, S, cap, nb_cnt, nb_jt,
                                                  nb_img, nb_vec);
  else
    k_refresh<float4><<<blocks, 256, 0, s>>>(n, geom, atom_struct, pos, S, cap, nb_cnt, nb_jt,
                                             nb_img, nb_vec);
  return (int)cudaGetLastError();
}

int ae_md_refresh_f32(int n, const StructGeom* geom, const int* atom_struct, const double* pos,
                      const double* S, float4* p32, int cap, const int* nb_cnt, const int* nb_jt,
                      const int* nb_img, void* nb_vec, cudaStream_t s) {
  if (n <= 0) return 0;
  k_shifted_f32<<<(n + 255) / 256, 256, 0, s>>>(n, pos, S, p32);
  k_refresh_f32<<<(int)(((size_t)n * 32 + 255) / 256), 256, 0, s>>>(
      n, geom, atom_struct, p32, cap, nb_cnt, nb_jt, nb_img, reinterpret_cast<float4*>(nb_vec));
  return (int)cudaGetLastError();
}

int ae_md_ekin_blocks() { return 304; }

int ae_md_ekin(int n, const double* vel, const double* invm, double* part, double half_mass_unit,
               double* out, cudaStream_t s) {
  k_ekin_part<<<ae_md_ekin_blocks(), 256, 0, s>>>(n, vel, invm, part);
  k_ekin_sum<<<1, 256, 0, s>>>(ae_md_ekin_blocks(), part, half_mass_unit, out);
  return (int)cudaGetLastError();
}
