// Reference neighbour order and stale spins of the Chebyshev angular terms.
//
// sfb_eval (src/ext/sfbasis.f90:489-566) weighs the spin block of the pair
// (j, k), k after j in its neighbour list, with s_j s_k, where s_k is k's
// typespin but s_j is refreshed only inside the radial branch (line 514):
// for a neighbour beyond the radial cut-off (possible when a_Rc > r_Rc)
// s_j is the spin of the last earlier neighbour inside it, or 1 before any.
// The result depends on the order of the list, which for predict.x is the
// order lcl_nbdist_cart produces (src/ext/lclist.f90:520-677): the atom's
// own periodic images first, then every other atom in ascending index, each
// with its home copy before its images, the images in the loop order of
// translation_vectors (i3, i2, i1 with i1 fastest, lclist.f90:1302-1375).
//
// k_stale_order (one warp per atom) ranks the slots of each table row in
// that order -- or, for rows built from a caller's list (the per-atom
// libaenet calls, an MD engine's neighbour lists), in the caller's order,
// which is the slot order -- and writes per slot the rank and s_eff; the
// pair-form descriptor kernels then weigh each pair with s_eff(first)
// s(second).
#include "common.h"

namespace {

constexpr double TWO_PI_O = 6.283185307179586;
constexpr double SFB_EPS_O = 1.0e-12;

template <typename T4>
__global__ void __launch_bounds__(128) k_stale_order(int natoms, const StructGeom* __restrict__ geom,
                                                     const int* __restrict__ atom_struct,
                                                     const double* __restrict__ r_wrap,
                                                     PotDevice pd, DescBuffers b,
                                                     int caller_order, int* __restrict__ rank,
                                                     float* __restrict__ seff) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= natoms) return;
  const int cap = b.cap;
  // per block: keys [warps][cap] (u64), ranks [warps][cap], pass spins [warps][cap]
  const size_t wc = (size_t)(blockDim.x >> 5) * cap;
  unsigned long long* key0 = reinterpret_cast<unsigned long long*>(smem_raw);
  int* rank0 = reinterpret_cast<int*>(key0 + wc);
  float* pass0 = reinterpret_cast<float*>(rank0 + wc);
  unsigned long long* key = key0 + (size_t)warp * cap;
  int* srank = rank0 + (size_t)warp * cap;
  float* spass = pass0 + (size_t)warp * cap;
  const int n = min(b.nb_cnt[i], cap);
  const size_t row = (size_t)i * cap;
  const int ti = b.types[i];
  const ChebTable& ct = pd.sp[ti].cheb;
  const T4* __restrict__ vec = reinterpret_cast<const T4*>(b.nb_vec) + row;
  const int* __restrict__ jt = b.nb_jt + row;
  for (int q = lane; q < n; q += 32) {
    const T4 v = vec[q];
    const int j = jt[q] & AE_INDEX_MASK;
    const int tj = jt[q] >> AE_TYPE_SHIFT;
    const double d = (double)v.w;
    // the radial branch of sfb_eval refreshes s_j: the slot's spin if it
    // passes, NaN otherwise
    spass[q] = (d <= ct.r_Rc && d > SFB_EPS_O) ? ct.spin[tj] : __int_as_float(0x7fc00000);
    if (caller_order) {
      key[q] = (unsigned long long)q;
      continue;
    }
    const StructGeom& g = geom[atom_struct[i]];
    int T[3] = {0, 0, 0};
    if (g.pbc) {
      // R_ij = L (s_j + T) - L s_i, so L T = R_ij - (r_j - r_i) on the
      // wrapped coordinates and T = B (L T) / (2 pi), an integer
      const double d0 = (double)v.x - (r_wrap[3 * j] - r_wrap[3 * i]);
      const double d1 = (double)v.y - (r_wrap[3 * j + 1] - r_wrap[3 * i + 1]);
      const double d2 = (double)v.z - (r_wrap[3 * j + 2] - r_wrap[3 * i + 2]);
      for (int a = 0; a < 3; ++a)
        T[a] = (int)rint((g.B[3 * a] * d0 + g.B[3 * a + 1] * d1 + g.B[3 * a + 2] * d2) / TWO_PI_O);
    }
    const unsigned long long primary = (j == i) ? 0ull : (unsigned long long)(j - g.atom_off + 1);
    const bool home = T[0] == 0 && T[1] == 0 && T[2] == 0;
    const unsigned long long secondary =
        home ? 0ull
             : 1ull + ((unsigned long long)(T[2] + 512) * 1024ull + (unsigned long long)(T[1] + 512)) *
                          1024ull +
                   (unsigned long long)(T[0] + 512);
    key[q] = (primary << 32) | secondary;
  }
  __syncwarp();
  for (int q = lane; q < n; q += 32) {
    const unsigned long long kq = key[q];
    int r = 0;
    for (int p = 0; p < n; ++p) r += key[p] < kq ? 1 : 0;
    srank[q] = r;
  }
  __syncwarp();
  // s_eff of a slot: the spin of the last slot up to it (in rank order) that
  // passed the radial branch, 1 before any
  for (int q = lane; q < n; q += 32) {
    const int rq = srank[q];
    int best = -1;
    float s = 1.0f;
    for (int p = 0; p < n; ++p) {
      const int rp = srank[p];
      const float sp = spass[p];
      if (rp <= rq && rp > best && sp == sp) {
        best = rp;
        s = sp;
      }
    }
    rank[row + q] = rq;
    seff[row + q] = s;
  }
}

}  // namespace

int ae_launch_stale_order(int natoms, const StructGeom* geom, const int* atom_struct,
                          const double* r_wrap, const PotDevice& pd, const DescBuffers& b,
                          int fp64, int caller_order, int* rank, float* seff, cudaStream_t s) {
  if (natoms <= 0) return 0;
  const int warps = 4;
  const size_t smem = (size_t)warps * b.cap * (8 + 4 + 4);
  if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
  const int blocks = (natoms + warps - 1) / warps;
  if (fp64) {
    auto kern = k_stale_order<double4_32a>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, s>>>(natoms, geom, atom_struct, r_wrap, pd, b, caller_order,
                                          rank, seff);
  } else {
    auto kern = k_stale_order<float4>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, s>>>(natoms, geom, atom_struct, r_wrap, pd, b, caller_order,
                                          rank, seff);
  }
  return (int)cudaGetLastError();
}
