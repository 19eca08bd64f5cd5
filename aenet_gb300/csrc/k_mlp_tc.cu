// Tensor-core (tcgen05) networks of the mixed-precision path: energy and
// dE/dG of every atom for networks with two hidden layers (replaces
// ff_eval / ff_deriv of src/ext/feedforward.f90:586-757 and the energy
// assembly of src/aenet.f90:464-469; same results as k_mlp within the
// mixed-precision tolerance).
//
// One CTA (128 threads, one warpgroup) per tile of 128 atoms of one
// species; thread m owns atom row m, which is TMEM lane m of the FP32
// accumulator.  Per tile, four MMA rounds (M = 128, K-major BF16 operands
// in shared memory, accumulator in TMEM):
//   z1 = X W1^T          X = normalised descriptors         N = h
//   z2 = a1 W2^T         a1 = f1(z1 + b1)                   N = h
//   d1 = g2 W2           g2 = f3'(z3) w3 * f2'(z2 + b2)     N = h
//   gin = (d1 * f1') W1                                     N = kin
// with y = f3(w3 . a2 + b3) and dE/dG = E_scale * gin / s (the adjoint
// contracts it with the raw descriptor derivatives).  Activations and
// derivatives stay in registers; only the MMA operands go through shared
// memory.  Every operand is split x = hi + lo into two BF16 values and a
// product is accumulated as hi*hi + hi*lo + lo*hi (three MMAs per K-step,
// ~16 significant bits; plain BF16 would give errors near 10 meV/atom).
//
// Waits on the MMA-completion mbarrier are bounded; on a time-out the CTA
// sets AE_ST_TC_TIMEOUT, waits (bounded) once more for its MMAs, frees its
// TMEM and returns.
#include <cuda_bf16.h>

#include "common.h"

namespace {

constexpr int TILE = 128;
constexpr uint32_t TMEM_COLS = 64;
constexpr int WAIT_LIMIT = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of this architecture
  return d;                 // base offset 0, relative LBO, layout type 0 (no swizzle)
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                    uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int it = 0; it < WAIT_LIMIT; ++it)
    if (mbar_try_wait(mbar, parity)) return true;
  return false;
}

// 32 consecutive FP32 columns of this thread's TMEM lane.  The load and
// its wait are one asm statement: the destination registers are written
// asynchronously, so no instruction may read them before the wait, and
// the compiler only orders uses after the statement that defines them.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%"
      "15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float* v) {
#pragma unroll
  for (int c = 0; c < N; c += 32) tmem_ld32(taddr + c, v + c);
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// row m of a K-major operand with K = 8*KC columns: hi and lo parts
template <int KC>
__device__ __forceinline__ void store_split(unsigned char* hi, unsigned char* lo, int m,
                                            const float* x) {
#pragma unroll
  for (int j = 0; j < KC; ++j) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float x0 = x[8 * j + 2 * e], x1 = x[8 * j + 2 * e + 1];
      const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
      const __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
      const __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
      h[e] = pack2(h0, h1);
      l[e] = pack2(l0, l1);
    }
    const int off = ((m >> 3) * KC + j) * 128 + (m & 7) * 16;
    *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

// D[128 x N] = A[128 x K] B[N x K]^T with both operands split in hi/lo
template <int K, int N>
__device__ __forceinline__ void gemm_split(uint32_t tmem, uint32_t a_hi, uint32_t a_lo,
                                           uint32_t b_hi, uint32_t b_lo) {
  constexpr uint32_t SBO = (K / 8) * 128;
  const uint32_t id = idesc_bf16(TILE, N);
#pragma unroll
  for (int s = 0; s < K / 16; ++s) {
    const uint32_t o = 256u * s;
    const uint64_t ah = sdesc(a_hi + o, 128, SBO), al = sdesc(a_lo + o, 128, SBO);
    const uint64_t bh = sdesc(b_hi + o, 128, SBO), bl = sdesc(b_lo + o, 128, SBO);
    mma(tmem, ah, bh, id, s > 0 ? 1u : 0u);
    mma(tmem, ah, bl, id, 1u);
    mma(tmem, al, bh, id, 1u);
  }
}

__device__ __forceinline__ void activate(int t, float x, float& y, float& dy) {
  const float a = 1.7159f, b = 0.666666666666667f, c = 0.1f;
  switch (t) {
    case 0: y = x; dy = 1.f; break;
    case 1: y = tanhf(x); dy = 1.f - y * y; break;
    case 2: y = 1.f / (1.f + expf(-x)); dy = y * (1.f - y); break;
    case 3: { const float tb = tanhf(b * x); y = a * tb; dy = a * (1.f - tb * tb) * b; } break;
    case 4: { const float tb = tanhf(b * x); y = a * tb + c * x; dy = a * (1.f - tb * tb) * b + c; } break;
    default: y = 0.f; dy = 0.f;
  }
}

// tanh(x) = 1 - 2 / (exp(2x) + 1): absolute error ~1e-7, far below the
// ~1e-5 relative resolution of the split-BF16 operands it feeds
__device__ __forceinline__ float tanh_fast(float x) {
  return 1.f - __fdividef(2.f, __expf(2.f * x) + 1.f);
}

// activation of a whole row: a = f(z + bias), d = f'(z + bias)
template <int N, bool TANH>
__device__ __forceinline__ void act_row(int fa, float* z, const float* bias, float* d) {
  if (TANH) {
#pragma unroll
    for (int n = 0; n < N; ++n) {
      const float y = tanh_fast(z[n] + bias[n]);
      z[n] = y;
      d[n] = 1.f - y * y;
    }
  } else {
#pragma unroll
    for (int n = 0; n < N; ++n) {
      float y, dy;
      activate(fa, z[n] + bias[n], y, dy);
      z[n] = y;
      d[n] = dy;
    }
  }
}

template <int KIN, int H, bool TANH>
__global__ void __launch_bounds__(128) k_mlp_tc(PotDevice pd, DescBuffers b,
                                                const int* __restrict__ order,
                                                const int* __restrict__ spec_off, int tiles_ub) {
  extern __shared__ __align__(1024) unsigned char sm[];
  constexpr int KA = KIN > H ? KIN : H;
  const TcLayout L = tc_layout(KIN, H);
  unsigned char* img = sm;
  unsigned char* aHi = sm + L.bytes;
  unsigned char* aLo = aHi + TILE * KA * 2;
  unsigned char* bHi = aLo + TILE * KA * 2;
  unsigned char* bLo = bHi + TILE * H * 2;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(bLo + TILE * H * 2);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int m = threadIdx.x, warp = m >> 5;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (m == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
  const uint32_t mb = smem_u32(mbar);
  const uint32_t sImg = smem_u32(img), sAh = smem_u32(aHi), sAl = smem_u32(aLo),
                 sBh = smem_u32(bHi), sBl = smem_u32(bLo);
  uint32_t phase = 0;
  bool ok = true;
  int cur = -1;

  // tiles in species order; this CTA takes a contiguous range
  int tiles = 0;
  for (int t = 0; t < pd.ntypes; ++t) tiles += (spec_off[t + 1] - spec_off[t] + TILE - 1) / TILE;
  const int per = (tiles_ub + gridDim.x - 1) / gridDim.x;
  const int q0 = blockIdx.x * per, q1 = min(tiles, q0 + per);

  for (int q = q0; q < q1; ++q) {
    int t = 0, acc = 0;
    for (; t < pd.ntypes; ++t) {
      const int tt = (spec_off[t + 1] - spec_off[t] + TILE - 1) / TILE;
      if (q < acc + tt) break;
      acc += tt;
    }
    const int beg = spec_off[t] + (q - acc) * TILE;
    const int cnt = min(TILE, spec_off[t + 1] - beg);
    if (t != cur) {
      const uint4* src = reinterpret_cast<const uint4*>(pd.tc_img + (size_t)t * L.bytes);
      uint4* dst = reinterpret_cast<uint4*>(img);
      for (int k = m; k < L.bytes / 16; k += TILE) dst[k] = src[k];
      cur = t;
      __syncthreads();   // every thread reads parts of the image the others copied
    }
    const float* vec = reinterpret_cast<const float*>(img + L.vec);
    const float* b1 = vec;
    const float* b2 = vec + H;
    const float* w3 = vec + 2 * H;
    const float* nsc = vec + 3 * H;
    const float b3 = vec[3 * H + KIN];
    const int fa1 = (int)vec[3 * H + KIN + 1], fa2 = (int)vec[3 * H + KIN + 2],
              fa3 = (int)vec[3 * H + KIN + 3];
    const bool valid = m < cnt;
    const int atom = valid ? order[beg + m] : 0;
    const int nsf = pd.sp[t].nsf;
    // the next tile's atom: its descriptor row is prefetched into L2 once
    // the first MMA round of this tile has been issued
    int atom_next = -1;
    if (q + 1 < q1) {
      int tn = 0, acn = 0;
      for (; tn < pd.ntypes; ++tn) {
        const int tt = (spec_off[tn + 1] - spec_off[tn] + TILE - 1) / TILE;
        if (q + 1 < acn + tt) break;
        acn += tt;
      }
      const int bn = spec_off[tn] + (q + 1 - acn) * TILE;
      if (m < min(TILE, spec_off[tn + 1] - bn)) atom_next = order[bn + m];
    }

    // ---- descriptor row -> A operand
    {
      float x[KIN];
      const float* G = reinterpret_cast<const float*>(b.G) + (size_t)atom * pd.nsf_pad;
#pragma unroll
      for (int k = 0; k < KIN; k += 4) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid && k < nsf) v = *reinterpret_cast<const float4*>(G + k);   // nsf_pad % 4 == 0
        x[k] = v.x;
        x[k + 1] = (k + 1 < nsf) ? v.y : 0.f;
        x[k + 2] = (k + 2 < nsf) ? v.z : 0.f;
        x[k + 3] = (k + 3 < nsf) ? v.w : 0.f;
      }
      store_split<KIN / 8>(aHi, aLo, m, x);
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    if (m == 0) {
      gemm_split<KIN, H>(tmem, sAh, sAl, sImg + L.b1, sImg + L.b1 + 2 * H * KIN);
      mma_commit(mb);
    }
    if (atom_next >= 0) {
      const float* Gn = reinterpret_cast<const float*>(b.G) + (size_t)atom_next * pd.nsf_pad;
#pragma unroll
      for (int k = 0; k < KIN; k += 32)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(Gn + k)));
    }
    ok = __syncthreads_and(mbar_wait(mb, phase));
    phase ^= 1u;
    if (!ok) break;
    fence_after();
    float f1p[H];
    {
      float z[H];
      tmem_ld<H>(tlane, z);
      act_row<H, TANH>(fa1, z, b1, f1p);
      store_split<H / 8>(bHi, bLo, m, z);
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    if (m == 0) {
      gemm_split<H, H>(tmem, sBh, sBl, sImg + L.b2, sImg + L.b2 + 2 * H * H);
      mma_commit(mb);
    }
    ok = __syncthreads_and(mbar_wait(mb, phase));
    phase ^= 1u;
    if (!ok) break;
    fence_after();
    float y;
    {
      float z[H];
      tmem_ld<H>(tlane, z);
      float d2[H];
      act_row<H, TANH>(fa2, z, b2, d2);
      float s = b3;
#pragma unroll
      for (int n = 0; n < H; ++n) {
        s = fmaf(w3[n], z[n], s);
        z[n] = w3[n] * d2[n];
      }
      float dy = 1.f;
      y = s;
      if (!TANH) activate(fa3, s, y, dy);
#pragma unroll
      for (int n = 0; n < H; ++n) z[n] *= dy;
      store_split<H / 8>(aHi, aLo, m, z);
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    if (m == 0) {
      gemm_split<H, H>(tmem, sAh, sAl, sImg + L.b2t, sImg + L.b2t + 2 * H * H);
      mma_commit(mb);
    }
    ok = __syncthreads_and(mbar_wait(mb, phase));
    phase ^= 1u;
    if (!ok) break;
    fence_after();
    {
      float z[H];
      tmem_ld<H>(tlane, z);
#pragma unroll
      for (int n = 0; n < H; ++n) z[n] *= f1p[n];
      store_split<H / 8>(bHi, bLo, m, z);
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    if (m == 0) {
      gemm_split<H, KIN>(tmem, sBh, sBl, sImg + L.b1t, sImg + L.b1t + 2 * KIN * H);
      mma_commit(mb);
    }
    ok = __syncthreads_and(mbar_wait(mb, phase));
    phase ^= 1u;
    if (!ok) break;
    fence_after();
    {
      float g[KIN];
      tmem_ld<KIN>(tlane, g);
      if (valid) {
        float* out = reinterpret_cast<float*>(b.dEdG) + (size_t)atom * pd.nsf_pad;
#pragma unroll
        for (int k = 0; k < KIN; k += 4) {
          if (k < nsf) {
            float4 v = make_float4(g[k] * nsc[k], g[k + 1] * nsc[k + 1], g[k + 2] * nsc[k + 2],
                                   g[k + 3] * nsc[k + 3]);
            *reinterpret_cast<float4*>(out + k) = v;   // padding columns of the row are free
          }
        }
        const SpeciesTable& sp = pd.sp[t];
        b.E_atom[atom] = sp.E_scale * (double)y + sp.E_shift + sp.E_atom;
      }
    }
    fence_before();
    __syncthreads();
    fence_after();
  }
  if (!ok) {
    // let the MMAs this CTA issued finish before the accumulator is freed
    mbar_wait(mb, phase ^ 1u);
    if (m == 0) atomicOr(b.status, AE_ST_TC_TIMEOUT);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                 : "memory");
}

template <int KIN, int H>
size_t tc_smem() {
  constexpr int KA = KIN > H ? KIN : H;
  return (size_t)tc_layout(KIN, H).bytes + 2 * TILE * KA * 2 + 2 * TILE * H * 2 + 16;
}

template <int KIN, int H, bool TANH>
int launch_tc(const PotDevice& pd, const DescBuffers& b, const int* order, const int* spec_off,
              cudaStream_t s) {
  const size_t smem = tc_smem<KIN, H>();
  auto kern = k_mlp_tc<KIN, H, TANH>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int dev = 0, nsm = 148, smem_sm = 228 * 1024;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  // CTAs per SM by shared memory (1 KB reserved per CTA) and TMEM columns
  int occ = (int)(smem_sm / (smem + 1024));
  occ = max(1, min(occ, (int)(512 / TMEM_COLS)));
  const int tiles_ub = (b.natoms + TILE - 1) / TILE + pd.ntypes;
  const int grid = max(1, min(tiles_ub, nsm * occ));
  kern<<<grid, TILE, smem, s>>>(pd, b, order, spec_off, tiles_ub);
  return (int)cudaGetLastError();
}

}  // namespace

int ae_launch_mlp_tc(const PotDevice& pd, const DescBuffers& b, const int* order,
                     const int* spec_off, cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  if (!pd.tc_ok || !pd.tc_img) return (int)cudaErrorInvalidValue;
  if (pd.tc_tanh) {
    if (pd.tc_kin == 32 && pd.tc_h == 32) return launch_tc<32, 32, true>(pd, b, order, spec_off, s);
    if (pd.tc_kin == 64 && pd.tc_h == 32) return launch_tc<64, 32, true>(pd, b, order, spec_off, s);
    if (pd.tc_kin == 32 && pd.tc_h == 64) return launch_tc<32, 64, true>(pd, b, order, spec_off, s);
    if (pd.tc_kin == 64 && pd.tc_h == 64) return launch_tc<64, 64, true>(pd, b, order, spec_off, s);
  }
  if (pd.tc_kin == 32 && pd.tc_h == 32) return launch_tc<32, 32, false>(pd, b, order, spec_off, s);
  if (pd.tc_kin == 64 && pd.tc_h == 32) return launch_tc<64, 32, false>(pd, b, order, spec_off, s);
  if (pd.tc_kin == 32 && pd.tc_h == 64) return launch_tc<32, 64, false>(pd, b, order, spec_off, s);
  if (pd.tc_kin == 64 && pd.tc_h == 64) return launch_tc<64, 64, false>(pd, b, order, spec_off, s);
  return (int)cudaErrorInvalidValue;
}
