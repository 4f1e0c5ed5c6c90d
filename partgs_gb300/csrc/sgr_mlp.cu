// BF16 tensor-core GEMM for the superquadric proposal network (tcgen05, FP32
// accumulation in tensor memory), with the epilogues its forward and
// backward need.
//
//   C[M, N] = A[M, K] . B[N, K]^T        (A, B bf16; C accumulated in fp32)
//
// A is given K-major (row m holds K contiguous values) or, with a_trans,
// transposed (row k holds M contiguous values); likewise B.  The transposed
// forms serve the weight gradient dW = X^T dZ, whose reduction runs over the
// point rows.
//
// One CTA of 128 threads computes a 128 x NT tile (NT = 64, 128 or 256).
// Per K chunk of 64, all threads stage the A and B chunks in shared memory
// in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core
// matrix; core matrices adjacent in K 128 bytes apart, 8-row groups 1024
// bytes apart), one thread issues four tcgen05.mma (K = 16 each) into the
// tensor-memory accumulator (lane = row, column = output column) and commits
// them to an mbarrier, which every thread waits on before the stage is
// reused.  The epilogue reads the accumulator with tcgen05.ld, 32 lanes per
// warp, 16 columns at a time.  With split_k > 0 each CTA reduces one slice of
// K and adds its partial tile atomically (fp32).
//
// Every wait is bounded: on timeout the kernel raises SGR_MLP_TIMEOUT in the
// status word, waits once more (bounded) for its own MMAs, frees its tensor
// memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgrmlp {

constexpr int kTM = 128;        // rows per CTA tile (= tensor-memory lanes)
constexpr int kKC = 64;         // K per shared-memory chunk
constexpr int kThreads = 128;
// Every mbarrier wait gives up after this long (a healthy wait takes
// microseconds); the kernel then reports SGR_MLP_TIMEOUT.
constexpr unsigned long long kWaitNs = 1000000000ull;   // 1 s

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: no swizzle, K-major, start address and
// the two core-matrix strides (bytes, multiples of 16), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// The same descriptor for the 128-byte swizzled K-major layout: rows of
// 128 bytes (64 bf16 of K), 8-row groups 1024 bytes apart (SBO), the
// leading offset unused (1); the 16-byte chunks of row r are XOR-permuted by
// r % 8, as the TMA unit writes them with CU_TENSOR_MAP_SWIZZLE_128B.  The
// tile must start on a 1024-byte boundary; a K step of 16 advances the start
// address by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// The 32-byte swizzled form, for K chunks of 16: rows of 32 bytes, 8-row
// groups 256 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(256u >> 4) << 32) | (1ull << 46) |
         (6ull << 61);
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t instr_desc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// Waits for phase `parity` of the barrier, at most kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
#pragma unroll 1
    for (int k = 0; k < 64; ++k)
      if (mbar_try(bar, parity)) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

// Offset of element (row r, k) of a chunk in the core-matrix layout.
__device__ __forceinline__ uint32_t cm_offset(int r, int k) {
  return (uint32_t)(((r >> 3) * (kKC / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Stages rows [r0, r0 + rows) x K [k0, k0 + kKC) of an operand (zero outside
// [0, R) x [0, K)) in shared memory.  Row-major source: ld elements per row,
// K contiguous; transposed source: row k holds R contiguous values.
template <bool TRANS>
__device__ __forceinline__ void stage(uint8_t* dst, const __nv_bfloat16* __restrict__ src, long long ld, int r0,
                                      int rows, long long R, long long k0, long long K) {
  if (!TRANS) {
    // 16-byte chunks: 8 consecutive k of one row
    const int chunks = rows * (kKC / 8);
    for (int c = threadIdx.x; c < chunks; c += kThreads) {
      const int r = c / (kKC / 8), kk = (c % (kKC / 8)) * 8;
      const long long gr = r0 + r, gk = k0 + kk;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gr < R && gk + 8 <= K) {
        v = *reinterpret_cast<const uint4*>(src + gr * ld + gk);
      } else if (gr < R && gk < K) {
        __nv_bfloat16 t[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) t[e] = (gk + e < K) ? src[gr * ld + gk + e] : __float2bfloat16(0.f);
        v = *reinterpret_cast<const uint4*>(t);
      }
      *reinterpret_cast<uint4*>(dst + cm_offset(r, kk)) = v;
    }
  } else {
    // 16-byte chunks: 8 consecutive rows at one k, scattered into 8 core-matrix rows
    const int chunks = (rows / 8) * kKC;
    for (int c = threadIdx.x; c < chunks; c += kThreads) {
      const int kk = c / (rows / 8), r = (c % (rows / 8)) * 8;
      const long long gr = r0 + r, gk = k0 + kk;
      __nv_bfloat16 t[8];
      if (gk < K && gr + 8 <= R) {
        *reinterpret_cast<uint4*>(t) = *reinterpret_cast<const uint4*>(src + gk * ld + gr);
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) t[e] = (gk < K && gr + e < R) ? src[gk * ld + gr + e] : __float2bfloat16(0.f);
      }
#pragma unroll
      for (int e = 0; e < 8; ++e) *reinterpret_cast<__nv_bfloat16*>(dst + cm_offset(r + e, kk)) = t[e];
    }
  }
}

// Epilogue of 16 accumulator columns [col0, col0 + 16) of one row: 16-byte
// vector stores (loads of the mask, fp32 vector atomics) when the 16 columns
// are in range and aligned, element by element otherwise.
// `bias`: the bias vector (indexed by output column), from shared or global
// memory, or null.
__device__ __forceinline__ void epilogue16(const sgr_gemm_args& a, long long row, long long col0,
                                           const uint32_t (&v)[16], const float* bias) {
  float x[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    x[e] = __uint_as_float(v[e]);
    if (bias && col0 + e < a.N) x[e] += bias[col0 + e];
  }
  const bool vec = col0 + 16 <= a.N && (a.ldo & 7) == 0 && (reinterpret_cast<uintptr_t>(a.out) & 15) == 0 &&
                   (a.epilogue != SGR_GEMM_MASK_BF16 ||
                    ((a.ldmask & 7) == 0 && (reinterpret_cast<uintptr_t>(a.mask) & 15) == 0));
  if (vec) {
    const long long o = row * a.ldo + col0;
    switch (a.epilogue) {
      case SGR_GEMM_STORE_F32: {
        float4* dst = reinterpret_cast<float4*>(static_cast<float*>(a.out) + o);
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
        return;
      }
      case SGR_GEMM_ADD_F32: {
        float4* dst = reinterpret_cast<float4*>(static_cast<float*>(a.out) + o);
#pragma unroll
        for (int q = 0; q < 4; ++q) atomicAdd(dst + q, make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]));
        return;
      }
      case SGR_GEMM_RELU_BF16:
      case SGR_GEMM_MASK_BF16: {
        if (a.epilogue == SGR_GEMM_MASK_BF16) {
          const uint4* mp = reinterpret_cast<const uint4*>(static_cast<const __nv_bfloat16*>(a.mask) +
                                                           row * a.ldmask + col0);
          const uint4 m2[2] = {mp[0], mp[1]};
          const __nv_bfloat16* mh = reinterpret_cast<const __nv_bfloat16*>(m2);
#pragma unroll
          for (int e = 0; e < 16; ++e) x[e] = __bfloat162float(mh[e]) > 0.0f ? x[e] : 0.0f;
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e) x[e] = fmaxf(x[e], 0.0f);
        }
        uint4 w[2];
        __nv_bfloat162* wh = reinterpret_cast<__nv_bfloat162*>(w);
#pragma unroll
        for (int q = 0; q < 8; ++q) wh[q] = __floats2bfloat162_rn(x[2 * q], x[2 * q + 1]);
        uint4* dst = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(a.out) + o);
        dst[0] = w[0];
        dst[1] = w[1];
        return;
      }
      default:
        return;
    }
  }
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    const long long col = col0 + e;
    if (col >= a.N) break;
    const long long o = row * a.ldo + col;
    switch (a.epilogue) {
      case SGR_GEMM_STORE_F32:
        static_cast<float*>(a.out)[o] = x[e];
        break;
      case SGR_GEMM_ADD_F32:
        atomicAdd(static_cast<float*>(a.out) + o, x[e]);
        break;
      case SGR_GEMM_RELU_BF16:
        static_cast<__nv_bfloat16*>(a.out)[o] = __float2bfloat16(fmaxf(x[e], 0.0f));
        break;
      case SGR_GEMM_MASK_BF16: {
        const float h = __bfloat162float(static_cast<const __nv_bfloat16*>(a.mask)[row * a.ldmask + col]);
        static_cast<__nv_bfloat16*>(a.out)[o] = __float2bfloat16(h > 0.0f ? x[e] : 0.0f);
        break;
      }
      default:
        break;
    }
  }
}

template <int NT, bool A_T, bool B_T>
__global__ void __launch_bounds__(kThreads) k_gemm_tc(const sgr_gemm_args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;                                  // kTM x kKC bf16: 16 KB
  uint8_t* sB = smem + kTM * kKC * 2;                  // NT x kKC bf16
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * NT;
  long long k_begin = 0, k_end = a.K;
  if (a.split_k > 0) {
    k_begin = (long long)blockIdx.z * a.split_k;
    k_end = k_begin + a.split_k < a.K ? k_begin + a.split_k : a.K;
  }
  if (k_begin >= k_end) return;                        // CTA-uniform

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&s_tmem)),
                 "r"(NT)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = s_tmem;
  const uint32_t bar = smem_addr(&s_bar);
  const uint32_t idesc = instr_desc(NT);
  uint32_t phase = 0;
  bool ok = true;

  for (long long k0 = k_begin; k0 < k_end; k0 += kKC) {
    stage<A_T>(sA, static_cast<const __nv_bfloat16*>(a.A), a.lda, m0, kTM, a.M, k0, k_end);
    stage<B_T>(sB, static_cast<const __nv_bfloat16*>(a.B), a.ldb, n0, NT, a.N, k0, k_end);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB);
#pragma unroll
      for (int s = 0; s < kKC / 16; ++s) {
        const uint64_t da = smem_desc(a0 + 256u * s, 128u, 1024u);
        const uint64_t db = smem_desc(b0 + 256u * s, 128u, 1024u);
        const uint32_t acc = (k0 > k_begin || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                   : "memory");
    }
    ok = mbar_wait(bar, phase);
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (!__syncthreads_and(ok)) break;
  }

  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) {
      atomicOr(a.status, (unsigned)SGR_MLP_TIMEOUT);
      mbar_wait(bar, phase ^ 1u);                       // once more for the MMAs in flight
    }
  } else {
    // epilogue: warp w owns rows m0 + 32 w + lane (tensor-memory lanes 32 w ..)
    const long long row = (long long)m0 + 32 * warp + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < NT; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row >= a.M) continue;
      epilogue16(a, row, (long long)n0 + c0, v, a.bias);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(NT) : "memory");
  }
}

// ---------------------------------------------------------------------------
// K-major operands: persistent, TMA-fed, warp-specialised form.
//
// A TMA copy of a box of 8 columns x R rows (no swizzle) lands as R rows of
// 16 bytes, contiguous: the no-swizzle K-major core-matrix layout with 8-row
// groups 128 bytes apart (SBO) and adjacent 8-column slices R * 16 bytes
// apart (LBO).  A K chunk of 64 is 8 such copies per operand.
//
// Each CTA stays resident and takes output tiles blockIdx.x, + gridDim.x, ...
// Six warps:
//   warp 0 (one thread): TMA producer; fills a ring of ns stages (A and B
//     chunks), waiting on empty[s] before it reuses stage s;
//   warp 1 (one thread): MMA issuer; per tile, into one of two tensor-memory
//     accumulators (2 x NT columns), four MMAs per chunk once full[s] has
//     its bytes, each chunk's MMAs committed to empty[s], the tile's last
//     commit to tfull[b]; it waits on tempty[b] before reusing accumulator b;
//   warps 2 ..: epilogue, four per 64 output columns; warp w reads
//     tensor-memory lanes 32 (w % 4) .. + 31 (rows of the tile), columns of
//     group (w - 2) / 4, once tfull[b] fires, 32 columns per wait, applies
//     the epilogue, stores, and arrives on tempty[b].
// So one tile's epilogue runs while the next tile's loads and MMAs do.
// Every wait is bounded (kWaitNs) and also ends when another role has
// failed; a failure raises SGR_MLP_TIMEOUT, the producer then waits
// (bounded) for the copies it issued, everyone waits for the issuer's final
// commit (all MMAs done), and only then is the tensor memory freed.
// Out-of-range rows and columns are zero-filled by the TMA unit.
// ---------------------------------------------------------------------------
constexpr int kStages = 4;          // pipeline stages of K chunks of 64
constexpr int kStages16 = 8;        // of K chunks of 16 (layers with K <= 16)
// SGR_MLP_SW128 1: the persistent GEMM loads each K chunk of 64 as one
// 128-byte swizzled TMA box per operand (64 columns x rows); 0: as eight
// no-swizzle boxes of 8 columns (16-byte rows).
#ifndef SGR_MLP_SW128
#define SGR_MLP_SW128 1
#endif
constexpr int kBiasSmem = 1024;   // output columns whose bias the persistent GEMM keeps in shared memory
// epilogue warps of an NT-column tile: four (one per 32 rows) per 64 columns
template <int NT>
__host__ __device__ constexpr int epi_warps() { return 4 * (NT >= 64 ? NT / 64 : 1); }
template <int NT>
__host__ __device__ constexpr int persist_threads() { return 64 + 32 * epi_warps<NT>(); }
// CTAs per SM the persistent GEMM is compiled for: as many as tensor memory
// holds (512 columns, 2 NT per CTA), at most 4 (so 64-column tiles keep their
// registers at 85 or fewer)
template <int NT>
__host__ __device__ constexpr int persist_min_ctas() { return 512 / (2 * NT) < 4 ? 512 / (2 * NT) : 4; }

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

// mbar_wait that also gives up as soon as another role has raised `fail`.
__device__ __forceinline__ bool mbar_wait_or_fail(uint32_t bar, uint32_t parity, const volatile int* fail) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
#pragma unroll 1
    for (int k = 0; k < 64; ++k)
      if (mbar_try(bar, parity)) return true;
    if (*fail || global_ns() - t0 > kWaitNs) return false;
  }
}

// KC: K per chunk, 64 (128-byte swizzle) or 16 (32-byte swizzle, for K <= 16).
template <int NT, int KC>
__global__ void __launch_bounds__(persist_threads<NT>(), persist_min_ctas<NT>())
    k_gemm_persist(const sgr_gemm_args a, const __grid_constant__ CUtensorMap map_a,
                   const __grid_constant__ CUtensorMap map_b, int ns) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t kBytesA = kTM * KC * 2, kBytesB = NT * KC * 2, kStage = kBytesA + kBytesB;
  constexpr uint32_t kCols = 2 * NT;                 // two accumulators
  constexpr int kMaxStages = KC == 64 ? kStages : kStages16;
  __shared__ __align__(8) uint64_t s_full[kMaxStages], s_empty[kMaxStages], s_tfull[2], s_tempty[2], s_done;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  __shared__ float s_bias[kBiasSmem];
  volatile int* fail = &s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the bias, once per CTA, into shared memory (the epilogue reads 16
  // values per 16 columns; from global memory those loads were its stall)
  const bool bias_smem = a.bias && a.N <= kBiasSmem;
  if (bias_smem)
    for (int c = threadIdx.x; c < (int)a.N; c += persist_threads<NT>()) s_bias[c] = a.bias[c];
  const float* bias = bias_smem ? s_bias : a.bias;
  const int tiles_n = (int)((a.N + NT - 1) / NT);
  const int total = (int)((a.M + kTM - 1) / kTM) * tiles_n;
  const int chunks = (int)((a.K + KC - 1) / KC);

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&s_tmem)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < ns; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_full[i])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_empty[i])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_tfull[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(&s_tempty[b])),
                   "r"(epi_warps<NT>())
                   : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_done)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s_fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = s_tmem;
  // TMA destinations: 1024-byte aligned (the swizzle atom; stages are multiples of it)
  const uint32_t base = (smem_addr(smem) + 1023u) & ~1023u;

  int issued = 0;                                    // producer: chunks whose loads were issued
  if (warp == 0) {
    // producer (a.skip_loads: issues nothing, so that the MMA issuer's wait
    // runs out with no copy in flight -- the timeout path's test)
    if (lane == 0 && !a.skip_loads) {
      int g = 0;
      for (int t = blockIdx.x; t < total && !*fail; t += gridDim.x) {
        const int m0 = (t / tiles_n) * kTM, n0 = (t % tiles_n) * NT;
        for (int c = 0; c < chunks; ++c, ++g) {
          const int st = g % ns;
          if (g >= ns && !mbar_wait_or_fail(smem_addr(&s_empty[st]), (uint32_t)((g / ns - 1) & 1), fail)) {
            *fail = 1;
            break;
          }
          const uint32_t full = smem_addr(&s_full[st]);
          mbar_expect(full, kStage);
          const uint32_t sa = base + st * kStage, sb = sa + kBytesA;
#if SGR_MLP_SW128
          tma_load_2d(sa, &map_a, c * KC, m0, full);
          tma_load_2d(sb, &map_b, c * KC, n0, full);
#else
          for (int kb = 0; kb < KC / 8; ++kb) {
            tma_load_2d(sa + kb * kTM * 16, &map_a, c * KC + kb * 8, m0, full);
            tma_load_2d(sb + kb * NT * 16, &map_b, c * KC + kb * 8, n0, full);
          }
#endif
          issued = g + 1;
        }
      }
    }
  } else if (warp == 1) {
    // MMA issuer
    if (lane == 0) {
      const uint32_t idesc = instr_desc(NT);
      int g = 0, i = 0;
      for (int t = blockIdx.x; t < total; t += gridDim.x, ++i) {
        const int b = i & 1;
        if (i >= 2 && !mbar_wait_or_fail(smem_addr(&s_tempty[b]), (uint32_t)(((i >> 1) - 1) & 1), fail)) {
          *fail = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t acc_tmem = tmem + (uint32_t)(b * NT);
        bool bad = false;
        for (int c = 0; c < chunks; ++c, ++g) {
          const int st = g % ns;
          if (!mbar_wait_or_fail(smem_addr(&s_full[st]), (uint32_t)((g / ns) & 1), fail)) {
            bad = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t sa = base + st * kStage, sb = sa + kBytesA;
#pragma unroll
          for (int s = 0; s < KC / 16; ++s) {
#if SGR_MLP_SW128
            const uint64_t da = KC == 64 ? smem_desc_sw128(sa + 32u * s) : smem_desc_sw32(sa);
            const uint64_t db = KC == 64 ? smem_desc_sw128(sb + 32u * s) : smem_desc_sw32(sb);
#else
            const uint64_t da = smem_desc(sa + 2u * s * kTM * 16, kTM * 16, 128u);
            const uint64_t db = smem_desc(sb + 2u * s * NT * 16, NT * 16, 128u);
#endif
            const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc_tmem),
                "l"(da), "l"(db), "r"(idesc), "r"(acc)
                : "memory");
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                           smem_addr(&s_empty[st]))
                       : "memory");
        }
        if (bad) {
          *fail = 1;
          break;
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         smem_addr(&s_tfull[b]))
                     : "memory");
      }
      // tracks every MMA this thread issued: the teardown waits on it
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_addr(&s_done))
                   : "memory");
    }
  } else {
    // epilogue: this warp's quarter of the tensor-memory lanes (rows) and
    // its group of columns
    const int q = warp & 3;
    constexpr int kHalf = NT / (epi_warps<NT>() / 4);   // columns per warp
    const int h0 = ((warp - 2) >> 2) * kHalf;
    int i = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x, ++i) {
      const int b = i & 1;
      const bool ok = mbar_wait_or_fail(smem_addr(&s_tfull[b]), (uint32_t)((i >> 1) & 1), fail);
      if (!__all_sync(0xffffffffu, ok)) {              // one decision per warp (tcgen05.ld needs every lane)
        if (lane == 0) *fail = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const long long row = (long long)(t / tiles_n) * kTM + 32 * q + lane;
      const long long n0 = (long long)(t % tiles_n) * NT + h0;
#pragma unroll 1
      for (int c0 = 0; c0 < kHalf; c0 += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * NT + h0 + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr)
            : "memory");
        if (c0 + 16 < kHalf)
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
              "[%16];\n"
              : "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
                "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                "=r"(v[30]), "=r"(v[31])
              : "r"(taddr + 16u)
              : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (row < a.M) {
          if (n0 + c0 < a.N) epilogue16(a, row, n0 + c0, *reinterpret_cast<const uint32_t(*)[16]>(&v[0]), bias);
          if (c0 + 16 < kHalf && n0 + c0 + 16 < a.N)
            epilogue16(a, row, n0 + c0 + 16, *reinterpret_cast<const uint32_t(*)[16]>(&v[16]), bias);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(&s_tempty[b]));
    }
  }

  // teardown: one decision for the whole CTA
  if (__syncthreads_or(*fail)) {
    if (threadIdx.x == 0) {
      atomicOr(a.status, (unsigned)SGR_MLP_TIMEOUT);
      // let the copies this CTA issued land before it gives its shared
      // memory back: the last phase armed on each stage (bounded waits)
      for (int g = issued - 1; g >= 0 && g >= issued - ns; --g)
        mbar_wait(smem_addr(&s_full[g % ns]), (uint32_t)((g / ns) & 1));
    }
  }
  if (threadIdx.x == 32) mbar_wait(smem_addr(&s_done), 0u);   // every MMA has completed
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kCols) : "memory");
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static std::once_flag once;
  static EncodeTiled fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

// Tensor map of a row-major bf16 matrix [rows, cols] (ld elements per row)
// read in boxes of 8 columns x box_rows rows.
bool make_map(CUtensorMap* m, const void* base, long long rows, long long cols, long long ld, int box_rows,
              int kc = kKC) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
#if SGR_MLP_SW128
  // boxes of kc columns (the swizzle span: 128 bytes for 64, 32 for 16) x box_rows
  const cuuint32_t box[2] = {(cuuint32_t)kc, (cuuint32_t)box_rows};
  const CUtensorMapSwizzle swz = kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_32B;
#else
  const cuuint32_t box[2] = {8u, (cuuint32_t)box_rows};
  const CUtensorMapSwizzle swz = CU_TENSOR_MAP_SWIZZLE_NONE;
#endif
  const cuuint32_t estr[2] = {1u, 1u};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NT, int KC>
int launch_persist(const sgr_gemm_args& a, cudaStream_t st) {
  alignas(64) CUtensorMap ma, mb;
  if (!make_map(&ma, a.A, a.M, a.K, a.lda, kTM, KC) || !make_map(&mb, a.B, a.N, a.K, a.ldb, NT, KC))
    return SGR_ERR_CUDA;
  // ring stages: a layer whose K is one chunk needs two (the next tile's
  // operands load while this tile's MMA runs; two accumulators do the rest),
  // which leaves shared memory for more resident CTAs
  const long long chunks = (a.K + KC - 1) / KC;
  const int ns = chunks <= 1 ? 2 : (KC == 64 ? kStages : kStages16);
  const size_t smem = (size_t)ns * (kTM + NT) * KC * 2 + 1024;
  // per device and ring size, once: the shared-memory attribute and the
  // resident CTAs per SM, from the kernel's registers and static shared
  // memory and the SM's limits (register file in 256-register warp
  // allocations, shared memory with the per-CTA reserve, threads), and from
  // tensor memory (512 columns, 2 NT per CTA; a CTA beyond that would wait in
  // its allocation until another finished).  Counted here rather than by the
  // occupancy calculator, which answered 1 CTA per SM for this kernel where
  // the SMs ran 3 (ncu: 456 CTAs of the 64-column tile resident at once,
  // warps active 9% -> 26%, layer time -20%).
  constexpr int kMaxDev = 64;
  static int resident[kMaxDev][2] = {};
  static std::mutex resident_mutex;   // callers may launch from several host threads
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return SGR_ERR_CUDA;
  std::unique_lock<std::mutex> lock(resident_mutex);
  int& res = resident[dev][ns == 2 ? 0 : 1];
  if (res == 0) {
    const int full = KC == 64 ? kStages : kStages16;   // the attribute covers the largest ring
    cudaFuncAttributes fa{};
    int sms = 0, smem_sm = 0, reserve = 0, regs_sm = 0, threads_sm = 0;
    if (cudaFuncSetAttribute(k_gemm_persist<NT, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)((size_t)full * (kTM + NT) * KC * 2 + 1024)) != cudaSuccess ||
        cudaFuncSetAttribute(k_gemm_persist<NT, KC>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, k_gemm_persist<NT, KC>) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess)
      return SGR_ERR_CUDA;
    constexpr int threads = persist_threads<NT>();
    const int warp_regs = (fa.numRegs * 32 + 255) / 256 * 256;
    int per_sm = 512 / (2 * NT);
    per_sm = std::min(per_sm, regs_sm / std::max(1, warp_regs * (threads / 32)));
    per_sm = std::min(per_sm, smem_sm / (int)(fa.sharedSizeBytes + smem + (size_t)reserve));
    per_sm = std::min(per_sm, threads_sm / threads);
    if (per_sm < 1) return SGR_ERR_UNSUPPORTED;
    res = sms * per_sm;
  }
  const int resident_ctas = res;
  lock.unlock();
  const long long tiles = ((a.M + kTM - 1) / kTM) * ((a.N + NT - 1) / NT);
  const long long grid = tiles < (long long)resident_ctas ? tiles : (long long)resident_ctas;
  k_gemm_persist<NT, KC><<<(unsigned)grid, persist_threads<NT>(), smem, st>>>(a, ma, mb, ns);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

// K <= 16 (the first layer: 3 coordinates padded to 16) in chunks of 16,
// everything else in chunks of 64.
template <int NT>
int launch_tma(const sgr_gemm_args& a, cudaStream_t st) {
#if SGR_MLP_SW128
  if (a.K <= 16) return launch_persist<NT, 16>(a, st);
#endif
  return launch_persist<NT, 64>(a, st);
}

template <int NT, bool A_T, bool B_T>
int launch(const sgr_gemm_args& a, cudaStream_t st) {
  const size_t smem = (size_t)(kTM + NT) * kKC * 2;
  if (cudaFuncSetAttribute(k_gemm_tc<NT, A_T, B_T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SGR_ERR_CUDA;
  const unsigned gz = a.split_k > 0 ? (unsigned)((a.K + a.split_k - 1) / a.split_k) : 1u;
  dim3 grid((unsigned)((a.M + kTM - 1) / kTM), (unsigned)((a.N + NT - 1) / NT), gz);
  k_gemm_tc<NT, A_T, B_T><<<grid, kThreads, smem, st>>>(a);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

template <int NT>
int launch_nt(const sgr_gemm_args& a, cudaStream_t st) {
  if (!a.a_trans && !a.b_trans && a.split_k == 0) return launch_tma<NT>(a, st);
  if (!a.a_trans && !a.b_trans) return launch<NT, false, false>(a, st);
  if (a.a_trans && a.b_trans) return launch<NT, true, true>(a, st);
  return SGR_ERR_UNSUPPORTED;
}

// Max over each set's P rows of a [S*P, C] activation: g[s, c] (fp32 and
// bf16 copies) and the row that holds it (first on ties).  One CTA per set,
// threads over channels, rows read coalesced.
__global__ void k_maxpool(const __nv_bfloat16* __restrict__ h, int P, int C, float* __restrict__ g,
                          __nv_bfloat16* __restrict__ g_bf16, int* __restrict__ arg) {
  const int set = blockIdx.x;
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    const __nv_bfloat16* col = h + (size_t)set * P * C + c;
    float best = __bfloat162float(col[0]);
    int at = 0;
    for (int p = 1; p < P; ++p) {
      const float v = __bfloat162float(col[(size_t)p * C]);
      if (v > best) {
        best = v;
        at = p;
      }
    }
    g[(size_t)set * C + c] = best;
    if (g_bf16) g_bf16[(size_t)set * C + c] = __float2bfloat16(best);
    arg[(size_t)set * C + c] = set * P + at;
  }
}

// Backward of the max-pool and of the ReLU below it: dh[arg[s, c], c] =
// dg[s, c] where g[s, c] > 0; every other entry of dh is zero (cleared by
// the caller's launch sequence).
__global__ void k_maxpool_bwd(const float* __restrict__ dg, const float* __restrict__ g, const int* __restrict__ arg,
                              long long n, int C, __nv_bfloat16* __restrict__ dh) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  dh[(size_t)arg[i] * C + c] = __float2bfloat16(g[i] > 0.0f ? dg[i] : 0.0f);
}

}  // namespace sgrmlp

using namespace sgrmlp;

extern "C" {

int sgr_mlp_gemm(const sgr_gemm_args* a, void* stream) {
  if (!a || a->M < 0 || a->N < 0 || a->K < 0 || !a->status) return SGR_ERR_INVALID_ARGUMENT;
  if (a->M == 0 || a->N == 0) return SGR_OK;
  if (!a->A || !a->B || !a->out || a->K == 0) return SGR_ERR_INVALID_ARGUMENT;
  if (a->epilogue < SGR_GEMM_STORE_F32 || a->epilogue > SGR_GEMM_MASK_BF16) return SGR_ERR_INVALID_ARGUMENT;
  if (a->epilogue == SGR_GEMM_MASK_BF16 && !a->mask) return SGR_ERR_INVALID_ARGUMENT;
  if (a->split_k < 0 || (a->split_k > 0 && a->split_k % kKC != 0)) return SGR_ERR_INVALID_ARGUMENT;
  if (a->split_k > 0 && a->epilogue != SGR_GEMM_ADD_F32) return SGR_ERR_UNSUPPORTED;
  // 16-byte vector loads: row strides and base addresses in multiples of 8 bf16
  if (a->lda % 8 || a->ldb % 8 || (reinterpret_cast<uintptr_t>(a->A) & 15) || (reinterpret_cast<uintptr_t>(a->B) & 15))
    return SGR_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n = a->N <= 64 ? 64 : a->N <= 128 ? 128 : 256;
  switch (n) {
    case 64: return launch_nt<64>(*a, st);
    case 128: return launch_nt<128>(*a, st);
    default: return launch_nt<256>(*a, st);
  }
}

int sgr_mlp_maxpool(const void* h, int32_t sets, int32_t P, int32_t C, float* g, void* g_bf16, int32_t* arg,
                    void* stream) {
  if (sets < 0 || P < 1 || C < 1 || (sets > 0 && (!h || !g || !arg))) return SGR_ERR_INVALID_ARGUMENT;
  if (sets == 0) return SGR_OK;
  k_maxpool<<<sets, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const __nv_bfloat16*>(h), P, C, g,
                                                                  static_cast<__nv_bfloat16*>(g_bf16), arg);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

int sgr_mlp_maxpool_backward(const float* dg, const float* g, const int32_t* arg, int32_t sets, int32_t P,
                             int32_t C, void* dh, void* stream) {
  if (sets < 0 || P < 1 || C < 1 || (sets > 0 && (!dg || !g || !arg || !dh))) return SGR_ERR_INVALID_ARGUMENT;
  if (sets == 0) return SGR_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(dh, 0, (size_t)sets * P * C * 2, st) != cudaSuccess) return SGR_ERR_CUDA;
  const long long n = (long long)sets * C;
  k_maxpool_bwd<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dg, g, arg, n, C, static_cast<__nv_bfloat16*>(dh));
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // extern "C"
