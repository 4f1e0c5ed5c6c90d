// Stable LSD radix sort of (key, record id) pairs and prefix sums, the
// depth order and the offset / cell scans of the forward
// (replacing the library sort and scans the reference calls,
// cuda_rasterizer/rasterizer_impl.cu:278, 304-309).
//
// Sort: digits of up to 9 bits, as few passes as cover bits [0, end_bit)
// (36-bit (view, depth) keys: 4 passes of 9 bits).  Each pass is three
// kernels:
//   1. k_radix_hist: per 4096-key tile, the digit histogram, stored
//      digit-major (hist[digit][tile]);
//   2. k_radix_scan: per digit, the exclusive scan of its counts over the
//      tiles, and the digit's total;
//   3. k_radix_scatter: per tile, every key's rank among the tile's keys of
//      its digit in input order, the tile reordered by (digit, rank) in
//      shared memory, then written out in digit runs:
//      out[digit base + tile prefix + rank].  A warp owns 512 consecutive
//      keys of the tile and ranks them with warp-private digit counters
//      (match_any per 32 keys, no block barrier); the warps' counts are
//      then scanned per digit, so earlier warps' keys come first.
// Equal digits keep their input order in every pass, so the result is the
// stable order of the keys (ties by input position), the order of any
// stable radix sort of the same bits.
//
// Scans: a 2048-element tile per CTA; per-tile sums, one CTA scanning those,
// then each tile's scan plus its prefix.
#include "sgr_kernels.cuh"

namespace sgr {

namespace {

constexpr int kSortThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kWarpSpan = 32 * kRadixItems;              // 512 keys per warp
constexpr int kRadixTile = kSortThreads * kRadixItems;   // 4096 keys per sort CTA
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;     // 2048 elements per scan CTA
constexpr int kMaxDigitBits = 9;
constexpr int kBins = 1 << kMaxDigitBits;                // 512
constexpr int kBinsPerThread = kBins / kSortThreads;     // 2
constexpr int kSortWarps = kSortThreads / 32;

inline long long tiles_of(long long n) { return (n + kSortTile - 1) / kSortTile; }
inline long long radix_tiles_of(long long n) { return (n + kRadixTile - 1) / kRadixTile; }

// The pass's digit: bits [shift, shift + width) of the key (dmask keeps the
// width, cut at the sort's end bit).
template <class K>
__device__ __forceinline__ uint32_t digit_of(K key, int shift, uint32_t dmask) {
  return (uint32_t)(key >> shift) & dmask;
}

// The lanes of the warp holding the same digit d (d <= kBins, kBins marking
// an empty slot).  SGR_SORT_BALLOT 1: one ballot per digit bit (ten of
// them), each lane keeping the lanes that agree with it on every bit;
// 0: __match_any_sync.
#ifndef SGR_SORT_BALLOT
#define SGR_SORT_BALLOT 1
#endif
__device__ __forceinline__ unsigned digit_peers(uint32_t d) {
#if SGR_SORT_BALLOT
  unsigned m = 0xffffffffu;
#pragma unroll
  for (int b = 0; b <= kMaxDigitBits; ++b) {
    const bool bit = (d >> b) & 1u;
    const unsigned v = __ballot_sync(0xffffffffu, bit);
    m &= bit ? v : ~v;
  }
  return m;
#else
  return __match_any_sync(0xffffffffu, d);
#endif
}

// Exclusive scan of one value per thread over a 256-thread CTA; returns the
// CTA total in `total`.  Uses s_warp[kSortWarps].
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* s_warp, T& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  T before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) {
    const T x = s_warp[w];
    if (w < warp) before += x;
    all += x;
  }
  __syncthreads();
  total = all;
  return before + incl - v;
}

// Exclusive scan over the kBins digits, thread t holding digits
// t*kBinsPerThread .. +kBinsPerThread-1 (consecutive).
template <class T>
__device__ __forceinline__ void digits_exclusive_scan(const T (&v)[kBinsPerThread], T (&ex)[kBinsPerThread],
                                                      T* s_warp) {
  T sum = 0;
#pragma unroll
  for (int j = 0; j < kBinsPerThread; ++j) sum += v[j];
  T tot;
  T run = block_exclusive_scan<T>(sum, s_warp, tot);
#pragma unroll
  for (int j = 0; j < kBinsPerThread; ++j) {
    ex[j] = run;
    run += v[j];
  }
}

template <class K>
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const K* __restrict__ keys, long long n, int shift,
                                                             uint32_t dmask, uint32_t* __restrict__ hist,
                                                             long long ntiles) {
  __shared__ uint32_t s_cnt[kBins];
#pragma unroll
  for (int j = 0; j < kBinsPerThread; ++j) s_cnt[j * kSortThreads + threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRadixTile;
  const int lane = threadIdx.x & 31;
  uint32_t d[kRadixItems];
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {       // all loads first
    const long long i = base + k * kSortThreads + threadIdx.x;
    d[k] = i < n ? digit_of(keys[i], shift, dmask) : (uint32_t)kBins;
  }
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const unsigned peers = digit_peers(d[k]);
    if (d[k] < kBins && lane == __ffs(peers) - 1) atomicAdd(&s_cnt[d[k]], (uint32_t)__popc(peers));
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kBinsPerThread; ++j) {
    const int b = j * kSortThreads + threadIdx.x;
    hist[(size_t)b * ntiles + blockIdx.x] = s_cnt[b];
  }
}

// One CTA per digit: exclusive scan of its per-tile counts, in place.
__global__ void __launch_bounds__(kSortThreads) k_radix_scan(uint32_t* __restrict__ hist, long long ntiles,
                                                             uint32_t* __restrict__ totals) {
  __shared__ uint32_t s_warp[kSortWarps];
  uint32_t* h = hist + (size_t)blockIdx.x * ntiles;
  uint32_t carry = 0;
  for (long long c = 0; c < ntiles; c += kSortThreads) {
    const long long i = c + threadIdx.x;
    const uint32_t v = i < ntiles ? h[i] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan<uint32_t>(v, s_warp, tot);
    if (i < ntiles) h[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

template <class K>
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const K* __restrict__ keys_in,
                                                                const uint32_t* __restrict__ vals_in,
                                                                K* __restrict__ keys_out,
                                                                uint32_t* __restrict__ vals_out, long long n,
                                                                int shift, uint32_t dmask,
                                                                const uint32_t* __restrict__ hist,
                                                                const uint32_t* __restrict__ totals,
                                                                long long ntiles) {
  extern __shared__ __align__(16) unsigned char s_dyn[];   // the tile in (digit, rank) order: keys, then values
  K* s_keys = reinterpret_cast<K*>(s_dyn);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_dyn + sizeof(K) * kRadixTile);
  __shared__ uint32_t s_wc[kSortWarps][kBins];     // per warp: keys of each digit (then: keys in earlier warps)
  __shared__ uint32_t s_local[kBins];              // start of each digit in the tile's order
  __shared__ unsigned long long s_gbase[kBins];    // output position of the tile's first key of each digit
  __shared__ unsigned long long s_warp64[kSortWarps];
  __shared__ uint32_t s_warp32[kSortWarps];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const long long base = (long long)blockIdx.x * kRadixTile;
  const long long wbase = base + (long long)warp * kWarpSpan;

  K key[kRadixItems];
  uint32_t val[kRadixItems];
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {       // all loads first; a warp's keys are consecutive
    const long long i = wbase + k * 32 + lane;
    key[k] = i < n ? keys_in[i] : (K)0;
    val[k] = i < n ? vals_in[i] : 0u;
  }
#pragma unroll
  for (int j = 0; j < kBinsPerThread; ++j)
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) s_wc[w][j * kSortThreads + t] = 0;
  // global start of each digit: all smaller digits, then the tiles before this one
  {
    unsigned long long tot[kBinsPerThread], ex[kBinsPerThread];
#pragma unroll
    for (int j = 0; j < kBinsPerThread; ++j) tot[j] = totals[t * kBinsPerThread + j];
    digits_exclusive_scan<unsigned long long>(tot, ex, s_warp64);   // (its barriers also cover the zeroing)
#pragma unroll
    for (int j = 0; j < kBinsPerThread; ++j) {
      const int b = t * kBinsPerThread + j;
      s_gbase[b] = ex[j] + hist[(size_t)b * ntiles + blockIdx.x];
    }
  }
  // rank within the warp, in input order: (digit << 16) | rank
  uint32_t dr[kRadixItems];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const long long i = wbase + k * 32 + lane;
    const uint32_t d = i < n ? digit_of(key[k], shift, dmask) : (uint32_t)kBins;
    const unsigned peers = digit_peers(d);
    const int leader = __ffs(peers) - 1;
    uint32_t before = 0;
    if (lane == leader && d < kBins) {
      before = s_wc[warp][d];
      s_wc[warp][d] = before + (uint32_t)__popc(peers);
    }
    before = __shfl_sync(0xffffffffu, before, leader);
    __syncwarp();
    dr[k] = (d << 16) | (before + (uint32_t)__popc(peers & lt));
  }
  __syncthreads();
  // per digit: exclusive prefix over the warps, and the tile's count
  {
    uint32_t cnt[kBinsPerThread], ex[kBinsPerThread];
#pragma unroll
    for (int j = 0; j < kBinsPerThread; ++j) {
      const int b = t * kBinsPerThread + j;
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = s_wc[w][b];
        s_wc[w][b] = run;
        run += c;
      }
      cnt[j] = run;
    }
    digits_exclusive_scan<uint32_t>(cnt, ex, s_warp32);
#pragma unroll
    for (int j = 0; j < kBinsPerThread; ++j) s_local[t * kBinsPerThread + j] = ex[j];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kRadixItems; ++k) {
    const uint32_t d = dr[k] >> 16;
    if (d < kBins) {
      const uint32_t pos = s_local[d] + s_wc[warp][d] + (dr[k] & 0xffffu);
      s_keys[pos] = key[k];
      s_vals[pos] = val[k];
    }
  }
  __syncthreads();
  const int count = (int)min((long long)kRadixTile, n - base);
  for (int s = t; s < count; s += kSortThreads) {
    const K kv = s_keys[s];
    const uint32_t d = digit_of(kv, shift, dmask);
    const unsigned long long dst = s_gbase[d] + (unsigned long long)(s - (int)s_local[d]);
    keys_out[dst] = kv;
    vals_out[dst] = s_vals[s];
  }
}

// ---- scans ------------------------------------------------------------------

template <class T>
__global__ void __launch_bounds__(kSortThreads) k_scan_reduce(const T* __restrict__ in, long long n,
                                                              T* __restrict__ partials) {
  __shared__ T s_warp[kSortWarps];
  const long long base = (long long)blockIdx.x * kSortTile;
  T sum = 0;
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const long long i = base + k * kSortThreads + threadIdx.x;
    if (i < n) sum += in[i];
  }
  T tot;
  block_exclusive_scan<T>(sum, s_warp, tot);
  if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

template <class T>
__global__ void __launch_bounds__(kSortThreads) k_scan_partials(T* __restrict__ partials, long long ntiles) {
  __shared__ T s_warp[kSortWarps];
  T carry = 0;
  for (long long c = 0; c < ntiles; c += kSortThreads) {
    const long long i = c + threadIdx.x;
    const T v = i < ntiles ? partials[i] : (T)0;
    T tot;
    const T ex = block_exclusive_scan<T>(v, s_warp, tot);
    if (i < ntiles) partials[i] = carry + ex;
    carry += tot;
  }
}

// Each thread owns kSortItems consecutive elements of the tile.
template <class T, bool INCLUSIVE>
__global__ void __launch_bounds__(kSortThreads) k_scan_apply(const T* in, T* out, long long n,
                                                             const T* __restrict__ partials) {
  __shared__ T s_tile[kSortTile];
  __shared__ T s_warp[kSortWarps];
  const long long base = (long long)blockIdx.x * kSortTile;
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const long long i = base + k * kSortThreads + threadIdx.x;
    s_tile[k * kSortThreads + threadIdx.x] = i < n ? in[i] : (T)0;
  }
  __syncthreads();
  T v[kSortItems];
  T run = 0;
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    v[k] = s_tile[threadIdx.x * kSortItems + k];
    run += v[k];
  }
  T tot;
  T pre = block_exclusive_scan<T>(run, s_warp, tot) + partials[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const T x = v[k];
    if (INCLUSIVE) pre += x;
    s_tile[threadIdx.x * kSortItems + k] = pre;
    if (!INCLUSIVE) pre += x;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const long long i = base + k * kSortThreads + threadIdx.x;
    if (i < n) out[i] = s_tile[k * kSortThreads + threadIdx.x];
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

template <class K>
size_t radix_sort_temp_bytes(long long n) {
  if (n <= 0) return 0;
  const long long nt = radix_tiles_of(n);
  return align256((size_t)n * sizeof(K)) + align256((size_t)n * 4) + align256((size_t)kBins * nt * 4) +
         align256((size_t)kBins * 4);
}

template <class K>
int radix_sort_pairs(const K* keys_in, K* keys_out, const uint32_t* vals_in, uint32_t* vals_out, long long n,
                     int end_bit, void* temp, size_t temp_bytes, cudaStream_t st) {
  if (n <= 0) return SGR_OK;
  if (temp_bytes < radix_sort_temp_bytes<K>(n) || !temp) return SGR_ERR_WORKSPACE;
  const long long nt = radix_tiles_of(n);
  const size_t dyn = (sizeof(K) + 4) * (size_t)kRadixTile;
  if (cudaFuncSetAttribute(k_radix_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess)
    return SGR_ERR_CUDA;
  char* p = static_cast<char*>(temp);
  K* alt_keys = reinterpret_cast<K*>(p);
  p += align256((size_t)n * sizeof(K));
  uint32_t* alt_vals = reinterpret_cast<uint32_t*>(p);
  p += align256((size_t)n * 4);
  uint32_t* hist = reinterpret_cast<uint32_t*>(p);
  p += align256((size_t)kBins * nt * 4);
  uint32_t* totals = reinterpret_cast<uint32_t*>(p);
  // as few passes as cover the bits, digits as even as possible
  const int passes = (end_bit + kMaxDigitBits - 1) / kMaxDigitBits;
  const int width = passes ? (end_bit + passes - 1) / passes : 0;
  const K* src_k = keys_in;
  const uint32_t* src_v = vals_in;
  for (int pass = 0; pass < passes; ++pass) {
    // the last pass lands in the output buffers
    const bool to_out = ((passes - 1 - pass) % 2) == 0;
    K* dst_k = to_out ? keys_out : alt_keys;
    uint32_t* dst_v = to_out ? vals_out : alt_vals;
    const int shift = width * pass;
    const int bits = end_bit - shift < width ? end_bit - shift : width;
    const uint32_t dmask = (1u << bits) - 1u;
    k_radix_hist<K><<<(unsigned)nt, kSortThreads, 0, st>>>(src_k, n, shift, dmask, hist, nt);
    k_radix_scan<<<kBins, kSortThreads, 0, st>>>(hist, nt, totals);
    k_radix_scatter<K><<<(unsigned)nt, kSortThreads, dyn, st>>>(src_k, src_v, dst_k, dst_v, n, shift, dmask, hist,
                                                                totals, nt);
    count_launches(3);
    src_k = dst_k;
    src_v = dst_v;
  }
  if (passes == 0) {
    if (cudaMemcpyAsync(keys_out, keys_in, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(vals_out, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return SGR_ERR_CUDA;
  }
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

template <class T>
size_t scan_temp_bytes(long long n) {
  return n <= 0 ? 0 : align256((size_t)tiles_of(n) * sizeof(T));
}

template <class T, bool INCLUSIVE>
int prefix_sum(const T* in, T* out, long long n, void* temp, size_t temp_bytes, cudaStream_t st) {
  if (n <= 0) return SGR_OK;
  if (temp_bytes < scan_temp_bytes<T>(n) || !temp) return SGR_ERR_WORKSPACE;
  const long long nt = tiles_of(n);
  T* partials = static_cast<T*>(temp);
  k_scan_reduce<T><<<(unsigned)nt, kSortThreads, 0, st>>>(in, n, partials);
  k_scan_partials<T><<<1, kSortThreads, 0, st>>>(partials, nt);
  k_scan_apply<T, INCLUSIVE><<<(unsigned)nt, kSortThreads, 0, st>>>(in, out, n, partials);
  count_launches(3);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

template size_t radix_sort_temp_bytes<unsigned long long>(long long);
template size_t radix_sort_temp_bytes<uint32_t>(long long);
template int radix_sort_pairs<unsigned long long>(const unsigned long long*, unsigned long long*, const uint32_t*,
                                                  uint32_t*, long long, int, void*, size_t, cudaStream_t);
template int radix_sort_pairs<uint32_t>(const uint32_t*, uint32_t*, const uint32_t*, uint32_t*, long long, int, void*,
                                        size_t, cudaStream_t);
template size_t scan_temp_bytes<unsigned long long>(long long);
template size_t scan_temp_bytes<uint32_t>(long long);
template int prefix_sum<unsigned long long, true>(const unsigned long long*, unsigned long long*, long long, void*,
                                                  size_t, cudaStream_t);
template int prefix_sum<uint32_t, false>(const uint32_t*, uint32_t*, long long, void*, size_t, cudaStream_t);

}  // namespace sgr

extern "C" {

size_t sgr_radix_sort_temp_bytes(int64_t n, int key_bytes) {
  if (key_bytes == 8) return sgr::radix_sort_temp_bytes<unsigned long long>(n);
  if (key_bytes == 4) return sgr::radix_sort_temp_bytes<uint32_t>(n);
  return 0;
}

int sgr_radix_sort_pairs(const void* keys_in, void* keys_out, const uint32_t* vals_in, uint32_t* vals_out, int64_t n,
                         int key_bytes, int end_bit, void* temp, size_t temp_bytes, void* stream) {
  if (n < 0 || (key_bytes != 4 && key_bytes != 8) || end_bit < 0 || end_bit > 8 * key_bytes)
    return SGR_ERR_INVALID_ARGUMENT;
  if (n > 0 && (!keys_in || !keys_out || !vals_in || !vals_out)) return SGR_ERR_INVALID_ARGUMENT;
  if (n >= 0x7fffffffLL) return SGR_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (key_bytes == 8)
    return sgr::radix_sort_pairs<unsigned long long>(static_cast<const unsigned long long*>(keys_in),
                                                     static_cast<unsigned long long*>(keys_out), vals_in, vals_out, n,
                                                     end_bit, temp, temp_bytes, st);
  return sgr::radix_sort_pairs<uint32_t>(static_cast<const uint32_t*>(keys_in), static_cast<uint32_t*>(keys_out),
                                         vals_in, vals_out, n, end_bit, temp, temp_bytes, st);
}

size_t sgr_prefix_sum_temp_bytes(int64_t n, int elem_bytes) {
  if (elem_bytes == 8) return sgr::scan_temp_bytes<unsigned long long>(n);
  if (elem_bytes == 4) return sgr::scan_temp_bytes<uint32_t>(n);
  return 0;
}

int sgr_inclusive_sum_u64(const uint64_t* in, uint64_t* out, int64_t n, void* temp, size_t temp_bytes, void* stream) {
  if (n < 0 || (n > 0 && (!in || !out))) return SGR_ERR_INVALID_ARGUMENT;
  return sgr::prefix_sum<unsigned long long, true>(reinterpret_cast<const unsigned long long*>(in),
                                                   reinterpret_cast<unsigned long long*>(out), n, temp, temp_bytes,
                                                   static_cast<cudaStream_t>(stream));
}

int sgr_exclusive_sum_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp, size_t temp_bytes, void* stream) {
  if (n < 0 || (n > 0 && (!in || !out))) return SGR_ERR_INVALID_ARGUMENT;
  return sgr::prefix_sum<uint32_t, false>(in, out, n, temp, temp_bytes, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
