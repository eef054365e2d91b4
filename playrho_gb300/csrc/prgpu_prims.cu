// prgpu_prims.cu -- device-wide exclusive scan and stable LSD radix sort.
//
// Both primitives read their element count from device memory so that a step
// captured once in a CUDA graph replays with whatever counts the previous
// kernels produced.  The grid is fixed (a multiple of the SM count); block b
// owns the contiguous chunk [b*ceil(n/G), (b+1)*ceil(n/G)), which keeps the
// sort stable without a global look-back.
#include <algorithm>

#include "prgpu_internal.cuh"

namespace prgpu {

namespace {

constexpr int kScanThreads = 256;
constexpr uint32_t kScanItems = 8;
constexpr int kSortThreads = 256;
constexpr int kRadix = 256;

__device__ __forceinline__ uint32_t chunk_of(uint32_t n, uint32_t& lo, uint32_t& hi) {
    const uint32_t g = gridDim.x;
    const uint32_t chunk = (n + g - 1u) / g;
    lo = min(n, blockIdx.x * chunk);
    hi = min(n, lo + chunk);
    return chunk;
}

// Inclusive block scan of one value per thread (256 threads).
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t& block_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t prefix = (warp > 0) ? s_warp[warp - 1] : 0u;
    block_total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return v + prefix;
}

__global__ void k_scan_reduce(const uint32_t* __restrict__ in, const uint32_t* n_ptr, uint32_t* partial) {
    __shared__ uint32_t s[32];
    uint32_t lo, hi;
    chunk_of(*n_ptr, lo, hi);
    // four independent loads in flight per thread
    uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    const uint32_t step = blockDim.x;
    uint32_t i = lo + threadIdx.x;
    for (; i + 3u * step < hi; i += 4u * step) {
        s0 += in[i];
        s1 += in[i + step];
        s2 += in[i + 2u * step];
        s3 += in[i + 3u * step];
    }
    for (; i < hi; i += step) s0 += in[i];
    uint32_t sum = (s0 + s1) + (s2 + s3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) t += s[w];
        partial[blockIdx.x] = t;
    }
}

__global__ void k_scan_partials(uint32_t* partial, int g, uint32_t* total) {
    __shared__ uint32_t s_warp[32];
    // one block of 1024 threads, g <= 1024
    uint32_t v = (threadIdx.x < (unsigned)g) ? partial[threadIdx.x] : 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t incl = x + ((warp > 0) ? s_warp[warp - 1] : 0u);
    if (threadIdx.x < (unsigned)g) partial[threadIdx.x] = incl - v;
    if (threadIdx.x == blockDim.x - 1 && total) *total = incl;
}

__global__ void k_scan_down(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, const uint32_t* n_ptr,
                            const uint32_t* partial) {
    __shared__ uint32_t s_warp[32];
    uint32_t lo, hi;
    chunk_of(*n_ptr, lo, hi);
    // kScanItems consecutive elements per thread: one block scan per
    // kScanItems * blockDim elements
    uint32_t running = partial[blockIdx.x];
    for (uint32_t base = lo; base < hi; base += blockDim.x * kScanItems) {
        const uint32_t i0 = base + threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
        uint32_t sum = 0;
#pragma unroll
        for (uint32_t j = 0; j < kScanItems; ++j) {
            v[j] = (i0 + j < hi) ? in[i0 + j] : 0u;
            sum += v[j];
        }
        uint32_t tot;
        uint32_t r = running + block_inclusive_scan(sum, s_warp, tot) - sum;
#pragma unroll
        for (uint32_t j = 0; j < kScanItems; ++j) {
            if (i0 + j < hi) out[i0 + j] = r;
            r += v[j];
        }
        running += tot;
    }
}

// ---- radix sort -----------------------------------------------------------
// Multi-block path (n > kSmallSort): one cooperative launch runs every pass;
// per pass each block counts the digits of its chunk, the digit rows of those
// counts are scanned across blocks (a warp per digit, coalesced) with the digit
// totals, and each block scatters its chunk stably; a bounded grid barrier
// separates the three.  Small inputs (n <= kSmallSort, e.g. the few new
// contacts of a step) are sorted by a single block in shared memory, and the
// cooperative launch returns at once, as it does for n = 0 (a step that
// rebuilds no tree): one launch a sort instead of three a pass.
//
// Data that other blocks wrote earlier in the launch (the keys and values of
// the previous pass, the digit counts) is read through L2 (__ldcg): a block's
// L1 may hold lines of those arrays from before the barrier.
constexpr uint32_t kSmallSort = 4096;

__global__ void __launch_bounds__(kSortThreads) k_radix_coop(uint64_t* keys, uint64_t* keys_alt, uint32_t* vals,
                                                              uint32_t* vals_alt, const uint32_t* n_ptr, int passes,
                                                              uint32_t* hist, Counters* cnt) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ uint32_t s_cnt[kRadix];
    __shared__ uint32_t s_base[kRadix];
    __shared__ uint32_t s_wcnt[kWarps][kRadix];
    const uint32_t n = *n_ptr;
    if (n <= kSmallSort) return;
    const uint32_t g = gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t lo, hi;
    chunk_of(n, lo, hi);
    const uint64_t* kin = keys;
    const uint32_t* vin = vals;
    uint64_t* kout = keys_alt;
    uint32_t* vout = vals_alt;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * 8;
        // digit counts of this block's chunk
        for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) s_cnt[dd] = 0u;
        __syncthreads();
        for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
            atomicAdd(&s_cnt[(uint32_t)(__ldcg(kin + i) >> shift) & 0xffu], 1u);
        __syncthreads();
        for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) hist[dd * g + blockIdx.x] = s_cnt[dd];
        grid_barrier(cnt);
        // hist[d*g + b] becomes block b's exclusive offset within digit d,
        // hist[kRadix*g + d] digit d's total
        for (uint32_t dd = blockIdx.x * kWarps + warp; dd < (uint32_t)kRadix; dd += g * kWarps) {
            uint32_t run = 0;
            for (uint32_t b0 = 0; b0 < g; b0 += 32) {
                const uint32_t b = b0 + lane;
                const uint32_t v = (b < g) ? __ldcg(hist + dd * g + b) : 0u;
                uint32_t x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += t;
                }
                if (b < g) hist[dd * g + b] = run + x - v;
                run += __shfl_sync(0xffffffffu, x, 31);
            }
            if (lane == 0) hist[kRadix * g + dd] = run;
        }
        grid_barrier(cnt);
        // this block's base of each digit: the digits before it, then the blocks before it
        if (warp == 0) {
            uint32_t run = 0;
            for (int d0 = 0; d0 < kRadix; d0 += 32) {
                const uint32_t v = __ldcg(hist + kRadix * g + d0 + lane);
                uint32_t x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += t;
                }
                s_base[d0 + lane] = run + x - v;
                run += __shfl_sync(0xffffffffu, x, 31);
            }
        }
        __syncthreads();
        for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) s_base[dd] += __ldcg(hist + dd * g + blockIdx.x);
        // stable scatter of the chunk: ranks within a warp by match, warps in order
        for (uint32_t base = lo; base < hi; base += blockDim.x) {
            for (int k = threadIdx.x; k < kWarps * kRadix; k += blockDim.x) (&s_wcnt[0][0])[k] = 0u;
            __syncthreads();
            const uint32_t i = base + threadIdx.x;
            const bool valid = i < hi;
            uint64_t key = 0;
            uint32_t val = 0, d = 0xffffffffu;
            if (valid) {
                key = __ldcg(kin + i);
                val = __ldcg(vin + i);
                d = (uint32_t)(key >> shift) & 0xffu;
            }
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            const uint32_t rank = __popc(peers & lt);
            if (valid && rank == 0) s_wcnt[warp][d] = __popc(peers);
            __syncthreads();
            if (valid) {
                uint32_t off = s_base[d] + rank;
                for (int w = 0; w < warp; ++w) off += s_wcnt[w][d];
                kout[off] = key;
                vout[off] = val;
            }
            __syncthreads();
            for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) {
                uint32_t t = 0;
                for (int w = 0; w < kWarps; ++w) t += s_wcnt[w][dd];
                s_base[dd] += t;
            }
            __syncthreads();
        }
        grid_barrier(cnt);
        const uint64_t* tk = kout;
        kout = const_cast<uint64_t*>(kin);
        kin = tk;
        const uint32_t* tv = vout;
        vout = const_cast<uint32_t*>(vin);
        vin = tv;
    }
}

// Single-block LSD radix sort of n <= kSmallSort pairs in shared memory,
// reading (kin, vin) and writing the sorted result to (kout, vout).
constexpr int kSmallThreads = 1024;
__global__ void __launch_bounds__(kSmallThreads) k_small_sort(const uint64_t* kin, const uint32_t* vin,
                                                               uint64_t* kout, uint32_t* vout,
                                                               const uint32_t* n_ptr, int bits) {
    constexpr int kWarps = kSmallThreads / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t n = *n_ptr;
    if (n == 0 || n > kSmallSort) return;
    uint64_t* ka = reinterpret_cast<uint64_t*>(smem);
    uint64_t* kb = ka + kSmallSort;
    uint32_t* va = reinterpret_cast<uint32_t*>(kb + kSmallSort);
    uint32_t* vb = va + kSmallSort;
    __shared__ uint32_t s_base[kRadix];
    __shared__ uint32_t s_cnt[kRadix];
    __shared__ uint32_t s_wcnt[kWarps][kRadix];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) { ka[i] = kin[i]; va[i] = vin[i]; }
    __syncthreads();
    for (int shift = 0; shift < bits; shift += 8) {
        for (int d = threadIdx.x; d < kRadix; d += blockDim.x) s_cnt[d] = 0u;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&s_cnt[(uint32_t)(ka[i] >> shift) & 0xffu], 1u);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int d = 0; d < kRadix; ++d) { s_base[d] = run; run += s_cnt[d]; }
        }
        __syncthreads();
        for (uint32_t base = 0; base < n; base += blockDim.x) {
            for (int k = threadIdx.x; k < kWarps * kRadix; k += blockDim.x) (&s_wcnt[0][0])[k] = 0u;
            __syncthreads();
            const uint32_t i = base + threadIdx.x;
            const bool valid = i < n;
            uint64_t key = 0;
            uint32_t val = 0, d = 0xffffffffu;
            if (valid) { key = ka[i]; val = va[i]; d = (uint32_t)(key >> shift) & 0xffu; }
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            const uint32_t rank = __popc(peers & lt);
            if (valid && rank == 0) s_wcnt[warp][d] = __popc(peers);
            __syncthreads();
            if (valid) {
                uint32_t off = s_base[d] + rank;
                for (int w = 0; w < warp; ++w) off += s_wcnt[w][d];
                kb[off] = key;
                vb[off] = val;
            }
            __syncthreads();
            for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) {
                uint32_t t = 0;
                for (int w = 0; w < kWarps; ++w) t += s_wcnt[w][dd];
                s_base[dd] += t;
            }
            __syncthreads();
        }
        uint64_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) { kout[i] = ka[i]; vout[i] = va[i]; }
}

constexpr size_t kSmallSmem = (size_t)kSmallSort * 2 * (sizeof(uint64_t) + sizeof(uint32_t));

}  // namespace

void scan_exclusive(const Prims& P, const uint32_t* in, uint32_t* out, const uint32_t* n, uint32_t* total,
                    uint32_t* partial, cudaStream_t s) {
    k_scan_reduce<<<P.grid, kScanThreads, 0, s>>>(in, n, partial);
    k_scan_partials<<<1, 1024, 0, s>>>(partial, P.grid, total);
    k_scan_down<<<P.grid, kScanThreads, 0, s>>>(in, out, n, partial);
}

bool radix_sort(const Prims& P, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                const uint32_t* n, int bits, uint32_t* hist, Counters* cnt, cudaStream_t s) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_small_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmem);
        attr_set = true;
    }
    const int passes = (bits + 7) / 8;
    const bool alt = (passes % 2) == 1;
    // small inputs: one block, result written straight to where the passes would leave it
    k_small_sort<<<1, kSmallThreads, kSmallSmem, s>>>(keys, vals, alt ? keys_alt : keys, alt ? vals_alt : vals, n,
                                                      passes * 8);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)radix_coop_grid(P));
    cfg.blockDim = dim3((unsigned)kSortThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_radix_coop, keys, keys_alt, vals, vals_alt, n, passes, hist, cnt);
    return alt;
}

int radix_coop_grid(const Prims& P) {
    // every block of the cooperative sort must be resident at once
    static int per_sm = -1;
    if (per_sm < 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_radix_coop, kSortThreads, 0) != cudaSuccess) b = 1;
        per_sm = b < 1 ? 1 : b;
    }
    return std::min(P.grid, per_sm * P.sm_count);
}

}  // namespace prgpu
