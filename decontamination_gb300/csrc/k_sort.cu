// Row regrouping of a resident catalogue by key (a counting sort), used between training epochs with the keys the
// BMUs the epoch just found. The reference visits the catalogue in storage order (algo/som_batch.py:285-376); the
// regrouping changes which rows share a 128-row tile of the tensor-core pass, never a row's result: after it, the
// rows of a tile sit near one unit of the map, so the tile's second sweep recomputes only the few column tiles that
// hold candidates (csrc/k1_tc.cu). The per-BMU sums are order-free (exact fixed point).
#include "common.cuh"

namespace somgb {

namespace {

constexpr int SORT_THREADS = 256;

// bucket of a key: keys outside [0, m) go last
__device__ __forceinline__ unsigned long long sort_bucket(int32_t k, int64_t m) {
    return (k >= 0 && (int64_t)k < m) ? (unsigned long long)k : (unsigned long long)m;
}

// counts[b] = rows with bucket b ("+="; zeroed first). Lanes of a warp with the same bucket add once: regrouped keys
// repeat along the rows.
__global__ void __launch_bounds__(SORT_THREADS) sort_count_kernel(const int32_t* __restrict__ key, int64_t n,
                                                                  int64_t m, unsigned long long* __restrict__ counts) {
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * SORT_THREADS; base < n; base += (int64_t)gridDim.x * SORT_THREADS) {
        const int64_t i = base + threadIdx.x;
        const bool in = i < n;
        const unsigned long long b = in ? sort_bucket(key[i], m) : ~0ull;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        if (in && __ffs(same) - 1 == lane) atomicAdd(counts + b, (unsigned long long)__popc(same));
    }
}

// cursor[b] = sum of counts[0..b) (one CTA; the buckets are map units plus one)
__global__ void __launch_bounds__(1024) sort_scan_kernel(const unsigned long long* __restrict__ counts, int64_t nb,
                                                         unsigned long long* __restrict__ cursor) {
    __shared__ unsigned long long warp_sums[32];
    __shared__ unsigned long long carry_s;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const unsigned long long v = i < nb ? counts[i] : 0ull;
        unsigned long long s = v;   // inclusive scan within the warp
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        if (lane == 31) warp_sums[wid] = s;
        __syncthreads();
        if (wid == 0) {
            unsigned long long ws = warp_sums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long t = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += t;
            }
            warp_sums[lane] = ws;
        }
        __syncthreads();
        const unsigned long long carry = carry_s;
        const unsigned long long before = carry + (wid > 0 ? warp_sums[wid - 1] : 0ull) + s - v;
        if (i < nb) cursor[i] = before;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s = before + v;
        __syncthreads();
    }
}

// x_out/rho_out[cursor[b]++] = x/rho[i]; the lanes of a warp with the same bucket take consecutive positions with one
// atomic. VEC = 4: rows of d % 4 == 0 floats, 16-byte aligned, copied as float4.
template <int VEC>
__global__ void __launch_bounds__(SORT_THREADS) sort_scatter_kernel(const float* __restrict__ x,
                                                                    const double* __restrict__ rho,
                                                                    const int32_t* __restrict__ key, int64_t n, int d,
                                                                    int64_t m, unsigned long long* __restrict__ cursor,
                                                                    float* __restrict__ x_out,
                                                                    double* __restrict__ rho_out) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    for (int64_t base = (int64_t)blockIdx.x * SORT_THREADS; base < n; base += (int64_t)gridDim.x * SORT_THREADS) {
        const int64_t i = base + threadIdx.x;
        const bool in = i < n;
        const unsigned long long b = in ? sort_bucket(key[i], m) : ~0ull;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(same) - 1;
        unsigned long long first = 0;
        if (in && leader == lane) first = atomicAdd(cursor + b, (unsigned long long)__popc(same));
        first = __shfl_sync(0xffffffffu, first, leader);
        // one bucket for the whole warp (b names a bucket, so every lane's row exists): 32 consecutive rows to 32
        // consecutive slots
        if (VEC == 4 && same == 0xffffffffu && b != ~0ull) {
            const int64_t i0 = i - lane, p0 = (int64_t)first;
            const float4* src = (const float4*)(x + i0 * d);
            float4* dst = (float4*)(x_out + p0 * d);
#pragma unroll 4   // several loads in flight per lane
            for (int k = lane; k < 8 * d; k += 32) dst[k] = __ldg(src + k);
            if (rho) rho_out[p0 + lane] = rho[i];
            continue;
        }
        if (!in) continue;
        const int64_t pos = (int64_t)(first + (unsigned long long)__popc(same & below));
        if (VEC == 4) {
            const float4* src = (const float4*)(x + i * d);
            float4* dst = (float4*)(x_out + pos * d);
#pragma unroll 4
            for (int k = 0; k < d / 4; ++k) dst[k] = __ldg(src + k);
        } else {
            for (int k = 0; k < d; ++k) x_out[pos * d + k] = __ldg(x + i * d + k);
        }
        if (rho) rho_out[pos] = rho[i];
    }
}

// The same scatter for regrouped keys (long runs of one key along the rows) and m + 1 buckets in shared memory: block
// b moves the contiguous rows [b * chunk, (b + 1) * chunk), first counting its rows per bucket, then taking each
// bucket's slots with one global atomic, then placing its rows. Few blocks share a bucket, where the row-wise form
// makes every warp of a long run contend for the same counter.
constexpr int SORT_BLOCK_THREADS = 512;
template <int VEC>
__global__ void __launch_bounds__(SORT_BLOCK_THREADS) sort_scatter_block_kernel(
    const float* __restrict__ x, const double* __restrict__ rho, const int32_t* __restrict__ key, int64_t n, int d,
    int64_t m, int64_t chunk, unsigned long long* __restrict__ cursor, float* __restrict__ x_out,
    double* __restrict__ rho_out) {
    extern __shared__ unsigned long long slot[];   // [m + 1]: this block's rows per bucket, then its next slot
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int64_t r0 = (int64_t)blockIdx.x * chunk, r1 = min64(n, r0 + chunk);
    for (int64_t b = threadIdx.x; b <= m; b += SORT_BLOCK_THREADS) slot[b] = 0;
    __syncthreads();
    for (int64_t base = r0; base < r1; base += SORT_BLOCK_THREADS) {
        const int64_t i = base + threadIdx.x;
        const bool in = i < r1;
        const unsigned long long b = in ? sort_bucket(key[i], m) : ~0ull;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        if (in && __ffs(same) - 1 == lane) atomicAdd(slot + b, (unsigned long long)__popc(same));
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b <= m; b += SORT_BLOCK_THREADS) {
        const unsigned long long c = slot[b];
        if (c) slot[b] = atomicAdd(cursor + b, c);
    }
    __syncthreads();
    for (int64_t base = r0; base < r1; base += SORT_BLOCK_THREADS) {
        const int64_t i = base + threadIdx.x;
        const bool in = i < r1;
        const unsigned long long b = in ? sort_bucket(key[i], m) : ~0ull;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(same) - 1;
        unsigned long long first = 0;
        if (in && leader == lane) first = atomicAdd(slot + b, (unsigned long long)__popc(same));
        first = __shfl_sync(0xffffffffu, first, leader);
        // one bucket for the whole warp (b names a bucket, so every lane's row exists): 32 consecutive rows to 32
        // consecutive slots
        if (VEC == 4 && same == 0xffffffffu && b != ~0ull) {
            const int64_t i0 = i - lane, p0 = (int64_t)first;
            const float4* src = (const float4*)(x + i0 * d);
            float4* dst = (float4*)(x_out + p0 * d);
#pragma unroll 4   // several loads in flight per lane
            for (int k = lane; k < 8 * d; k += 32) dst[k] = __ldg(src + k);
            if (rho) rho_out[p0 + lane] = rho[i];
            continue;
        }
        if (!in) continue;
        const int64_t pos = (int64_t)(first + (unsigned long long)__popc(same & below));
        if (VEC == 4) {
            const float4* src = (const float4*)(x + i * d);
            float4* dst = (float4*)(x_out + pos * d);
#pragma unroll 4
            for (int k = 0; k < d / 4; ++k) dst[k] = __ldg(src + k);
        } else {
            for (int k = 0; k < d; ++k) x_out[pos * d + k] = __ldg(x + i * d + k);
        }
        if (rho) rho_out[pos] = rho[i];
    }
}

}  // namespace

size_t sort_rows_workspace(int64_t m) { return m >= 0 ? 2 * align_up((size_t)(m + 1) * 8, 256) : 0; }

int launch_sort_rows(const float* x, const double* rho, const int32_t* key, int64_t n, int d, int64_t m,
                     float* x_out, double* rho_out, void* ws, size_t ws_bytes, cudaStream_t stream) {
    if (ws_bytes < sort_rows_workspace(m)) return set_error(SOMGB_ERR_WORKSPACE, "sort workspace too small");
    if (n == 0) return SOMGB_OK;
    unsigned long long* counts = (unsigned long long*)ws;
    unsigned long long* cursor = (unsigned long long*)((uint8_t*)ws + align_up((size_t)(m + 1) * 8, 256));
    SOMGB_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)(m + 1) * 8, stream));
    const unsigned grid = (unsigned)std::min<int64_t>(ceil_div(n, SORT_THREADS), 8 * (int64_t)num_sms());
    sort_count_kernel<<<grid, SORT_THREADS, 0, stream>>>(key, n, m, counts);
    SOMGB_LAUNCH_CHECK();
    sort_scan_kernel<<<1, 1024, 0, stream>>>(counts, m + 1, cursor);
    SOMGB_LAUNCH_CHECK();
    const bool vec = d % 4 == 0 && ((uintptr_t)x) % 16 == 0 && ((uintptr_t)x_out) % 16 == 0;
    const size_t smem = (size_t)(m + 1) * 8;
    if (smem <= 96 * 1024) {   // the buckets fit shared memory: two blocks per SM, contiguous row ranges
        const int64_t blocks = std::min<int64_t>(ceil_div(n, SORT_BLOCK_THREADS), 2 * (int64_t)num_sms());
        const int64_t chunk = ceil_div(n, blocks);
        auto kern = vec ? sort_scatter_block_kernel<4> : sort_scatter_block_kernel<1>;
        SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<(unsigned)ceil_div(n, chunk), SORT_BLOCK_THREADS, smem, stream>>>(x, rho, key, n, d, m, chunk, cursor,
                                                                                 x_out, rho_out);
        SOMGB_LAUNCH_CHECK();
        return SOMGB_OK;
    }
    if (vec)
        sort_scatter_kernel<4><<<grid, SORT_THREADS, 0, stream>>>(x, rho, key, n, d, m, cursor, x_out, rho_out);
    else
        sort_scatter_kernel<1><<<grid, SORT_THREADS, 0, stream>>>(x, rho, key, n, d, m, cursor, x_out, rho_out);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

}  // namespace somgb
