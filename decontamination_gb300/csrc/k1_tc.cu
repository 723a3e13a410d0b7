// K1: BMU search on the tcgen05 tensor cores (split-BF16 distance GEMM), exact by construction.
//
// Distances are expanded as |x - w_j|^2 = |x'|^2 + s_j with s_j = |w'_j|^2 - 2 x'.w'_j, where x' = x - c and
// w' = w - c are centred on the mean unit c (the centring shrinks every error term below). One GEMM per 128-sample
// row tile and 256-unit column tile produces s~_j in TMEM:
//   A row (sample)  = [ x'_hi | x'_lo | x'_hi | 1 | 1 | 0 ... ]            (BF16, K padded to a multiple of 16)
//   B row (unit j)  = [ -2w'_hi | -2w'_hi | -2w'_lo | q_hi | q_lo | 0 ... ] with q = |w'_j|^2
// so that sum_k A.B = -2 (x_hi w_hi + x_lo w_hi + x_hi w_lo) + q ~ s_j, accumulated in FP32.
//
// Error bound. With BF16 unit roundoff 2^-8, dropping x_lo w_lo and the two-term residuals costs at most
// 3.01 * 2^-16 |x'_k||w'_k| per product; q's split and float32 evaluation cost 2.5 * 2^-16 |w'|^2; the FP32 accumulation of
// the K non-zero products is bounded by K * 2^-23 * sum|terms| (one rounding per product, the worst case).
// Using |w'_j|^2 <= 2|x'|^2 + 2 d'_j (d'_j = |x' - w'_j|^2) every term is bounded by
//   |s~_j - s_j| <= alpha |x'|^2 + beta d'_j,
// with alpha, beta computed on the host (tc_error_coefficients). A unit can beat the tile's best (or, for the
// error sums, the second best) only if s~_j <= m + 2 (alpha |x'|^2 + beta (m + |x'|^2)) / (1 - beta), m being the
// best (second-best) s~ of the row.
//
// Epilogue, per row tile: sweep 1 streams the TMEM tiles and keeps the best (and second-best) s~ per row with
// FP32 min/max (full-rate ALU); sweep 2 recomputes the same MMAs (the tensor pipe has slack) and collects every
// unit under that threshold — the only units that can be the reference's BMU (or second BMU). Each candidate's
// distance is then evaluated on CUDA cores with float32 differences (the reference's terms) and, when two
// candidates are within float32 rounding of each other, with the reference's float64 sum. Rows with more than
// CAP candidates, non-finite features or overflowing distances go to an exact per-row recheck kernel.
//
// Pipeline (one persistent CTA per SM, 192 threads):
//   warp 5      TMA producer: the unit operand B once (bulk copy), sample tiles (2-D tiled TMA, 3-stage ring);
//   warp 4      TMEM allocator and MMA issuer (one thread), two 256-column TMEM accumulators;
//   warps 0-3   converter (FP32 tile -> centred split-BF16 A tile) and epilogue; thread r owns TMEM lane r.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "tc.cuh"
#include "tc_ptx.cuh"

namespace somgb {

// Sticky device status: bit set by any bounded wait of the tensor-core pass that gave up (0 = healthy).
__device__ unsigned int g_tc_status;

// Optional per-phase cycle counters of the epilogue warps (compiled in only with -DSOMGB_TC_PHASE_TIMING; read with
// cudaMemcpyFromSymbol). Phases: 0 wait for TMEM (sweep 1), 1 sweep 1, 2 wait (sweep 2), 3 sweep 2, 4 convert,
// 5 row barriers, 6 resolution, 7 slice-0 decision.
#ifdef SOMGB_TC_PHASE_TIMING
__device__ unsigned long long g_tc_phase_cycles[8];
#define TC_T0() _tc_t0 = clock64()
#define TC_T(ph)                                    \
    do {                                            \
        const long long _tc_t1 = clock64();         \
        _tc_acc[ph] += (unsigned long long)(_tc_t1 - _tc_t0); \
        _tc_t0 = _tc_t1;                            \
    } while (0)
#else
#define TC_T0() \
    do {        \
    } while (0)
#define TC_T(ph) \
    do {         \
    } while (0)
#endif

namespace {

constexpr int TM = 128;           // samples per row tile (MMA M)
constexpr int TN = 256;           // units per column tile (MMA N)
constexpr int SLICES = 4;         // epilogue warps per TMEM lane quarter, each owning 64 of 256 columns
constexpr int CAPR = 32;          // candidates kept per row (a pool shared by the row's four slices)
constexpr int XSTAGES = 3;
constexpr int EPI_WARPS = 4 * SLICES;
constexpr int MMA_WARP = EPI_WARPS;
constexpr int TMA_WARP = EPI_WARPS + 1;
constexpr int NUM_THREADS = (EPI_WARPS + 2) * 32;
constexpr float BIG = 3.0e38f;    // s~ of padding / invalid units
constexpr float HUGE_S = 1.0e30f; // rows whose best s~ + |x'|^2 reaches this go to the exact recheck
constexpr uint32_t IDESC = ptx::idesc_bf16_f32(TM, TN);

struct TcShape {
    int d = 0, kpad = 0, knz = 0;
    int64_t mpad = 0;
    int utiles = 0;
    size_t b_bytes = 0, a_bytes = 0, x_bytes = 0;
    size_t off_a = 0, off_x = 0, off_cand = 0, off_part = 0, off_res = 0, off_center = 0, off_bar = 0, smem = 0;
};

TcShape tc_shape(int64_t m, int d) {
    TcShape s;
    s.d = d;
    s.knz = 3 * d + 2;
    s.kpad = (int)align_up((size_t)s.knz, 16);
    s.mpad = (int64_t)align_up((size_t)m, TN);
    s.utiles = (int)(s.mpad / TN);
    s.b_bytes = (size_t)s.mpad * s.kpad * 2;
    s.a_bytes = (size_t)TM * s.kpad * 2;
    s.x_bytes = align_up((size_t)TM * d * 4, 128);
    size_t off = align_up(s.b_bytes, 1024);
    s.off_a = off;
    off += 2 * align_up(s.a_bytes, 1024);
    s.off_x = off;
    off += XSTAGES * s.x_bytes;
    s.off_cand = off;
    off += (size_t)CAPR * TM * 4;
    s.off_part = off;
    off += (size_t)SLICES * TM * 8;
    s.off_res = off;
    off += (size_t)(CAPR + 1) * TM * 4;
    s.off_center = off;
    off += align_up((size_t)d * 4, 16);
    s.off_bar = align_up(off, 8);
    off = s.off_bar + 16 * 8;
    s.smem = off + 1024;   // slack for aligning the dynamic base to 1024
    return s;
}

// Scratch: [B operand | centre (d floats) | recheck row list (n int32)]
struct TcWs {
    uint8_t* b = nullptr;
    float* center = nullptr;
    int32_t* rows = nullptr;
};

size_t tc_ws_layout(int64_t n, int64_t m, int d, TcWs* out, void* base) {
    TcShape s = tc_shape(m, d);
    size_t off = 0;
    size_t ob = off;
    off += align_up(s.b_bytes, 256);
    size_t oc = off;
    off += align_up((size_t)d * 4, 256);
    size_t orow = off;
    off += align_up((size_t)std::max<int64_t>(n, 1) * 4, 256);
    if (out && base) {
        uint8_t* p = (uint8_t*)base;
        out->b = p + ob;
        out->center = (float*)(p + oc);
        out->rows = (int32_t*)(p + orow);
    }
    return off;
}

void tc_error_coefficients(int d, float* alpha, float* beta) {
    const double u16 = std::ldexp(1.0, -16);
    const double knz = 3.0 * d + 2.0;
    const double acc = knz * std::ldexp(1.0, -23);       // one rounding per product, worst case
    // representation: 3.01*2^-16 (|x'|^2 + |w'|^2) from -2 x'.w'; 2.5*2^-16 |w'|^2 from q; |w'|^2 <= 2|x'|^2 + 2d'
    double a = 3.01 * u16 * 3.0 + 2.5 * u16 * 2.0 + acc * 5.05;
    double b = 3.01 * u16 * 2.0 + 2.5 * u16 * 2.0 + acc * 4.04;
    // centring rounding and the reference's own float32 rounding of each term
    a += std::ldexp(1.0, -21);
    b += std::ldexp(1.0, -21);
    *alpha = (float)(1.25 * a);   // 25% safety margin
    *beta = (float)(1.25 * b);
}

// ---------------------------------------------------------------------------------------------------------------------
// prep: centre and unit operand
// ---------------------------------------------------------------------------------------------------------------------

__global__ void tc_center_kernel(const float* __restrict__ w, int64_t m, int d, float* __restrict__ center) {
    // mean of the finite unit rows, per feature, in float64
    __shared__ double part[256];
    __shared__ unsigned long long cnt_s;
    if (threadIdx.x == 0) cnt_s = 0;
    __syncthreads();
    for (int k = 0; k < d; ++k) {
        double s = 0.0;
        unsigned long long c = 0;
        for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
            bool ok = true;
            for (int q = 0; q < d; ++q) ok = ok && isfinite(w[j * d + q]);
            if (ok) { s += (double)w[j * d + k]; ++c; }
        }
        part[threadIdx.x] = s;
        if (k == 0 && c) atomicAdd(&cnt_s, c);
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) center[k] = cnt_s ? (float)(part[0] / (double)cnt_s) : 0.0f;
        __syncthreads();
    }
}

__device__ __forceinline__ size_t canon_off(int64_t row, int k, int kpad) {
    return (size_t)(row >> 3) * (kpad >> 3) * 128 + (size_t)(k >> 3) * 128 + (size_t)(row & 7) * 16 + (size_t)(k & 7) * 2;
}

__global__ void tc_prep_b_kernel(const float* __restrict__ w, int64_t m, int d, int kpad, int64_t mpad,
                                 const float* __restrict__ center, uint8_t* __restrict__ b) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mpad) return;
    __nv_bfloat16* out = (__nv_bfloat16*)b;
    auto put = [&](int k, float v) { *(__nv_bfloat16*)((uint8_t*)out + canon_off(j, k, kpad)) = __float2bfloat16_rn(v); };
    bool valid = j < m;
    float q = 0.0f;
    if (valid) {
        for (int k = 0; k < d; ++k) {
            float v = w[j * d + k];
            if (!isfinite(v)) valid = false;
            float t = v - center[k];
            q = fmaf(t, t, q);
        }
        if (!(q < HUGE_S)) valid = false;
    }
    for (int k = 0; k < kpad; ++k) put(k, 0.0f);
    if (!valid) {
        put(3 * d, BIG);   // never the minimum; s~ = BIG
        return;
    }
    for (int k = 0; k < d; ++k) {
        float t = w[j * d + k] - center[k];
        __nv_bfloat16 hi = __float2bfloat16_rn(t);
        __nv_bfloat16 lo = __float2bfloat16_rn(t - __bfloat162float(hi));
        put(k, -2.0f * __bfloat162float(hi));
        put(d + k, -2.0f * __bfloat162float(hi));
        put(2 * d + k, -2.0f * __bfloat162float(lo));
    }
    __nv_bfloat16 qh = __float2bfloat16_rn(q);
    put(3 * d, __bfloat162float(qh));
    put(3 * d + 1, q - __bfloat162float(qh));
}

// ---------------------------------------------------------------------------------------------------------------------
// main pass
// ---------------------------------------------------------------------------------------------------------------------

struct TcArgs {
    PassArgs a;
    const uint8_t* b;
    const float* center;
    int32_t* rows;
    unsigned long long* row_count;
    int kpad;
    int utiles;
    float alpha, beta;
    size_t off_a, off_x, off_cand, off_part, off_res, off_center, off_bar, a_stride, x_stride;
    uint32_t b_bytes;
};

// float32 distance over the reference's float32 differences (FMA chain): |df - d_ref| <= (D+2) 2^-24 d_ref
template <int DT>
__device__ __forceinline__ float cand_dist32v(const float* __restrict__ wr, const float (&xr)[DT]) {
    float acc = 0.0f;
    const float4* w4 = (const float4*)wr;
#pragma unroll
    for (int k4 = 0; k4 < DT / 4; ++k4) {
        const float4 w = __ldg(w4 + k4);
        float t = w.x - xr[4 * k4]; acc = fmaf(t, t, acc);
        t = w.y - xr[4 * k4 + 1]; acc = fmaf(t, t, acc);
        t = w.z - xr[4 * k4 + 2]; acc = fmaf(t, t, acc);
        t = w.w - xr[4 * k4 + 3]; acc = fmaf(t, t, acc);
    }
    return acc;
}

// Reference distance (float64 sum of float32 squares) as an exact float32 pair; used for d1 of QE.
template <int DT>
__device__ __forceinline__ DFloat ref_dist_pair(const float* __restrict__ wr, const float (&xr)[DT]) {
    DFAcc acc;
    const float4* w4 = (const float4*)wr;
#pragma unroll
    for (int k4 = 0; k4 < DT / 4; ++k4) {
        const float4 w = __ldg(w4 + k4);
        const float t0 = __fsub_rn(w.x, xr[4 * k4]), t1 = __fsub_rn(w.y, xr[4 * k4 + 1]);
        const float t2 = __fsub_rn(w.z, xr[4 * k4 + 2]), t3 = __fsub_rn(w.w, xr[4 * k4 + 3]);
        acc.add(__fmul_rn(t0, t0));
        acc.add(__fmul_rn(t1, t1));
        acc.add(__fmul_rn(t2, t2));
        acc.add(__fmul_rn(t3, t3));
    }
    return DFloat{acc.hi, acc.lo};
}

template <bool ERR, int DT>
__global__ void __launch_bounds__(NUM_THREADS, 1) tc_pass_kernel(const __grid_constant__ CUtensorMap tmap, TcArgs P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sB = smem;
    float* sCenter = (float*)(smem + P.off_center);
    int32_t* sCand = (int32_t*)(smem + P.off_cand);   // [CAPR][TM]: candidate units of each row
    float2* sPart = (float2*)(smem + P.off_part);     // [slice][TM]: (m1, m2) of the slice
    float* sCandD = (float*)(smem + P.off_res);       // [CAPR][TM]: float32 distance of each candidate
    int* sCandN = (int*)(smem + P.off_res + (size_t)CAPR * TM * 4);   // [TM]: candidates claimed by the row
    uint64_t* bars = (uint64_t*)(smem + P.off_bar);
    uint64_t* b_full = bars + 0;
    uint64_t* x_full = bars + 1;    // [3]
    uint64_t* x_empty = bars + 4;   // [3]
    uint64_t* a_full = bars + 7;    // [2]
    uint64_t* a_empty = bars + 9;   // [2]
    uint64_t* t_full = bars + 11;   // [2]
    uint64_t* t_empty = bars + 13;  // [2]
    uint64_t* drain = bars + 15;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_s;

    const PassArgs& a = P.a;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int d = DT;
    constexpr int kpad = (3 * DT + 2 + 15) / 16 * 16;
    const int U = P.utiles;
    const int64_t num_tiles = (a.n + TM - 1) / TM;
    const int64_t n_my = blockIdx.x < num_tiles ? (num_tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

    if (tid == 0) {
        ptx::mbar_init(b_full, 1);
        for (int s = 0; s < XSTAGES; ++s) {
            ptx::mbar_init(x_full + s, 1);
            ptx::mbar_init(x_empty + s, EPI_WARPS);
        }
        for (int s = 0; s < 2; ++s) {
            ptx::mbar_init(a_full + s, EPI_WARPS);
            ptx::mbar_init(a_empty + s, 1);
            ptx::mbar_init(t_full + s, 1);
            ptx::mbar_init(t_empty + s, EPI_WARPS);
        }
        ptx::mbar_init(drain, 1);
        ptx::fence_mbar_init();
        abort_s = 0;
    }
    for (int k = tid; k < d; k += NUM_THREADS) sCenter[k] = P.center[k];
    if (warp == MMA_WARP) {
        ptx::tmem_alloc(&tmem_base_s, 512);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tbase = tmem_base_s;

    volatile int* abort_v = &abort_s;
    auto fail = [&](unsigned code) {
        atomicOr(&g_tc_status, code);
        *abort_v = 1;
    };

    if (warp == TMA_WARP) {
        if (lane == 0 && n_my > 0) {
            ptx::prefetch_tensormap(&tmap);
            ptx::mbar_arrive_expect_tx(b_full, P.b_bytes);
            for (uint32_t off = 0; off < P.b_bytes; off += 32768u) {
                const uint32_t len = P.b_bytes - off < 32768u ? P.b_bytes - off : 32768u;
                ptx::bulk_g2s(sB + off, P.b + off, len, b_full);
            }
            int64_t issued = 0;
            for (int64_t it = 0; it < n_my && !*abort_v; ++it) {
                const int s = (int)(it % XSTAGES);
                if (it >= XSTAGES && !ptx::mbar_wait(x_empty + s, (uint32_t)((it / XSTAGES - 1) & 1))) {
                    fail(1u);
                    break;
                }
                const int64_t t = blockIdx.x + it * gridDim.x;
                ptx::mbar_arrive_expect_tx(x_full + s, (uint32_t)(TM * d * 4));
                ptx::tma_load_2d(smem + P.off_x + s * P.x_stride, &tmap, 0, (int32_t)(t * TM), x_full + s);
                issued = it + 1;
            }
            if (*abort_v) {
                // let the copies still in flight land before the CTA releases its shared memory
                ptx::mbar_wait(b_full, 0);
                for (int64_t k = issued > XSTAGES ? issued - XSTAGES : 0; k < issued; ++k)
                    ptx::mbar_wait(x_full + (int)(k % XSTAGES), (uint32_t)((k / XSTAGES) & 1));
            }
        }
    } else if (warp == MMA_WARP) {
        if (lane == 0 && n_my > 0) {
            bool ok = ptx::mbar_wait(b_full, 0);
            if (!ok) fail(2u);
            const uint32_t sbo = (uint32_t)(kpad / 8) * 128u;
            const uint32_t b_addr = ptx::smem_u32(sB);
            int64_t g = 0;
            for (int64_t it = 0; ok && it < n_my && !*abort_v; ++it) {
                const int s = (int)(it & 1);
                if (!ptx::mbar_wait(a_full + s, (uint32_t)((it >> 1) & 1))) { fail(4u); break; }
                ptx::tc_fence_after();
                const uint32_t a_addr = ptx::smem_u32(smem + P.off_a + s * P.a_stride);
                for (int sweep = 0; ok && sweep < 2; ++sweep) {
                    for (int u = 0; u < U; ++u, ++g) {
                        const int buf = (int)(g & 1);
                        if (g >= 2 && !ptx::mbar_wait(t_empty + buf, (uint32_t)(((g >> 1) - 1) & 1))) {
                            fail(8u);
                            ok = false;
                            break;
                        }
                        ptx::tc_fence_after();
                        const uint32_t dt = tbase + (uint32_t)(buf * TN);
                        const uint32_t bu = b_addr + (uint32_t)u * (uint32_t)(TN / 8) * sbo;
                        for (int kb = 0; kb < kpad / 16; ++kb) {
                            const uint64_t ad = ptx::smem_desc(a_addr + kb * 256, 128, sbo);
                            const uint64_t bd = ptx::smem_desc(bu + kb * 256, 128, sbo);
                            ptx::mma_bf16(dt, ad, bd, IDESC, kb > 0);
                        }
                        ptx::mma_commit(t_full + buf);
                    }
                }
                ptx::mma_commit(a_empty + s);
            }
            // every MMA issued by this thread has completed once `drain` flips
            ptx::mma_commit(drain);
            if (!ptx::mbar_wait(drain, 0)) fail(256u);
        }
    } else {
        // ------------------------------ converter + epilogue (warps 0..15) -----------------------------------------
        // warp e: TMEM lane quarter q = e & 3 (rows 32q..32q+31), column slice sl = e >> 2 (64 of each 256 columns)
        const int q = warp & 3, sl = warp >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;
        const float g32 = (float)(d + 2) * 5.9604645e-8f;
        const float fac = 1.0f + 8.0f * g32;
        DFAcc e0, e1, e2;
        int64_t gcons = 0;   // TMEM tiles consumed
#ifdef SOMGB_TC_PHASE_TIMING
        unsigned long long _tc_acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        long long _tc_t0 = 0;
#endif

        auto qbar = [&]() { asm volatile("bar.sync %0, 128;" ::"r"(1 + q) : "memory"); };

        // centred split-BF16 A row of `row`: this thread writes the 16-byte chunks kc = sl, sl + 4, ... of kpad / 8;
        // returns |x'|^2 (infinite when a feature is not finite)
        auto convert = [&](int64_t it, float& xn_out) -> bool {
            const int s2 = (int)(it & 1), s3 = (int)(it % XSTAGES);
            if (it >= 2 && !ptx::mbar_wait(a_empty + s2, (uint32_t)(((it >> 1) - 1) & 1))) { fail(16u); return false; }
            if (!ptx::mbar_wait(x_full + s3, (uint32_t)((it / XSTAGES) & 1))) { fail(32u); return false; }
            const float4* xs4 = (const float4*)(smem + P.off_x + s3 * P.x_stride) + row * (DT / 4);
            float xp[DT];
            bool finite = true;
            float xn = 0.0f;
#pragma unroll
            for (int k4 = 0; k4 < DT / 4; ++k4) {
                const float4 v = xs4[k4];
                xp[4 * k4 + 0] = v.x - sCenter[4 * k4 + 0];
                xp[4 * k4 + 1] = v.y - sCenter[4 * k4 + 1];
                xp[4 * k4 + 2] = v.z - sCenter[4 * k4 + 2];
                xp[4 * k4 + 3] = v.w - sCenter[4 * k4 + 3];
            }
#pragma unroll
            for (int k = 0; k < DT; ++k) {
                finite = finite && isfinite(xp[k]);
                xn = fmaf(xp[k], xp[k], xn);
            }
            finite = finite && (xn < HUGE_S);
            xn_out = finite ? xn : INFINITY;
            uint8_t* at = smem + P.off_a + s2 * P.a_stride;
#pragma unroll
            for (int kc = 0; kc < kpad / 8; ++kc) {
                if (kc % SLICES != sl) continue;
                __align__(16) __nv_bfloat16 v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int k = kc * 8 + i;
                    float val = 0.0f;
                    if (k < 3 * DT) {
                        const float t = xp[k % DT];
                        const float hi = __bfloat162float(__float2bfloat16_rn(t));
                        val = (k >= DT && k < 2 * DT) ? t - hi : hi;
                    } else if (k == 3 * DT || k == 3 * DT + 1) {
                        val = 1.0f;
                    }
                    v[i] = __float2bfloat16_rn(finite ? val : 0.0f);
                }
                *(uint4*)(at + canon_off(row, kc * 8, kpad)) = *(const uint4*)v;
            }
            ptx::fence_proxy_async();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(a_full + s2);
            return true;
        };

        // two 32-column chunks of this warp's slice of TMEM tile `buf`, loaded back to back
        auto load64 = [&](int buf, float (&v0)[32], float (&v1)[32]) {
            const uint32_t base = tbase + lane_base + (uint32_t)(buf * TN + sl * 64);
            uint32_t r0[32], r1[32];
            ptx::tmem_ld32_raw(base, r0);
            ptx::tmem_ld32_raw(base + 32, r1);
            ptx::tmem_wait_ld2(r0, r1);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                v0[i] = __uint_as_float(r0[i]);
                v1[i] = __uint_as_float(r1[i]);
            }
        };

        float xn_next = 0.0f;
        bool ok = n_my > 0 ? convert(0, xn_next) : true;
        for (int64_t it = 0; ok && it < n_my && !*abort_v; ++it) {
            const float xn = xn_next;
            TC_T0();
            if (it + 1 < n_my && !(ok = convert(it + 1, xn_next))) break;
            TC_T(4);
            const int s3 = (int)(it % XSTAGES);
            const int64_t tile = blockIdx.x + it * gridDim.x;
            const int64_t grow = tile * TM + row;
            const bool live = grow < a.n;
            const float* xs = (const float*)(smem + P.off_x + s3 * P.x_stride) + row * d;
            bool flagged = !(xn < HUGE_S);

            // ---- sweep 1: best (and second best) s~ of the row over this warp's columns -------------------------
            float a1 = INFINITY, a2 = INFINITY, b1 = INFINITY, b2 = INFINITY;
            for (int u = 0; u < U && ok; ++u, ++gcons) {
                const int buf = (int)(gcons & 1);
                if (!ptx::mbar_wait(t_full + buf, (uint32_t)((gcons >> 1) & 1))) { fail(64u); ok = false; break; }
                TC_T(0);
                ptx::tc_fence_after();
                float v0[32], v1[32];
                load64(buf, v0, v1);
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(t_empty + buf);
#pragma unroll
                for (int g8 = 0; g8 < 32; g8 += 8) {
                    const float ga = fminf(fminf(fminf(v0[g8], v0[g8 + 1]), fminf(v0[g8 + 2], v0[g8 + 3])),
                                           fminf(fminf(v0[g8 + 4], v0[g8 + 5]), fminf(v0[g8 + 6], v0[g8 + 7])));
                    const float gb = fminf(fminf(fminf(v1[g8], v1[g8 + 1]), fminf(v1[g8 + 2], v1[g8 + 3])),
                                           fminf(fminf(v1[g8 + 4], v1[g8 + 5]), fminf(v1[g8 + 6], v1[g8 + 7])));
                    if (ERR) {
                        a2 = fminf(a2, fmaxf(a1, ga));
                        a1 = fminf(a1, ga);
                        b2 = fminf(b2, fmaxf(b1, gb));
                        b1 = fminf(b1, gb);
                    } else {
                        a1 = fminf(a1, ga);
                        b1 = fminf(b1, gb);
                    }
                }
                TC_T(1);
            }
            if (!ok) break;
            {
                const float m1 = fminf(a1, b1);
                const float m2 = fminf(fmaxf(a1, b1), fminf(a2, b2));
                sPart[sl * TM + row] = make_float2(m1, m2);
            }
            qbar();
            TC_T(5);
            float M1 = INFINITY, M2 = INFINITY;
#pragma unroll
            for (int t = 0; t < SLICES; ++t) {
                const float2 p = sPart[t * TM + row];
                M2 = fminf(fminf(M2, p.y), fmaxf(M1, p.x));
                M1 = fminf(M1, p.x);
            }
            // ERR: M2 is the second smallest 8-unit group minimum, an upper bound of the second smallest s~ (two
            // groups have a unit at or below it), so the threshold derived from it keeps every possible second BMU
            const float mref = ERR ? M2 : M1;
            // every slice has read sPart; the previous row tile's resolution finished before this tile's qbar
            if (sl == 0) sCandN[row] = 0;
            if (!(M1 + xn < HUGE_S) || !(mref < HUGE_S)) flagged = true;
            const float dref = fmaxf(0.0f, mref + xn);
            const float thr = flagged ? -INFINITY
                                      : mref + 2.0f * (P.alpha * xn + P.beta * dref) / (1.0f - P.beta) + 1.0e-30f;

            qbar();   // the pool count is reset before any slice claims a slot
            TC_T(5);
            // ---- sweep 2: every unit of this warp's columns under the threshold --------------------------------

            for (int u = 0; u < U && ok; ++u, ++gcons) {
                const int buf = (int)(gcons & 1);
                if (!ptx::mbar_wait(t_full + buf, (uint32_t)((gcons >> 1) & 1))) { fail(128u); ok = false; break; }
                TC_T(2);
                ptx::tc_fence_after();
                float v0[32], v1[32];
                load64(buf, v0, v1);
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(t_empty + buf);
                const int jb = u * TN + sl * 64;
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const float* v = half ? v1 : v0;
#pragma unroll
                    for (int g4 = 0; g4 < 32; g4 += 4) {
                        const float gm = fminf(fminf(v[g4], v[g4 + 1]), fminf(v[g4 + 2], v[g4 + 3]));
                        if (__any_sync(0xffffffffu, gm <= thr)) {
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const int j = jb + half * 32 + g4 + i;
                                if (v[g4 + i] <= thr && j < (int)a.m) {
                                    const int slot = atomicAdd(sCandN + row, 1);
                                    if (slot < CAPR) sCand[slot * TM + row] = j;
                                }
                            }
                        }
                    }
                }
                TC_T(3);
            }
            if (!ok) break;

            // ---- resolution: float32 distances of the row's candidates (slot k by slice k % 4), then slice 0 decides
            qbar();
            TC_T(5);
            const int total = sCandN[row];
            if (live && !flagged && total <= CAPR) {
                float xr[DT];
                const float4* xs4 = (const float4*)xs;
#pragma unroll
                for (int k4 = 0; k4 < DT / 4; ++k4) {
                    const float4 t = xs4[k4];
                    xr[4 * k4] = t.x; xr[4 * k4 + 1] = t.y; xr[4 * k4 + 2] = t.z; xr[4 * k4 + 3] = t.w;
                }
                for (int k = sl; k < total; k += SLICES) {
                    const int32_t j = sCand[k * TM + row];
                    sCandD[k * TM + row] = cand_dist32v<DT>(a.w + (int64_t)j * DT, xr);
                }
            }
            TC_T(6);
            qbar();
            TC_T(5);
            if (sl == 0 && live) {
                // best two candidates in (float32 distance, unit) order
                float f1 = INFINITY, f2 = INFINITY;
                int32_t c1 = -1, c2 = -1;
                const bool overflow = total > CAPR;
                const int nlist = overflow ? 0 : total;
                for (int k = 0; k < nlist; ++k) {
                    const float df = sCandD[k * TM + row];
                    const int32_t j = sCand[k * TM + row];
                    if (df < f1 || (df == f1 && j < c1)) { f2 = f1; c2 = c1; f1 = df; c1 = j; }
                    else if (df < f2 || (df == f2 && j < c2)) { f2 = df; c2 = j; }
                }
                if (flagged || overflow || total == 0) {
                    const unsigned long long slotq = atomicAdd(P.row_count, 1ull);
                    P.rows[slotq] = (int32_t)grow;
                } else {
                    // contenders: candidates the float32 distances cannot separate from the best (second best)
                    const float lim = ERR ? f2 : f1;
                    const float climit = lim < 1.0e37f ? fmaf(lim, fac, 1.0e-37f) : INFINITY;
                    int ncont = 0;
                    for (int k = 0; k < nlist; ++k) ncont += sCandD[k * TM + row] <= climit;
                    int32_t r1, r2;
                    DFloat rd1{0.0f, 0.0f};
                    if (ncont <= (ERR ? 2 : 1)) {
                        r1 = c1;
                        r2 = ERR ? c2 : -1;
                        if (ERR && c1 >= 0) {
                            float xr[DT];
                            const float4* xs4 = (const float4*)xs;
#pragma unroll
                            for (int k4 = 0; k4 < DT / 4; ++k4) {
                                const float4 t = xs4[k4];
                                xr[4 * k4] = t.x; xr[4 * k4 + 1] = t.y; xr[4 * k4 + 2] = t.z; xr[4 * k4 + 3] = t.w;
                            }
                            rd1 = ref_dist_pair<DT>(a.w + (int64_t)c1 * DT, xr);
                        }
                    } else {
                        // float64 reference sums of every contender, ranked in (distance, unit) order
                        Top2Lex tt;
                        tt.init();
                        for (int k = 0; k < nlist; ++k) {
                            if (!(sCandD[k * TM + row] <= climit)) continue;
                            const int32_t j = sCand[k * TM + row];
                            tt.push(ref_sqdist(a.w + (int64_t)j * d, xs, d), j);
                        }
                        r1 = tt.i1;
                        r2 = ERR ? tt.i2 : -1;
                        rd1.hi = (float)tt.d1;
                        rd1.lo = (float)(tt.d1 - (double)rd1.hi);
                    }
                    emit_sample32(a, grow, r1, r2, rd1, e0, e1, e2);
                }
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(x_empty + s3);
            TC_T(7);
        }
#ifdef SOMGB_TC_PHASE_TIMING
        if (lane == 0)
            for (int ph = 0; ph < 8; ++ph) atomicAdd(&g_tc_phase_cycles[ph], _tc_acc[ph]);
#endif
        if (ERR) {
            double v0 = e0.value(), v1 = e1.value(), v2 = e2.value();
            for (int o = 16; o > 0; o >>= 1) {
                v0 += __shfl_xor_sync(0xffffffffu, v0, o);
                v1 += __shfl_xor_sync(0xffffffffu, v1, o);
                v2 += __shfl_xor_sync(0xffffffffu, v2, o);
            }
            if (lane == 0 && (a.outs & OUT_ERR)) {
                if (v0 != 0.0) atomicAdd(a.err3 + 0, v0);
                if (v1 != 0.0) atomicAdd(a.err3 + 1, v1);
                if (v2 != 0.0) atomicAdd(a.err3 + 2, v2);
            }
        }
    }

    // teardown: the MMA thread has drained its MMAs and, after an abort, the producer its copies (both bounded)
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == MMA_WARP) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tbase, 512);
    }
}

template <bool ERR, int DT>
int launch_main(const CUtensorMap& tmap, const TcArgs& P, unsigned grid, size_t smem, cudaStream_t stream) {
    SOMGB_CUDA_TRY(cudaFuncSetAttribute(tc_pass_kernel<ERR, DT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    timer_begin(stream);
    tc_pass_kernel<ERR, DT><<<grid, NUM_THREADS, smem, stream>>>(tmap, P);
    timer_end(stream);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

bool device_is_sm103() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (dev < 0 || dev >= 64) return false;
    if (!cached[dev]) {
        int major = 0, minor = 0;
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
        cached[dev] = (major == 10 && minor == 3) ? 1 : 2;
    }
    return cached[dev] == 1;
}

size_t max_smem_optin() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (size_t)v;
}

}  // namespace

bool tc_shape_ok(int64_t m, int d) {
    if (d != 4 && d != 8 && d != 16 && d != 32) return false;
    if (m <= 0 || m > (int64_t)1 << 24) return false;
    return tc_shape(m, d).smem <= 227 * 1024;
}

bool tc_device_ok(int64_t m, int d) {
    return device_is_sm103() && encode_fn() != nullptr && max_smem_optin() >= tc_shape(m, d).smem;
}

bool tc_supported(int64_t n, int64_t m, int d, int algo) {
    if (algo == SOMGB_ALGO_FP32) return false;
    if (!tc_shape_ok(m, d)) return false;
    if (algo == SOMGB_ALGO_AUTO && n * m < ((int64_t)1 << 22)) return false;   // small passes: K0 has no prep cost
    return device_is_sm103() && encode_fn() != nullptr && max_smem_optin() >= tc_shape(m, d).smem;
}

#ifdef SOMGB_TC_PHASE_TIMING
// Instrumented builds only: copies out (and optionally clears) the eight phase counters.
extern "C" int somgb_tc_phase_cycles(unsigned long long* out8, int reset) {
    SOMGB_CUDA_TRY(cudaDeviceSynchronize());
    SOMGB_CUDA_TRY(cudaMemcpyFromSymbol(out8, g_tc_phase_cycles, 8 * sizeof(unsigned long long)));
    if (reset) {
        unsigned long long z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        SOMGB_CUDA_TRY(cudaMemcpyToSymbol(g_tc_phase_cycles, z, sizeof(z)));
    }
    return SOMGB_OK;
}
#endif

int read_device_status(unsigned int* status, bool clear, cudaStream_t stream) {
    SOMGB_CUDA_TRY(cudaMemcpyFromSymbolAsync(status, g_tc_status, sizeof(unsigned int), 0, cudaMemcpyDeviceToHost,
                                             stream));
    SOMGB_CUDA_TRY(cudaStreamSynchronize(stream));
    if (clear) {
        const unsigned int zero = 0;
        SOMGB_CUDA_TRY(cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, stream));
        SOMGB_CUDA_TRY(cudaStreamSynchronize(stream));
    }
    return SOMGB_OK;
}

size_t tc_workspace_bytes(int64_t n, int64_t m, int d) { return tc_ws_layout(n, m, d, nullptr, nullptr); }

int launch_tc_pass(const PassArgs& a, void* ws, size_t ws_bytes, cudaStream_t stream) {
    if (((uintptr_t)a.x) % 16) return set_error(SOMGB_ERR_INVALID, "tensor-core pass needs 16-byte aligned x");
    const TcShape s = tc_shape(a.m, a.d);
    TcWs W;
    if (tc_ws_layout(a.n, a.m, a.d, &W, ws) > ws_bytes) return set_error(SOMGB_ERR_WORKSPACE, "tc workspace too small");

    // unit operand
    tc_center_kernel<<<1, 256, 0, stream>>>(a.w, a.m, a.d, W.center);
    SOMGB_LAUNCH_CHECK();
    tc_prep_b_kernel<<<(unsigned)ceil_div(s.mpad, 128), 128, 0, stream>>>(a.w, a.m, a.d, s.kpad, s.mpad, W.center,
                                                                          W.b);
    SOMGB_LAUNCH_CHECK();

    // sample tensor map: rows of d float32, boxes of 128 rows
    CUtensorMap tmap;
    cuuint64_t gdim[2] = {(cuuint64_t)a.d, (cuuint64_t)a.n};
    cuuint64_t gstride[1] = {(cuuint64_t)a.d * 4};
    cuuint32_t box[2] = {(cuuint32_t)a.d, (cuuint32_t)TM};
    cuuint32_t estride[2] = {1, 1};
    CUresult cr = encode_fn()(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)a.x, gdim, gstride, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(SOMGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)cr);

    TcArgs P{};
    P.a = a;
    P.b = W.b;
    P.center = W.center;
    P.rows = W.rows;
    P.row_count = a.recheck_count;
    P.kpad = s.kpad;
    P.utiles = s.utiles;
    tc_error_coefficients(a.d, &P.alpha, &P.beta);
    P.off_a = s.off_a;
    P.off_x = s.off_x;
    P.off_cand = s.off_cand;
    P.off_part = s.off_part;
    P.off_res = s.off_res;
    P.off_center = s.off_center;
    P.off_bar = s.off_bar;
    P.a_stride = align_up(s.a_bytes, 1024);
    P.x_stride = s.x_bytes;
    P.b_bytes = (uint32_t)s.b_bytes;

    const int64_t tiles = ceil_div(a.n, TM);
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, num_sms());
    // at least half of an SM's shared memory, so that one CTA (the sole TMEM owner) runs per SM
    const size_t smem = std::max<size_t>(s.smem, 120 * 1024);
    int st = SOMGB_OK;
    if (a.outs & OUT_ERR) {
        switch (a.d) {
            case 4: st = launch_main<true, 4>(tmap, P, grid, smem, stream); break;
            case 8: st = launch_main<true, 8>(tmap, P, grid, smem, stream); break;
            case 16: st = launch_main<true, 16>(tmap, P, grid, smem, stream); break;
            case 32: st = launch_main<true, 32>(tmap, P, grid, smem, stream); break;
            default: return set_error(SOMGB_ERR_UNSUPPORTED, "tensor-core pass: D=%d not in {4, 8, 16, 32}", a.d);
        }
    } else {
        switch (a.d) {
            case 4: st = launch_main<false, 4>(tmap, P, grid, smem, stream); break;
            case 8: st = launch_main<false, 8>(tmap, P, grid, smem, stream); break;
            case 16: st = launch_main<false, 16>(tmap, P, grid, smem, stream); break;
            case 32: st = launch_main<false, 32>(tmap, P, grid, smem, stream); break;
            default: return set_error(SOMGB_ERR_UNSUPPORTED, "tensor-core pass: D=%d not in {4, 8, 16, 32}", a.d);
        }
    }
    if (st) return st;
    // rows the tensor-core pass could not decide: the exact CUDA-core pass over the listed rows (it must not count
    // into the list length it reads)
    PassArgs b = a;
    b.recheck_count = nullptr;
    return launch_k0_pass(b, stream, W.rows, a.recheck_count);
}

}  // namespace somgb
