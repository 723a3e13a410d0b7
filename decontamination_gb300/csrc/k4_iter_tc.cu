// K4: iteration mode ("n_vectors", algo/som_batch.py:154-210, 378-495) as a contraction on the tcgen05 tensor cores.
//
// Iteration mode gives every sample its own neighbourhood width, so its sums do not factor through per-BMU sums; they
// are the dense contraction over the samples s
//   num[u, k] = sum_s h[s, u] rho_s x_s[k],   den[u] = sum_s h[s, u] rho_s,
//   h[s, u] = exp(-|t_u - t_b(s)|^2 / (2 sigma_s^2)) = Ex_s[row(u), col(u) mod 2] * Ey_s[col(u)]
// on the reference's square and hexagonal grids (a unit's x depends on its row and its column's parity, its y on its
// column). Each CTA owns 512 units (four 128-unit M tiles; 384 units, three tiles, for D >= 32) and a chunk of the
// samples, taken in batches of 32 samples (two MMA K-steps); each of its threads (16 warps, or 12) owns one unit:
//   * thread t holds TMEM lane t mod 128 of M tile t / 128 and the unit of slot t in the CTA's order (even grid columns
//     first, then odd, rows ascending within a column), so that a warp's 32 units share few table rows;
//   * a batch has two CTA barriers. Between them the CTA writes the batch's B operand to shared memory (rows
//     [0, NB) the FP16 hi parts and rows [NB, 2 NB) the lo parts of B[n, s] = rho_s x_s[n] (n < D), rho_s (n = D),
//     0 (D < n < NB), each feature scaled by a power of two from the catalogue's bounds) and stages the next batch's
//     samples (loaded into registers a batch earlier);
//   * after the second, lane 0 of warps 0, 5, 10 (, 15) (one per scheduler) issues its M tile's MMAs of the previous
//     batch, 128 x 2 NB x 16 with A from TMEM and B from shared memory: per K-step A_lo.B then A_hi.B (accumulator
//     columns [0, NB) sum A.B_hi, [NB, 2 NB) A.B_lo); an issuing thread waits while the tensor core takes each MMA
//     (about 46 cycles), which is why those warps compute no tables;
//   * meanwhile each thread writes its unit's factors A[u, s] = 2^15 h[s, u] of this batch, split into FP16 hi (h
//     truncated to 11 significant bits) + lo (the exact rest, rounded) parts, into its TMEM lane (tcgen05.st), and the
//     other warps compute the next batch's exponential tables over the grid rows (by column parity) and grid
//     columns of the CTA's units (float32 arguments as the float32 CUDA-core pass forms them, the exponential from the
//     hardware base-2 approximation with an extended-precision argument, k4_exp), half of them before their A and
//     half after, so that every scheduler has both kinds of work;
//   * every `group` batches each thread reads its unit's accumulator row (tcgen05.ld), adds the two halves and adds
//     them to compensated float32 sums; at the end of the chunk it adds those to num, den in float64.
// The tables, samples and operands are double-buffered by batch parity.
// TMEM (512 columns): NB = 16 (D <= 15) two accumulator sets of 4 x 32 columns, NB = 32 (D <= 31) one set of 4 x 64,
// NB = 48 (D <= 47) one set of 3 x 96, from column 0; then the A operands, (buffer, split, M tile, K-step) at
// ACC + 8 (((buffer * 2 + split) * tiles + tile) * 2 + K-step). An MMA of N <= 64 columns takes as long as one of
// 64, so the hi and lo parts of B share one MMA.
// Error budget: 2^-21 relative per product from the FP16 parts, then the tensor core's FP32 accumulation, which loses
// low bits with every MMA (measured: ~20 float32 ulps over 16 MMAs, ~8 over the 8 MMAs of a 2-batch group, ~3 over 4),
// then float32 rounding of the compensated sums, besides the float32 tables (k4_exp: within the ex2 approximation's
// error of e^x). With `group` = 2 the sums differ from the float32 CUDA-core pass (expf) by at most 6e-7 relative
// (12.6 M samples on a 64 x 64 map), for 8% of the time a 1-batch group would take.
// Every wait is bounded: one that gives up sets bit 65536 of the status words and the CTA returns.
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "tc.cuh"
#include "tc_ptx.cuh"

namespace somgb {

namespace {

constexpr int K4_UNITS_MAX = 512;              // units per CTA: 128 per M tile, 4 tiles (3 for D >= 32)
constexpr int K4_SB = 32;                      // samples per batch: two K-steps of 16
constexpr int K4_NB_MAX = 48;                  // B rows per FP16 part: the D features, the density, zero rows
constexpr int K4_TPAD = 36;                    // floats per table row: 32 samples + 4 (conflict-free 16-byte reads)
constexpr int K4_TAB_MAX = 320;                // table rows (2 per grid row + 1 per grid column) of a CTA
constexpr uint32_t K4_B_MAX = 2 * K4_NB_MAX * K4_SB * 2;   // bytes of one batch's B operand
constexpr uint32_t K4_SBO = (K4_SB / 8) * 128;      // bytes between the 8-row groups of the canonical layout
constexpr unsigned K4_FAIL = 65536u;
constexpr float K4_ASCALE = 32768.0f;          // A = 2^15 h: FP16 normals down to h = 2^-29

struct K4Args {
    const float* x;
    const double* rho;
    const int32_t* bmu;
    int64_t n;
    int d;
    const float* topo;
    int64_t rows, cols;
    double inv_coef, clamp_q;   // 1 / (2 sigma_i^2) = inv_coef q_i^2, q_i = n_vectors + 2 (cur + i) <= clamp_q
    float inv_clamp_f;          // 1 / (2 FLOAT_EPS^2) beyond
    int64_t cur_vector, n_vectors, chunk;
    const float* bounds;   // d + 1 floats: max |rho x_k|, max rho (somgb_feature_bounds)
    double* num;
    double* den;
    unsigned int* status;
    unsigned int* gstatus;
    int group;             // batches per accumulator set before it is folded
    int withhold_group;    // test hook: this group's completion is never signalled (-1: none)
    uint32_t wait_limit;
};

// byte offset of element (row, k) of a K-major canonical operand with K4_SB columns (8-row x 16-byte core matrices)
__device__ __forceinline__ uint32_t k4_off(int row, int k) {
    return (uint32_t)((row >> 3) * K4_SBO + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t h2_bits(__half2 v) { return *reinterpret_cast<uint32_t*>(&v); }
__device__ __forceinline__ float trunc11(float v) { return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u); }

// Two-lane float32 arithmetic (sm_100 and later): each lane rounds to nearest as __fmul_rn / __fadd_rn / __fsub_rn.
__device__ __forceinline__ unsigned long long f2_bits(float2 v) {
    unsigned long long u;
    asm("mov.b64 %0, {%1, %2};" : "=l"(u) : "f"(v.x), "f"(v.y));
    return u;
}
__device__ __forceinline__ float2 f2_of(unsigned long long u) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(u));
    return v;
}
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return f2_of(r);
}
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return f2_of(r);
}
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return f2_of(r);
}
__device__ __forceinline__ uint32_t h2_of(float2 v) { return h2_bits(__floats2half2_rn(v.x, v.y)); }

// e^x from the hardware base-2 exponential (ex2.approx): y = x log2(e) is carried as y_hi + y_lo with log2(e) split
// into float32 hi and lo parts and the FMA product error, and e^x = 2^y_hi (1 + y_lo ln 2), first order in
// |y_lo| < 2^-23 |y|; the result is within the ex2 approximation's error of e^x (results below 2^-126 flush to zero).
constexpr float K4_LOG2E_HI = 1.44269502162933349609375f;   // log2(e) rounded to float32
constexpr float K4_LOG2E_LO = 1.925963033500011e-08f;       // log2(e) - K4_LOG2E_HI
constexpr float K4_LN2 = 0.693147180559945309f;
__device__ __forceinline__ float k4_exp(float x) {
    const float yh = __fmul_rn(x, K4_LOG2E_HI);
    const float yl = __fmaf_rn(x, K4_LOG2E_LO, __fmaf_rn(x, K4_LOG2E_HI, -yh));
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(yh));
    return __fmaf_rn(e, __fmul_rn(yl, K4_LN2), e);
}

// c (Q + t)^2 in float32 arithmetic from Q = c[0] + c[1] (integers) and c = c[2] + c[3], for integer t < 2^24: q = Q + t
// exactly as qh + ql (Knuth's two-sum; ql a small integer), qh^2 exactly as p + pe (FMA product error), then
// (p + pe + 2 qh ql) (c[2] + c[3]) with the product p c[2] split the same way: about 2^-44 relative before the one
// rounding, so the result is the correctly rounded float32 except in rare near-ties.
__device__ __forceinline__ float inv_sigma_of(const float* c, float t) {
    const float qh = __fadd_rn(c[0], t);
    const float bv = __fsub_rn(qh, c[0]);
    const float e = __fadd_rn(__fsub_rn(c[0], __fsub_rn(qh, bv)), __fsub_rn(t, bv));
    const float ql = __fadd_rn(e, c[1]);
    const float p = __fmul_rn(qh, qh);
    const float pe = __fmaf_rn(qh, qh, -p);
    const float r = __fadd_rn(pe, __fmul_rn(__fmul_rn(2.0f, qh), ql));
    const float v = __fmul_rn(p, c[2]);
    const float ve = __fmaf_rn(p, c[2], -v);
    return __fadd_rn(v, __fadd_rn(ve, __fmaf_rn(p, c[3], __fmul_rn(r, c[2]))));
}

template <int DMAX, int NB, int K4_MT>
__global__ void __launch_bounds__(128 * K4_MT, 1) k4_iter_kernel(const K4Args P) {
    constexpr int K4_UNITS = 128 * K4_MT;
    constexpr int K4_THREADS = K4_UNITS;            // one thread per unit
    constexpr int TW = K4_THREADS / 32 - K4_MT;     // the warps that issue no MMAs compute the tables
    constexpr int N = 2 * NB;                       // MMA N: hi rows then lo rows of B
    constexpr int NSET = NB == 16 ? 2 : 1;          // accumulator sets
    constexpr uint32_t IDESC = ptx::idesc_f16_f32(128, N);
    constexpr uint32_t B_BYTES = N * K4_SB * 2;
    constexpr uint32_t K4_ACC_COLS = NSET * K4_MT * N;   // accumulator columns; the A operands follow
    static_assert(K4_ACC_COLS + 64 * K4_MT <= 512 && DMAX < NB && N <= 256 && K4_MT <= 4, "the TMEM layout fits");
    extern __shared__ __align__(128) uint8_t k4_raw[];
    uint8_t* sB = k4_raw;                              // [buffer] B operands
    float* tab0 = (float*)(k4_raw + 2 * K4_B_MAX);     // [batch parity][table row][K4_TPAD]; row ntab is all zeros
    __shared__ float inv_s[K4_SB], bx_s[K4_SB], by_s[K4_SB], scale_s[K4_NB_MAX];
    __shared__ float rho_s[2][K4_SB];                  // [batch parity]
    __shared__ int valid_s[2][K4_SB];
    __shared__ float poly_s[5];
    __shared__ int perm_s[K4_UNITS_MAX];
    __shared__ __align__(8) uint64_t bars[5];
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    uint64_t* a_empty = bars + 0;    // [2] the MMAs reading operand buffer b have completed (one commit per issuer)
    uint64_t* acc_full = bars + 2;   // [NSET] an accumulator set holds a finished group
    uint64_t* drain = bars + 4;      // every MMA has completed

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int d = P.d;
    const int64_t m = P.rows * P.cols, cols = P.cols;
    const int64_t u0 = (int64_t)blockIdx.x * K4_UNITS;
    const int64_t ulast = min64(u0 + K4_UNITS, m) - 1;
    const int nunits = (int)(ulast - u0 + 1);
    const int64_t r0 = u0 / cols;
    const int nrow = (int)(ulast / cols - r0 + 1);
    const int64_t c0 = nrow > 1 ? 0 : u0 % cols;
    const int ncol = nrow > 1 ? (int)cols : (int)(ulast % cols - c0 + 1);
    const int ntab = 2 * nrow + ncol;
    const int tabn = (ntab + 1) * K4_TPAD;            // floats per table buffer
    float* xs0 = tab0 + 2 * tabn;                     // [batch parity][K4_SB][d]
    float* gc = xs0 + 2 * K4_SB * d;                  // [ntab] the table rows' grid coordinates
    const int64_t s0 = (int64_t)blockIdx.y * P.chunk;
    const int64_t s1 = min64(P.n, s0 + P.chunk);
    const int nbatch = s1 > s0 ? (int)((s1 - s0 + K4_SB - 1) / K4_SB) : 0;
    const int G = P.group;
    const uint32_t lim = P.wait_limit;
    const int mt = tid >> 7;
    const bool issuer = lane == 0 && warp == 5 * mt;   // warps 0, 5, 10, 15: one per scheduler
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            ptx::mbar_init(a_empty + i, K4_MT);
            ptx::mbar_init(acc_full + i, K4_MT);
        }
        ptx::mbar_init(drain, K4_MT);
        ptx::fence_mbar_init();
        abort_s = 0;
        // 1 / (2 sigma_i^2) = inv_coef (Q + t)^2 for sample i = s0 + t / 2 of this chunk, Q = n_vectors + 2 (cur + s0):
        // Q and inv_coef as float32 pairs (hi, lo) once per CTA, so that the per-sample value in float32 arithmetic
        // is the correctly rounded one (inv_sigma_of)
        const double Q = (double)P.n_vectors + 2.0 * (double)(P.cur_vector + s0);
        poly_s[0] = (float)Q;
        poly_s[1] = (float)(Q - (double)poly_s[0]);
        poly_s[2] = (float)P.inv_coef;
        poly_s[3] = (float)(P.inv_coef - (double)poly_s[2]);
        poly_s[4] = (float)(P.clamp_q - Q);   // sigma_i < FLOAT_EPS beyond this t
    }
    if (tid < K4_NB_MAX) {   // B row scales 2^(14 - e), the feature's bound below 2^e: |B| < 2^14
        int e = 0;
        const float b = P.bounds[tid < d ? tid : d];
        if (b > 0.0f) frexpf(b, &e);
        e = max(e, -60);
        scale_s[tid] = tid <= d ? ldexpf(1.0f, 14 - e) : 0.0f;
    }
    for (int q = tid; q < 2 * K4_TPAD; q += K4_THREADS) tab0[(q / K4_TPAD) * tabn + ntab * K4_TPAD + q % K4_TPAD] = 0.0f;
    // table row e < 2 nrow: x of grid row r0 + e mod nrow at column parity e / nrow; else y of grid column c0 + e - 2 nrow
    for (int e = tid; e < ntab; e += K4_THREADS) {
        const int p = e / nrow;
        const int64_t ua = e < 2 * nrow ? (r0 + e % nrow) * cols + (p < cols ? p : 0) : c0 + e - 2 * nrow;
        gc[e] = __ldg(P.topo + 2 * ua + (e < 2 * nrow ? 0 : 1));
    }
    {   // slot of unit u0 + tid: the CTA's units of the even columns (ascending), then of the odd ones, each column's
        // rows ascending; a column's rows are contiguous, and only the first and last grid rows can be partial
        if (tid < nunits) {
            auto E = [](int64_t v) -> int64_t { return v > 0 ? (v + 1) / 2 : 0; };   // even integers in [0, v)
            auto O = [](int64_t v) -> int64_t { return v > 0 ? v / 2 : 0; };         // odd integers in [0, v)
            const int64_t uu = u0 + tid, r = uu / cols, c = uu % cols;
            const int64_t a = u0 % cols, z = ulast % cols;
            int64_t pre, rlo = r0;
            if (nrow > 1) {   // column c holds nrow rows, less one when c < a (first row) or c > z (last row)
                auto below = [&](auto F, int64_t v) { return F(v) * nrow - F(min64(v, a)) - (F(v) - F(min64(v, z + 1))); };
                pre = (c & 1) == 0 ? below(E, c) : below(E, cols) + below(O, c);
                rlo = r0 + (c < a ? 1 : 0);
            } else {          // one grid row: columns [c0, c0 + ncol)
                pre = (c & 1) == 0 ? E(c) - E(c0) : E(c0 + ncol) - E(c0) + O(c) - O(c0);
            }
            perm_s[pre + (r - rlo)] = tid;
        } else {
            perm_s[tid] = tid;
        }
    }
    if (warp == 0) {
        ptx::tmem_alloc(&tmem_s, 512);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tbase = tmem_s;
    volatile int* abort_v = &abort_s;
    auto fail = [&]() {
        atomicOr(P.gstatus, K4_FAIL);
        if (P.status) atomicOr(P.status, K4_FAIL);
        *abort_v = 1;
    };

    // unit indices fit 32 bits (shapes of at most 2^26 units)
    const int tu = perm_s[tid];
    const int u = (int)u0 + tu;
    const bool live = tu < nunits;
    const int urow = u / (int)cols, ucol = u % (int)cols;
    const int ix = live ? (ucol & 1) * nrow + (urow - (int)r0) : ntab;   // Ex row: (column parity, grid row)
    const int iy = live ? 2 * nrow + (ucol - (int)c0) : ntab;           // Ey row: grid column
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    const int tx = ix * K4_TPAD, ty = iy * K4_TPAD;   // offsets in a table buffer
    // compensated float32 sums of the scaled accumulator columns, features k and k + 1 in the lanes of one pair
    constexpr int NP = DMAX / 2 + 1;
    float2 asum[NP], aerr[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) asum[k] = aerr[k] = make_float2(0.0f, 0.0f);

    // M tile mt's MMAs of K-step ks of batch b: A_lo.B, then A_hi.B
    auto issue = [&](int b, int ks) {
        const int sb = b & 1, g = b / G, ab = g % NSET;
        const uint64_t bd = ptx::smem_desc(ptx::smem_u32(sB) + (uint32_t)sb * B_BYTES + (uint32_t)ks * 256u, 128,
                                           K4_SBO);
        const uint32_t dt = tbase + (uint32_t)((ab * K4_MT + mt) * N);
        const uint32_t ahi = tbase + K4_ACC_COLS + (uint32_t)((((sb * 2 + 0) * K4_MT + mt) * 2 + ks) * 8);
        const uint32_t alo = tbase + K4_ACC_COLS + (uint32_t)((((sb * 2 + 1) * K4_MT + mt) * 2 + ks) * 8);
        ptx::mma_f16_ta(dt, alo, bd, IDESC, (b % G == 0 && ks == 0) ? 0u : 1u);
        ptx::mma_f16_ta(dt, ahi, bd, IDESC, 1u);
        if (ks == 1) {
            ptx::mma_commit(a_empty + sb);
            if ((b % G == G - 1 || b == nbatch - 1) && g != P.withhold_group) ptx::mma_commit(acc_full + ab);
        }
    };
    // folds group g's accumulator set into acc; false when its wait gave up
    auto fold = [&](int g) -> bool {
        const int ab = g % NSET;
        const bool ok = ptx::mbar_wait(acc_full + ab, (uint32_t)((g / NSET) & 1), lim);
        if (!__all_sync(0xffffffffu, ok)) return false;
        ptx::tc_fence_after();
        const uint32_t base = tbase + lane_base + (uint32_t)((ab * K4_MT + mt) * N);
#pragma unroll
        for (int c = 0; c <= DMAX / 8; ++c) {
            uint32_t rh[8], rl[8];
            ptx::tmem_ld8_raw(base + (uint32_t)(8 * c), rh);
            ptx::tmem_ld8_raw(base + (uint32_t)(NB + 8 * c), rl);
            ptx::tmem_wait_ld8(rh);
            ptx::tmem_tie8(rl);
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
                const int k2 = (8 * c + j) / 2;
                if (k2 >= NP) break;
                // the hi and lo halves, then Kahan's compensated addition, two features at a time
                const float2 v = add2_rn(make_float2(__uint_as_float(rh[j]), __uint_as_float(rh[j + 1])),
                                         make_float2(__uint_as_float(rl[j]), __uint_as_float(rl[j + 1])));
                const float2 y = sub2_rn(v, aerr[k2]);
                const float2 t = add2_rn(asum[k2], y);
                aerr[k2] = sub2_rn(sub2_rn(t, asum[k2]), y);
                asum[k2] = t;
            }
        }
        ptx::tc_fence_before();
        return true;
    };

    // the samples two batches ahead are loaded while this batch runs: XPT features per thread; warp 1 lane s:
    // sample s's BMU, weight and 1 / (2 sigma^2), then the BMU's grid coordinates
    constexpr int XPT = (K4_SB * DMAX + K4_THREADS - 1) / K4_THREADS;
    float xr[XPT];
    int32_t bm_r = -1;
    double rho_r = 1.0;
    float inv_r = 0.0f, bx_r = 0.0f, by_r = 0.0f;
    auto prefetch = [&](int b) {
        const int64_t i0 = s0 + (int64_t)b * K4_SB;
        const int nb = (int)min64(K4_SB, s1 - i0);
#pragma unroll
        for (int j = 0; j < XPT; ++j) {
            const int q = tid + j * K4_THREADS;
            xr[j] = q < nb * d ? __ldg(P.x + i0 * d + q) : 0.0f;
        }
        if (warp == 1) {
            const int64_t i = i0 + lane;
            bm_r = lane < nb ? __ldg(P.bmu + i) : -1;
            rho_r = (lane < nb && P.rho) ? __ldg(P.rho + i) : 1.0;
            // sigma_i = sigma0 / (1 + 2 (cur + i) / n_vectors) clamped at FLOAT_EPS (som_batch.py:167-170), so
            // 1 / (2 sigma_i^2) = q^2 / (2 sigma0^2 n_vectors^2) with q = n_vectors + 2 (cur + i) = Q + t
            const float t = (float)(2 * (i - s0));   // exact below 2^24
            inv_r = t > poly_s[4] ? P.inv_clamp_f : inv_sigma_of(poly_s, t);
        }
    };
    auto prefetch_bmu = [&]() {
        if (warp == 1 && bm_r >= 0) {
            bx_r = __ldg(P.topo + 2 * (int64_t)bm_r);
            by_r = __ldg(P.topo + 2 * (int64_t)bm_r + 1);
        }
    };
    // batch b's samples from the registers into shared memory (its parity's buffers)
    auto stage = [&](int b) {
        const int64_t i0 = s0 + (int64_t)b * K4_SB;
        const int nb = (int)min64(K4_SB, s1 - i0);
        float* xs = xs0 + (b & 1) * K4_SB * d;
#pragma unroll
        for (int j = 0; j < XPT; ++j) {
            const int q = tid + j * K4_THREADS;
            if (q < nb * d) xs[q] = xr[j];
        }
        if (warp == 1) {
            const bool v = bm_r >= 0;
            inv_s[lane] = inv_r;
            rho_s[b & 1][lane] = v ? (float)rho_r : 0.0f;   // float32 training density
            valid_s[b & 1][lane] = v;
            bx_s[lane] = bx_r;
            by_s[lane] = by_r;
        }
    };
    // batch b's tables: lane s of the w-th warp that issues no MMAs computes sample s's entries of rows w, w + 12, ...;
    // 2^15 is folded into the column factors; zero for absent samples
    auto tables = [&](int b) {
        if (warp % 5 == 0) return;
        const int tw = warp - warp / 5 - 1;   // 0 .. TW - 1
        float* tab = tab0 + (b & 1) * tabn;
        const bool vs = valid_s[b & 1][lane] != 0;
        const float ninv = -inv_s[lane], bx = bx_s[lane], by = by_s[lane];
        // rows e and e + TW in the two lanes of the float32 pairs
        for (int e = tw; e < ntab; e += 2 * TW) {
            const int e2 = e + TW;
            const bool two = e2 < ntab, x1 = e < 2 * nrow, x2 = e2 < 2 * nrow;
            const float2 dd = sub2_rn(make_float2(gc[e], two ? gc[e2] : 0.0f), make_float2(x1 ? bx : by, x2 ? bx : by));
            const float2 xa = mul2_rn(mul2_rn(dd, dd), make_float2(ninv, ninv));   // -dd^2 / (2 sigma^2)
            const float2 v = mul2_rn(make_float2(k4_exp(xa.x), k4_exp(xa.y)),
                                     make_float2(x1 ? 1.0f : K4_ASCALE, x2 ? 1.0f : K4_ASCALE));
            tab[e * K4_TPAD + lane] = vs ? v.x : 0.0f;
            if (two) tab[e2 * K4_TPAD + lane] = vs ? v.y : 0.0f;
        }
    };
    // batch b's B operand: item p < 16 NB (items strided over the threads): feature row n = p mod NB, samples
    // 2 (p / NB) + {0, 1}: rho x (scaled), rho, zeros; the hi parts to row n, the lo parts to row NB + n (a warp's lanes
    // read consecutive features)
    auto bgen = [&](int b) {
        const float* xs = xs0 + (b & 1) * K4_SB * d;
        const float* rs = rho_s[b & 1];
        const int* vs = valid_s[b & 1];
        for (int p = tid; p < 16 * NB; p += K4_THREADS) {
            const int nn = p % NB, s = (p / NB) * 2;
            float v0 = 0.0f, v1 = 0.0f;
            if (nn <= d) {
                const float sc = scale_s[nn];
                v0 = (nn < d ? rs[s] * xs[s * d + nn] : rs[s]) * sc;
                v1 = (nn < d ? rs[s + 1] * xs[(s + 1) * d + nn] : rs[s + 1]) * sc;
                if (!vs[s]) v0 = 0.0f;
                if (!vs[s + 1]) v1 = 0.0f;
            }
            const __half2 hi = __floats2half2_rn(v0, v1);
            const float2 hf = __half22float2(hi);
            const __half2 lo = __floats2half2_rn(__fsub_rn(v0, hf.x), __fsub_rn(v1, hf.y));
            *(uint32_t*)(sB + (b & 1) * B_BYTES + k4_off(nn, s)) = h2_bits(hi);
            *(uint32_t*)(sB + (b & 1) * B_BYTES + k4_off(NB + nn, s)) = h2_bits(lo);
        }
    };
    // batch b's A operand: this unit's factors, one K-step (16 samples, 8 TMEM columns) at a time
    auto agen = [&](int b) {
        const int sb = b & 1;
        const float* tab = tab0 + sb * tabn;
#pragma unroll
        for (int ks = 0; ks < K4_SB / 16; ++ks) {
            uint32_t hv[8], lv[8];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 ex = *(const float4*)(tab + tx + ks * 16 + q * 4);
                const float4 ey = *(const float4*)(tab + ty + ks * 16 + q * 4);
                const float2 h01 = mul2_rn(make_float2(ex.x, ex.y), make_float2(ey.x, ey.y));
                const float2 h23 = mul2_rn(make_float2(ex.z, ex.w), make_float2(ey.z, ey.w));
                // hi: h truncated to FP16's 11 significant bits (exact in FP16 for h >= 2^-29); lo = h - hi exactly
                const float2 g01 = make_float2(trunc11(h01.x), trunc11(h01.y));
                const float2 g23 = make_float2(trunc11(h23.x), trunc11(h23.y));
                hv[2 * q] = h2_of(g01);
                hv[2 * q + 1] = h2_of(g23);
                lv[2 * q] = h2_of(sub2_rn(h01, g01));
                lv[2 * q + 1] = h2_of(sub2_rn(h23, g23));
            }
            const uint32_t chi = K4_ACC_COLS + (uint32_t)((((sb * 2 + 0) * K4_MT + mt) * 2 + ks) * 8);
            const uint32_t clo = K4_ACC_COLS + (uint32_t)((((sb * 2 + 1) * K4_MT + mt) * 2 + ks) * 8);
            ptx::tmem_st8(tbase + lane_base + chi, hv);
            ptx::tmem_st8(tbase + lane_base + clo, lv);
        }
    };

    // Batch b: its tables were computed during batch b - 1, its samples staged then. Between the two barriers the CTA
    // writes B and stages batch b + 1's samples; after the second the issuers take batch b - 1's MMAs, and the other
    // warps write their units' A of batch b and compute batch b + 1's tables (half of the warps in each order, so that
    // each scheduler has both kinds of work).
    bool bad = false;
    if (nbatch > 0) {
        prefetch(0);
        prefetch_bmu();
        stage(0);
        __syncthreads();
        tables(0);
        if (nbatch > 1) {
            prefetch(1);
            prefetch_bmu();
        }
    }
    for (int b = 0; b <= nbatch; ++b) {
        // every thread has finished batch b - 1 (operands written and fenced, folds done) and batch b's tables
        if (__syncthreads_or(bad || *abort_v)) {
            bad = true;
            break;
        }
        if (b == nbatch) {   // the last batch's MMAs
            if (b >= 1 && issuer) {
                ptx::tc_fence_after();
                issue(b - 1, 0);
                issue(b - 1, 1);
            }
            break;
        }
        // operand buffer b mod 2 is free once the MMAs of batch b - 2 have completed
        if (b >= 2) bad |= !ptx::mbar_wait(a_empty + (b & 1), (uint32_t)(((b >> 1) - 1) & 1), lim);
        bgen(b);
        ptx::fence_proxy_async();   // the B operand's generic writes, before the MMAs read them
        if (b + 1 < nbatch) stage(b + 1);
        __syncthreads();
        ptx::tc_fence_after();
        if (b >= 1 && issuer) {   // the issuers wait while the tensor core takes each MMA
            issue(b - 1, 0);
            issue(b - 1, 1);
        }
        if (b + 2 < nbatch) prefetch(b + 2);
        const bool tables_first = ((warp >> 2) & 1) != 0;
        if (tables_first && b + 1 < nbatch) tables(b + 1);
        agen(b);
        if (!tables_first && b + 1 < nbatch) tables(b + 1);
        ptx::tmem_wait_st();
        ptx::tc_fence_before();
        prefetch_bmu();   // batch b + 2's BMU indices have arrived by now
        // the group that ended with batch b - 1 (its MMAs were issued during this batch): fold it now
        if (b >= 1 && (b - 1) % G == G - 1 && !bad) bad = !fold((b - 1) / G);
    }
    if (!bad && nbatch > 0) bad = !fold((nbatch - 1) / G);   // the last group
    if (!bad && live) {
#pragma unroll
        for (int k = 0; k <= DMAX; ++k) {
            if (k > d) break;
            const double sc = (double)K4_ASCALE * (double)scale_s[k];
            const float sk = (k & 1) ? asum[k / 2].y : asum[k / 2].x, ek = (k & 1) ? aerr[k / 2].y : aerr[k / 2].x;
            const double v = ((double)sk - (double)ek) / sc;
            if (v != 0.0) atomicAdd(k < d ? P.num + (int64_t)u * d + k : P.den + u, v);
        }
    }
    if (bad) fail();
    if (issuer) ptx::mma_commit(drain);
    __syncthreads();
    if (warp == 0) {
        const bool ok = ptx::mbar_wait(drain, 0, lim);
        if (!__all_sync(0xffffffffu, ok) && lane == 0) fail();
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tbase, 512);
    }
}

// Test hook (somgb_debug_iter_withhold): the next contraction on this thread withholds one group's completion and
// bounds its waits by `limit` polls; one-shot.
thread_local int t_withhold_group = -1;
thread_local uint32_t t_wait_limit = 0;

}  // namespace

void iter_tc_debug_withhold(int group, uint32_t wait_limit) {
    t_withhold_group = group;
    t_wait_limit = wait_limit;
}

// Units per CTA: four 128-unit M tiles, three for D >= 32 (wider B operand, so wider accumulators).
int iter_tc_units(int d) { return d + 1 <= 32 ? 512 : 384; }

// Table rows of the CTA with the most: 2 per grid row that its units touch, plus its grid columns.
int64_t iter_tc_table_rows(int64_t rows, int64_t cols, int units) {
    const int64_t m = rows * cols;
    int64_t best = 0;
    for (int64_t u0 = 0; u0 < m; u0 += units) {
        const int64_t ul = std::min<int64_t>(u0 + units, m) - 1;
        const int64_t nrow = ul / cols - u0 / cols + 1;
        const int64_t ncol = nrow > 1 ? cols : ul % cols - u0 % cols + 1;
        best = std::max<int64_t>(best, 2 * nrow + ncol);
    }
    return best;
}

bool iter_tc_shape_ok(int64_t rows, int64_t cols, int d) {
    return d >= 1 && d + 1 <= K4_NB_MAX && rows >= 1 && cols >= 1 && rows * cols <= ((int64_t)1 << 26) &&
           iter_tc_table_rows(rows, cols, iter_tc_units(d)) <= K4_TAB_MAX;
}

int launch_iter_tc(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, const float* topo,
                   int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors,
                   const float* bounds, double* num, double* den, unsigned int* status, cudaStream_t stream) {
    if (n == 0) return SOMGB_OK;
    const int64_t m = rows * cols;
    const int units = iter_tc_units(d);
    const int64_t tiles = ceil_div(m, units);
    int64_t chunks = std::max<int64_t>(1, num_sms() / tiles);
    const int64_t chunk = ceil_div(std::max<int64_t>(K4_SB, ceil_div(n, chunks)), K4_SB) * K4_SB;
    chunks = ceil_div(n, chunk);
    K4Args P{};
    P.x = x; P.rho = rho; P.bmu = bmu; P.n = n; P.d = d; P.topo = topo; P.rows = rows; P.cols = cols;
    // 1 / (2 sigma_i^2) = q^2 inv_coef with q = n_vectors + 2 (cur + i); sigma_i falls below FLOAT_EPS when
    // q > sigma0 n_vectors / FLOAT_EPS, and then 1 / (2 FLOAT_EPS^2) applies
    const double nv = (double)n_vectors;
    P.inv_coef = 1.0 / (2.0 * sigma0 * sigma0 * nv * nv);
    P.inv_clamp_f = (float)(1.0 / (2.0 * FLOAT_EPS * FLOAT_EPS));
    P.clamp_q = sigma0 * nv / FLOAT_EPS;
    P.cur_vector = cur_vector; P.n_vectors = n_vectors; P.chunk = chunk; P.bounds = bounds;
    P.num = num; P.den = den; P.status = status; P.gstatus = device_status_word();
    P.group = 2;
    P.withhold_group = t_withhold_group;
    P.wait_limit = t_wait_limit ? t_wait_limit : (1u << 22);
    t_withhold_group = -1;   // one-shot
    t_wait_limit = 0;
    if (!P.gstatus) return set_error(SOMGB_ERR_CUDA, "device status word unavailable");
    const int64_t ntab = iter_tc_table_rows(rows, cols, units);
    // at least 120 KB, so that one CTA (which holds all 512 TMEM columns) is resident per SM
    const size_t smem = std::max<size_t>(
        2 * K4_B_MAX + 2 * (size_t)(ntab + 1) * K4_TPAD * 4 + 2 * (size_t)K4_SB * d * 4 + (size_t)ntab * 4, 120 * 1024);
    auto kern = d <= 7    ? k4_iter_kernel<7, 16, 4>
                : d <= 15 ? k4_iter_kernel<15, 16, 4>
                : d <= 16 ? k4_iter_kernel<16, 32, 4>
                : d <= 23 ? k4_iter_kernel<23, 32, 4>
                : d <= 31 ? k4_iter_kernel<31, 32, 4>
                : d <= 39 ? k4_iter_kernel<39, 48, 3>
                          : k4_iter_kernel<47, 48, 3>;
    SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<dim3((unsigned)tiles, (unsigned)chunks), units, smem, stream>>>(P);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

}  // namespace somgb
