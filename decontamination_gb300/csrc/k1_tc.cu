// K1: BMU search on the tcgen05 tensor cores (split-FP16 distance GEMM), exact by construction.
//
// Distances are expanded as |x - w_j|^2 = |x'|^2 + s_j with s_j = |w'_j|^2 - 2 x'.w'_j, where x' = (x - c) S and
// w' = (w - c) S are centred on the mean unit c (the centring shrinks every error term below) and scaled by a power
// of two S that puts the largest unit coordinate in [2^5, 2^6) (samples up to 512 times farther out stay in FP16
// range; the scaling is exact in float32). One GEMM per
// 128-sample row tile and TN-unit column tile produces s~_j in TMEM:
//   A row (sample)  = [ x'_hi | x'_lo | x'_hi | 2^11 | 2^11 | 0 ... ]             (FP16, K padded to a multiple of 16)
//   B row (unit j)  = [ -2w'_hi | -2w'_hi | -2w'_lo | q_hi | q_lo | 0 ... ] with q_hi + q_lo = 2^-11 |w'_j|^2
// so that sum_k A.B = -2 (x_hi w_hi + x_lo w_hi + x_hi w_lo) + |w'|^2 ~ s_j, accumulated in FP32. (For D a multiple
// of 16 the repeated blocks are stored once and the MMA K-steps point at them twice; see k_step_cols.) Invalid and padding
// units carry q_hi = +inf (s~ = +inf); rows with a coordinate at or above 2^15 after scaling, or non-finite, go to
// the exact recheck.
//
// Error bound. With FP16 unit roundoff 2^-11, dropping x_lo w_lo and the two-term residuals costs at most
// 3.01 * 2^-22 |x'_k||w'_k| per product; q's split and float32 evaluation cost 2.5 * 2^-22 |w'|^2 + (D+2) 2^-24 |w'|^2;
// the FP32 accumulation of the K non-zero products is bounded by K * 2^-23 * sum|terms| (one rounding per product,
// the worst case); FP16 subnormals add at most 2^-21 |x'|^2 plus an absolute 2^-8.
// Using |w'_j|^2 <= 2|x'|^2 + 2 d'_j (d'_j = |x' - w'_j|^2) every term is bounded by
//   |s~_j - s_j| <= alpha |x'|^2 + beta d'_j + gamma,
// with alpha, beta computed on the host (tc_error_coefficients). A unit can beat the tile's best (or, for the
// error sums, the second best) only if s~_j <= thr(m) = m + 2 (alpha |x'|^2 + beta (m + |x'|^2) + gamma) / (1 - beta)
// + gamma, m being the best (second-best) s~ of the row; thr is non-decreasing in m, so any upper bound of m gives a
// threshold that keeps every such unit.
//
// Epilogue: two sweeps per row tile. Sweep 1 computes every column tile and reads each row's s~ in 32-column chunks,
// keeping the smallest value (for the error sums, the two smallest 8-unit group minima: an upper bound of the
// second-best s~) and each column tile's minimum; the two column halves combine theirs into the row's threshold, and
// the column tiles where some row of the 128-row tile has a tile minimum at or under its threshold make the tile set
// of sweep 2. Sweep 2 recomputes only those column tiles (every candidate lies in one; with the rows grouped by their
// previous BMU, somgb_sort_rows, a tile's rows share a neighbourhood of the map and the set is small): where a row of
// the warp can have a candidate in a chunk (chunk minimum at or under its threshold), the warp builds the chunk's
// candidate bit masks, a branch-free subtraction and shift of the sign bit per value, and every row with a non-zero
// mask appends (mask word, chunk) to its own short list. The MMAs run sweep 1 of row tile k, then sweep 2 of row
// tile k - 1, so that sweep 2's tile set is known a whole sweep ahead. The
// resolvers evaluate each row's candidates on CUDA cores with float32 differences (the reference's terms) and rank
// them; ranks within float32 rounding of each other are decided by compensated float32 sums and, failing that, by
// the reference's float64 sum. Rows with more than CAPR candidates, a full list, non-finite features or overflowing
// distances go to an exact per-row recheck.
//
// Pipeline (one persistent CTA per SM, 480 threads, every hand-off an mbarrier):
//   warp 13     TMA producer: the unit operand B (resident: one bulk copy; else a ring of column tiles in the MMAs'
//               order), sample tiles (2-D tiled TMA, one row tile ahead);
//   warp 12     TMEM allocator; two TMEM accumulators of TN columns each;
//   warps 12/14 MMA issuers (one thread each): warp 12 the even column tiles (accumulator 0), warp 14 the odd ones
//               (accumulator 1);
//   warps 0-7   converters (FP32 tile -> centred split-FP16 A tile, three A stages: two row tiles' MMAs read them
//               while the next is written) and sweeps; warp e reads TMEM lanes
//               32(e&3).. and column half e>>2 and writes its rows' candidate lists (two list buffers, so the sweeps
//               of row tile t+1 do not wait for the resolvers of row tile t);
//   warps 8-11  resolvers: thread r of warp 8+q decides row 32q+r of a row tile while the sweeps run the next one:
//               candidates' distances from the unit rows (shared memory when they fit, else L2), ranking, decision,
//               outputs.
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "tc.cuh"
#include "tc_ptx.cuh"

namespace somgb {

// Sticky device status: bit set by any bounded wait of the tensor-core pass that gave up (0 = healthy).
__device__ unsigned int g_tc_status;

// Optional per-phase cycle counters of the epilogue warps (compiled in only with -DSOMGB_TC_PHASE_TIMING; read with
// cudaMemcpyFromSymbol). Sweep warps: 0 wait for TMEM, 1 sweep, 4 convert, 5 wait for a free list buffer; resolver
// warps: 6 wait for candidates, 7 emit, 8 recheck listing, 9 candidate loop, 10 decision; the MMA thread: 12 wait for
// a free TMEM accumulator, 13 wait for a unit-operand tile.
#ifdef SOMGB_TC_PHASE_TIMING
constexpr int TC_PHASES = 14;
__device__ unsigned long long g_tc_phase_cycles[TC_PHASES];
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
constexpr int NACC = 512 / TN;    // TMEM accumulators (512 columns), so the MMAs run up to NACC - 1 tiles ahead
constexpr int HW = TN / 2;        // columns of a tile per sweep warp (two column halves)
constexpr int CPW = HW / 32;      // 32-column chunks per tile and sweep warp
constexpr int HALVES = 2;         // sweep warps per TMEM lane quarter, each owning half of a tile's columns
constexpr int CAPR = 24;          // candidates a resolver ranks per row
constexpr int CAP = 4;            // candidate-list entries per row and column half
constexpr size_t SMEM_LIMIT = 227 * 1024;   // opt-in shared memory of one CTA
constexpr int MAX_U = 16384 / TN; // column tiles per row tile (a list entry names its chunk, CPW per tile and half, in a byte)
constexpr int NBARS = 56;         // mbarrier slots
constexpr int ASTAGES = 3;        // A tiles: sweep 1 of row tile k and sweep 2 of k - 1 read two, the converters write a third
constexpr int BMAX = 4;           // deepest ring of streamed unit-operand tiles (slots 32 .. 32 + 2 BMAX - 1)
static_assert(32 + 2 * BMAX <= 40 && 44 + 2 * ASTAGES <= NBARS, "mbarrier slots");
static_assert(CPW * MAX_U <= 256, "chunk ids are bytes");
static_assert(NACC * TN == 512 && CPW * 32 == HW, "TMEM and chunk layout");
constexpr int XSTAGES = 1;   // a sample tile is converted a whole row tile before its MMAs: one stage is ahead enough
constexpr int SWEEP_WARPS = 4 * HALVES;
constexpr int RES_GROUP = 4;    // resolver warps per row tile (one thread per row)
constexpr int RES_GROUPS = 1;   // groups of resolvers taking the row tiles in turn (1 or 2; list buffers: 2)
constexpr int RES_WARPS = RES_GROUPS * RES_GROUP;
constexpr int MMA_WARP = SWEEP_WARPS + RES_WARPS;   // issuer of the tiles of accumulator 0; allocates TMEM
constexpr int TMA_WARP = MMA_WARP + 1;
constexpr int MMA_WARP2 = TMA_WARP + 1;              // issuer of the tiles of accumulator 1
constexpr int NUM_THREADS = (MMA_WARP2 + 1) * 32;
constexpr float X_LIMIT = 32768.0f;   // scaled sample coordinates at or above this go to the exact recheck
constexpr float Q_COLUMN = 2048.0f;   // A's value in the two q columns (B holds q / 2^11)
constexpr float GAMMA = 0.00390625f;  // 2^-8: absolute error bound of the FP16 subnormal range, in scaled units
constexpr float HUGE_S = 1.0e30f; // rows whose best s~ + |x'|^2 reaches this go to the exact recheck
// One MMA of N = TN = 256 per K-step: two of N = 128, each half of the accumulator with its own barriers, were
// measured slower (they read the A tile twice).
static_assert(NACC == 2, "one MMA issuer per accumulator (issuer k: column tiles g with g % 2 == k)");
constexpr uint32_t IDESC = ptx::idesc_f16_f32(TM, TN);
constexpr uint32_t WAIT_LIMIT = 1u << 22;   // polls of a bounded mbarrier wait (each at most about 1 us)
// K layout of the operands (elements per row, FP16). D a multiple of 16: A = [x_hi | x_lo | q columns],
// B = [-2w_hi | -2w_lo | q_hi q_lo 0...], and the MMA K-steps pair the blocks (lo.hi, hi.lo, hi.hi, then q), so no
// block is stored twice. Other D: A = [x_lo | x_hi | x_hi | 2^11 2^11 | 0...], B = [-2w_hi | -2w_lo | -2w_hi | q_hi
// q_lo | 0...] padded to a multiple of 16, one K-step per 16 columns. Either way the small (lo) products enter the
// FP32 accumulator first, while it is small, so their roundings are small too (tc_error_coefficients).
__host__ __device__ constexpr bool k_dedup(int d) { return d % 16 == 0; }
__host__ __device__ constexpr int k_width(int d) { return k_dedup(d) ? 2 * d + 16 : (3 * d + 2 + 15) / 16 * 16; }
__host__ __device__ constexpr int k_steps(int d) { return k_dedup(d) ? 3 * (d / 16) + 1 : k_width(d) / 16; }
__host__ __device__ constexpr int k_qcol(int d) { return k_dedup(d) ? 2 * d : 3 * d; }   // first q column
// column offsets of K-step i in A and in B
__host__ __device__ __forceinline__ void k_step_cols(int d, int i, int& ka, int& kb) {
    if (!k_dedup(d)) {
        ka = kb = 16 * i;
        return;
    }
    const int nb = d / 16;
    if (i == 3 * nb) {
        ka = kb = 2 * d;
        return;
    }
    const int blk = i % nb, kind = i / nb;   // kind 0: lo.hi, 1: hi.lo, 2: hi.hi
    ka = (kind == 0 ? d : 0) + 16 * blk;
    kb = (kind == 1 ? d : 0) + 16 * blk;
}

struct TcShape {
    int d = 0, kpad = 0;
    int64_t mpad = 0;
    int utiles = 0;
    int bstages = 0;   // 0: the whole unit operand resident in shared memory; else a ring of this many column tiles
    size_t b_bytes = 0, b_tile = 0, a_bytes = 0, x_bytes = 0;
    size_t off_a = 0, off_x = 0, off_lw = 0, off_part = 0, off_thr = 0, off_lc = 0, off_cnt = 0, off_flag = 0,
           off_tmin = 0, off_union = 0, off_center = 0, off_bar = 0, off_w = 0, smem = 0;
};

// Layout after a unit-operand region of `bregion` bytes; returns the end offset (before the unit rows).
size_t tc_layout(TcShape& s, size_t bregion) {
    size_t off = align_up(bregion, 1024);
    s.off_a = off;
    off += ASTAGES * align_up(s.a_bytes, 1024);
    s.off_x = off;
    off += XSTAGES * s.x_bytes;
    // candidate lists, [buffer][half][entry][row]: mask words and chunk ids; per buffer, half and row the half's
    // bounds (a1, a2) and the entry count; per buffer and row the final threshold and the recheck flag
    s.off_lw = off;
    off += (size_t)2 * HALVES * CAP * TM * 4;
    s.off_part = off;
    off += (size_t)2 * HALVES * TM * 8;
    s.off_thr = off;
    off += (size_t)2 * TM * 4;
    s.off_lc = off;
    off += (size_t)2 * HALVES * CAP * TM;
    s.off_cnt = off;
    off += (size_t)2 * HALVES * TM;
    s.off_flag = off;
    off += (size_t)2 * TM;
    // per row, column half and column tile the tile's minimum (FP16), and per list buffer the column tiles with a
    // candidate, one word per sweep warp
    s.off_tmin = align_up(off, 16);
    off = s.off_tmin + (size_t)HALVES * s.utiles * TM * 2;
    s.off_union = align_up(off, 16);
    off = s.off_union + (size_t)2 * SWEEP_WARPS * 8;
    s.off_center = align_up(off, 16);
    off = s.off_center + align_up((size_t)(s.d + 1) * 4, 16);
    s.off_bar = align_up(off, 8);
    return s.off_bar + NBARS * 8;
}

TcShape tc_shape(int64_t m, int d) {
    TcShape s;
    s.d = d;
    s.kpad = k_width(d);
    s.mpad = (int64_t)align_up((size_t)m, TN);
    s.utiles = (int)(s.mpad / TN);
    s.b_bytes = (size_t)s.mpad * s.kpad * 2;
    s.b_tile = (size_t)TN * s.kpad * 2;
    s.a_bytes = (size_t)TM * s.kpad * 2;
    s.x_bytes = align_up((size_t)TM * d * 4, 128);
    const size_t w_bytes = (size_t)m * d * 4;   // the float32 unit rows, for the resolvers' candidate distances
    // In order of preference: the unit operand resident with the unit rows; a ring of BMAX (down to 2) column tiles
    // streamed from L2 with the unit rows; then the same without the unit rows (the resolvers read them from L2).
    for (int rows = 1; rows >= 0; --rows) {
        for (int st = 0; st == 0 || st >= 2; st = st == 0 ? BMAX : st - 1) {
            s.bstages = st;
            size_t off = tc_layout(s, st == 0 ? s.b_bytes : (size_t)st * align_up(s.b_tile, 1024));
            s.off_w = 0;
            if (rows) {
                s.off_w = align_up(off, 16);
                off = s.off_w + w_bytes;
            }
            s.smem = off + 128;   // slack for aligning the dynamic base to 128 bytes (TMA tile destinations)
            if (s.smem <= SMEM_LIMIT) return s;
        }
    }
    return s;   // does not fit (smem > SMEM_LIMIT): refused by tc_shape_ok
}

// Scratch: [B operand | centre (d floats) and scale | recheck row list (n int32)]
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
    off += align_up((size_t)(d + 1) * 4, 256);   // centre and scale
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

// Operand classes of the K columns (tc_error_coefficients walks the layout with them).
enum KCol { KC_ZERO = 0, KC_HI, KC_LO, KC_Q, KC_QL };
inline int k_col_a(int d, int k) {
    if (k_dedup(d)) return k < d ? KC_HI : k < 2 * d ? KC_LO : (k == 2 * d || k == 2 * d + 1) ? KC_Q : KC_ZERO;
    return k < d ? KC_LO : k < 3 * d ? KC_HI : (k == 3 * d || k == 3 * d + 1) ? KC_Q : KC_ZERO;
}
inline int k_col_b(int d, int k) {
    const int qc = k_qcol(d);
    if (k == qc) return KC_Q;
    if (k == qc + 1) return KC_QL;
    if (k_dedup(d)) return k < d ? KC_HI : k < 2 * d ? KC_LO : KC_ZERO;
    return k < d ? KC_HI : k < 2 * d ? KC_LO : k < 3 * d ? KC_HI : KC_ZERO;
}

// |s~_j - s_j| <= alpha |x'|^2 + beta d'_j + gamma. With P = |x'|^2 + |w'|^2 <= 3|x'|^2 + 2d' and
// Q = |w'|^2 <= 2|x'|^2 + 2d':
//  * representation: dropping x_lo w_lo and the two-term residuals costs 3.01 * 2^-22 |x'_k||w'_k| per product, so
//    3.01 * 2^-22 P over the row; q's split (computed in float64) 2.5 * 2^-22 Q;
//  * accumulation: each non-zero product is one FP32 rounding of the running sum (2^-23 of it, a worst case that also
//    covers truncation). The MMA K-steps run in order and the running sum after step s is bounded by the magnitudes of
//    the product classes seen so far: hi.hi products sum to at most 1.0011 P, each lo class (lo.hi, hi.lo) to
//    2^-11 * 1.0011 P, the q pair to (1 + 2^-10) Q. The bound is summed step by step over the actual layout, so the
//    small products placed first cost almost nothing;
//  * centring rounding and the reference's own float32 rounding of each term: 2^-21 (|x'|^2 + d');
//  * FP16 subnormal split residuals (absolute 2^-25) times |x'_k| summed over k: below 2^-24 sqrt(D) (1 + |x'|^2) / 2,
//    a further 2^-21 |x'|^2 and an absolute part inside gamma.
// 25% is added to alpha and beta as a safety margin.
void tc_error_coefficients(int d, float* alpha, float* beta) {
    const double u22 = std::ldexp(1.0, -22), u23 = std::ldexp(1.0, -23), u11 = std::ldexp(1.0, -11);
    double cp = 0.0, cq = 0.0;   // accumulated rounding bound, in units of 2^-23 P and 2^-23 Q
    bool seen_hi = false, seen_lo_a = false, seen_lo_b = false, seen_q = false;
    for (int st = 0; st < k_steps(d); ++st) {
        int ka = 0, kb = 0;
        k_step_cols(d, st, ka, kb);
        int nz = 0;
        for (int i = 0; i < 16; ++i) {
            const int ca = k_col_a(d, ka + i), cb = k_col_b(d, kb + i);
            if (ca == KC_ZERO || cb == KC_ZERO) continue;
            ++nz;
            if (ca == KC_HI && cb == KC_HI) seen_hi = true;
            else if (ca == KC_LO && cb == KC_HI) seen_lo_a = true;
            else if (ca == KC_HI && cb == KC_LO) seen_lo_b = true;
            else if (ca == KC_Q) seen_q = true;
            else seen_hi = seen_lo_a = seen_lo_b = seen_q = true;   // not produced by the layouts; counted in full
        }
        const double run_p = (seen_hi ? 1.0011 : 0.0) + (seen_lo_a ? u11 * 1.0011 : 0.0) + (seen_lo_b ? u11 * 1.0011 : 0.0);
        const double run_q = seen_q ? 1.0 + 2.0 * u11 : 0.0;
        cp += nz * run_p;
        cq += nz * run_q;
    }
    const double rep_p = 3.01 * u22, rep_q = 2.5 * u22;
    const double kp = rep_p + cp * u23, kq = rep_q + cq * u23;   // error <= kp P + kq Q
    double a = 3.0 * kp + 2.0 * kq, b = 2.0 * kp + 2.0 * kq;
    a += std::ldexp(1.0, -21);   // centring and the reference's float32 terms
    b += std::ldexp(1.0, -21);
    a += std::ldexp(1.0, -21);   // FP16 subnormal residuals
    *alpha = (float)(1.25 * a);
    *beta = (float)(1.25 * b);
}

// ---------------------------------------------------------------------------------------------------------------------
// prep: centre and unit operand
// ---------------------------------------------------------------------------------------------------------------------

// Mean of the finite unit rows, per feature, in float64; then center[d] = the power-of-two scale S that puts the
// largest |w - c| coordinate of those rows in [2^5, 2^6). One CTA, three coalesced passes over the m x d values
// (d divides the block, so thread t always holds feature t % d): rows with a non-finite value are marked in a shared
// bitmap, then the finite rows are summed per feature (each thread its own float64 sum, combined per feature), then
// their largest scaled deviation is taken. Any centre keeps the pass exact (the error bound holds for every centre);
// a central one keeps the bound tight.
constexpr int CENTER_THREADS = 1024;
constexpr int CENTER_MAXM = 16384;   // the largest map of the tensor-core pass (rows of the shared bitmap)
__global__ void __launch_bounds__(CENTER_THREADS) tc_center_kernel(const float* __restrict__ w, int64_t m, int d,
                                                                   float* __restrict__ center) {
    __shared__ uint32_t bad[CENTER_MAXM / 32];
    __shared__ double part[CENTER_THREADS];
    __shared__ unsigned int nvalid_s, maxbits_s;
    const int tid = threadIdx.x;
    const int total = (int)m * d;   // m <= CENTER_MAXM (tc_shape_ok)
    for (int i = tid; i < CENTER_MAXM / 32; i += CENTER_THREADS) bad[i] = 0u;
    if (tid == 0) {
        nvalid_s = 0u;
        maxbits_s = 0u;
    }
    __syncthreads();
    for (int idx = tid; idx < total; idx += CENTER_THREADS)
        if (!isfinite(__ldg(w + idx))) atomicOr(&bad[(idx / d) >> 5], 1u << ((idx / d) & 31));
    __syncthreads();
    unsigned int nv = 0;
    for (int j = tid; j < (int)m; j += CENTER_THREADS) nv += ((bad[j >> 5] >> (j & 31)) & 1u) ? 0u : 1u;
    atomicAdd(&nvalid_s, nv);
    double s = 0.0;
    for (int idx = tid; idx < total; idx += CENTER_THREADS) {
        const int j = idx / d;
        if (!((bad[j >> 5] >> (j & 31)) & 1u)) s += (double)__ldg(w + idx);
    }
    part[tid] = s;
    __syncthreads();
    const unsigned int cnt = nvalid_s;
    for (int k = tid; k < d; k += CENTER_THREADS) {
        double t = 0.0;
        for (int q = k; q < CENTER_THREADS; q += d) t += part[q];
        center[k] = cnt ? (float)(t / (double)cnt) : 0.0f;
    }
    __syncthreads();
    const float ck = center[tid % d];   // this thread's feature
    unsigned int mx = 0u;
    for (int idx = tid; idx < total; idx += CENTER_THREADS) {
        const int j = idx / d;
        if (!((bad[j >> 5] >> (j & 31)) & 1u)) mx = max(mx, __float_as_uint(fabsf(__ldg(w + idx) - ck)));
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((tid & 31) == 0 && mx) atomicMax(&maxbits_s, mx);
    __syncthreads();
    if (tid == 0) {
        const float mxf = __uint_as_float(maxbits_s);
        int e = 0;
        if (mxf > 0.0f && isfinite(mxf)) frexpf(mxf, &e);   // mx < 2^e
        else e = 10;
        center[d] = ldexpf(1.0f, min(max(6 - e, -100), 100));
    }
}

__device__ __forceinline__ size_t canon_off(int64_t row, int k, int kpad) {
    return (size_t)(row >> 3) * (kpad >> 3) * 128 + (size_t)(k >> 3) * 128 + (size_t)(row & 7) * 16 + (size_t)(k & 7) * 2;
}

__global__ void tc_prep_b_kernel(const float* __restrict__ w, int64_t m, int d, int kpad, int64_t mpad,
                                 const float* __restrict__ center, uint8_t* __restrict__ b) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mpad) return;
    auto put = [&](int k, float v) { *(__half*)(b + canon_off(j, k, kpad)) = __float2half_rn(v); };
    const float scale = center[d];
    bool valid = j < m;
    double q = 0.0;   // |w'|^2 of the float32 coordinates, to float64 rounding (once per unit and pass)
    if (valid) {
        for (int k = 0; k < d; ++k) {
            const float v = w[j * d + k];
            if (!isfinite(v)) valid = false;
            const float t = (v - center[k]) * scale;
            q = fma((double)t, (double)t, q);
        }
        if (!(q < 1.0e30)) valid = false;
    }
    for (int k = 0; k < kpad; ++k) put(k, 0.0f);
    const int qc = k_qcol(d);
    if (!valid) {
        put(qc, INFINITY);   // never the minimum, never under a threshold: s~ = +inf
        return;
    }
    const bool dedup = k_dedup(d);
    for (int k = 0; k < d; ++k) {
        const float t = (w[j * d + k] - center[k]) * scale;
        const __half hi = __float2half_rn(t);
        const __half lo = __float2half_rn(t - __half2float(hi));
        put(k, -2.0f * __half2float(hi));
        put(d + k, -2.0f * __half2float(lo));
        if (!dedup) put(2 * d + k, -2.0f * __half2float(hi));
    }
    // q_hi + q_lo = 2^-11 |w'|^2 to 2^-22 relative
    const double qs = q * (1.0 / Q_COLUMN);
    const __half qh = __float2half_rn((float)qs);
    put(qc, __half2float(qh));
    put(qc + 1, (float)(qs - (double)__half2float(qh)));
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
    float alpha, beta, kthr;   // kthr = 2 / (1 - beta), rounded up
    size_t off_a, off_x, off_lw, off_part, off_thr, off_lc, off_cnt, off_flag, off_tmin, off_union, off_center,
        off_bar, off_w, a_stride, x_stride;
    uint32_t b_bytes;
    uint32_t b_tile;         // bytes of one column tile of the unit operand
    int bstages;             // 0: resident unit operand; else the ring depth
    uint32_t wait_limit;     // polls of the protocol waits (WAIT_LIMIT; shorter only under the test hook)
    int64_t withhold_tile;   // test hook: the row tile whose samples the producer never loads (-1: none)
};

// thr(m): the largest s~ a unit can have and still be the best (second best) unit of a row whose best (second-best)
// s~ is m; axg = alpha |x'|^2 + gamma. Non-decreasing in m (every operation is, in round-to-nearest).
__device__ __forceinline__ float thr_of(float mref, float xn, float axg, float beta, float kthr) {
    const float dref = fmaxf(0.0f, mref + xn);
    return fmaf(kthr, fmaf(beta, dref, axg), mref) + GAMMA;
}

// float32 distance over the reference's float32 differences: four FMA chains (features k mod 4) summed at the end,
// so the dependent chain is D/4 + 2 long; any summation order keeps |df - d_ref| <= (D+2) 2^-24 d_ref
template <int DT>
__device__ __forceinline__ float cand_dist32v(const float* __restrict__ wr, const float (&xr)[DT]) {
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
    const float4* w4 = (const float4*)wr;
#pragma unroll
    for (int k4 = 0; k4 < DT / 4; ++k4) {
        const float4 w = w4[k4];
        float t = w.x - xr[4 * k4]; c0 = fmaf(t, t, c0);
        t = w.y - xr[4 * k4 + 1]; c1 = fmaf(t, t, c1);
        t = w.z - xr[4 * k4 + 2]; c2 = fmaf(t, t, c2);
        t = w.w - xr[4 * k4 + 3]; c3 = fmaf(t, t, c3);
    }
    return (c0 + c1) + (c2 + c3);
}

// Bit 31-i set when v[i] - thr_up < 0, i.e. v[i] < thr_up (false for NaN): a subtraction and a shift-or per value.
// Two independent 16-bit chains (columns 0-15 in the high half), so the shift-ors do not form one 32-long dependency.
__device__ __forceinline__ uint32_t sign_mask32(const uint32_t (&v)[32], float thr_up) {
    uint32_t m0 = 0u, m1 = 0u;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        m0 = (m0 << 1) | (__float_as_uint(__fsub_rn(__uint_as_float(v[i]), thr_up)) >> 31);
        m1 = (m1 << 1) | (__float_as_uint(__fsub_rn(__uint_as_float(v[16 + i]), thr_up)) >> 31);
    }
    return (m0 << 16) | m1;
}

// min(a, b, c) in one instruction (three-input form of min.f32, sm_100 and later); NaN inputs are ignored as by fminf
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// (da, ja) ranks before (db, jb): lexicographic, empty entries (unit < 0) last
__device__ __forceinline__ bool lex_before(float da, int32_t ja, float db, int32_t jb) {
    return ja >= 0 && (jb < 0 || da < db || (da == db && ja < jb));
}

// minimum of v[B .. B + 16) (NaN ignored)
template <int B>
__device__ __forceinline__ float min16(const uint32_t (&v)[32]) {
    auto f = [&](int i) { return __uint_as_float(v[B + i]); };
    const float t0 = fmin3(f(0), f(1), f(2)), t1 = fmin3(f(3), f(4), f(5)), t2 = fmin3(f(6), f(7), f(8));
    const float t3 = fmin3(f(9), f(10), f(11)), t4 = fmin3(f(12), f(13), f(14));
    return fminf(fmin3(t0, t1, t2), fmin3(t3, t4, f(15)));
}

// minimum of v[b .. b + 8) (NaN ignored)
__device__ __forceinline__ float min8(const uint32_t (&v)[32], int b) {
    auto f = [&](int i) { return __uint_as_float(v[b + i]); };
    return fmin3(fmin3(f(0), f(1), f(2)), fmin3(f(3), f(4), f(5)), fminf(f(6), f(7)));
}

// The tensor-core pass. ERR: the error sums (second BMU ranked too); the bound of the second-best s~ is the
// second-smallest 8-unit group minimum.
template <bool ERR, int DT>
__global__ void __launch_bounds__(NUM_THREADS, 1) tc_pass_kernel(const __grid_constant__ CUtensorMap tmap, TcArgs P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
    uint8_t* sB = smem;
    float* sCenter = (float*)(smem + P.off_center);
    uint32_t* sLw = (uint32_t*)(smem + P.off_lw);   // [2][HALVES][CAP][TM] mask words: bit 31-i = column 32c+i
    uint8_t* sLc = smem + P.off_lc;                 // [2][HALVES][CAP][TM] chunk id u * CPW + c
    uint8_t* sCnt = smem + P.off_cnt;               // [2][HALVES][TM] entries; bit 7: the list overflowed
    float2* sPart = (float2*)(smem + P.off_part);   // [2][HALVES][TM] (a1, a2) of the half
    float* sThr = (float*)(smem + P.off_thr);       // [2][TM] the row's threshold
    uint8_t* sFlag = smem + P.off_flag;             // [2][TM] the row goes to the exact recheck
    __half* sTmin = (__half*)(smem + P.off_tmin);   // [HALVES][U][TM] tile minimum of s~ + |x'|^2, rounded down
    uint64_t* sUnion = (uint64_t*)(smem + P.off_union);   // [2][SWEEP_WARPS] column tiles with a candidate
    uint64_t* bars = (uint64_t*)(smem + P.off_bar);
    uint64_t* b_full = bars + 0;
    uint64_t* x_full = bars + 1;    // [XSTAGES]
    uint64_t* x_empty = bars + 4;   // [XSTAGES]
    uint64_t* a_full = bars + 44;   // [ASTAGES]
    uint64_t* a_empty = bars + 47;  // [ASTAGES]
    uint64_t* t_full = bars + 11;   // [NACC]: an accumulator holds a computed column tile
    uint64_t* t_empty = bars + 15;  // [NACC]: the sweeps have read it
    uint64_t* m_full = bars + 19;   // [2]: the sweeps have written the candidate lists of a row tile
    uint64_t* m_empty = bars + 21;  // [2]: the resolvers are done with them
    uint64_t* drain = bars + 40;    // [NACC]: every MMA of one issuer has completed
    uint64_t* u_full = bars + 42;   // [2]: every sweep warp has published its column tiles with a candidate
    uint64_t* p_full = bars + 24;   // [2][4] both halves of a lane quarter have published (a1, a2)
    uint64_t* bs_full = bars + 32;  // [BMAX]: a column tile of the unit operand has landed (streamed operand)
    uint64_t* bs_empty = bars + 32 + BMAX; // [BMAX]: the MMAs reading it have completed
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_s;

    const PassArgs& a = P.a;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int d = DT;
    constexpr int kpad = k_width(DT);
    const int U = P.utiles;
    const uint32_t lim = P.wait_limit;
    const int64_t num_tiles = (a.n + TM - 1) / TM;
    const int64_t n_my = blockIdx.x < num_tiles ? (num_tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

    if (tid == 0) {
        ptx::mbar_init(b_full, 1);
        for (int s = 0; s < BMAX; ++s) {
            ptx::mbar_init(bs_full + s, 1);
            ptx::mbar_init(bs_empty + s, 1);
        }
        for (int s = 0; s < XSTAGES; ++s) {
            ptx::mbar_init(x_full + s, 1);
            ptx::mbar_init(x_empty + s, SWEEP_WARPS);
        }
        static_assert(NACC <= 4, "barrier slots 11-14 and 15-18");
        for (int s = 0; s < NACC; ++s) {
            ptx::mbar_init(t_full + s, 1);
            ptx::mbar_init(t_empty + s, SWEEP_WARPS);
        }
        for (int s = 0; s < 2; ++s) {
            ptx::mbar_init(m_full + s, SWEEP_WARPS);
            ptx::mbar_init(m_empty + s, RES_GROUP);
            ptx::mbar_init(u_full + s, SWEEP_WARPS);
            for (int qq = 0; qq < 4; ++qq) ptx::mbar_init(p_full + s * 4 + qq, HALVES);
        }
        for (int s = 0; s < NACC; ++s) ptx::mbar_init(drain + s, 1);
        for (int s = 0; s < ASTAGES; ++s) {
            ptx::mbar_init(a_full + s, SWEEP_WARPS);
            ptx::mbar_init(a_empty + s, NACC);   // a commit from each issuer
        }
        ptx::fence_mbar_init();
        abort_s = 0;
    }
    for (int k = tid; k <= d; k += NUM_THREADS) sCenter[k] = P.center[k];   // centre and scale
    if (P.off_w) {   // unit rows for the resolvers (16-byte aligned: checked on the host)
        const float4* src = (const float4*)a.w;
        float4* dst = (float4*)(smem + P.off_w);
        for (int64_t i = tid; i < a.m * DT / 4; i += NUM_THREADS) dst[i] = __ldg(src + i);
    }
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
        if (a.status) atomicOr(a.status, code);
        *abort_v = 1;
    };
    // Whole-warp forms for the sweep and resolver warps: a wait's outcome and the abort flag are made the same for
    // every lane, so that no lane leaves a loop whose warp-wide votes the others still execute.
    auto wwait = [&](uint64_t* bar, uint32_t parity) -> bool {
        return __all_sync(0xffffffffu, ptx::mbar_wait(bar, parity, lim));
    };
    auto waborted = [&]() -> bool { return __any_sync(0xffffffffu, *abort_v != 0); };
    // the column tiles of sweep 2 of the row tiles with list buffer lb (after their u_full phase)
    auto union_of = [&](int lb) -> uint64_t {
        uint64_t un = 0;
#pragma unroll
        for (int k = 0; k < SWEEP_WARPS; ++k) un |= sUnion[lb * SWEEP_WARPS + k];
        return un;
    };
#ifdef SOMGB_TC_PHASE_TIMING
    unsigned long long _tc_acc[TC_PHASES] = {};
    long long _tc_t0 = 0;
#endif

    if (warp == TMA_WARP) {
        if (lane == 0 && n_my > 0) {
            ptx::prefetch_tensormap(&tmap);
            const int BST = P.bstages;
            const int BSTD = BST > 0 ? BST : 1;   // divisor in the ring arithmetic (used only when BST > 0)
            if (BST == 0) {
                ptx::mbar_arrive_expect_tx(b_full, P.b_bytes);
                for (uint32_t off = 0; off < P.b_bytes; off += 32768u) {
                    const uint32_t len = P.b_bytes - off < 32768u ? P.b_bytes - off : 32768u;
                    ptx::bulk_g2s(sB + off, P.b + off, len, b_full);
                }
            }
            const uint32_t b_stride = (P.b_tile + 1023u) & ~1023u;
            int64_t issued = 0, kb = 0, withheld = -1;
            bool ok = true;
            auto issue_x = [&](int64_t it) -> bool {
                const int s = (int)(it % XSTAGES);
                if (it >= XSTAGES && !ptx::mbar_wait(x_empty + s, (uint32_t)((it / XSTAGES - 1) & 1), lim)) {
                    fail(1u);
                    return false;
                }
                const int64_t t = blockIdx.x + it * gridDim.x;
                issued = it + 1;
                if (t == P.withhold_tile) {   // test hook: this tile is never loaded, so its consumer's wait runs out
                    withheld = it;
                    return true;
                }
                ptx::mbar_arrive_expect_tx(x_full + s, (uint32_t)(TM * d * 4));
                ptx::tma_load_2d(smem + P.off_x + s * P.x_stride, &tmap, 0, (int32_t)(t * TM), x_full + s);
                return true;
            };
            if (BST == 0) {
                for (int64_t it = 0; ok && it < n_my && !*abort_v; ++it) ok = issue_x(it);
            } else {
                // sample tiles one row tile ahead of the unit-operand tiles, which go in the MMAs' order: every
                // column tile for sweep 1, then those with a candidate for sweep 2, once the sweeps have published them
                auto stream_b = [&](int u) -> bool {
                    const int st = (int)(kb % BSTD);
                    if (kb >= BST && !ptx::mbar_wait(bs_empty + st, (uint32_t)((kb / BSTD - 1) & 1), lim)) {
                        fail(4096u);
                        return false;
                    }
                    ptx::mbar_arrive_expect_tx(bs_full + st, P.b_tile);
                    const uint8_t* src = P.b + (size_t)u * P.b_tile;
                    for (uint32_t off = 0; off < P.b_tile; off += 32768u) {
                        const uint32_t len = P.b_tile - off < 32768u ? P.b_tile - off : 32768u;
                        ptx::bulk_g2s(sB + (size_t)st * b_stride + off, src + off, len, bs_full + st);
                    }
                    ++kb;
                    return true;
                };
                for (int64_t k = 0; ok && k <= n_my && !*abort_v; ++k) {   // phase k: sweep 1 of k, sweep 2 of k - 1
                    while (ok && issued < n_my && issued <= k + 1) ok = issue_x(issued);
                    for (int u = 0; ok && k < n_my && u < U && !*abort_v; ++u) ok = stream_b(u);
                    if (!ok || *abort_v || k == 0) continue;
                    const int64_t j = k - 1;
                    if (!ptx::mbar_wait(u_full + (j & 1), (uint32_t)((j >> 1) & 1), lim)) {
                        fail(32768u);
                        ok = false;
                        break;
                    }
                    for (uint64_t rest = union_of((int)(j & 1)); ok && rest != 0 && !*abort_v; rest &= rest - 1)
                        ok = stream_b(__ffsll((long long)rest) - 1);
                }
            }
            if (*abort_v || !ok) {
                // let the copies still in flight land before the CTA releases its shared memory (these waits end:
                // every copy waited for was issued)
                if (BST == 0) ptx::mbar_wait(b_full, 0);
                for (int64_t k = issued > XSTAGES ? issued - XSTAGES : 0; k < issued; ++k)
                    if (k != withheld) ptx::mbar_wait(x_full + (int)(k % XSTAGES), (uint32_t)((k / XSTAGES) & 1));
                for (int64_t k = kb > BST ? kb - BST : 0; BST > 0 && k < kb; ++k)
                    ptx::mbar_wait(bs_full + (int)(k % BSTD), (uint32_t)((k / BSTD) & 1));
            }
        }
    } else if (warp == MMA_WARP || warp == MMA_WARP2) {
        // Two issuers, one per accumulator: issuer k issues the MMAs of the column tiles g with g % NACC == k, so the
        // waits for one accumulator never hold up the other's MMAs.
        const int ik = warp == MMA_WARP ? 0 : 1;
        if (lane == 0 && n_my > 0) {
            const int BST = P.bstages;
            bool ok = BST > 0 || ptx::mbar_wait(b_full, 0, lim);
            if (!ok) fail(2u);
            const uint32_t sbo = (uint32_t)(kpad / 8) * 128u;
            const uint32_t b_addr = ptx::smem_u32(sB);
            const uint32_t b_stride = (P.b_tile + 1023u) & ~1023u;
            int64_t g = 0;
            int bst = 0;              // ring stage of column tile g, and the parity of its use
            uint32_t bpar = 0;
            // column tile g, unit tile u: its MMAs when it is this issuer's
            auto tile = [&](uint32_t a_addr, int u) -> bool {
                const int cur_bst = bst;
                const uint32_t cur_bpar = bpar;
                if (BST > 0 && ++bst == BST) {
                    bst = 0;
                    bpar ^= 1u;
                }
                const int64_t gg = g++;
                if ((int)(gg & (NACC - 1)) != ik) return true;
                const int buf = ik;
                TC_T0();
                // The unit-operand tile and the accumulator. With an even ring depth the stage's previous use,
                // column tile g - BST, was issued by this thread after its own wait, so that phase has completed
                // and the parity names this use: the tile is waited for first, off the critical path (the
                // accumulator is the wait that ends last). With an odd depth the previous use belongs to the
                // other issuer; the accumulator comes first, and once the sweeps have released tile g - NACC every
                // tile before it has completed its MMAs, so that use is over.
                const bool b_first = (BST & 1) == 0;
                if (b_first && BST > 0 && !ptx::mbar_wait(bs_full + cur_bst, cur_bpar, lim)) {
                    fail(8192u);
                    return false;
                }
                TC_T(13);
                if (gg >= NACC && !ptx::mbar_wait(t_empty + buf, (uint32_t)((gg / NACC - 1) & 1), lim)) {
                    fail(8u);
                    return false;
                }
                TC_T(12);
                if (!b_first && !ptx::mbar_wait(bs_full + cur_bst, cur_bpar, lim)) {
                    fail(8192u);
                    return false;
                }
                ptx::tc_fence_after();
                const uint32_t bu = BST > 0 ? b_addr + (uint32_t)cur_bst * b_stride
                                            : b_addr + (uint32_t)u * (uint32_t)(TN / 8) * sbo;
                const uint32_t dt = tbase + (uint32_t)(buf * TN);
#pragma unroll
                for (int ks = 0; ks < k_steps(DT); ++ks) {
                    int ka, kb;
                    k_step_cols(DT, ks, ka, kb);
                    const uint64_t ad = ptx::smem_desc(a_addr + (uint32_t)(ka / 8) * 128u, 128, sbo);
                    const uint64_t bd = ptx::smem_desc(bu + (uint32_t)(kb / 8) * 128u, 128, sbo);
                    ptx::mma_f16(dt, ad, bd, IDESC, ks > 0);
                }
                ptx::mma_commit(t_full + buf);
                // the stage is free once these MMAs have completed
                if (BST > 0) ptx::mma_commit(bs_empty + cur_bst);
                return true;
            };
            // phase k: sweep 1 of row tile k (every column tile), then sweep 2 of row tile k - 1 (the column tiles
            // with a candidate, published by the sweeps at the end of its sweep 1)
            for (int64_t k = 0; ok && k <= n_my && !*abort_v; ++k) {
                if (k < n_my) {
                    const int sa = (int)(k % ASTAGES);
                    if (!ptx::mbar_wait(a_full + sa, (uint32_t)((k / ASTAGES) & 1), lim)) { fail(4u); break; }
                    ptx::tc_fence_after();
                    const uint32_t a_addr = ptx::smem_u32(smem + P.off_a + sa * P.a_stride);
                    for (int u = 0; ok && u < U; ++u) ok = tile(a_addr, u);
                    if (!ok) break;
                }
                if (k >= 1) {
                    const int64_t j = k - 1;
                    const int sa = (int)(j % ASTAGES);
                    if (!ptx::mbar_wait(u_full + (j & 1), (uint32_t)((j >> 1) & 1), lim)) {
                        fail(32768u);
                        break;
                    }
                    const uint64_t un = union_of((int)(j & 1));
                    if (ik == 0 && a.sweep2_tiles) atomicAdd(a.sweep2_tiles, (unsigned long long)__popcll(un));
                    const uint32_t a_addr = ptx::smem_u32(smem + P.off_a + sa * P.a_stride);
                    for (uint64_t rest = un; ok && rest != 0; rest &= rest - 1)
                        ok = tile(a_addr, __ffsll((long long)rest) - 1);
                    if (!ok) break;
                    ptx::mma_commit(a_empty + sa);   // A tile j is no longer read once these MMAs have completed
                }
            }
            // every MMA issued by this thread has completed once its drain barrier flips
            ptx::mma_commit(drain + ik);
            if (!ptx::mbar_wait(drain + ik, 0)) fail(256u);
        }
    } else if (warp < SWEEP_WARPS) {
        // ------------------------------ converter + sweep (warps 0..7) ----------------------------------------------
        // warp e: TMEM lane quarter q = e & 3 (rows 32q..32q+31), column half h = e >> 2 (HW of each tile's TN columns)
        const int q = warp & 3, h = warp >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;

        // centred, scaled split-FP16 A row of `row`: this thread writes the 16-byte chunks kc = h, h + 2, ... of
        // kpad / 8; returns |x'|^2 (infinite when a coordinate is not finite or outside the FP16 split's range)
        auto convert = [&](int64_t it, float& xn_out) -> bool {
            const int s2 = (int)(it % ASTAGES), s3 = (int)(it % XSTAGES);
            if (it >= ASTAGES && !wwait(a_empty + s2, (uint32_t)((it / ASTAGES - 1) & 1))) { fail(16u); return false; }
            if (!wwait(x_full + s3, (uint32_t)((it / XSTAGES) & 1))) { fail(32u); return false; }
            const float4* xs4 = (const float4*)(smem + P.off_x + s3 * P.x_stride) + row * (DT / 4);
            const float scale = sCenter[DT];
            float xp[DT];
            bool finite = true;
            float xn = 0.0f;
#pragma unroll
            for (int k4 = 0; k4 < DT / 4; ++k4) {
                const float4 v = xs4[k4];
                xp[4 * k4 + 0] = (v.x - sCenter[4 * k4 + 0]) * scale;
                xp[4 * k4 + 1] = (v.y - sCenter[4 * k4 + 1]) * scale;
                xp[4 * k4 + 2] = (v.z - sCenter[4 * k4 + 2]) * scale;
                xp[4 * k4 + 3] = (v.w - sCenter[4 * k4 + 3]) * scale;
            }
#pragma unroll
            for (int k = 0; k < DT; ++k) {
                finite = finite && fabsf(xp[k]) < X_LIMIT;   // false for inf and NaN as well
                xn = fmaf(xp[k], xp[k], xn);
            }
            xn_out = finite ? xn : INFINITY;
            uint8_t* at = smem + P.off_a + s2 * P.a_stride;
            // chunks kc = H, H + HALVES, ... with H the warp's half as a compile-time constant (one branch per call)
            auto write_chunks = [&](auto hc) {
                constexpr int H = decltype(hc)::value;
#pragma unroll
                for (int kc = H; kc < kpad / 8; kc += HALVES) {
                    __align__(16) __half v[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int k = kc * 8 + i;
                        constexpr int nx = k_dedup(DT) ? 2 * DT : 3 * DT;   // x_hi | x_lo, or x_lo | x_hi | x_hi
                        constexpr int klo = k_dedup(DT) ? DT : 0;              // first x_lo column
                        float val = 0.0f;
                        if (k < nx) {
                            const float t = xp[k % DT];
                            const float hi = __half2float(__float2half_rn(t));
                            val = (k >= klo && k < klo + DT) ? t - hi : hi;
                        } else if (k == k_qcol(DT) || k == k_qcol(DT) + 1) {
                            val = Q_COLUMN;
                        }
                        v[i] = __float2half_rn(finite ? val : 0.0f);
                    }
                    *(uint4*)(at + canon_off(row, kc * 8, kpad)) = *(const uint4*)v;
                }
            };
            if (h == 0) write_chunks(std::integral_constant<int, 0>{});
            else write_chunks(std::integral_constant<int, 1>{});
            ptx::fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                ptx::mbar_arrive(a_full + s2);
                ptx::mbar_arrive(x_empty + s3);   // the sample tile is no longer read from shared memory
            }
            return true;
        };

        // the warp's last read of TMEM tile `buf` is complete: hand the accumulator back to the MMA issuer
        auto release = [&](int buf) {
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(t_empty + buf);
        };

        // This warp's HW columns of TMEM tile `buf` in CPW 32-column chunks, software-pipelined: chunk c + 1 is loading
        // while chunk c is processed (tcgen05.wait::ld waits for every load issued before it, so one load is in flight
        // at a time). The accumulator is handed back as soon as the last load has landed.
        auto stream_tile = [&](int buf, auto&& process) {
            const uint32_t base = tbase + lane_base + (uint32_t)(buf * TN + h * HW);
            uint32_t ra[32], rb[32];
            ptx::tmem_ld32_raw(base, ra);
            ptx::tmem_wait_ld1(ra);
#pragma unroll
            for (int c = 0; c + 2 < CPW; c += 2) {
                ptx::tmem_ld32_raw(base + 32 * (c + 1), rb);
                process(c, ra);
                ptx::tmem_wait_ld1(rb);
                ptx::tmem_ld32_raw(base + 32 * (c + 2), ra);
                process(c + 1, rb);
                ptx::tmem_wait_ld1(ra);
            }
            ptx::tmem_ld32_raw(base + 32 * (CPW - 1), rb);
            process(CPW - 2, ra);
            ptx::tmem_wait_ld1(rb);
            release(buf);
            process(CPW - 1, rb);
        };

        // The same with loads that also return each lane's chunk minimum: process(c, values, minimum).
        auto stream_tile_red = [&](int buf, auto&& process) {
            const uint32_t base = tbase + lane_base + (uint32_t)(buf * TN + h * HW);
            uint32_t ra[32], rb[32];
            float fa, fb;
            ptx::tmem_ldred32_raw(base, ra, fa);
            ptx::tmem_wait_ld_red(ra, fa);
#pragma unroll
            for (int c = 0; c + 2 < CPW; c += 2) {
                ptx::tmem_ldred32_raw(base + 32 * (c + 1), rb, fb);
                process(c, ra, fa);
                ptx::tmem_wait_ld_red(rb, fb);
                ptx::tmem_ldred32_raw(base + 32 * (c + 2), ra, fa);
                process(c + 1, rb, fb);
                ptx::tmem_wait_ld_red(ra, fa);
            }
            ptx::tmem_ldred32_raw(base + 32 * (CPW - 1), rb, fb);
            process(CPW - 2, ra, fa);
            ptx::tmem_wait_ld_red(rb, fb);
            release(buf);
            process(CPW - 1, rb, fb);
        };

        // the chunk's minimum; for ERR it also folds the chunk's four 8-unit group minima into the running two
        // smallest (a1, a2), else the minimum into a1
        auto chunk_min = [&](const uint32_t (&r)[32], float& a1, float& a2) -> float {
            if constexpr (ERR) {
                const float g0 = min8(r, 0), g1 = min8(r, 8), g2 = min8(r, 16), g3 = min8(r, 24);
                const float l01 = fminf(g0, g1), h01 = fmaxf(g0, g1), l23 = fminf(g2, g3), h23 = fmaxf(g2, g3);
                const float c1 = fminf(l01, l23), c2 = fmin3(fmaxf(l01, l23), h01, h23);   // the chunk's two smallest
                a2 = fmin3(a2, c2, fmaxf(a1, c1));
                a1 = fminf(a1, c1);
                return c1;
            } else {
                const float c = fminf(min16<0>(r), min16<16>(r));
                a1 = fminf(a1, c);
                return c;
            }
        };

        int64_t gcons = 0;   // TMEM tiles consumed
        float xn_next = 0.0f;
        bool ok = n_my > 0 ? convert(0, xn_next) : true;
        // Phase k: sweep 1 of row tile k, then sweep 2 of row tile k - 1 (the MMAs run in this order), so that the
        // column tiles of a sweep 2 are known one sweep 1 ahead and the tensor pipe never waits for them. thr_p,
        // thr_up_p, flagged_p: row tile k - 1's threshold state.
        float thr_p = -INFINITY, thr_up_p = -INFINITY;
        bool flagged_p = true;
        for (int64_t k = 0; ok && k <= n_my && !waborted(); ++k) {
            const float xn = xn_next;
            TC_T0();
            if (k + 1 < n_my && !(ok = convert(k + 1, xn_next))) break;
            TC_T(4);
            float thr = -INFINITY, thr_up = -INFINITY;
            bool flagged = true;
            float a1 = INFINITY, a2 = INFINITY;   // row tile k's bounds over this half's columns
            __half* const tmin = sTmin + (size_t)h * U * TM + row;   // the row's minimum over its half of each tile
            if (k < n_my) {
                // ---- sweep 1: the row's bounds over this half's columns --------------------------------------------
                for (int u = 0; u < U && ok; ++u, ++gcons) {
                    const int buf = (int)(gcons % NACC);
                    if (!wwait(t_full + buf, (uint32_t)((gcons / NACC) & 1))) {
                        fail(64u);
                        ok = false;
                        break;
                    }
                    TC_T(0);
                    ptx::tc_fence_after();
                    float tm = INFINITY;
                    stream_tile(buf, [&](int, const uint32_t (&r)[32]) { tm = fminf(tm, chunk_min(r, a1, a2)); });
                    // as |x' - w'|^2 = s~ + |x'|^2 (non-negative up to rounding, so FP16 holds it), rounded down
                    tmin[(size_t)u * TM] = __float2half_rd(__fadd_rd(tm, xn));
                    TC_T(1);
                }
                if (!ok) break;
            }
            if (k >= 1) {
                const int64_t j = k - 1;
                const int lb = (int)(j & 1);
                // the resolvers are done with list buffer lb (row tile j - 2)
                if (j >= 2 && !wwait(m_empty + lb, (uint32_t)(((j >> 1) - 1) & 1))) { fail(512u); break; }
                TC_T(5);
                if (!wwait(u_full + lb, (uint32_t)((j >> 1) & 1))) { fail(32768u); break; }
                const uint64_t un = union_of(lb);
                // ---- sweep 2: the candidate lists -------------------------------------------------------------------
                const size_t lbase = (size_t)((lb * HALVES + h) * CAP) * TM + row;
                uint32_t* lw = sLw + lbase;
                uint8_t* lc = sLc + lbase;
                int cnt = 0;
                bool ovf = false;
                for (uint64_t rest = un; rest != 0 && ok; rest &= rest - 1, ++gcons) {
                    const int u = __ffsll((long long)rest) - 1;
                    const int buf = (int)(gcons % NACC);
                    if (!wwait(t_full + buf, (uint32_t)((gcons / NACC) & 1))) {
                        fail(128u);
                        ok = false;
                        break;
                    }
                    TC_T(0);
                    ptx::tc_fence_after();
                    stream_tile_red(buf, [&](int c, const uint32_t (&r)[32], float red) {
                        // the chunk's masks only when a row of the warp has a candidate in it
                        if (__any_sync(0xffffffffu, red <= thr_p)) {
                            const uint32_t mw = sign_mask32(r, thr_up_p);
                            if (mw != 0u) {
                                if (cnt < CAP) {
                                    lw[cnt * TM] = mw;
                                    lc[cnt * TM] = (uint8_t)(u * CPW + c);
                                    ++cnt;
                                } else {
                                    ovf = true;
                                }
                            }
                        }
                    });
                    TC_T(1);
                }
                if (!ok) break;
                sCnt[(lb * HALVES + h) * TM + row] = (uint8_t)(cnt | (ovf ? 0x80 : 0));
                if (h == 0) {
                    sThr[lb * TM + row] = thr_p;
                    sFlag[lb * TM + row] = flagged_p ? 1 : 0;
                }
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(m_full + lb);
            }
            // Row tile k's threshold and the column tiles of its sweep 2, after sweep 2 of row tile k - 1: its MMAs
            // were issued behind those of sweep 1, so the tensor pipe computes the next sweep 1's first column tiles
            // while this exchange runs, and the tile set is still published a whole sweep 1 before it is needed.
            if (k < n_my) {
                const int lb = (int)(k & 1);
                // both halves' bounds: the row's threshold. ERR: M2 is the second smallest 8-unit group minimum, an
                // upper bound of the second smallest s~ (two groups have a unit at or below it), so the threshold
                // derived from it keeps every possible second BMU.
                sPart[(lb * HALVES + h) * TM + row] = make_float2(a1, a2);
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(p_full + lb * 4 + q);
                if (!wwait(p_full + lb * 4 + q, (uint32_t)((k >> 1) & 1))) { fail(2048u); break; }
                const float2 p0 = sPart[(lb * HALVES + 0) * TM + row], p1 = sPart[(lb * HALVES + 1) * TM + row];
                const float M1 = fminf(p0.x, p1.x);
                const float M2 = fminf(fmaxf(p0.x, p1.x), fminf(p0.y, p1.y));
                const float mref = ERR ? M2 : M1;
                flagged = !(xn < HUGE_S) || !(M1 + xn < HUGE_S) || !(mref < HUGE_S);
                thr = flagged ? -INFINITY : thr_of(mref, xn, fmaf(P.alpha, xn, GAMMA), P.beta, P.kthr);
                // v <= thr  <=>  v - thr_up < 0 with thr_up the next float above thr (exact: a difference of distinct
                // floats never rounds to zero), so each value costs one subtraction and one shift of its sign bit
                thr_up = nextafterf(thr, INFINITY);
                // ---- the column tiles of sweep 2: those where a row of the tile has a candidate --------------------
                // (a tile minimum at or under the threshold; both rounded outwards, so no candidate's tile is missed)
                uint32_t ulo = 0, uhi = 0;
                if (!flagged) {
                    const float dlim = __fadd_ru(thr, xn);
                    for (int u = 0; u < U; ++u) {
                        if (__half2float(tmin[(size_t)u * TM]) <= dlim) {
                            if (u < 32) ulo |= 1u << u;
                            else uhi |= 1u << (u - 32);
                        }
                    }
                }
                ulo = __reduce_or_sync(0xffffffffu, ulo);
                uhi = __reduce_or_sync(0xffffffffu, uhi);
                if (lane == 0) {
                    sUnion[lb * SWEEP_WARPS + warp] = ((uint64_t)uhi << 32) | ulo;
                    ptx::mbar_arrive(u_full + lb);
                }
            }
            thr_p = thr;
            thr_up_p = thr_up;
            flagged_p = flagged;
        }
    } else if (warp < SWEEP_WARPS + RES_WARPS) {
        // ------------------------------ resolvers: group g takes the row tiles it with it % RES_GROUPS == g ---------
        // (list buffer it % 2) while the sweeps run the next ones; thread r of the group's warp q owns row 32q + r:
        // float32 distances of its candidates, the decision, the outputs
        const int grp = (warp - SWEEP_WARPS) / RES_GROUP, q = (warp - SWEEP_WARPS) % RES_GROUP;
        const int row = q * 32 + lane;
        const float g32 = (float)(d + 2) * 5.9604645e-8f;
        const float fac = 1.0f + 8.0f * g32;
        DFAcc e0, e1, e2;
        const float* wrows = P.off_w ? (const float*)(smem + P.off_w) : a.w;   // unit rows: shared memory or L2
        for (int64_t it = grp; it < n_my && !waborted(); it += RES_GROUPS) {
            const int lb = (int)(it & 1);
            TC_T0();
            if (!wwait(m_full + lb, (uint32_t)((it >> 1) & 1))) { fail(1024u); break; }
            TC_T(6);
            const int64_t grow = (blockIdx.x + it * gridDim.x) * TM + row;
            const bool live = grow < a.n;
            const double rho_v = (live && a.rho) ? __ldg(a.rho + grow) : 1.0;   // issued early, used at the end
            // the sample row from global memory (just read by the tile load, so in L2)
            const float* xg = a.x + (live ? grow : 0) * DT;
            float xr[DT];   // loads issued before the candidate extraction, whose latency they overlap
#pragma unroll
            for (int k4 = 0; k4 < DT / 4; ++k4) {
                const float4 t = __ldg((const float4*)xg + k4);
                xr[4 * k4] = t.x; xr[4 * k4 + 1] = t.y; xr[4 * k4 + 2] = t.z; xr[4 * k4 + 3] = t.w;
            }
            const bool flagged = sFlag[lb * TM + row] != 0;
            const uint8_t c0 = sCnt[(lb * HALVES + 0) * TM + row], c1 = sCnt[(lb * HALVES + 1) * TM + row];
            const bool ovf = ((c0 | c1) & 0x80) != 0;
            const int n0 = c0 & 0x7f, nwc = n0 + (c1 & 0x7f);
            // list entry wi of the row (half 0's entries, then half 1's): its index in the list arrays
            auto entry = [&](int wi) -> size_t {
                const int hh = wi >= n0 ? 1 : 0;
                return (size_t)((lb * HALVES + hh) * CAP + (wi - hh * n0)) * TM + row;
            };
            auto entry_top = [&](int wi, size_t ix) -> int {   // the unit of bit 0 of the entry's word
                const int ch = sLc[ix];
                return (ch / CPW) * TN + (wi >= n0 ? HW : 0) + (ch % CPW) * 32 + 31;
            };
            // The candidates, one per lane and iteration (the next entry fetched in the same iteration), each one's
            // float32 distance computed and ranked (float32 top-3 in (distance, unit) order) as it is found. A row with
            // more than CAPR candidates stops there and goes to the exact recheck.
            int cnt = 0;
            float f1 = INFINITY, f2 = INFINITY, f3 = INFINITY;
            int32_t j1 = -1, j2 = -1, j3 = -1;
            auto push = [&](float df, int32_t j) {
                if (!lex_before(df, j, f3, j3)) return;
                if (lex_before(df, j, f2, j2)) {
                    f3 = f2; j3 = j2;
                    if (lex_before(df, j, f1, j1)) { f2 = f1; j2 = j1; f1 = df; j1 = j; }
                    else { f2 = df; j2 = j; }
                } else { f3 = df; j3 = j; }
            };
            {
                int wi = 0, jtop = 0;
                uint32_t word = 0u;
                bool more = live && !flagged && !ovf && nwc > 0;
                while (__any_sync(0xffffffffu, more)) {
                    const bool need = word == 0u;
                    if (need && wi < nwc) {
                        const size_t ix = entry(wi);
                        word = sLw[ix];
                        jtop = entry_top(wi, ix);
                    }
                    wi += need ? 1 : 0;
                    const int j = jtop - (__ffs(word) - 1);
                    const bool take = more && word != 0u && j < (int)a.m;
                    word &= word - 1u;
                    if (take) {
                        ++cnt;
                        push(cand_dist32v<DT>(wrows + (int64_t)j * DT, xr), j);
                    }
                    more = more && (word != 0u || wi < nwc) && cnt <= CAPR;
                }
            }
            // every candidate of the row again (the rare slower paths)
            auto for_each_cand = [&](auto&& f) {
                for (int wi = 0; wi < nwc; ++wi) {
                    const size_t ix = entry(wi);
                    uint32_t word = sLw[ix];
                    const int jt = entry_top(wi, ix);
                    while (word) {
                        const int j = jt - (__ffs(word) - 1);
                        word &= word - 1u;
                        if (j < (int)a.m) f(j);
                    }
                }
            };
            TC_T(9);
            const bool recheck = live && (flagged || ovf || cnt == 0 || cnt > CAPR);
            if (recheck) {
                const unsigned long long slotq = atomicAdd(P.row_count, 1ull);
                P.rows[slotq] = (int32_t)grow;
            } else if (live) {
                const float2* topo2 = (const float2*)a.topo;
                TC_T(8);
                // The float32 ranking decides when every rank that matters is separated by more than the float32
                // rounding bound: best vs second (both modes) and, for the error sums, second vs third. Otherwise the
                // contenders, the candidates within that bound of the best (second best), are ranked by the
                // reference's float64 sums.
                const float c1lim = f1 < 1.0e37f ? fmaf(f1, fac, 1.0e-37f) : INFINITY;
                const float c2lim = f2 < 1.0e37f ? fmaf(f2, fac, 1.0e-37f) : INFINITY;
                const bool gap12 = j2 < 0 || !(f2 <= c1lim);
                const bool separated = ERR ? (gap12 && (j3 < 0 || !(f3 <= c2lim))) : gap12;
                const float climit = ERR ? c2lim : c1lim;
                int32_t r1, r2;
                float2 tr1 = make_float2(0.0f, 0.0f), tr2 = tr1;
                DFloat rd1{0.0f, 0.0f};
                if (separated) {
                    r1 = j1;
                    r2 = ERR ? j2 : -1;
                    // the error sums' topographic coordinates of the best two, loaded while rd1 is computed
                    if (ERR && j1 >= 0 && j2 >= 0) {
                        tr1 = __ldg(topo2 + j1);
                        tr2 = __ldg(topo2 + j2);
                    }
                    if (ERR && j1 >= 0) rd1 = ref_dist_pair<DT>(wrows + (int64_t)j1 * DT, xr);
                } else {
                    // Contenders ranked by the compensated sum of the reference's float32 squares as a normalised
                    // float32 pair; ranks whose pairs differ by more than 2^-36 of the larger are the reference's
                    // ranks (df_apart). Closer ones (equal units, in practice) take the reference's float64 sums.
                    DFloat p1{INFINITY, 0.0f}, p2{INFINITY, 0.0f}, p3{INFINITY, 0.0f};
                    int32_t q1 = -1, q2 = -1, q3 = -1;
                    for_each_cand([&](int32_t j) {
                        if (!(cand_dist32v<DT>(wrows + (int64_t)j * DT, xr) <= climit)) return;
                        const DFloat t = ref_dist_pair<DT>(wrows + (int64_t)j * DT, xr);
                        const DFloat v = two_sum(t.hi, t.lo);
                        if (df_before(v, j, p3, q3)) {
                            if (df_before(v, j, p2, q2)) {
                                p3 = p2; q3 = q2;
                                if (df_before(v, j, p1, q1)) { p2 = p1; q2 = q1; p1 = v; q1 = j; }
                                else { p2 = v; q2 = j; }
                            } else { p3 = v; q3 = j; }
                        }
                    });
                    const bool sure = df_apart(p1, p2, q2) && (!ERR || df_apart(p2, p3, q3));
                    if (sure) {
                        r1 = q1;
                        r2 = ERR ? q2 : -1;
                        rd1 = p1;
                    } else {
                        const float* xs = xg;
                        Top2Lex tt;
                        tt.init();
                        for_each_cand([&](int32_t j) {
                            if (!(cand_dist32v<DT>(wrows + (int64_t)j * DT, xr) <= climit)) return;
                            tt.push(ref_sqdist(a.w + (int64_t)j * d, xs, d), j);
                        });
                        r1 = tt.i1;
                        r2 = ERR ? tt.i2 : -1;
                        rd1.hi = (float)tt.d1;
                        rd1.lo = (float)(tt.d1 - (double)rd1.hi);
                    }
                    if (ERR && r1 >= 0 && r2 >= 0) {
                        tr1 = topo2[r1];
                        tr2 = topo2[r2];
                    }
                }
                TC_T(10);
                emit_sample32(a, grow, rho_v, r1, r2, rd1, tr1, tr2, e0, e1, e2);
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(m_empty + lb);   // the sweeps may refill list buffer lb
            TC_T(7);
        }
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
#ifdef SOMGB_TC_PHASE_TIMING
    if (lane == 0 && (warp <= MMA_WARP || warp == MMA_WARP2))
        for (int ph = 0; ph < TC_PHASES; ++ph) atomicAdd(&g_tc_phase_cycles[ph], _tc_acc[ph]);
#endif

    // teardown: the MMA thread has drained its MMAs and, after an abort, the producer its copies
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == MMA_WARP) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tbase, 512);
    }
}

template <bool ERR, int DT>
int launch_main(const CUtensorMap& tmap, const TcArgs& P, unsigned grid, size_t smem, cudaStream_t stream) {
    auto kern = tc_pass_kernel<ERR, DT>;
    SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    timer_begin(stream);
    kern<<<grid, NUM_THREADS, smem, stream>>>(tmap, P);
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

// Test hook (somgb_debug_tc_withhold): the next tensor-core pass on this thread withholds one row tile's samples and
// bounds its protocol waits by `limit` polls; one-shot.
thread_local int64_t t_withhold_tile = -1;
thread_local uint32_t t_wait_limit = 0;

}  // namespace

unsigned int* device_status_word() {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tc_status) != cudaSuccess) return nullptr;
    return (unsigned int*)p;
}

bool device_has_tc() { return device_is_sm103(); }

bool tc_shape_ok(int64_t m, int d) {
    if (d != 4 && d != 8 && d != 16 && d != 32) return false;
    if (m <= 0 || m > (int64_t)MAX_U * TN) return false;   // a list entry names its chunk in a byte
    static_assert(MAX_U * TN <= CENTER_MAXM, "the centre kernel's bitmap covers every map of the pass");
    return tc_shape(m, d).smem <= SMEM_LIMIT;
}

bool tc_device_ok(int64_t m, int d) {
    return device_is_sm103() && encode_fn() != nullptr && max_smem_optin() >= tc_shape(m, d).smem;
}

bool tc_supported(int64_t n, int64_t m, int d, int algo) {
    if (algo == SOMGB_ALGO_FP32) return false;
    if (!tc_shape_ok(m, d)) return false;
    // AUTO: small passes (no prep cost on CUDA cores) and maps of fewer than 32 units stay on K0
    if (algo == SOMGB_ALGO_AUTO && (n * m < ((int64_t)1 << 22) || m < 32)) return false;
    return device_is_sm103() && encode_fn() != nullptr && max_smem_optin() >= tc_shape(m, d).smem;
}

#ifdef SOMGB_TC_PHASE_TIMING
// Instrumented builds only: copies out (and optionally clears) the TC_PHASES phase counters.
extern "C" int somgb_tc_phase_cycles(unsigned long long* out8, int reset) {
    SOMGB_CUDA_TRY(cudaDeviceSynchronize());
    SOMGB_CUDA_TRY(cudaMemcpyFromSymbol(out8, g_tc_phase_cycles, TC_PHASES * sizeof(unsigned long long)));
    if (reset) {
        unsigned long long z[TC_PHASES] = {};
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

void tc_debug_withhold(int64_t row_tile, uint32_t wait_limit) {
    t_withhold_tile = row_tile;
    t_wait_limit = wait_limit;
}

size_t tc_workspace_bytes(int64_t n, int64_t m, int d) { return tc_ws_layout(n, m, d, nullptr, nullptr); }

int launch_tc_pass(const PassArgs& a, void* ws, size_t ws_bytes, cudaStream_t stream) {
    if (((uintptr_t)a.x) % 16 || ((uintptr_t)a.w) % 16 || ((a.outs & OUT_ERR) && ((uintptr_t)a.topo) % 8))
        return set_error(SOMGB_ERR_INVALID, "tensor-core pass needs 16-byte aligned x and w, 8-byte aligned topo");
    const TcShape s = tc_shape(a.m, a.d);
    TcWs W;
    if (tc_ws_layout(a.n, a.m, a.d, &W, ws) > ws_bytes) return set_error(SOMGB_ERR_WORKSPACE, "tc workspace too small");
    const bool err = (a.outs & OUT_ERR) != 0;

    TcArgs P{};
    tc_error_coefficients(a.d, &P.alpha, &P.beta);
    P.kthr = nextafterf((float)(2.0 / (1.0 - (double)P.beta)), INFINITY);

    // unit operand
    tc_center_kernel<<<1, CENTER_THREADS, 0, stream>>>(a.w, a.m, a.d, W.center);
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

    P.a = a;
    P.b = W.b;
    P.center = W.center;
    P.rows = W.rows;
    P.row_count = a.recheck_count;
    P.kpad = s.kpad;
    P.utiles = s.utiles;
    P.off_a = s.off_a;
    P.off_x = s.off_x;
    P.off_lw = s.off_lw;
    P.off_part = s.off_part;
    P.off_thr = s.off_thr;
    P.off_lc = s.off_lc;
    P.off_cnt = s.off_cnt;
    P.off_flag = s.off_flag;
    P.off_tmin = s.off_tmin;
    P.off_union = s.off_union;
    P.off_w = s.off_w;
    P.off_center = s.off_center;
    P.off_bar = s.off_bar;
    P.a_stride = align_up(s.a_bytes, 1024);
    P.x_stride = s.x_bytes;
    P.b_bytes = (uint32_t)s.b_bytes;
    P.b_tile = (uint32_t)s.b_tile;
    P.bstages = s.bstages;
    P.wait_limit = t_wait_limit ? t_wait_limit : WAIT_LIMIT;
    P.withhold_tile = t_withhold_tile;
    t_withhold_tile = -1;
    t_wait_limit = 0;

    const int64_t tiles = ceil_div(a.n, TM);
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, num_sms());
    // at least half of an SM's shared memory, so that one CTA (the sole TMEM owner) runs per SM
    const size_t smem = std::max<size_t>(s.smem, 120 * 1024);
    int st = SOMGB_OK;
    if (err) {
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
