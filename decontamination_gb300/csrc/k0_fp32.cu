// K0: BMU search on CUDA cores — the plain FP32 form of the path.
//
// One thread per sample, 128 samples per CTA; the units stream through shared memory in tiles of 128
// (broadcast reads). Each (sample, unit) distance is the reference formula (algo/__init__.py:89-98) with the
// float64 sum replaced by a float32 FMA chain over the same float32 differences. All terms are non-negative,
// so that float32 sum df and the reference's float64 sum d of float32 squares satisfy |df - d| <= g*d with
// g = (D+2)*2^-24. A running top-2 (top-3 when the exact second BMU is needed) in float32 is certified when
// each next candidate exceeds the previous one by the factor (1+8g); otherwise the sample takes the exact
// path: it re-screens every unit in float32 and evaluates the reference formula in float64 for each unit
// whose df is within (1+8g) of the float32 second-best — the only units that can rank first or second.
#include "pass.cuh"

namespace somgb {

namespace {

constexpr int K0_THREADS = 128;
constexpr int K0_TILE = 128;

template <int DMAX>
__device__ __forceinline__ float fp32_dist(const float* __restrict__ wrow, const float (&xr)[DMAX], int d) {
    float acc = 0.0f;
    if constexpr (DMAX > 0) {
#pragma unroll
        for (int k = 0; k < DMAX; ++k) {
            float t = wrow[k] - xr[k];
            acc = fmaf(t, t, acc);
        }
    }
    return acc;
}

// Exact path of one sample: candidates are units with fp32 distance <= thr (thr = +inf: every unit).
// Reads the sample from global memory so that the register copy in the main loop keeps static indexing.
__device__ SampleResult exact_top2(const PassArgs& a, const float* __restrict__ xg, float thr) {
    Top2 t;
    t.init();
    const int d = a.d;
    for (int64_t j = 0; j < a.m; ++j) {
        const float* wr = a.w + j * d;
        float df = 0.0f;
        for (int k = 0; k < d; ++k) {
            float u = wr[k] - xg[k];
            df = fmaf(u, u, df);
        }
        if (!(df <= thr)) continue;   // also drops NaN, whose reference distance is NaN as well
        t.push(ref_sqdist(wr, xg, d), (int32_t)j);
    }
    SampleResult r;
    r.i1 = t.i1;
    r.i2 = t.i2;
    r.d1 = t.d1;
    return r;
}

template <int DMAX, bool TOP3>
__device__ __forceinline__ void k0_block(const PassArgs& a, int64_t i, bool live);

// Units j0 .. j0 + K0_TILE - 1 into the block's shared tile (rows padded to DMAX with zeros, past the map too);
// returns how many are real. Every thread of the block calls it.
template <int DMAX>
__device__ __forceinline__ int k0_load_tile(const PassArgs& a, float* wsh, int64_t j0) {
    const int tu = (int)min64(K0_TILE, a.m - j0);
    const int d = a.d;
    __syncthreads();
    for (int idx = threadIdx.x; idx < K0_TILE * DMAX; idx += K0_THREADS) {
        int jj = idx / DMAX, k = idx - jj * DMAX;
        wsh[idx] = (jj < tu && k < d) ? a.w[(j0 + jj) * d + k] : 0.0f;
    }
    __syncthreads();
    return tu;
}

// Thread t of block b handles sample b*128 + t.
template <int DMAX, bool TOP3>
__global__ void __launch_bounds__(K0_THREADS) k0_pass_kernel(PassArgs a) {
    const int64_t e = (int64_t)blockIdx.x * K0_THREADS + threadIdx.x;
    const bool live = e < a.n;
    k0_block<DMAX, TOP3>(a, live ? e : 0, live);
}

template <int DMAX, bool TOP3>
__device__ __forceinline__ void k0_block(const PassArgs& a, int64_t i, bool live) {
    constexpr int DS = DMAX > 0 ? DMAX : 4;
    __shared__ __align__(16) float wsh[K0_TILE * DS];
    const int d = a.d;
    const float* xg = a.x + (live ? i : 0) * d;

    float xr[DMAX > 0 ? DMAX : 1];
    if constexpr (DMAX > 0) {
#pragma unroll
        for (int k = 0; k < DMAX; ++k) xr[k] = (live && k < d) ? xg[k] : 0.0f;
    }

    float m1 = INFINITY, m2 = INFINITY, m3 = INFINITY;
    int32_t u1 = -1, u2 = -1, u3 = -1;
    for (int64_t j0 = 0; j0 < a.m; j0 += K0_TILE) {
        const int tu = (int)min64(K0_TILE, a.m - j0);
        if constexpr (DMAX > 0) k0_load_tile<DMAX>(a, wsh, j0);
        for (int jj = 0; jj < tu; ++jj) {
            float df;
            if constexpr (DMAX > 0) {
                df = fp32_dist<DMAX>(wsh + jj * DMAX, xr, d);
            } else {
                const float* wr = a.w + (j0 + jj) * d;
                df = 0.0f;
                for (int k = 0; k < d; ++k) {
                    float u = wr[k] - xg[k];
                    df = fmaf(u, u, df);
                }
            }
            const int32_t j = (int32_t)(j0 + jj);
            if (TOP3) {
                if (df < m3) {
                    if (df < m2) {
                        m3 = m2; u3 = u2;
                        if (df < m1) { m2 = m1; u2 = u1; m1 = df; u1 = j; }
                        else { m2 = df; u2 = j; }
                    } else { m3 = df; u3 = j; }
                }
            } else {
                if (df < m2) {
                    if (df < m1) { m2 = m1; u2 = u1; m1 = df; u1 = j; }
                    else { m2 = df; u2 = j; }
                }
            }
        }
    }

    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    const float g = (float)(d + 2) * 5.9604645e-8f;
    const float fac = 1.0f + 8.0f * g;
    bool ok = m1 < 1.0e37f && m2 < 1.0e37f && m2 > fmaf(m1, fac, 1.0e-37f);
    if (TOP3) ok = ok && m3 < 1.0e37f && m3 > fmaf(m2, fac, 1.0e-37f);
    const bool exact = live && !ok;
    SampleResult r;
    if (live && ok) {
        r.i1 = u1;
        r.i2 = TOP3 ? u2 : -1;
        r.d1 = (a.outs & OUT_ERR) ? ref_sqdist(a.w + (int64_t)u1 * d, xg, d) : 0.0;
    }
    if (exact && a.recheck_count) atomicAdd(a.recheck_count, 1ull);
    const float thr = m2 < 1.0e37f ? fmaf(m2, fac, 1.0e-37f) : INFINITY;
    if constexpr (DMAX > 0) {
        // Exact path: more passes over the same shared-memory unit tiles, for the rows of the block that need them.
        // First the units the float32 screen cannot exclude are ranked by compensated float32 sums of the reference's
        // squares; ranks that pass df_apart are the reference's (D <= 32). Rows left undecided (equal units,
        // non-finite sums) take the reference's float64 sums in a last pass.
        bool fp64 = exact && !(DMAX <= 32 && thr < 1.0e37f);
        if (__syncthreads_or(exact && !fp64)) {
            DFloat p1{INFINITY, 0.0f}, p2{INFINITY, 0.0f}, p3{INFINITY, 0.0f};
            int32_t q1 = -1, q2 = -1, q3 = -1;
            for (int64_t j0 = 0; j0 < a.m; j0 += K0_TILE) {
                const int tu = k0_load_tile<DMAX>(a, wsh, j0);
                if (exact && !fp64) {
                    for (int jj = 0; jj < tu; ++jj) {
                        if (!(fp32_dist<DMAX>(wsh + jj * DMAX, xr, d) <= thr)) continue;
                        const DFloat t = ref_dist_pair<DMAX>(wsh + jj * DMAX, xr);
                        const DFloat v = two_sum(t.hi, t.lo);
                        const int32_t j = (int32_t)(j0 + jj);
                        if (TOP3) {
                            if (df_before(v, j, p3, q3)) {
                                if (df_before(v, j, p2, q2)) {
                                    p3 = p2; q3 = q2;
                                    if (df_before(v, j, p1, q1)) { p2 = p1; q2 = q1; p1 = v; q1 = j; }
                                    else { p2 = v; q2 = j; }
                                } else { p3 = v; q3 = j; }
                            }
                        } else if (df_before(v, j, p2, q2)) {
                            if (df_before(v, j, p1, q1)) { p2 = p1; q2 = q1; p1 = v; q1 = j; }
                            else { p2 = v; q2 = j; }
                        }
                    }
                }
            }
            if (exact && !fp64) {
                const bool finite = q1 >= 0 && p1.hi < 1.0e37f && (q2 < 0 || p2.hi < 1.0e37f) &&
                                    (!TOP3 || q3 < 0 || p3.hi < 1.0e37f);
                if (finite && df_apart(p1, p2, q2) && (!TOP3 || df_apart(p2, p3, q3))) {
                    r.i1 = q1;
                    r.i2 = q2;
                    r.d1 = (a.outs & OUT_ERR) ? ref_sqdist(a.w + (int64_t)q1 * d, xg, d) : 0.0;
                } else {
                    fp64 = true;
                }
            }
        }
        if (__syncthreads_or(fp64)) {
            Top2 t;
            t.init();
            for (int64_t j0 = 0; j0 < a.m; j0 += K0_TILE) {
                const int tu = k0_load_tile<DMAX>(a, wsh, j0);
                if (fp64) {
                    for (int jj = 0; jj < tu; ++jj) {
                        if (!(fp32_dist<DMAX>(wsh + jj * DMAX, xr, d) <= thr)) continue;   // drops NaN, as the reference
                        t.push(ref_sqdist(wsh + jj * DMAX, xg, d), (int32_t)(j0 + jj));
                    }
                }
            }
            if (fp64) {
                r.i1 = t.i1;
                r.i2 = t.i2;
                r.d1 = t.d1;
            }
        }
    } else {
        if (exact) r = exact_top2(a, xg, thr);
    }
    if (live) emit_sample(a, i, r, e0, e1, e2);
    if (a.outs & OUT_ERR) block_add3(e0, e1, e2, a.err3);
    __syncthreads();   // the shared tile and reduction buffers are reused by the next row block
}

template <int DMAX>
int launch_dmax(const PassArgs& a, cudaStream_t stream) {
    const dim3 grid((unsigned)ceil_div(a.n, K0_THREADS));
    timer_begin(stream);
    if (a.outs & OUT_ERR)
        k0_pass_kernel<DMAX, true><<<grid, K0_THREADS, 0, stream>>>(a);
    else
        k0_pass_kernel<DMAX, false><<<grid, K0_THREADS, 0, stream>>>(a);
    timer_end(stream);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

// ---------------------------------------------------------------------------------------------------------------------
// Listed rows: one warp per sample. The rows the tensor-core pass leaves undecided are few (typically 1e-4 of a
// catalogue) and scattered, so a thread per sample would leave most SMs idle and run each sample's unit scan as one
// latency-bound chain. Here lane l scans units l, l+32, ...; the per-lane rankings are merged across the warp in
// (distance, unit) order, which is the order the one-thread scan ranks in (strict comparisons in ascending unit
// order keep the lowest unit among equal distances).
// ---------------------------------------------------------------------------------------------------------------------

constexpr int KR_THREADS = 256;

// (da, ja) ranks before (db, jb): lexicographic, empty entries (unit < 0) last
__device__ __forceinline__ bool lex_before32(float da, int32_t ja, float db, int32_t jb) {
    return ja >= 0 && (jb < 0 || da < db || (da == db && ja < jb));
}
__device__ __forceinline__ bool lex_before64(double da, int32_t ja, double db, int32_t jb) {
    return ja >= 0 && (jb < 0 || da < db || (da == db && ja < jb));
}

// float32 FMA-chain distance in feature order (the chain of k0_block)
template <int DMAX>
__device__ __forceinline__ float row_dist32(const float* __restrict__ wr, const float* __restrict__ xr, int d) {
    float acc = 0.0f;
    if constexpr (DMAX > 0) {
#pragma unroll
        for (int k = 0; k < DMAX; ++k) {
            const float t = __ldg(wr + k) - xr[k];
            acc = fmaf(t, t, acc);
        }
    } else {
        for (int k = 0; k < d; ++k) {
            const float t = __ldg(wr + k) - xr[k];
            acc = fmaf(t, t, acc);
        }
    }
    return acc;
}

template <int DMAX, bool TOP3>
__global__ void __launch_bounds__(KR_THREADS) k0_rows_kernel(PassArgs a, const int32_t* __restrict__ rows,
                                                             const unsigned long long* __restrict__ count,
                                                             long long max_rows) {
    const int lane = threadIdx.x & 31;
    const int64_t total = (int64_t)*count;
    if (total > max_rows) return;   // a long list: k0_rows_block_kernel takes it
    const int64_t nwarps = (int64_t)gridDim.x * (KR_THREADS / 32);
    const int d = a.d;
    const float g = (float)(d + 2) * 5.9604645e-8f;
    const float fac = 1.0f + 8.0f * g;
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    // listed row r to warp r / gridDim.x of block r % gridDim.x: a short list spreads over every SM, one row per
    // block, instead of filling the warps of a few blocks (each row scans the whole map)
    for (int64_t r = (int64_t)blockIdx.x + (int64_t)(threadIdx.x >> 5) * gridDim.x; r < total; r += nwarps) {
        const int64_t i = rows[r];
        const float* xg = a.x + i * d;
        float xl[DMAX > 0 ? DMAX : 1];
        if constexpr (DMAX > 0) {
#pragma unroll
            for (int k = 0; k < DMAX; ++k) xl[k] = __ldg(xg + k);
        }
        const float* xr = DMAX > 0 ? xl : xg;

        // float32 top-3 of this lane's units, then of the warp
        float m1 = INFINITY, m2 = INFINITY, m3 = INFINITY;
        int32_t u1 = -1, u2 = -1, u3 = -1;
        for (int64_t j = lane; j < a.m; j += 32) {
            const float df = row_dist32<DMAX>(a.w + j * d, xr, d);
            if (df < m3) {
                if (df < m2) {
                    m3 = m2; u3 = u2;
                    if (df < m1) { m2 = m1; u2 = u1; m1 = df; u1 = (int32_t)j; }
                    else { m2 = df; u2 = (int32_t)j; }
                } else { m3 = df; u3 = (int32_t)j; }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float p1 = __shfl_xor_sync(0xffffffffu, m1, o), p2 = __shfl_xor_sync(0xffffffffu, m2, o),
                        p3 = __shfl_xor_sync(0xffffffffu, m3, o);
            const int32_t q1 = __shfl_xor_sync(0xffffffffu, u1, o), q2 = __shfl_xor_sync(0xffffffffu, u2, o),
                          q3 = __shfl_xor_sync(0xffffffffu, u3, o);
            const float pv[3] = {p1, p2, p3};
            const int32_t qv[3] = {q1, q2, q3};
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const float dv = pv[t];
                const int32_t jv = qv[t];
                if (lex_before32(dv, jv, m3, u3)) {
                    if (lex_before32(dv, jv, m2, u2)) {
                        m3 = m2; u3 = u2;
                        if (lex_before32(dv, jv, m1, u1)) { m2 = m1; u2 = u1; m1 = dv; u1 = jv; }
                        else { m2 = dv; u2 = jv; }
                    } else { m3 = dv; u3 = jv; }
                }
            }
        }

        bool ok = m1 < 1.0e37f && m2 < 1.0e37f && m2 > fmaf(m1, fac, 1.0e-37f);
        if (TOP3) ok = ok && m3 < 1.0e37f && m3 > fmaf(m2, fac, 1.0e-37f);
        SampleResult res;
        if (ok) {
            res.i1 = u1;
            res.i2 = TOP3 ? u2 : -1;
            res.d1 = (a.outs & OUT_ERR) ? ref_sqdist(a.w + (int64_t)u1 * d, xg, d) : 0.0;
        } else {
            // exact path: the reference's float64 sum for every unit the float32 screen cannot exclude
            if (a.recheck_count && lane == 0) atomicAdd(a.recheck_count, 1ull);
            const float thr = m2 < 1.0e37f ? fmaf(m2, fac, 1.0e-37f) : INFINITY;
            Top2 t;
            t.init();
            for (int64_t j = lane; j < a.m; j += 32) {
                const float* wr = a.w + j * d;
                const float df = row_dist32<DMAX>(wr, xr, d);
                if (!(df <= thr)) continue;   // also drops NaN, whose reference distance is NaN as well
                t.push(ref_sqdist(wr, xg, d), (int32_t)j);
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double p1 = __shfl_xor_sync(0xffffffffu, t.d1, o), p2 = __shfl_xor_sync(0xffffffffu, t.d2, o);
                const int32_t q1 = __shfl_xor_sync(0xffffffffu, t.i1, o), q2 = __shfl_xor_sync(0xffffffffu, t.i2, o);
                const double pv[2] = {p1, p2};
                const int32_t qv[2] = {q1, q2};
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    if (lex_before64(pv[k], qv[k], t.d2, t.i2)) {
                        if (lex_before64(pv[k], qv[k], t.d1, t.i1)) { t.d2 = t.d1; t.i2 = t.i1; t.d1 = pv[k]; t.i1 = qv[k]; }
                        else { t.d2 = pv[k]; t.i2 = qv[k]; }
                    }
                }
            }
            res.i1 = t.i1;
            res.i2 = t.i2;
            res.d1 = t.d1;
        }
        if (lane == 0) emit_sample(a, i, res, e0, e1, e2);
    }
    if (a.outs & OUT_ERR) block_add3(e0, e1, e2, a.err3);
}

// A long list: thread t of block b takes listed row 128 i + t for the blocks' turns i; the unit tiles are shared
// through shared memory by the block's 128 rows (k0_block), instead of each row reading the whole map.
template <int DMAX, bool TOP3>
__global__ void __launch_bounds__(K0_THREADS) k0_rows_block_kernel(PassArgs a, const int32_t* __restrict__ rows,
                                                                   const unsigned long long* __restrict__ count,
                                                                   long long min_rows) {
    const int64_t total = (int64_t)*count;
    if (total < min_rows) return;   // a short list: k0_rows_kernel takes it
    for (int64_t base = (int64_t)blockIdx.x * K0_THREADS; base < total; base += (int64_t)gridDim.x * K0_THREADS) {
        const int64_t e = base + threadIdx.x;
        const bool live = e < total;
        k0_block<DMAX, TOP3>(a, live ? (int64_t)rows[e] : 0, live);
    }
}

template <int DMAX>
int launch_rows(const PassArgs& a, const int32_t* rows, const unsigned long long* count, cudaStream_t stream) {
    // the list length is known on the device only: both kernels launch and the one whose range it is in runs. Above
    // a thousand rows the block form wins: its rows share each unit tile through shared memory, where a warp per row
    // reads the whole map from L2 for every row.
    const long long split = 1024;
    const dim3 grid((unsigned)(4 * num_sms())), bgrid((unsigned)(2 * num_sms()));
    if (a.outs & OUT_ERR) {
        k0_rows_kernel<DMAX, true><<<grid, KR_THREADS, 0, stream>>>(a, rows, count, split - 1);
        k0_rows_block_kernel<DMAX, true><<<bgrid, K0_THREADS, 0, stream>>>(a, rows, count, split);
    } else {
        k0_rows_kernel<DMAX, false><<<grid, KR_THREADS, 0, stream>>>(a, rows, count, split - 1);
        k0_rows_block_kernel<DMAX, false><<<bgrid, K0_THREADS, 0, stream>>>(a, rows, count, split);
    }
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

// Float64 maps: the reference formula is float64 end to end, computed exactly as written.
__global__ void __launch_bounds__(128) exact_pass_f64_kernel(const double* __restrict__ x,
                                                             const double* __restrict__ rho, int64_t n, int d,
                                                             const double* __restrict__ w, int64_t m,
                                                             const double* __restrict__ topo, double penalty,
                                                             int outs, int32_t* bmu_out, double* hist,
                                                             double* err3, int32_t* train_bmu) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    if (i < n) {
        const double* xr = x + i * d;
        Top2 t;
        t.init();
        for (int64_t j = 0; j < m; ++j) t.push(ref_sqdist(w + j * d, xr, d), (int32_t)j);
        const double r = rho ? rho[i] : 1.0;
        if (outs & OUT_BMU) bmu_out[i] = t.i1 < 0 ? 0 : t.i1;
        if ((outs & OUT_HIST) && r > 0.0) atomicAdd(hist + (t.i1 < 0 ? 0 : t.i1), r);
        if (outs & OUT_TRAIN) train_bmu[i] = (r > 0.0 && t.i1 >= 0) ? t.i1 : -1;
        if ((outs & OUT_ERR) && r > 0.0 && t.i1 >= 0 && t.i2 >= 0) {
            e0 += r * sqrt(t.d1);
            if (topo_sqdist(topo, t.i1, t.i2) > penalty) e1 += r;
            e2 += r;
        }
    }
    if (outs & OUT_ERR) block_add3(e0, e1, e2, err3);
}

}  // namespace

int launch_k0_pass(const PassArgs& a, cudaStream_t stream, const int32_t* rows, const unsigned long long* count) {
    if (a.n == 0) return SOMGB_OK;
    if (rows) {
        switch (a.d) {
            case 4: return launch_rows<4>(a, rows, count, stream);
            case 8: return launch_rows<8>(a, rows, count, stream);
            case 16: return launch_rows<16>(a, rows, count, stream);
            case 32: return launch_rows<32>(a, rows, count, stream);
            default: return launch_rows<0>(a, rows, count, stream);
        }
    }
    if (a.d <= 4) return launch_dmax<4>(a, stream);
    if (a.d <= 8) return launch_dmax<8>(a, stream);
    if (a.d <= 16) return launch_dmax<16>(a, stream);
    if (a.d <= 32) return launch_dmax<32>(a, stream);
    if (a.d <= 64) return launch_dmax<64>(a, stream);
    return launch_dmax<0>(a, stream);
}

int launch_exact_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                          const double* topo, double penalty, int outs, int32_t* bmu_out, double* hist,
                          double* err3, int32_t* train_bmu, cudaStream_t stream) {
    if (n == 0) return SOMGB_OK;
    exact_pass_f64_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, stream>>>(x, rho, n, d, w, m, topo, penalty, outs,
                                                                         bmu_out, hist, err3, train_bmu);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

}  // namespace somgb
