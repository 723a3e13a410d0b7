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

// rows == NULL: thread t of block b handles sample b*128 + t. Otherwise the blocks stride over the first *count
// entries of `rows` (a list of sample indices), 128 per block and iteration.
template <int DMAX, bool TOP3>
__global__ void __launch_bounds__(K0_THREADS) k0_pass_kernel(PassArgs a, const int32_t* __restrict__ rows,
                                                             const unsigned long long* __restrict__ count) {
    const int64_t total = rows ? (int64_t)*count : a.n;
    const int64_t step = rows ? (int64_t)gridDim.x * K0_THREADS : total + 1;
    for (int64_t base = (int64_t)blockIdx.x * K0_THREADS; base < total; base += step) {
        const int64_t e = base + threadIdx.x;
        const bool live = e < total;
        const int64_t i = !live ? 0 : (rows ? (int64_t)rows[e] : e);
        k0_block<DMAX, TOP3>(a, i, live);
    }
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
        if constexpr (DMAX > 0) {
            __syncthreads();
            for (int idx = threadIdx.x; idx < K0_TILE * DMAX; idx += K0_THREADS) {
                int jj = idx / DMAX, k = idx - jj * DMAX;
                wsh[idx] = (jj < tu && k < d) ? a.w[(j0 + jj) * d + k] : 0.0f;
            }
            __syncthreads();
        }
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
    if (live) {
        const float g = (float)(d + 2) * 5.9604645e-8f;
        const float fac = 1.0f + 8.0f * g;
        bool ok = m1 < 1.0e37f && m2 < 1.0e37f && m2 > fmaf(m1, fac, 1.0e-37f);
        if (TOP3) ok = ok && m3 < 1.0e37f && m3 > fmaf(m2, fac, 1.0e-37f);
        SampleResult r;
        if (ok) {
            r.i1 = u1;
            r.i2 = TOP3 ? u2 : -1;
            r.d1 = (a.outs & OUT_ERR) ? ref_sqdist(a.w + (int64_t)u1 * d, xg, d) : 0.0;
        } else {
            if (a.recheck_count) atomicAdd(a.recheck_count, 1ull);
            const float thr = m2 < 1.0e37f ? fmaf(m2, fac, 1.0e-37f) : INFINITY;
            r = exact_top2(a, xg, thr);
        }
        emit_sample(a, i, r, e0, e1, e2);
    }
    if (a.outs & OUT_ERR) block_add3(e0, e1, e2, a.err3);
    __syncthreads();   // the shared tile and reduction buffers are reused by the next row block
}

template <int DMAX>
int launch_dmax(const PassArgs& a, const int32_t* rows, const unsigned long long* count, cudaStream_t stream) {
    dim3 grid(rows ? (unsigned)(2 * num_sms()) : (unsigned)ceil_div(a.n, K0_THREADS));
    if (!rows) timer_begin(stream);
    if (a.outs & OUT_ERR)
        k0_pass_kernel<DMAX, true><<<grid, K0_THREADS, 0, stream>>>(a, rows, count);
    else
        k0_pass_kernel<DMAX, false><<<grid, K0_THREADS, 0, stream>>>(a, rows, count);
    if (!rows) timer_end(stream);
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
    if (a.d <= 4) return launch_dmax<4>(a, rows, count, stream);
    if (a.d <= 8) return launch_dmax<8>(a, rows, count, stream);
    if (a.d <= 16) return launch_dmax<16>(a, rows, count, stream);
    if (a.d <= 32) return launch_dmax<32>(a, rows, count, stream);
    if (a.d <= 64) return launch_dmax<64>(a, rows, count, stream);
    return launch_dmax<0>(a, rows, count, stream);
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
