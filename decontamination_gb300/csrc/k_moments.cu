// Weighted first and second moments of a catalogue: the covariance behind the PCA initialisation of a map
// (algo/covariance.py:124-258 computes it with Welford's update over the samples, algo/som_pca.py:181-225 uses it).
//
// Samples count when every feature is finite and the weight is finite and positive (covariance.py:33-38); without
// weights every sample weighs 1. All sums are float64. Two passes over the resident rows:
//   1. W = sum w, S = sum w x (lanes over features, warp-level reductions, one float64 atomic per feature and warp);
//      the mean is S / W;
//   2. M2 = sum w (x - mean)(x - mean)^T over the upper triangle: sample tiles staged in shared memory as
//      sqrt(w) (x - mean) in float64, each thread owning pairs (j, k) and samples of its group, one FMA per pair and
//      sample; block partial sums go to global memory with one atomic per pair.
// The host combines chunks (Chan's pairwise update) and divides by W - ddof.
#include <cmath>

#include "common.cuh"

namespace somgb {
namespace {

constexpr int MOM_THREADS = 256;

template <typename T>
__device__ __forceinline__ bool sample_weight(const double* __restrict__ rho, int64_t i, double& w) {
    w = rho ? rho[i] : 1.0;
    return isfinite(w) && w > 0.0;
}

// Pass 1: out[0] += W, out[1 + k] += sum w x_k. Lanes over features: DP lanes per sample (DP a power of two >= d,
// at most 32; wider rows take ceil(d / 32) features per lane).
template <typename T>
__global__ void __launch_bounds__(MOM_THREADS) moments1_kernel(const T* __restrict__ x, const double* __restrict__ rho,
                                                               int64_t n, int d, int dp, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int spw = 32 / dp, slot = lane / dp, k0 = lane % dp;
    const int fpl = (d + dp - 1) / dp;   // features per lane (1 unless d > 32)
    const uint32_t slot_mask = dp == 32 ? 0xffffffffu : (((1u << dp) - 1u) << (slot * dp));
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double sw = 0.0, sx[2] = {0.0, 0.0};
    for (int64_t base = gw * spw; base < n; base += nw * spw) {
        const int64_t i = base + slot;
        const bool in = i < n;
        double w = 0.0;
        const bool wok = in && sample_weight<T>(rho, in ? i : 0, w);
        double v[2] = {0.0, 0.0};
        bool fin = true;
        for (int f = 0; f < fpl && f < 2; ++f) {
            const int k = k0 + f * dp;
            if (in && k < d) {
                v[f] = (double)x[i * d + k];
                fin = fin && isfinite(v[f]);
            }
        }
        const bool bad = __ballot_sync(0xffffffffu, !fin) & slot_mask;
        if (wok && !bad) {
            if (k0 == 0) sw += w;
            sx[0] = fma(w, v[0], sx[0]);
            sx[1] = fma(w, v[1], sx[1]);
        }
    }
    for (int o = dp; o < 32; o <<= 1) {
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
        sx[0] += __shfl_xor_sync(0xffffffffu, sx[0], o);
        sx[1] += __shfl_xor_sync(0xffffffffu, sx[1], o);
    }
    if (lane < dp) {
        if (lane == 0 && sw != 0.0) atomicAdd(out, sw);
        for (int f = 0; f < fpl && f < 2; ++f) {
            const int k = k0 + f * dp;
            if (k < d && sx[f] != 0.0) atomicAdd(out + 1 + k, sx[f]);
        }
    }
}

// mean_k = S_k / W in place (one thread per feature)
__global__ void moments_mean_kernel(int d, double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < d) out[1 + k] = out[0] > 0.0 ? out[1 + k] / out[0] : 0.0;
}

// Pass 2: out[1 + d + j*d + k] += sum w (x_j - mean_j)(x_k - mean_k) for j <= k. A tile of `tile` samples is read
// coalesced into shared memory as float64, each sample's weight and validity are taken from it, and the tile is
// centred and scaled by sqrt(w) in place (zero for samples that do not count). Thread t owns pair t % P (and, when
// the pairs are more than the block, t + blockDim ...) over the samples g, g + G, ... with g = t / P.
template <typename T>
__global__ void __launch_bounds__(1024) moments2_kernel(const T* __restrict__ x, const double* __restrict__ rho,
                                                        int64_t n, int d, int tile, double* __restrict__ out) {
    extern __shared__ double sm[];   // [tile][d] centred rows, then [tile] sqrt(w), then [d] mean
    double* rows = sm;
    double* sw = sm + (size_t)tile * d;
    double* mean = sw + tile;
    double* m2 = out + 1 + d;
    const int P = d * (d + 1) / 2;
    const int nt = blockDim.x;
    const int G = P >= nt ? 1 : nt / P;
    const int g = threadIdx.x / (P >= nt ? nt : P);
    const int p0 = threadIdx.x % (P >= nt ? nt : P);
    constexpr int MAXP = 3;   // d <= 64: P <= 2080 <= 3 * 1024 (blocks of fewer threads only when P is smaller)
    double acc[MAXP];
    int pj[MAXP], pk[MAXP];
#pragma unroll
    for (int q = 0; q < MAXP; ++q) {
        acc[q] = 0.0;
        int p = p0 + q * nt, j = 0;
        while (j < d && p >= d - j) { p -= d - j; ++j; }   // pair p of the row-major upper triangle
        pj[q] = j < d ? j : 0;
        pk[q] = j < d ? j + p : 0;
    }
    for (int k = threadIdx.x; k < d; k += nt) mean[k] = out[1 + k];
    for (int64_t t0 = (int64_t)blockIdx.x * tile; t0 < n; t0 += (int64_t)gridDim.x * tile) {
        const int rows_here = (int)min64(tile, n - t0);
        __syncthreads();
        for (int q = threadIdx.x; q < tile * d; q += nt)
            rows[q] = q < rows_here * d ? (double)x[t0 * d + q] : 0.0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < tile; idx += nt) {
            double w = 0.0;
            bool ok = idx < rows_here && sample_weight<T>(rho, t0 + (idx < rows_here ? idx : 0), w);
            for (int k = 0; ok && k < d; ++k) ok = isfinite(rows[idx * d + k]);
            sw[idx] = ok ? sqrt(w) : 0.0;
        }
        __syncthreads();
        for (int q = threadIdx.x; q < tile * d; q += nt) {
            const double s = sw[q / d];
            rows[q] = s != 0.0 ? s * (rows[q] - mean[q % d]) : 0.0;
        }
        __syncthreads();
        if (g < G) {
            for (int sidx = g; sidx < rows_here; sidx += G) {
                const double* r = rows + sidx * d;
#pragma unroll
                for (int q = 0; q < MAXP; ++q)
                    if (p0 + q * nt < P) acc[q] = fma(r[pj[q]], r[pk[q]], acc[q]);
            }
        }
    }
    if (g < G) {
#pragma unroll
        for (int q = 0; q < MAXP; ++q)
            if (p0 + q * nt < P && acc[q] != 0.0) atomicAdd(m2 + pj[q] * d + pk[q], acc[q]);
    }
}

// lower triangle = upper triangle
__global__ void moments_mirror_kernel(int d, double* __restrict__ out) {
    double* m2 = out + 1 + d;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < d * d; idx += gridDim.x * blockDim.x) {
        const int j = idx / d, k = idx % d;
        if (j > k) m2[idx] = m2[k * d + j];
    }
}

template <typename T>
int launch_moments(const T* x, const double* rho, int64_t n, int d, double* out, cudaStream_t stream) {
    if (!out) return set_error(SOMGB_ERR_INVALID, "out is NULL");
    if (d < 1 || d > 64) return set_error(SOMGB_ERR_UNSUPPORTED, "moments support 1 <= D <= 64 (got %d)", d);
    if (n < 0 || (n > 0 && !x)) return set_error(SOMGB_ERR_INVALID, "bad catalogue");
    SOMGB_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)(1 + d + d * d) * sizeof(double), stream));
    if (n == 0) return SOMGB_OK;
    int dp = 1;
    while (dp < d && dp < 32) dp <<= 1;
    const int64_t per_block = (int64_t)(MOM_THREADS / 32) * (32 / dp);
    const int64_t b1 = std::min<int64_t>(ceil_div(n, per_block), 8 * (int64_t)num_sms());
    moments1_kernel<T><<<(unsigned)b1, MOM_THREADS, 0, stream>>>(x, rho, n, d, dp, out);
    SOMGB_LAUNCH_CHECK();
    moments_mean_kernel<<<1, 64, 0, stream>>>(d, out);
    SOMGB_LAUNCH_CHECK();
    // block: every pair once, repeated over sample groups up to 1024 threads; tile: up to 96 KB of float64 rows
    const int P = d * (d + 1) / 2;
    const int threads2 = P >= 1024 ? 1024 : (1024 / P) * P;
    const int tile = (int)std::max<int64_t>(32, std::min<int64_t>(1024, (96 * 1024) / (8 * d)));
    const size_t smem = ((size_t)tile * d + tile + d) * sizeof(double);
    auto k2 = moments2_kernel<T>;
    if (smem > 48 * 1024) SOMGB_CUDA_TRY(cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t b2 = std::min<int64_t>(ceil_div(n, tile), 2 * (int64_t)num_sms());
    k2<<<(unsigned)b2, threads2, smem, stream>>>(x, rho, n, d, tile, out);
    SOMGB_LAUNCH_CHECK();
    moments_mirror_kernel<<<(unsigned)ceil_div((int64_t)d * d, 256), 256, 0, stream>>>(d, out);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

}  // namespace
}  // namespace somgb

using namespace somgb;

extern "C" int somgb_weighted_moments(const float* x, const double* rho, int64_t n, int d, double* out,
                                      somgb_stream_t stream) {
    return launch_moments<float>(x, rho, n, d, out, (cudaStream_t)stream);
}

extern "C" int somgb_weighted_moments_f64(const double* x, const double* rho, int64_t n, int d, double* out,
                                          somgb_stream_t stream) {
    return launch_moments<double>(x, rho, n, d, out, (cudaStream_t)stream);
}
