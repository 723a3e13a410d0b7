// Training-side kernels: per-BMU segmented sums, the neighbourhood contraction with the divide, iteration
// mode, and the plain divide.
//
// The reference scatters every sample into every unit with float32 atomics
// (algo/som_batch.py:552-566): num_j += rho*exp(-|t_j - t_b|^2/(2 sigma^2))*x, N*M*(D+1) atomics per epoch.
// Because the factor depends on the sample only through its BMU b, the same sums factor exactly as
//   num = H.S, den = H.c,  S_b = sum_{i: bmu_i = b} rho_i x_i,  c_b = sum_{i: bmu_i = b} rho_i,
// so an epoch needs N*(D+1) additions into M*(D+1) float64 bins plus an M x M x (D+1) contraction.
#include "common.cuh"

namespace somgb {

namespace {

// ---------------------------------------------------------------------------------------------------------------------
// Segmented sums in exact fixed point. Every term v = (float)rho * x_k is quantised as q = rint(v * 2^(47 - e_k)), with
// 2^e_k above the largest |v| of feature k over the dataset (somgb_feature_bounds), so |q| < 2^47 and the quantisation
// error is below 2^-48 of that bound. q is split into three 16-bit limbs accumulated with shared-memory int32 atomics
// (native and fast on sm_100-class GPUs, unlike float atomics); a window of at most 2^15 samples keeps every limb sum
// inside int32. At the end of each window the limbs of every bin recombine exactly in int64 and are added to the
// float64 sums in global memory. The result is the exact sum to ~1e-14 relative, independent of summation order.
// CTA (chunk, range) owns the bins of units [lo, lo+cnt); ranges exist only when M*(D+1) bins exceed shared memory.
// ---------------------------------------------------------------------------------------------------------------------

constexpr int FX_BITS = 47;
constexpr int64_t FX_WINDOW = 1 << 15;

__device__ __forceinline__ int fx_exponent(float bound) {
    int e = 0;
    if (bound > 0.0f) frexpf(bound, &e);   // bound < 2^e
    return max(e, -60);
}

__device__ __forceinline__ void fx_add(int32_t* limbs, int64_t nb, int64_t bin, long long q) {
    atomicAdd(limbs + bin, (int32_t)(q & 0xFFFF));
    atomicAdd(limbs + nb + bin, (int32_t)((q >> 16) & 0xFFFF));
    atomicAdd(limbs + 2 * nb + bin, (int32_t)(q >> 32));
}

// Nearest integer of a float32 in [-2^22, 2^22], exactly, with full-rate float and integer ops: adding 1.5 * 2^23
// rounds to an integer and puts it in the low mantissa bits.
__device__ __forceinline__ int32_t fx_small_int(float v) {
    return (int32_t)__float_as_uint(__fadd_rn(v, 12582912.0f)) - 0x4B400000;
}

// Adds q = rint(f) (|f| < 2^47) as three signed limbs, q = L2 * 2^32 + L1 * 2^16 + L0 with |L| <= 2^15, without a
// 64-bit conversion: adding 1.5 * 2^55 rounds f to a multiple of 2^32 (f2), 1.5 * 2^39 rounds the exact remainder to
// a multiple of 2^16 (f1), and 1.5 * 2^23 rounds the last remainder to an integer; every step is exact float32.
// The limbs of 2^15 samples stay inside int32 and recombine as in the unsigned split.
__device__ __forceinline__ void fx_add_float(int32_t* limbs, int64_t nb, int64_t bin, float f) {
    const float f2 = __fsub_rn(__fadd_rn(f, 54043195528445952.0f), 54043195528445952.0f);   // 1.5 * 2^55
    const float r = __fsub_rn(f, f2);                                                      // |r| <= 2^31
    const float f1 = __fsub_rn(__fadd_rn(r, 824633720832.0f), 824633720832.0f);           // 1.5 * 2^39
    const float r0 = __fsub_rn(r, f1);                                                     // |r0| <= 2^15
    atomicAdd(limbs + bin, fx_small_int(r0));
    atomicAdd(limbs + nb + bin, fx_small_int(__fmul_rn(f1, 1.52587890625e-05f)));          // f1 / 2^16
    atomicAdd(limbs + 2 * nb + bin, fx_small_int(__fmul_rn(f2, 2.3283064365386963e-10f))); // f2 / 2^32
}

__global__ void __launch_bounds__(256) feature_bounds_kernel(const float* __restrict__ x, const double* __restrict__ rho,
                                                             int64_t n, int d, unsigned int* __restrict__ bounds) {
    extern __shared__ unsigned int smax[];   // d + 1
    for (int k = threadIdx.x; k <= d; k += blockDim.x) smax[k] = 0u;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float r = rho ? (float)rho[i] : 1.0f;
        if (!(r > 0.0f)) continue;
        const float* xr = x + i * d;
        bool finite = true;
        for (int k = 0; k < d; ++k) finite = finite && isfinite(xr[k]);
        if (!finite) continue;   // such a sample never has a training BMU
        for (int k = 0; k < d; ++k) {
            const float v = fabsf(r * xr[k]);
            // the float product may round down: one ulp up keeps the bound above the exact product
            atomicMax(smax + k, __float_as_uint(v) + (v > 0.0f ? 1u : 0u));
        }
        atomicMax(smax + d, __float_as_uint(r));
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= d; k += blockDim.x)
        if (smax[k]) atomicMax(bounds + k, smax[k]);
}

// The same bounds with the lanes of a warp over features (DP lanes per sample, DP a power of two >= d): the loads of a
// warp are 32 consecutive floats, each lane keeps the running maximum of its feature in a register, and shared
// memory sees one atomic per feature and warp at the end. A sample counts when all its features are finite
// (a vote over its DP lanes) and its float32 weight is positive. UNR groups are loaded before any is used.
template <int DP>
__global__ void __launch_bounds__(256) feature_bounds_lanes_kernel(const float* __restrict__ x,
                                                                   const double* __restrict__ rho, int64_t n, int d,
                                                                   unsigned int* __restrict__ bounds) {
    __shared__ unsigned int smax[33];
    for (int k = threadIdx.x; k <= d; k += blockDim.x) smax[k] = 0u;
    __syncthreads();
    constexpr int SPW = 32 / DP;
    constexpr int UNR = 4;
    const int lane = threadIdx.x & 31, slot = lane / DP, k = lane % DP;
    const bool kval = k < d;
    const uint32_t slot_mask = DP == 32 ? 0xffffffffu : (((1u << DP) - 1u) << (slot * DP));
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned int mx = 0u, mr = 0u;
    for (int64_t base = gw * SPW * UNR; base < n; base += nw * SPW * UNR) {
        float v[UNR], r[UNR];
#pragma unroll
        for (int t = 0; t < UNR; ++t) {
            const int64_t i = base + t * SPW + slot;
            v[t] = (i < n && kval) ? __ldg(x + i * d + k) : 0.0f;
            r[t] = i < n ? (rho ? (float)__ldg(rho + i) : 1.0f) : 0.0f;
        }
#pragma unroll
        for (int t = 0; t < UNR; ++t) {
            const bool bad = __ballot_sync(0xffffffffu, !isfinite(v[t])) & slot_mask;
            if (!bad && r[t] > 0.0f) {
                const float av = fabsf(r[t] * v[t]);
                // the float product may round down: one ulp up keeps the bound above the exact product
                mx = max(mx, __float_as_uint(av) + (av > 0.0f ? 1u : 0u));
                mr = max(mr, __float_as_uint(r[t]));
            }
        }
    }
#pragma unroll
    for (int o = DP; o < 32; o <<= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mr = max(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    }
    if (lane < DP && kval && mx) atomicMax(smax + k, mx);
    if (lane == 0 && mr) atomicMax(smax + d, mr);
    __syncthreads();
    for (int q = threadIdx.x; q <= d; q += blockDim.x)
        if (smax[q]) atomicMax(bounds + q, smax[q]);
}

// DT > 0: the feature count known at compile time (rows loaded as float4); DT == 0: any d.
template <int DT>
__global__ void __launch_bounds__(1024) accumulate_kernel(const float* __restrict__ x, const double* __restrict__ rho,
                                                          const int32_t* __restrict__ bmu, int64_t n, int d_rt,
                                                          int64_t units_per_range, int64_t m, int64_t chunk,
                                                          const float* __restrict__ bounds, double* __restrict__ S,
                                                          double* __restrict__ c) {
    extern __shared__ int32_t limbs[];   // [3][cnt * (d + 1)]
    __shared__ float scale_s[65];
    __shared__ int exp_s[65];
    const int d = DT > 0 ? DT : d_rt;
    const int64_t lo = (int64_t)blockIdx.y * units_per_range;
    const int64_t cnt = min64(units_per_range, m - lo);
    const int stride = d + 1;
    const int64_t nb = cnt * stride;
    for (int64_t q = threadIdx.x; q < 3 * nb; q += blockDim.x) limbs[q] = 0;
    for (int k = threadIdx.x; k <= d; k += blockDim.x) {
        const int e = fx_exponent(bounds[k]);
        exp_s[k] = e;
        scale_s[k] = ldexpf(1.0f, FX_BITS - e);
    }
    __syncthreads();
    const int64_t s0 = (int64_t)blockIdx.x * chunk;
    const int64_t s1 = min64(n, s0 + chunk);
    for (int64_t w0 = s0; w0 < s1; w0 += FX_WINDOW) {
        const int64_t w1 = min64(s1, w0 + FX_WINDOW);
        for (int64_t i = w0 + threadIdx.x; i < w1; i += blockDim.x) {
            const int32_t b = __ldg(bmu + i);
            if (b < lo || b >= lo + cnt) continue;   // also skips b == -1
            const float r = rho ? (float)__ldg(rho + i) : 1.0f;  // float32 training density (som_batch.py:312)
            const int64_t bin = (b - lo) * stride;
            const float* xr = x + i * d;
            if constexpr (DT > 0) {
                float xv[DT];
                const float4* x4 = (const float4*)xr;
#pragma unroll
                for (int k4 = 0; k4 < DT / 4; ++k4) {
                    const float4 t = __ldg(x4 + k4);
                    xv[4 * k4] = t.x; xv[4 * k4 + 1] = t.y; xv[4 * k4 + 2] = t.z; xv[4 * k4 + 3] = t.w;
                }
                if (r == 1.0f) {
#pragma unroll
                    for (int k = 0; k < DT; ++k) fx_add_float(limbs, nb, bin + k, xv[k] * scale_s[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < DT; ++k) {
                        const float hi = r * xv[k];
                        const float lo_ = fmaf(r, xv[k], -hi);   // r * x exactly as hi + lo
                        fx_add(limbs, nb, bin + k, __float2ll_rn(hi * scale_s[k]) + __float2ll_rn(lo_ * scale_s[k]));
                    }
                }
            } else {
                for (int k = 0; k < d; ++k) {
                    const float xv = __ldg(xr + k);
                    const float hi = r * xv;
                    const float lo_ = fmaf(r, xv, -hi);
                    fx_add(limbs, nb, bin + k, __float2ll_rn(hi * scale_s[k]) + __float2ll_rn(lo_ * scale_s[k]));
                }
            }
            fx_add_float(limbs, nb, bin + d, r * scale_s[d]);
        }
        __syncthreads();
        for (int64_t q = threadIdx.x; q < nb; q += blockDim.x) {
            const long long v = (long long)limbs[q] + ((long long)limbs[nb + q] << 16) +
                                ((long long)limbs[2 * nb + q] << 32);
            limbs[q] = 0;
            limbs[nb + q] = 0;
            limbs[2 * nb + q] = 0;
            if (v == 0) continue;
            const int64_t u = lo + q / stride;
            const int k = (int)(q % stride);
            const double val = ldexp((double)v, exp_s[k] - FX_BITS);
            if (k < d) atomicAdd(S + u * d + k, val);
            else atomicAdd(c + u, val);
        }
        __syncthreads();
    }
}

// The same sums with the lanes of a warp spread over features: DP lanes (a power of two >= d) per sample, 32 / DP
// samples per warp instruction. The DP lanes of a sample add d contiguous words of one unit's bins, so an atomic
// instruction touches 32 / DP short runs of banks instead of 32 random banks. Unweighted samples add 1 to an
// integer count per unit; weighted ones add their float32 weight in fixed point like a feature.
// A warp takes 128 samples at a time: each lane loads four BMUs (one 16-byte load), and the samples whose BMU lies in
// this CTA's unit range are listed in shared memory (ballot prefix sums) as (offset << 16 | unit - lo). The list is
// then processed UNR groups at a time, every group's feature loads issued before any is added. With several unit
// ranges only the CTA of a sample's range reads its features, and scanning the other ranges' samples costs a few
// instructions per 128. The bins are flushed to the float64 sums once the samples added since the last flush could
// reach FX_WINDOW (the limbs' headroom): each sample adds to one unit's bins, so no bin has more adds than that.
// HOT (maps split into unit ranges): each sample slot also keeps one unit's sums in 64-bit registers (the first unit
// it meets after a flush), so that a unit winning most samples, as on the contracted maps of early epochs, does not
// serialise every warp on the same shared-memory words; those sums go to the float64 sums at each flush.
constexpr int ACC_BATCH = 128;    // samples a warp scans at once (four per lane)
constexpr int ACC_THREADS = 1024;

template <int DP, bool HOT>
__global__ void __launch_bounds__(ACC_THREADS) accumulate_lanes_kernel(const float* __restrict__ x,
                                                                       const double* __restrict__ rho,
                                                                       const int32_t* __restrict__ bmu, int64_t n,
                                                                       int d, int64_t units_per_range, int64_t m,
                                                                       int64_t chunk, int stripes,
                                                                       const float* __restrict__ bounds,
                                                                       double* __restrict__ S, double* __restrict__ c) {
    // [3][cnt * d] feature limbs, [cnt] counts or [3][cnt] weight limbs, then the warps' sample lists [32][128]
    extern __shared__ int32_t lane_bins[];
    __shared__ float scale_s[33];
    __shared__ int exp_s[33];
    __shared__ int added_s;   // samples added to the bins since the last flush
    constexpr int SPW = 32 / DP;
    constexpr int UNR = 8;
    constexpr int64_t SCAN = FX_WINDOW / 4;   // samples scanned between flush decisions
    const int64_t lo = (int64_t)blockIdx.y * units_per_range;
    const int64_t cnt = min64(units_per_range, m - lo);
    const int64_t nbf = cnt * d;
    int32_t* limbs = lane_bins;
    int32_t* csum = lane_bins + 3 * nbf;
    const int64_t nbc = rho ? 3 * cnt : cnt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint32_t* list = (uint32_t*)(lane_bins + 3 * nbf + nbc) + warp * ACC_BATCH;
    for (int64_t q = threadIdx.x; q < 3 * nbf + nbc; q += blockDim.x) lane_bins[q] = 0;
    for (int k = threadIdx.x; k <= d; k += blockDim.x) {
        const int e = fx_exponent(bounds[k]);
        exp_s[k] = e;
        scale_s[k] = ldexpf(1.0f, FX_BITS - e);
    }
    if (threadIdx.x == 0) added_s = 0;
    __syncthreads();
    const int slot = lane / DP, k = lane % DP;
    const bool kval = k < d;
    const float sk = kval ? scale_s[k] : 0.0f;
    const bool vec = ((uintptr_t)bmu & 15u) == 0u;   // chunk starts are multiples of ACC_BATCH samples
    const uint32_t lt_mask = (1u << lane) - 1u;
    int32_t hot = -1;              // HOT: this slot's register-held unit (relative to lo), -1 before the first sample
    long long hacc = 0, hw = 0;    // its feature-k sum and its count (or weight sum) in fixed point
    // CTA x takes slice x of each of the `stripes` stripes of gridDim.x * chunk samples: on rows grouped by BMU every
    // unit range then meets samples in every CTA, instead of a few CTAs holding all of a range's samples
    const int64_t span = (int64_t)gridDim.x * chunk, first = (int64_t)blockIdx.x * chunk;
    const int t_last = first < n ? (int)min64(stripes - 1, (n - 1 - first) / span) : -1;   // its last non-empty slice
    for (int t = 0; t <= t_last; ++t) {
    const bool last_stripe = t == t_last;   // the bins are flushed at the end of it
    const int64_t s0 = t * span + first;
    const int64_t s1 = min64(n, s0 + chunk);
    for (int64_t w0 = s0; w0 < s1; w0 += SCAN) {
        const int64_t w1 = min64(s1, w0 + SCAN);
        for (int64_t base = w0 + (int64_t)warp * ACC_BATCH; base < w1; base += (int64_t)nwarps * ACC_BATCH) {
            const int64_t i0 = base + 4 * lane;
            int32_t b[4];
            if (vec && i0 + 3 < w1) {
                const int4 v = __ldg((const int4*)(bmu + i0));
                b[0] = v.x; b[1] = v.y; b[2] = v.z; b[3] = v.w;
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = i0 + j < w1 ? __ldg(bmu + i0 + j) : -1;
            }
            int total = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const bool in = b[j] >= lo && b[j] < lo + cnt;   // never for b == -1
                const uint32_t mk = __ballot_sync(0xffffffffu, in);
                if (in) list[total + __popc(mk & lt_mask)] = ((uint32_t)(4 * lane + j) << 16) | (uint32_t)(b[j] - lo);
                total += __popc(mk);
            }
            __syncwarp();
            for (int p0 = 0; p0 < total; p0 += SPW * UNR) {
                uint32_t e[UNR];
                float xv[UNR];
#pragma unroll
                for (int t = 0; t < UNR; ++t) {
                    const int p = p0 + t * SPW + slot;
                    e[t] = p < total ? list[p] : 0xFFFFFFFFu;
                }
#pragma unroll
                for (int t = 0; t < UNR; ++t)
                    xv[t] = (e[t] != 0xFFFFFFFFu && kval) ? __ldg(x + (base + (e[t] >> 16)) * d + k) : 0.0f;
#pragma unroll
                for (int t = 0; t < UNR; ++t) {
                    if (e[t] == 0xFFFFFFFFu) continue;
                    const int64_t u = e[t] & 0xFFFFu;
                    if (HOT) {
                        if (hot < 0) hot = (int32_t)u;   // the slot's lanes share the sample, so the choice too
                        if (u == hot) {
                            if (!rho) {
                                if (kval) hacc += __float2ll_rn(xv[t] * sk);
                                if (k == 0) hw += 1;
                            } else {
                                const float r = (float)__ldg(rho + base + (e[t] >> 16));
                                if (kval) {
                                    const float hi = r * xv[t];
                                    const float lo_ = fmaf(r, xv[t], -hi);
                                    hacc += __float2ll_rn(hi * sk) + __float2ll_rn(lo_ * sk);
                                }
                                if (k == 0) hw += __float2ll_rn(r * scale_s[d]);
                            }
                            continue;
                        }
                    }
                    if (!rho) {
                        if (kval) fx_add_float(limbs, nbf, u * d + k, xv[t] * sk);
                        if (k == 0) atomicAdd(csum + u, 1);
                    } else {
                        const float r = (float)__ldg(rho + base + (e[t] >> 16));   // float32 density (som_batch.py:312)
                        if (kval) {
                            const float hi = r * xv[t];
                            const float lo_ = fmaf(r, xv[t], -hi);   // r * x exactly as hi + lo
                            fx_add(limbs, nbf, u * d + k, __float2ll_rn(hi * sk) + __float2ll_rn(lo_ * sk));
                        }
                        if (k == 0) fx_add_float(csum, cnt, u, r * scale_s[d]);
                    }
                }
            }
            if (lane == 0 && total) atomicAdd(&added_s, total);
            __syncwarp();   // the list is rewritten by the next batch
        }
        __syncthreads();
        const bool flush = (w1 == s1 && last_stripe) || added_s + SCAN > FX_WINDOW;
        __syncthreads();   // every thread has read added_s
        if (!flush) continue;
        if (threadIdx.x == 0) added_s = 0;
        if (HOT && hot >= 0) {
            if (kval && hacc) atomicAdd(S + (lo + hot) * d + k, ldexp((double)hacc, exp_s[k] - FX_BITS));
            if (k == 0 && hw) atomicAdd(c + lo + hot, rho ? ldexp((double)hw, exp_s[d] - FX_BITS) : (double)hw);
            hacc = 0;
            hw = 0;
            hot = -1;
        }
        for (int64_t q = threadIdx.x; q < nbf + cnt; q += blockDim.x) {
            long long v;
            int kk;
            int64_t uu;
            if (q < nbf) {
                v = (long long)limbs[q] + ((long long)limbs[nbf + q] << 16) + ((long long)limbs[2 * nbf + q] << 32);
                limbs[q] = 0;
                limbs[nbf + q] = 0;
                limbs[2 * nbf + q] = 0;
                uu = q / d;
                kk = (int)(q % d);
            } else {
                const int64_t qc = q - nbf;
                if (!rho) {
                    v = csum[qc];
                    csum[qc] = 0;
                } else {
                    v = (long long)csum[qc] + ((long long)csum[cnt + qc] << 16) + ((long long)csum[2 * cnt + qc] << 32);
                    csum[qc] = 0;
                    csum[cnt + qc] = 0;
                    csum[2 * cnt + qc] = 0;
                }
                uu = qc;
                kk = d;
            }
            if (v == 0) continue;
            const double val = (kk < d || rho) ? ldexp((double)v, exp_s[kk] - FX_BITS) : (double)v;
            if (kk < d) atomicAdd(S + (lo + uu) * d + kk, val);
            else atomicAdd(c + lo + uu, val);
        }
        __syncthreads();
    }
    }
}

// Float64 maps keep float64 bins (their sums must stay float64-accurate).
__global__ void __launch_bounds__(256) accumulate_f64_kernel(const double* __restrict__ x,
                                                             const double* __restrict__ rho,
                                                             const int32_t* __restrict__ bmu, int64_t n, int d,
                                                             double* __restrict__ S, double* __restrict__ c) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = bmu[i];
        if (b < 0) continue;
        const double r = rho ? rho[i] : 1.0;
        for (int k = 0; k < d; ++k) atomicAdd(S + (int64_t)b * d + k, r * x[i * d + k]);
        atomicAdd(c + b, r);
    }
}

// ---------------------------------------------------------------------------------------------------------------------
// Neighbourhood contraction: one CTA per unit j, threads stride over the source units b with a non-empty BMU bin.
// h_jb = exp(-|t_j - t_b|^2 * inv2s2) with |t_j - t_b|^2 typed as the reference types it (float32 differences and
// squares, float64 sum), exp in float64 (algo/som_batch.py:548-556).
// ---------------------------------------------------------------------------------------------------------------------

template <typename T, int DMAX>
__global__ void __launch_bounds__(256) neighbourhood_kernel(const double* __restrict__ S, const double* __restrict__ c,
                                                            const T* __restrict__ topo, int64_t m, int d,
                                                            double inv2s2, T* __restrict__ w_out,
                                                            double* __restrict__ num_out,
                                                            double* __restrict__ den_out) {
    const int64_t j = blockIdx.x;
    double acc[DMAX + 1];
#pragma unroll
    for (int k = 0; k <= DMAX; ++k) acc[k] = 0.0;
    for (int64_t b = threadIdx.x; b < m; b += blockDim.x) {
        const double cb = c[b];
        if (cb == 0.0) continue;
        const double h = exp(-topo_sqdist(topo, j, b) * inv2s2);
        const double* Sb = S + b * d;
#pragma unroll
        for (int k = 0; k < DMAX; ++k)
            if (k < d) acc[k] = fma(h, Sb[k], acc[k]);
        acc[DMAX] = fma(h, cb, acc[DMAX]);
    }
    __shared__ double red[DMAX + 1][8];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k <= DMAX; ++k) {
        if (k < d || k == DMAX) {
            double v = acc[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[k][wid] = v;
        }
    }
    __syncthreads();
    __shared__ double den_s;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[DMAX][q];
        den_s = s;
        if (den_out) den_out[j] = s;
    }
    __syncthreads();
    const double den = den_s;
    for (int k = threadIdx.x; k < d; k += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[k][q];
        if (num_out) num_out[j * d + k] = s;
        w_out[j * d + k] = den > FLOAT_EPS ? (T)(s / den) : (T)0;
    }
}

// Large D: the per-thread accumulators live in shared memory.
template <typename T>
__global__ void __launch_bounds__(128) neighbourhood_wide_kernel(const double* __restrict__ S,
                                                                 const double* __restrict__ c,
                                                                 const T* __restrict__ topo, int64_t m, int d,
                                                                 double inv2s2, T* __restrict__ w_out,
                                                                 double* __restrict__ num_out,
                                                                 double* __restrict__ den_out) {
    extern __shared__ double hs[];   // blockDim.x factors
    __shared__ double den_s;
    const int64_t j = blockIdx.x;
    double den_part = 0.0;
    // pass 1: den
    for (int64_t b = threadIdx.x; b < m; b += blockDim.x) {
        const double cb = c[b];
        if (cb != 0.0) den_part = fma(exp(-topo_sqdist(topo, j, b) * inv2s2), cb, den_part);
    }
    for (int o = 16; o > 0; o >>= 1) den_part += __shfl_xor_sync(0xffffffffu, den_part, o);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = den_part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
        den_s = s;
        if (den_out) den_out[j] = s;
    }
    __syncthreads();
    const double den = den_s;
    // pass 2: every thread owns features k = tid, tid + blockDim, ...; factors are staged per block of units
    for (int k0 = 0; k0 < d; k0 += blockDim.x) {
        const int k = k0 + threadIdx.x;
        double acc = 0.0;
        for (int64_t b0 = 0; b0 < m; b0 += blockDim.x) {
            __syncthreads();
            const int64_t b = b0 + threadIdx.x;
            hs[threadIdx.x] = (b < m && c[b] != 0.0) ? exp(-topo_sqdist(topo, j, b) * inv2s2) : 0.0;
            __syncthreads();
            const int64_t nb = min64(blockDim.x, m - b0);
            if (k < d)
                for (int64_t q = 0; q < nb; ++q) acc = fma(hs[q], S[(b0 + q) * d + k], acc);
        }
        if (k < d) {
            if (num_out) num_out[j * d + k] = acc;
            w_out[j * d + k] = den > FLOAT_EPS ? (T)(acc / den) : (T)0;
        }
    }
}

// ---------------------------------------------------------------------------------------------------------------------
// Iteration mode (algo/som_batch.py:154-210): every sample has its own radius, so the update does not factor through
// per-BMU sums. CTA (unit tile, sample chunk): each thread owns one unit and accumulates over the chunk; samples are
// staged in shared memory.
// ---------------------------------------------------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(128) iter_kernel(const T* __restrict__ x, const double* __restrict__ rho,
                                                   const int32_t* __restrict__ bmu, int64_t n, int d,
                                                   const T* __restrict__ topo, int64_t m, double sigma0,
                                                   int64_t cur_vector, int64_t n_vectors, int64_t chunk,
                                                   double* __restrict__ num, double* __restrict__ den) {
    constexpr int SB = 32;                       // samples staged per round
    extern __shared__ double sm[];               // SB x d samples, then SB factors info
    double* xs = sm;
    double* inv_s = sm + SB * d;
    double* r_s = inv_s + SB;
    int* b_s = (int*)(r_s + SB);
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s0 = (int64_t)blockIdx.y * chunk;
    const int64_t s1 = min64(n, s0 + chunk);
    double dacc = 0.0;
    // per-thread numerator partials are kept in global memory order: one pass per feature block of 8
    for (int k0 = 0; k0 < d; k0 += 8) {
        double acc[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = 0.0;
        for (int64_t i0 = s0; i0 < s1; i0 += SB) {
            __syncthreads();
            const int nb = (int)min64(SB, s1 - i0);
            for (int q = threadIdx.x; q < nb * d; q += blockDim.x) xs[q] = (double)x[i0 * d + q];
            for (int q = threadIdx.x; q < nb; q += blockDim.x) {
                const int64_t i = i0 + q;
                double r = rho ? rho[i] : 1.0;
                if (sizeof(T) == 4) r = (double)(float)r;
                // sigma_i = sigma0 * 1/(1 + 2 (cur + i)/n_vectors), clamped (som_batch.py:167-170)
                double sg = sigma0 * (1.0 / (1.0 + 2.0 * (double)(cur_vector + i) / (double)n_vectors));
                if (sg < FLOAT_EPS) sg = FLOAT_EPS;
                inv_s[q] = 1.0 / (2.0 * sg * sg);
                r_s[q] = r;
                b_s[q] = bmu[i];
            }
            __syncthreads();
            if (j < m) {
                for (int q = 0; q < nb; ++q) {
                    const int b = b_s[q];
                    if (b < 0) continue;
                    const double h = r_s[q] * exp(-topo_sqdist(topo, j, (int64_t)b) * inv_s[q]);
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk)
                        if (k0 + kk < d) acc[kk] = fma(h, xs[q * d + k0 + kk], acc[kk]);
                    if (k0 == 0) dacc += h;
                }
            }
        }
        if (j < m) {
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                if (k0 + kk < d && acc[kk] != 0.0) atomicAdd(num + j * d + k0 + kk, acc[kk]);
        }
    }
    if (j < m && dacc != 0.0) atomicAdd(den + j, dacc);
}

// Iteration mode on the reference's square and hexagonal grids, in float32 with the grid factorisation. Unit
// u = i * cols + j has x depending on (i, j mod 2) and y on j, so with b the sample's BMU
//   h_u = rho exp(-|t_u - t_b|^2 / (2 sigma_i^2)) = rho Ex[i, j mod 2] Ey[j],
// Ex = exp(-dx^2 / (2 sigma_i^2)) over the 2 * rows (row, parity) pairs and Ey over the cols columns, dx and dy the
// float32 differences (the reference's typing of the topographic distance). Per staged batch of IG_SB samples a CTA
// computes the tables (expf, within a few ulp of the float64 factor the reference casts to float32 for its atomics),
// then each thread adds h * x for its units in float32 and folds the partial sums of every IG_FOLD batches into
// compensated float32 accumulators in shared memory (no float64 arithmetic in the loop); at the end of its sample
// chunk the CTA adds them to num, den (float64 atomics). Work: N * M * (D+1) float32 FMAs and N * (2 rows + cols)
// exponentials per unit tile.
constexpr int IG_SB = 32;
constexpr int IG_FOLD = 2;   // batches summed in float32 before each compensated fold (64 samples)
constexpr int IG_THREADS = 128;
template <int DMAX, int UPT>
__global__ void __launch_bounds__(IG_THREADS) iter_grid_kernel(const float* __restrict__ x,
                                                               const double* __restrict__ rho,
                                                               const int32_t* __restrict__ bmu, int64_t n, int d,
                                                               const float* __restrict__ topo, int64_t rows,
                                                               int64_t cols, double sigma0, int64_t cur_vector,
                                                               int64_t n_vectors, int64_t chunk,
                                                               double* __restrict__ num, double* __restrict__ den) {
    extern __shared__ double ig_sm[];
    const int64_t m = rows * cols;
    const int ntab = (int)(2 * rows + cols);
    constexpr int UPB = IG_THREADS * UPT;                 // units of this CTA's tile
    float2* sacc = (float2*)ig_sm;                        // [UPB][d + 1] compensated float32 sums (sum, error)
    float* xs = (float*)(sacc + (size_t)UPB * (d + 1));   // [IG_SB][d]
    float* tab = xs + IG_SB * d;                          // [IG_SB][2 rows + cols]: Ex then rho * Ey
    __shared__ float inv_s[IG_SB], rho_s[IG_SB], bx_s[IG_SB], by_s[IG_SB];   // per staged sample
    __shared__ int valid_s[IG_SB];
    const int64_t u0 = (int64_t)blockIdx.x * UPB;
    for (int q = threadIdx.x; q < UPB * (d + 1); q += IG_THREADS) sacc[q] = make_float2(0.0f, 0.0f);
    int tx_i[UPT], tx_j[UPT];
    bool live[UPT];
#pragma unroll
    for (int t = 0; t < UPT; ++t) {
        const int64_t u = u0 + t * IG_THREADS + threadIdx.x;
        live[t] = u < m;
        tx_i[t] = live[t] ? (int)(2 * (u / cols) + ((u % cols) & 1)) : 0;   // Ex column: (row, parity)
        tx_j[t] = live[t] ? (int)(2 * rows + u % cols) : 0;                // Ey column
    }
    const int64_t s0 = (int64_t)blockIdx.y * chunk;
    const int64_t s1 = min64(n, s0 + chunk);
    float acc[UPT][DMAX];   // float32 sums of IG_FOLD batches, then folded into float64
    float hacc[UPT];
#pragma unroll
    for (int t = 0; t < UPT; ++t) {
        hacc[t] = 0.0f;
#pragma unroll
        for (int k = 0; k < DMAX; ++k) acc[t][k] = 0.0f;
    }
    int batch = 0;
    for (int64_t i0 = s0; i0 < s1; i0 += IG_SB, ++batch) {
        const int nb = (int)min64(IG_SB, s1 - i0);
        __syncthreads();   // the previous batch's tables and samples are no longer read
        for (int q = threadIdx.x; q < nb * d; q += IG_THREADS) xs[q] = __ldg(x + i0 * d + q);
        if (threadIdx.x < nb) {
            const int64_t i = i0 + threadIdx.x;
            const int32_t b = __ldg(bmu + i);
            // sigma_i = sigma0 / (1 + 2 (cur + i) / n_vectors), clamped (som_batch.py:167-170); 1 / (2 sigma_i^2)
            double sg = sigma0 * (1.0 / (1.0 + 2.0 * (double)(cur_vector + i) / (double)n_vectors));
            if (sg < FLOAT_EPS) sg = FLOAT_EPS;
            inv_s[threadIdx.x] = (float)(1.0 / (2.0 * sg * sg));
            rho_s[threadIdx.x] = rho ? (float)__ldg(rho + i) : 1.0f;   // float32 training density
            valid_s[threadIdx.x] = b >= 0;
            bx_s[threadIdx.x] = b >= 0 ? topo[2 * (int64_t)b] : 0.0f;
            by_s[threadIdx.x] = b >= 0 ? topo[2 * (int64_t)b + 1] : 0.0f;
        }
        __syncthreads();
        for (int sidx = 0; sidx < nb; ++sidx) {
            const bool ok = valid_s[sidx] != 0;
            const float inv = inv_s[sidx], bx = bx_s[sidx], by = by_s[sidx], rr = rho_s[sidx];
            float* t = tab + sidx * ntab;
            for (int r = threadIdx.x; r < ntab; r += IG_THREADS) {
                float v = 0.0f;
                if (ok) {
                    // exp(-dx^2 / (2 sigma^2)) in float32: within a few ulp of the float64 factor where it is above
                    // 2^-24 of the BMU's own (|exponent| < 17), negligibly small beyond
                    if (r < 2 * rows) {
                        const int64_t ua = (r >> 1) * cols + ((r & 1) < cols ? (r & 1) : 0);
                        const float dx = __fsub_rn(topo[2 * ua], bx);
                        v = expf(-__fmul_rn(dx, dx) * inv);
                    } else {
                        const float dy = __fsub_rn(topo[2 * (r - 2 * rows) + 1], by);
                        v = rr * expf(-__fmul_rn(dy, dy) * inv);
                    }
                }
                t[r] = v;
            }
        }
        __syncthreads();
        for (int sidx = 0; sidx < nb; ++sidx) {
            const float* tb = tab + sidx * ntab;
            const float* xr = xs + sidx * d;
            // a sample without a training BMU (non-finite features or weight <= 0) adds nothing: its factors are 0 and
            // its features are read as 0, so that 0 * NaN cannot reach the sums
            const bool ok = valid_s[sidx] != 0;
            float xv[DMAX];
#pragma unroll
            for (int k = 0; k < DMAX; ++k) xv[k] = (k < d && ok) ? xr[k] : 0.0f;
#pragma unroll
            for (int t = 0; t < UPT; ++t) {
                const float h = tb[tx_i[t]] * tb[tx_j[t]];
                hacc[t] += h;
#pragma unroll
                for (int k = 0; k < DMAX; ++k) acc[t][k] = fmaf(h, xv[k], acc[t][k]);
            }
        }
        if ((batch + 1) % IG_FOLD == 0 || i0 + IG_SB >= s1) {
            // compensated (Kahan) float32 accumulation: the running error stays at float32 rounding of the total
            auto kahan = [](float2& a, float v) {
                const float y = __fsub_rn(v, a.y);
                const float t2 = __fadd_rn(a.x, y);
                a.y = __fsub_rn(__fsub_rn(t2, a.x), y);
                a.x = t2;
            };
#pragma unroll
            for (int t = 0; t < UPT; ++t) {
                float2* sa = sacc + (size_t)(t * IG_THREADS + threadIdx.x) * (d + 1);
#pragma unroll
                for (int k = 0; k < DMAX; ++k)
                    if (k < d) kahan(sa[k], acc[t][k]);
                kahan(sa[d], hacc[t]);
                hacc[t] = 0.0f;
#pragma unroll
                for (int k = 0; k < DMAX; ++k) acc[t][k] = 0.0f;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < UPT; ++t) {
        const int64_t u = u0 + t * IG_THREADS + threadIdx.x;
        if (!live[t]) continue;
        const float2* sa = sacc + (size_t)(t * IG_THREADS + threadIdx.x) * (d + 1);
        for (int k = 0; k < d; ++k) {
            const double v = (double)sa[k].x - (double)sa[k].y;
            if (v != 0.0) atomicAdd(num + u * d + k, v);
        }
        const double v = (double)sa[d].x - (double)sa[d].y;
        if (v != 0.0) atomicAdd(den + u, v);
    }
}

template <typename T>
__global__ void divide_kernel(const double* __restrict__ num, const double* __restrict__ den, int64_t m, int d,
                              T* __restrict__ w_out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m * d) return;
    const double dn = den[q / d];
    w_out[q] = dn > FLOAT_EPS ? (T)(num[q] / dn) : (T)0;
}

}  // namespace

// Both activation maps of a footprint from its BMUs (the fused form of two get_activation_map calls,
// decontamination_som.py:640-641): hist_w[b_i] += rho_i for rho_i > 0, hist_c[b_i] += 1 for every sample. Per-CTA
// bins in shared memory when the map fits (float64 shared atomics), flushed with one global atomic per non-zero bin.
constexpr int HIST_THREADS = 1024;
constexpr int64_t HIST_SMEM_UNITS = 6144;   // 2 x 6144 float64 bins = 96 KB

__global__ void __launch_bounds__(HIST_THREADS) bmu_histograms_kernel(const int32_t* __restrict__ bmu,
                                                                      const double* __restrict__ rho, int64_t n,
                                                                      int64_t m, double* __restrict__ hist_w,
                                                                      double* __restrict__ hist_c) {
    extern __shared__ double hbins[];   // [2][m] when m <= HIST_SMEM_UNITS
    const bool local = m <= HIST_SMEM_UNITS;
    double* hw = local ? hbins : hist_w;
    double* hc = local ? hbins + m : hist_c;
    if (local) {
        for (int64_t q = threadIdx.x; q < 2 * m; q += blockDim.x) hbins[q] = 0.0;
        __syncthreads();
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = __ldg(bmu + i);
        if (b < 0 || b >= m) continue;
        if (hist_c) atomicAdd(hc + b, 1.0);
        if (hist_w) {
            const double r = rho ? __ldg(rho + i) : 1.0;
            if (r > 0.0) atomicAdd(hw + b, r);
        }
    }
    if (local) {
        __syncthreads();
        for (int64_t q = threadIdx.x; q < m; q += blockDim.x) {
            if (hist_w && hbins[q] != 0.0) atomicAdd(hist_w + q, hbins[q]);
            if (hist_c && hbins[m + q] != 0.0) atomicAdd(hist_c + q, hbins[m + q]);
        }
    }
}

int launch_bmu_histograms(const int32_t* bmu, const double* rho, int64_t n, int64_t m, double* hist_w, double* hist_c,
                          cudaStream_t stream) {
    if (n == 0 || m == 0) return SOMGB_OK;
    const bool local = m <= HIST_SMEM_UNITS;
    const size_t smem = local ? (size_t)(2 * m) * sizeof(double) : 0;
    if (smem > 48 * 1024)
        SOMGB_CUDA_TRY(cudaFuncSetAttribute(bmu_histograms_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
    const int64_t blocks = std::min<int64_t>(ceil_div(n, HIST_THREADS), (int64_t)num_sms());
    bmu_histograms_kernel<<<(unsigned)blocks, HIST_THREADS, smem, stream>>>(bmu, rho, n, m, hist_w, hist_c);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

int launch_feature_bounds(const float* x, const double* rho, int64_t n, int d, float* bounds, cudaStream_t stream) {
    if (n == 0) return SOMGB_OK;
    if (d <= 32) {
        auto kern = feature_bounds_lanes_kernel<32>;
        if (d <= 4) kern = feature_bounds_lanes_kernel<4>;
        else if (d <= 8) kern = feature_bounds_lanes_kernel<8>;
        else if (d <= 16) kern = feature_bounds_lanes_kernel<16>;
        const int dp = d <= 4 ? 4 : d <= 8 ? 8 : d <= 16 ? 16 : 32;
        const int64_t per_block = (int64_t)(256 / 32) * (32 / dp) * 4;   // samples per block and step
        const int64_t blocks = std::min<int64_t>(ceil_div(n, per_block), 8 * (int64_t)num_sms());
        kern<<<(unsigned)blocks, 256, 0, stream>>>(x, rho, n, d, (unsigned int*)bounds);
        SOMGB_LAUNCH_CHECK();
        return SOMGB_OK;
    }
    const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), 4 * (int64_t)num_sms());
    feature_bounds_kernel<<<(unsigned)blocks, 256, (size_t)(d + 1) * 4, stream>>>(x, rho, n, d, (unsigned int*)bounds);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

template <typename T>
int launch_accumulate(const T* x, const double* rho, const int32_t* bmu, int64_t n, int d, int64_t m,
                      const float* bounds, double* S, double* c, cudaStream_t stream) {
    if (n == 0 || m == 0) return SOMGB_OK;
    if (sizeof(T) == 8) {
        accumulate_f64_kernel<<<(unsigned)(4 * num_sms()), 256, 0, stream>>>((const double*)x, rho, bmu, n, d, S, c);
        SOMGB_LAUNCH_CHECK();
        return SOMGB_OK;
    }
    if (d > 64) return set_error(SOMGB_ERR_UNSUPPORTED, "fixed-point segmented sums support D <= 64");
    // three int32 limbs per bin; up to ~204 KB of bins per CTA (beside the warps' sample lists), so that a 32x32 map
    // with D = 16 fits one CTA and every sample is read once
    const bool lanes = d <= 32;
    const size_t lists = lanes ? (size_t)(ACC_THREADS / 32) * ACC_BATCH * 4 : 0;
    const size_t budget = 220 * 1024 - lists;
    const int64_t per_unit = lanes ? (int64_t)d * 12 + (rho ? 12 : 4) : (int64_t)(d + 1) * 12;
    int64_t upr = std::max<int64_t>(1, (int64_t)(budget / per_unit));
    upr = std::min(upr, m);
    const int64_t ranges = ceil_div(m, upr);
    upr = ceil_div(m, ranges);
    const size_t smem = (size_t)(upr * per_unit) + lists;
    const int64_t ctas_per_sm = smem <= 100 * 1024 ? 2 : 1;
    const int64_t ctas_wanted = ctas_per_sm * (int64_t)num_sms();
    // Every unit range gets as many sample chunks as one wave has CTAs: a range that wins most samples (a contracted
    // early map) is then spread over the whole GPU, and the block scheduler balances the ranges' unequal work.
    int64_t chunks = std::max<int64_t>(1, ctas_wanted);
    int64_t chunk = std::max<int64_t>(4096, ceil_div(n, chunks));
    chunk = ceil_div(chunk, ACC_BATCH) * ACC_BATCH;
    chunks = ceil_div(n, chunk);
    // with several unit ranges, each CTA's samples come from `ranges` stripes of the dataset (slices of chunk / ranges
    // samples, multiples of ACC_BATCH), so that rows grouped by BMU still give every range CTA a share
    int stripes = 1;
    if (ranges > 1 && chunk >= ranges * (int64_t)ACC_BATCH) {
        stripes = (int)ranges;
        chunk = ceil_div(ceil_div(n, chunks * stripes), ACC_BATCH) * ACC_BATCH;
    }
    const dim3 grid((unsigned)chunks, (unsigned)ranges);
    if (lanes) {
        const bool hot = ranges > 1;
        auto kern = hot ? accumulate_lanes_kernel<32, true> : accumulate_lanes_kernel<32, false>;
        if (d <= 4) kern = hot ? accumulate_lanes_kernel<4, true> : accumulate_lanes_kernel<4, false>;
        else if (d <= 8) kern = hot ? accumulate_lanes_kernel<8, true> : accumulate_lanes_kernel<8, false>;
        else if (d <= 16) kern = hot ? accumulate_lanes_kernel<16, true> : accumulate_lanes_kernel<16, false>;
        if (smem > 48 * 1024)
            SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, ACC_THREADS, smem, stream>>>((const float*)x, rho, bmu, n, d, upr, m, chunk, stripes, bounds, S,
                                                  c);
        SOMGB_LAUNCH_CHECK();
        return SOMGB_OK;
    }
    auto kern = accumulate_kernel<0>;
    if (smem > 48 * 1024)
        SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, 1024, smem, stream>>>((const float*)x, rho, bmu, n, d, upr, m, chunk, bounds, S, c);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

// ---------------------------------------------------------------------------------------------------------------------
// Neighbourhood contraction on a grid topography, by separation. On the reference's square and hexagonal grids the
// x coordinate of unit (i, j) (unit i*cols + j) depends only on (i, j mod 2) and the y coordinate only on j, so
//   h = exp(-(dx^2 + dy^2) / (2 sigma^2)) = exp(-dx^2 / (2 sigma^2)) * exp(-dy^2 / (2 sigma^2))
// (dx^2, dy^2 the float32 squares of the float32 differences, as the reference types them) and num = H S becomes two
// one-dimensional contractions: T[i, j', p] = sum_i' Ex[(i, p), (i', j' mod 2)] S[i', j'] for the two parities p of
// the output column, then num[i, j] = sum_j' Ey[j, j'] T[i, j', j mod 2]: rows*cols*(rows + cols) terms instead of
// (rows*cols)^2, and (2 rows)^2 + cols^2 exponentials. Same float64 arithmetic per term; h differs from the exponential
// of the sum by a few float64 ulps.
// ---------------------------------------------------------------------------------------------------------------------

template <typename T>
__global__ void grid_tables_kernel(const T* __restrict__ topo, int64_t rows, int64_t cols, double inv2s2,
                                   double* __restrict__ ex, double* __restrict__ ey) {
    const int64_t nx = 2 * rows, total = nx * nx + cols * cols;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        if (q < nx * nx) {
            const int64_t a = q / nx, b = q % nx;   // (i, p) and (i', p')
            const int64_t ua = (a >> 1) * cols + ((a & 1) < cols ? (a & 1) : 0);
            const int64_t ub = (b >> 1) * cols + ((b & 1) < cols ? (b & 1) : 0);
            const T dx = topo[2 * ua] - topo[2 * ub];
            ex[q] = exp(-(double)(dx * dx) * inv2s2);
        } else {
            const int64_t r = q - nx * nx, j = r / cols, jp = r % cols;
            const T dy = topo[2 * j + 1] - topo[2 * jp + 1];
            ey[r] = exp(-(double)(dy * dy) * inv2s2);
        }
    }
}

// tmp[((i * cols + j') * 2 + p) * (d + 1) + k] = sum_i' ex[(2i + p) * 2 rows + 2i' + j' mod 2] * S_k[i' * cols + j']
// (feature k = d: the count c)
__global__ void grid_step1_kernel(const double* __restrict__ S, const double* __restrict__ c, int64_t rows,
                                  int64_t cols, int d, const double* __restrict__ ex, double* __restrict__ tmp) {
    const int64_t total = rows * cols * 2 * (d + 1);
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % (d + 1));
        const int64_t r = q / (d + 1);
        const int p = (int)(r & 1);
        const int64_t jp = (r >> 1) % cols, i = (r >> 1) / cols;
        const double* erow = ex + (2 * i + p) * (2 * rows) + (jp & 1);
        double acc = 0.0;
        for (int64_t ip = 0; ip < rows; ++ip) {
            const int64_t u = ip * cols + jp;
            acc = fma(erow[2 * ip], k < d ? S[u * d + k] : c[u], acc);
        }
        tmp[q] = acc;
    }
}

// num[i * cols + j][k] = sum_j' ey[j * cols + j'] * tmp[i, j', j mod 2][k]; w_out = num / den where den > 1e-12
template <typename T>
__global__ void grid_step2_kernel(const double* __restrict__ tmp, int64_t rows, int64_t cols, int d,
                                  const double* __restrict__ ey, T* __restrict__ w_out, double* __restrict__ num_out,
                                  double* __restrict__ den_out) {
    const int64_t total = rows * cols * d;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % d);
        const int64_t u = q / d, j = u % cols, i = u / cols;
        const double* eyr = ey + j * cols;
        const double* trow = tmp + (i * cols * 2 + (j & 1)) * (d + 1);
        double num = 0.0, den = 0.0;
        for (int64_t jp = 0; jp < cols; ++jp) {
            const double* t = trow + jp * 2 * (d + 1);
            num = fma(eyr[jp], t[k], num);
            den = fma(eyr[jp], t[d], den);
        }
        if (num_out) num_out[u * d + k] = num;
        if (den_out && k == 0) den_out[u] = den;
        w_out[u * d + k] = den > FLOAT_EPS ? (T)(num / den) : (T)0;
    }
}

size_t grid_neighbourhood_workspace(int64_t rows, int64_t cols, int d) {
    return (size_t)(4 * rows * rows + cols * cols + rows * cols * 2 * (d + 1)) * sizeof(double);
}

template <typename T>
int launch_neighbourhood_grid(const double* S, const double* c, const T* topo, int64_t rows, int64_t cols, int d,
                              double sigma, T* w_out, double* num, double* den, void* ws, size_t ws_bytes,
                              cudaStream_t stream) {
    if (rows <= 0 || cols <= 0 || d <= 0) return SOMGB_OK;
    if (!ws || ws_bytes < grid_neighbourhood_workspace(rows, cols, d))
        return set_error(SOMGB_ERR_WORKSPACE, "grid neighbourhood workspace too small");
    const double inv2s2 = 1.0 / (2.0 * sigma * sigma);
    double* ex = (double*)ws;
    double* ey = ex + 4 * rows * rows;
    double* tmp = ey + cols * cols;
    const int64_t nt = 4 * rows * rows + cols * cols;
    grid_tables_kernel<T><<<(unsigned)std::min<int64_t>(ceil_div(nt, 256), 4 * (int64_t)num_sms()), 256, 0, stream>>>(
        topo, rows, cols, inv2s2, ex, ey);
    SOMGB_LAUNCH_CHECK();
    const int64_t n1 = rows * cols * 2 * (d + 1);
    grid_step1_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n1, 256), 8 * (int64_t)num_sms()), 256, 0, stream>>>(
        S, c, rows, cols, d, ex, tmp);
    SOMGB_LAUNCH_CHECK();
    const int64_t n2 = rows * cols * d;
    grid_step2_kernel<T><<<(unsigned)std::min<int64_t>(ceil_div(n2, 256), 8 * (int64_t)num_sms()), 256, 0, stream>>>(
        tmp, rows, cols, d, ey, w_out, num, den);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

template <typename T>
int launch_neighbourhood(const double* S, const double* c, const T* topo, int64_t m, int d, double sigma, T* w_out,
                         double* num, double* den, cudaStream_t stream) {
    if (m == 0) return SOMGB_OK;
    const double inv2s2 = 1.0 / (2.0 * sigma * sigma);
    if (d <= 8) {
        neighbourhood_kernel<T, 8><<<(unsigned)m, 256, 0, stream>>>(S, c, topo, m, d, inv2s2, w_out, num, den);
    } else if (d <= 16) {
        neighbourhood_kernel<T, 16><<<(unsigned)m, 256, 0, stream>>>(S, c, topo, m, d, inv2s2, w_out, num, den);
    } else if (d <= 32) {
        neighbourhood_kernel<T, 32><<<(unsigned)m, 256, 0, stream>>>(S, c, topo, m, d, inv2s2, w_out, num, den);
    } else {
        neighbourhood_wide_kernel<T><<<(unsigned)m, 128, 128 * sizeof(double), stream>>>(S, c, topo, m, d, inv2s2,
                                                                                        w_out, num, den);
    }
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

template <typename T>
int launch_iter(const T* x, const double* rho, const int32_t* bmu, int64_t n, int d, const T* topo, int64_t m,
                double sigma0, int64_t cur_vector, int64_t n_vectors, double* num, double* den,
                cudaStream_t stream) {
    if (n == 0 || m == 0) return SOMGB_OK;
    const int64_t tiles = ceil_div(m, 128);
    int64_t chunks = std::max<int64_t>(1, (2 * num_sms()) / tiles);
    int64_t chunk = std::max<int64_t>(256, ceil_div(n, chunks));
    chunks = ceil_div(n, chunk);
    const size_t smem = 32 * (size_t)d * sizeof(double) + 32 * (2 * sizeof(double) + sizeof(int));
    auto kern = iter_kernel<T>;
    if (smem > 48 * 1024) SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                              (int)smem));
    kern<<<dim3((unsigned)tiles, (unsigned)chunks), 128, smem, stream>>>(x, rho, bmu, n, d, topo, m, sigma0,
                                                                        cur_vector, n_vectors, chunk, num, den);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

template <int DMAX, int UPT>
int launch_iter_grid_d(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, const float* topo,
                       int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors, double* num,
                       double* den, cudaStream_t stream) {
    constexpr int UPB = IG_THREADS * UPT;
    const int64_t m = rows * cols;
    const int64_t tiles = ceil_div(m, UPB);
    int64_t chunks = std::max<int64_t>(1, (4 * num_sms()) / tiles);
    int64_t chunk = std::max<int64_t>(4 * IG_SB, ceil_div(n, chunks));
    chunk = ceil_div(chunk, IG_SB) * IG_SB;
    chunks = ceil_div(n, chunk);
    const size_t smem = (size_t)UPB * (d + 1) * 8 + (size_t)IG_SB * d * 4 + (size_t)IG_SB * (2 * rows + cols) * 4;
    // (the float2 sums take the 8 bytes per unit and feature that float64 ones would)
    if (smem > 200 * 1024) return set_error(SOMGB_ERR_UNSUPPORTED, "grid too large for the grid iteration pass");
    auto kern = iter_grid_kernel<DMAX, UPT>;
    SOMGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<dim3((unsigned)tiles, (unsigned)chunks), IG_THREADS, smem, stream>>>(x, rho, bmu, n, d, topo, rows, cols,
                                                                              sigma0, cur_vector, n_vectors, chunk,
                                                                              num, den);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

int launch_iter_grid(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, const float* topo,
                     int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors, double* num,
                     double* den, cudaStream_t stream) {
    if (n == 0) return SOMGB_OK;
    if (d <= 4) return launch_iter_grid_d<4, 4>(x, rho, bmu, n, d, topo, rows, cols, sigma0, cur_vector, n_vectors,
                                                num, den, stream);
    if (d <= 8) return launch_iter_grid_d<8, 4>(x, rho, bmu, n, d, topo, rows, cols, sigma0, cur_vector, n_vectors,
                                                num, den, stream);
    if (d <= 16) return launch_iter_grid_d<16, 4>(x, rho, bmu, n, d, topo, rows, cols, sigma0, cur_vector,
                                                  n_vectors, num, den, stream);
    if (d <= 32) return launch_iter_grid_d<32, 2>(x, rho, bmu, n, d, topo, rows, cols, sigma0, cur_vector,
                                                  n_vectors, num, den, stream);
    if (d <= 64) return launch_iter_grid_d<64, 1>(x, rho, bmu, n, d, topo, rows, cols, sigma0, cur_vector,
                                                  n_vectors, num, den, stream);
    return set_error(SOMGB_ERR_UNSUPPORTED, "the grid iteration pass supports D <= 64");
}

template <typename T>
int launch_divide(const double* num, const double* den, int64_t m, int d, T* w_out, cudaStream_t stream) {
    const int64_t total = m * d;
    if (total == 0) return SOMGB_OK;
    divide_kernel<T><<<(unsigned)ceil_div(total, 256), 256, 0, stream>>>(num, den, m, d, w_out);
    SOMGB_LAUNCH_CHECK();
    return SOMGB_OK;
}

template int launch_accumulate<float>(const float*, const double*, const int32_t*, int64_t, int, int64_t,
                                      const float*, double*, double*, cudaStream_t);
template int launch_accumulate<double>(const double*, const double*, const int32_t*, int64_t, int, int64_t,
                                       const float*, double*, double*, cudaStream_t);
template int launch_neighbourhood<float>(const double*, const double*, const float*, int64_t, int, double, float*,
                                         double*, double*, cudaStream_t);
template int launch_neighbourhood<double>(const double*, const double*, const double*, int64_t, int, double, double*,
                                          double*, double*, cudaStream_t);
template int launch_iter<float>(const float*, const double*, const int32_t*, int64_t, int, const float*, int64_t,
                                double, int64_t, int64_t, double*, double*, cudaStream_t);
template int launch_iter<double>(const double*, const double*, const int32_t*, int64_t, int, const double*, int64_t,
                                 double, int64_t, int64_t, double*, double*, cudaStream_t);
template int launch_neighbourhood_grid<float>(const double*, const double*, const float*, int64_t, int64_t, int, double,
                                              float*, double*, double*, void*, size_t, cudaStream_t);
template int launch_neighbourhood_grid<double>(const double*, const double*, const double*, int64_t, int64_t, int,
                                               double, double*, double*, double*, void*, size_t, cudaStream_t);
template int launch_divide<float>(const double*, const double*, int64_t, int, float*, cudaStream_t);
template int launch_divide<double>(const double*, const double*, int64_t, int, double*, cudaStream_t);

}  // namespace somgb
