// Per-sample outputs shared by every BMU-search kernel (CUDA-core and tensor-core).
#pragma once

#include "common.cuh"

namespace somgb {

// What a BMU pass produces for each sample.
enum PassOutputs : int {
    OUT_BMU = 1,        // bmu_out[i] = b1, or 0 when no unit is valid (_find_bmu_xpu semantics)
    OUT_HIST = 2,       // hist[b1 or 0] += rho for rho > 0 (_count_bmus_kernel)
    OUT_ERR = 4,        // error sums of _compute_errors_xpu; needs the exact second BMU
    OUT_TRAIN = 8,      // train_bmu[i] = b1 when (float)rho > 0 and b1 valid, else -1 (_train_step2_xpu)
};

struct PassArgs {
    const float* x;        // n x d
    const double* rho;     // n or NULL (= 1)
    int64_t n;
    int d;
    const float* w;        // m x d
    int64_t m;
    const float* topo;     // m x 2 (OUT_ERR)
    double penalty;        // OUT_ERR
    int32_t* bmu_out;      // OUT_BMU
    double* hist;          // OUT_HIST (m)
    double* err3;          // OUT_ERR (3)
    int32_t* train_bmu;    // OUT_TRAIN (n)
    unsigned long long* recheck_count;  // optional: samples that took the exact path
    unsigned int* status;  // optional: this call's status word (bounded waits that gave up), besides the global one
    unsigned long long* sweep2_tiles;   // optional: column tiles the tensor-core pass's second sweeps computed
    int outs;
};

// Exact top-2 of one sample over a set of candidate units, in ascending unit order.
// `is_candidate(j)` screens units; the distance is the reference's (ref_sqdist).
// Consumes the sample's result and performs the per-sample outputs. Returns the error-sum contributions.
struct SampleResult {
    int32_t i1, i2;
    double d1;
};

__device__ __forceinline__ void emit_sample(const PassArgs& a, int64_t i, const SampleResult& r, double& e0,
                                            double& e1, double& e2) {
    const int outs = a.outs;
    double rho = a.rho ? a.rho[i] : 1.0;
    if (outs & OUT_BMU) a.bmu_out[i] = r.i1 < 0 ? 0 : r.i1;
    if ((outs & OUT_HIST) && rho > 0.0) atomicAdd(a.hist + (r.i1 < 0 ? 0 : r.i1), rho);
    if (outs & OUT_TRAIN) {
        float r32 = (float)rho;
        a.train_bmu[i] = (r32 > 0.0f && r.i1 >= 0) ? r.i1 : -1;
    }
    if ((outs & OUT_ERR) && rho > 0.0 && r.i1 >= 0 && r.i2 >= 0 && r.i1 != r.i2) {
        e0 += rho * sqrt(r.d1);
        if (topo_sqdist(a.topo, r.i1, r.i2) > a.penalty) e1 += rho;
        e2 += rho;
    }
}

// ---------------------------------------------------------------------------------------------------------------------
// Float32 double-float helpers: exact sums and products without the (slow on this GPU) float64 pipe.
// ---------------------------------------------------------------------------------------------------------------------

struct DFloat {
    float hi, lo;
};

// hi + lo == a + b exactly (Knuth's two-sum)
__device__ __forceinline__ DFloat two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return DFloat{s, e};
}

// running sum with a compensation term (error of the order of 2^-48 of the total)
struct DFAcc {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const DFloat t = two_sum(hi, v);
        hi = t.hi;
        lo = __fadd_rn(lo, t.lo);
    }
    __device__ __forceinline__ void add(DFloat v) {
        add(v.hi);
        lo = __fadd_rn(lo, v.lo);
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// sqrt of the double-float hi + lo (hi >= 0), to about 2^-46 relative: one Newton step on the float32 root
__device__ __forceinline__ DFloat df_sqrt(float hi, float lo) {
    if (!(hi > 0.0f)) return DFloat{0.0f, 0.0f};
    const float s = sqrtf(hi);
    const float r = __fadd_rn(fmaf(-s, s, hi), lo);
    return DFloat{s, __fdiv_rn(r, __fmul_rn(2.0f, s))};
}

// (a.hi + a.lo) * (b.hi + b.lo) to about 2^-46 relative
__device__ __forceinline__ DFloat df_mul(DFloat a, DFloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = fmaf(a.hi, b.hi, -p);
    return DFloat{p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e))};
}

// Normalised float32 pairs (|lo| <= ulp(hi) / 2) in (value, unit) order; empty entries (unit < 0) last.
__device__ __forceinline__ bool df_before(DFloat a, int32_t ja, DFloat b, int32_t jb) {
    return ja >= 0 && (jb < 0 || a.hi < b.hi || (a.hi == b.hi && (a.lo < b.lo || (a.lo == b.lo && ja < jb))));
}
// b (unit jb; absent when jb < 0) exceeds a by more than 2^-36 of b. Each pair is the compensated float32 sum of
// the D float32 squares: its low word carries at most (D-1)^2 2^-48 of the sum in rounding (2^-38 at D = 32), and the
// reference's float64 sum of the same squares is within (D-1) 2^-53 of the exact one; so pairs that far apart stand
// for float64 sums ordered the same way.
__device__ __forceinline__ bool df_apart(DFloat a, DFloat b, int32_t jb) {
    if (jb < 0) return true;
    const float gap = __fadd_rn(__fsub_rn(b.hi, a.hi), __fsub_rn(b.lo, a.lo));
    return gap > 1.4551915e-11f * b.hi;   // 2^-36
}

// The reference distance (float64 sum of the float32 squares in feature order) as a compensated float32 pair, within
// (D-1)^2 2^-48 of the sum; unnormalised (two_sum(hi, lo) normalises). wr: 16-byte aligned, DT a multiple of 4.
template <int DT>
__device__ __forceinline__ DFloat ref_dist_pair(const float* __restrict__ wr, const float (&xr)[DT]) {
    DFAcc acc;
    const float4* w4 = (const float4*)wr;
#pragma unroll
    for (int k4 = 0; k4 < DT / 4; ++k4) {
        const float4 w = w4[k4];
        const float t0 = __fsub_rn(w.x, xr[4 * k4]), t1 = __fsub_rn(w.y, xr[4 * k4 + 1]);
        const float t2 = __fsub_rn(w.z, xr[4 * k4 + 2]), t3 = __fsub_rn(w.w, xr[4 * k4 + 3]);
        acc.add(__fmul_rn(t0, t0));
        acc.add(__fmul_rn(t1, t1));
        acc.add(__fmul_rn(t2, t2));
        acc.add(__fmul_rn(t3, t3));
    }
    return DFloat{acc.hi, acc.lo};
}

// Is the reference's float64 sum of the float32 squares of the float32 topographic differences above `penalty`
// (exactly representable)? The two squares are summed exactly in float32 pairs. ta, tb: the two units' coordinates.
__device__ __forceinline__ bool topo_far32(float2 ta, float2 tb, float penalty) {
    const float t0 = __fsub_rn(ta.x, tb.x);
    const float t1 = __fsub_rn(ta.y, tb.y);
    const DFloat s = two_sum(__fmul_rn(t0, t0), __fmul_rn(t1, t1));
    return s.hi > penalty || (s.hi == penalty && s.lo > 0.0f);
}

// Per-sample outputs from float32 quantities; d1 is the reference distance of b1 as a double-float, r the sample's
// weight (a.rho[i], or 1 when a.rho is NULL) and t1, t2 the topographic coordinates of b1 and b2, all loaded by the
// caller.
__device__ __forceinline__ void emit_sample32(const PassArgs& a, int64_t i, double r, int32_t i1, int32_t i2, DFloat d1,
                                              float2 t1, float2 t2, DFAcc& e0, DFAcc& e1, DFAcc& e2) {
    const int outs = a.outs;
    const long long bits = __double_as_longlong(r);
    const bool pos = bits > 0 && bits <= 0x7FF0000000000000LL;   // r > 0 (NaN excluded)
    DFloat rho{1.0f, 0.0f};
    if (a.rho) {   // no float64 work for unweighted samples
        rho.hi = (float)r;
        rho.lo = (float)(r - (double)rho.hi);
    }
    if (outs & OUT_BMU) a.bmu_out[i] = i1 < 0 ? 0 : i1;
    if ((outs & OUT_HIST) && pos) atomicAdd(a.hist + (i1 < 0 ? 0 : i1), (double)rho.hi + (double)rho.lo);
    if (outs & OUT_TRAIN) a.train_bmu[i] = (rho.hi > 0.0f && i1 >= 0) ? i1 : -1;
    if ((outs & OUT_ERR) && pos && i1 >= 0 && i2 >= 0 && i1 != i2) {
        e0.add(df_mul(rho, df_sqrt(d1.hi, d1.lo)));
        if (topo_far32(t1, t2, (float)a.penalty)) e1.add(rho);
        e2.add(rho);
    }
}

// Launches (defined in the .cu files).
// The CUDA-core pass over all samples, or over the first *count samples listed in `rows` (device memory).
int launch_k0_pass(const PassArgs& a, cudaStream_t stream, const int32_t* rows = nullptr,
                   const unsigned long long* count = nullptr);
int launch_exact_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                          const double* topo, double penalty, int outs, int32_t* bmu_out, double* hist,
                          double* err3, int32_t* train_bmu, cudaStream_t stream);

}  // namespace somgb
