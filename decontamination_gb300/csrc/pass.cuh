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

// Launches (defined in the .cu files).
// The CUDA-core pass over all samples, or over the first *count samples listed in `rows` (device memory).
int launch_k0_pass(const PassArgs& a, cudaStream_t stream, const int32_t* rows = nullptr,
                   const unsigned long long* count = nullptr);
int launch_exact_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                          const double* topo, double penalty, int outs, int32_t* bmu_out, double* hist,
                          double* err3, int32_t* train_bmu, cudaStream_t stream);

}  // namespace somgb
