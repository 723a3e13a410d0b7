// Shared definitions of the somgb CUDA library (batch self-organising maps on GB300 / sm_103a).
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/somgb.h"

namespace somgb {

// Records a message for somgb_last_error() (per host thread) and returns `status`.
int set_error(int status, const char* fmt, ...);

#define SOMGB_CUDA_TRY(expr)                                                                                \
    do {                                                                                                    \
        cudaError_t _e = (expr);                                                                            \
        if (_e != cudaSuccess)                                                                              \
            return ::somgb::set_error(SOMGB_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                                      __FILE__, __LINE__);                                                  \
    } while (0)

#define SOMGB_LAUNCH_CHECK() \
    do {                     \
        ::somgb::count_launch(); \
        SOMGB_CUDA_TRY(cudaGetLastError()); \
    } while (0)

constexpr double FLOAT_EPS = 1.0e-12;   // algo/som_batch.py:24

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
inline size_t align_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

int num_sms();

// Launch bookkeeping (api.cu): the process-wide launch counter and the optional per-thread kernel timer.
void count_launch();
void timer_begin(cudaStream_t s);
void timer_end(cudaStream_t s);

// ---------------------------------------------------------------------------------------------------------------------
// Device helpers shared by the kernels.
// ---------------------------------------------------------------------------------------------------------------------

// One term of square_distance_xpu (algo/__init__.py:89-98) as the compiled reference types it for float32 operands:
// the difference and its square stay float32 (Numba types float32**int as float32) and the sum is float64 (the
// accumulator starts at the literal 0.0). The _rn intrinsics forbid contraction into an FMA.
__device__ __forceinline__ double ref_term(float a, float b) {
    float t = __fsub_rn(a, b);
    return (double)__fmul_rn(t, t);
}
__device__ __forceinline__ double ref_term(double a, double b) {
    double t = __dsub_rn(a, b);
    return __dmul_rn(t, t);
}

// Exact reference distance between two rows (sum in feature order).
template <typename T>
__device__ __forceinline__ double ref_sqdist(const T* __restrict__ a, const T* __restrict__ b, int d) {
    double acc = 0.0;
    for (int k = 0; k < d; ++k) acc = __dadd_rn(acc, ref_term(a[k], b[k]));
    return acc;
}

// Topographic distance |t_a - t_b|^2 with the same typing (topography is stored in the map's dtype).
template <typename T>
__device__ __forceinline__ double topo_sqdist(const T* __restrict__ topo, int64_t a, int64_t b) {
    double acc = 0.0;
    acc = __dadd_rn(acc, ref_term(topo[2 * a + 0], topo[2 * b + 0]));
    acc = __dadd_rn(acc, ref_term(topo[2 * a + 1], topo[2 * b + 1]));
    return acc;
}

// Exact top-2 in the reference's order: (distance, index) lexicographic, strict comparisons, NaN skipped
// (_compute_errors_xpu, algo/som_abstract.py:822-850; its first entry is also _find_bmu_xpu's argmin).
struct Top2 {
    double d1, d2;
    int32_t i1, i2;
    __device__ __forceinline__ void init() { d1 = 1.0e99; d2 = 1.0e99; i1 = -1; i2 = -1; }
    __device__ __forceinline__ void push(double d, int32_t j) {
        if (d != d) return;
        if (d1 > d) { d2 = d1; i2 = i1; d1 = d; i1 = j; }
        else if (d2 > d) { d2 = d; i2 = j; }
    }
};

// The same ranking for entries arriving in any order: (distance, index) compared lexicographically.
struct Top2Lex {
    double d1, d2;
    int32_t i1, i2;
    __device__ __forceinline__ void init() { d1 = 1.0e99; d2 = 1.0e99; i1 = -1; i2 = -1; }
    __device__ __forceinline__ static bool before(double da, int32_t ja, double db, int32_t jb) {
        return jb < 0 || da < db || (da == db && ja < jb);
    }
    __device__ __forceinline__ void push(double d, int32_t j) {
        if (d != d || !(d < 1.0e99)) return;
        if (before(d, j, d1, i1)) { d2 = d1; i2 = i1; d1 = d; i1 = j; }
        else if (before(d, j, d2, i2)) { d2 = d; i2 = j; }
    }
};

// Block-wide sum of three doubles into out[0..2] with one atomic per block and value.
__device__ __forceinline__ void block_add3(double a, double b, double c, double* out) {
    __shared__ double red[3][32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { red[0][w] = a; red[1][w] = b; red[2][w] = c; }
    __syncthreads();
    if (w == 0) {
        int nw = (blockDim.x + 31) >> 5;
        a = l < nw ? red[0][l] : 0.0;
        b = l < nw ? red[1][l] : 0.0;
        c = l < nw ? red[2][l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        if (l == 0) {
            if (a != 0.0) atomicAdd(out + 0, a);
            if (b != 0.0) atomicAdd(out + 1, b);
            if (c != 0.0) atomicAdd(out + 2, c);
        }
    }
}

}  // namespace somgb
