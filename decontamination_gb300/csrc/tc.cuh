// K1: tensor-core (tcgen05, split-FP16) BMU search.
#pragma once

#include "pass.cuh"

namespace somgb {

// True when the tensor-core pass handles this shape on the current device for `algo`.
bool tc_supported(int64_t n, int64_t m, int d, int algo);
// Shape limits of the tensor-core pass (host-only check, no device query).
bool tc_shape_ok(int64_t m, int d);
// Scratch bytes of the tensor-core pass (prepared unit operand, recheck list).
size_t tc_workspace_bytes(int64_t n, int64_t m, int d);
int launch_tc_pass(const PassArgs& a, void* ws, size_t ws_bytes, cudaStream_t stream);
// Reads (and optionally clears) the device status word that bounded waits set when they give up.
int read_device_status(unsigned int* status, bool clear, cudaStream_t stream);
// Test hook: the next tensor-core pass on this thread never loads the samples of row tile `row_tile` and bounds its
// protocol waits by `wait_limit` polls, so that a wait runs out and the pass returns with its status set.
void tc_debug_withhold(int64_t row_tile, uint32_t wait_limit);

// The sticky device status word above, as a device pointer (NULL if it cannot be resolved).
unsigned int* device_status_word();
// True on an sm_103 device (the tensor-core kernels' target).
bool device_has_tc();

// K4: the iteration-mode contraction on the tensor cores (k4_iter_tc.cu). Shape limits (host-only check): D <= 47 and
// at most 320 exponential-table rows per unit tile of the grid (512 units, 384 for D >= 32).
bool iter_tc_shape_ok(int64_t rows, int64_t cols, int d);
int iter_tc_units(int d);
int64_t iter_tc_table_rows(int64_t rows, int64_t cols, int units);
// num[u, :] += sum_i h_iu rho_i x_i, den[u] += sum_i h_iu rho_i over the samples with bmu[i] >= 0 (iteration-mode
// neighbourhood of sample cur_vector + i), `bounds` from launch_feature_bounds over the same samples.
// Test hook: the next K4 launch on this thread never signals that accumulator group `group` is complete and bounds its
// waits by `wait_limit` polls, so that the fold's wait runs out.
void iter_tc_debug_withhold(int group, uint32_t wait_limit);
int launch_iter_tc(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, const float* topo,
                   int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors,
                   const float* bounds, double* num, double* den, unsigned int* status, cudaStream_t stream);

}  // namespace somgb
