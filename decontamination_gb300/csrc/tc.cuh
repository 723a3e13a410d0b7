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

}  // namespace somgb
