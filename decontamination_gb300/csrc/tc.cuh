// K1: tensor-core (tcgen05, split-BF16) BMU search.
#pragma once

#include "pass.cuh"

namespace somgb {

// True when the tensor-core pass handles this shape on the current device for `algo`.
bool tc_supported(int64_t n, int64_t m, int d, int algo);
// Scratch bytes of the tensor-core pass (prepared unit operand, recheck list).
size_t tc_workspace_bytes(int64_t n, int64_t m, int d);
int launch_tc_pass(const PassArgs& a, void* ws, size_t ws_bytes, cudaStream_t stream);

}  // namespace somgb
