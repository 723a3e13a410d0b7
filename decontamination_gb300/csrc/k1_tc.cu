// K1: tcgen05 split-BF16 BMU search (not yet enabled).
#include "tc.cuh"

namespace somgb {

bool tc_supported(int64_t, int64_t, int, int) { return false; }
size_t tc_workspace_bytes(int64_t, int64_t, int) { return 0; }
int launch_tc_pass(const PassArgs&, void*, size_t, cudaStream_t) {
    return set_error(SOMGB_ERR_UNSUPPORTED, "tensor-core pass not built");
}

}  // namespace somgb
