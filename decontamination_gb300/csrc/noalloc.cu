// BMU search that allocates nothing: somgb_find_bmus with its scratch in a fixed, file-scope device array.
//
// Some callers cannot allocate device memory when they need BMUs: a host framework that hands out a fixed
// device-memory budget up front and owns every allocation, or a C/Fortran pipeline that only passes the catalogue and
// output buffers it already owns and has no allocator to call. For them this entry point keeps its working memory in
// one static device array instead of a caller workspace. That array is part of the library's module: every GPU that
// loads libsomgb holds it from module load until the process exits.
//
// The array is shared by every call on a device. The pass rewrites everything it reads before reading it (the unit
// operand, the centre, the recheck list) and clears the recheck counter at the start of each pass, so results never
// depend on what an earlier call left there; two calls that overlap on the GPU (for example on two streams) race on it.
#include "common.cuh"

#include <algorithm>
#include <mutex>

namespace somgb {
namespace {

// Large enough for the tensor-core unit operand of any supported shape (at most ~230 KB) plus the recheck list of a
// chunk of about a million rows; inputs with more rows are processed in chunks.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(4) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of the array, per device. Only a successful lookup is cached: a failed one is retried by the next
// call, so one failure does not disable the entry point on that device for the rest of the process.
std::mutex g_addr_mutex;
void* g_addr[64] = {};

// Device address of the scratch array on the current device, looked up with that device current. The lookup is the
// first call's set-up on a device; it is refused while `stream` is being captured (the lookup is not a stream
// operation), so that first call has to come before any stream capture.
int scratch_address(cudaStream_t stream, void** out) {
    int dev = 0;
    SOMGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(SOMGB_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        SOMGB_CUDA_TRY(cudaStreamIsCapturing(stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return set_error(SOMGB_ERR_INVALID,
                             "the first somgb_find_bmus_noalloc call on device %d looks up its static scratch and must "
                             "be made outside a stream capture",
                             dev);
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();   // leave no stale error for the next launch check of another entry point
            return set_error(SOMGB_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed: %s",
                             cudaGetErrorString(e));
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return SOMGB_OK;
}

}  // namespace
}  // namespace somgb

using namespace somgb;

extern "C" {

size_t somgb_find_bmus_noalloc_scratch_bytes(void) { return NOALLOC_SCRATCH_BYTES; }

int somgb_find_bmus_noalloc(const float* x, int64_t n, int d, const float* w, int64_t m, int algo, int32_t* bmu_out,
                            somgb_stream_t stream) {
    if (n < 0 || m <= 0 || d <= 0)
        return set_error(SOMGB_ERR_INVALID, "invalid sizes n=%lld m=%lld d=%d", (long long)n, (long long)m, d);
    // the largest row chunk whose workspace fits the static array
    int64_t chunk = std::max<int64_t>(n, 1);
    while (chunk > 128 && somgb_workspace_bytes(SOMGB_OP_FIND_BMUS, chunk, m, d, algo) > NOALLOC_SCRATCH_BYTES)
        chunk = std::max<int64_t>(128, chunk / 2);
    if (somgb_workspace_bytes(SOMGB_OP_FIND_BMUS, std::min<int64_t>(chunk, std::max<int64_t>(n, 1)), m, d, algo) >
        NOALLOC_SCRATCH_BYTES)
        return set_error(SOMGB_ERR_WORKSPACE,
                         "m=%lld d=%d needs more scratch than the %zu-byte static array of somgb_find_bmus_noalloc",
                         (long long)m, d, NOALLOC_SCRATCH_BYTES);
    void* scratch = nullptr;
    if (int s = scratch_address((cudaStream_t)stream, &scratch)) return s;
    if (n == 0) return somgb_find_bmus(x, 0, d, w, m, algo, bmu_out, scratch, NOALLOC_SCRATCH_BYTES, stream);
    for (int64_t s0 = 0; s0 < n; s0 += chunk) {
        const int64_t len = std::min<int64_t>(chunk, n - s0);
        const int st = somgb_find_bmus(x + s0 * d, len, d, w, m, algo, bmu_out + s0, scratch, NOALLOC_SCRATCH_BYTES,
                                       stream);
        if (st) return st;
    }
    return SOMGB_OK;
}

}  // extern "C"
