// C ABI of libsomgb (declared in include/somgb.h): argument checks, workspace layout and kernel dispatch.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <string>

#include "pass.cuh"
#include "tc.cuh"

namespace somgb {

template <typename T>
int launch_accumulate(const T* x, const double* rho, const int32_t* bmu, int64_t n, int d, int64_t m,
                      const float* bounds, double* S, double* c, cudaStream_t stream);
int launch_feature_bounds(const float* x, const double* rho, int64_t n, int d, float* bounds, cudaStream_t stream);
template <typename T>
int launch_neighbourhood_grid(const double* S, const double* c, const T* topo, int64_t rows, int64_t cols, int d,
                              double sigma, T* w_out, double* num, double* den, void* ws, size_t ws_bytes,
                              cudaStream_t stream);
size_t grid_neighbourhood_workspace(int64_t rows, int64_t cols, int d);
size_t sort_rows_workspace(int64_t m);
int launch_iter_grid(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, const float* topo,
                     int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors, double* num,
                     double* den, cudaStream_t stream);
int launch_sort_rows(const float* x, const double* rho, const int32_t* key, int64_t n, int d, int64_t m,
                     float* x_out, double* rho_out, void* ws, size_t ws_bytes, cudaStream_t stream);
int launch_bmu_histograms(const int32_t* bmu, const double* rho, int64_t n, int64_t m, double* hist_w, double* hist_c,
                          cudaStream_t stream);
template <typename T>
int launch_neighbourhood(const double* S, const double* c, const T* topo, int64_t m, int d, double sigma, T* w_out,
                         double* num, double* den, cudaStream_t stream);
template <typename T>
int launch_iter(const T* x, const double* rho, const int32_t* bmu, int64_t n, int d, const T* topo, int64_t m,
                double sigma0, int64_t cur_vector, int64_t n_vectors, double* num, double* den, cudaStream_t stream);
template <typename T>
int launch_divide(const double* num, const double* den, int64_t m, int d, T* w_out, cudaStream_t stream);

namespace {
thread_local std::string g_last_error;
thread_local unsigned long long* g_last_counter = nullptr;
}  // namespace

std::atomic<int64_t> g_launches{0};
thread_local cudaEvent_t g_timer_start = nullptr;
thread_local cudaEvent_t g_timer_stop = nullptr;

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void timer_begin(cudaStream_t s) {
    if (g_timer_start) cudaEventRecord(g_timer_start, s);
}
void timer_end(cudaStream_t s) {
    if (g_timer_stop) cudaEventRecord(g_timer_stop, s);
}

int set_error(int status, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = v > 0 ? v : 1;
    }
    return cached[dev];
}

namespace {

// Workspace layout: [0, 256) header (u64 recheck counter at 0, u32 status word of the call at 8), then op-specific
// arrays, each 256-byte aligned.
constexpr size_t WS_HEADER = 256;

struct Workspace {
    unsigned long long* counter = nullptr;
    int32_t* train_bmu = nullptr;
    float* bounds = nullptr;
    void* tc = nullptr;
    size_t tc_bytes = 0;
};

size_t ws_bytes_for(int op, int64_t n, int64_t m, int d, int algo, bool* tc_used) {
    size_t b = WS_HEADER;
    if (op == SOMGB_OP_EPOCH) b += align_up((size_t)std::max<int64_t>(n, 1) * sizeof(int32_t), 256) + 512;
    bool tc = tc_supported(n, m, d, algo);
    if (tc_used) *tc_used = tc;
    if (tc) b += align_up(tc_workspace_bytes(n, m, d), 256);
    return b;
}

int carve(void* ws, size_t ws_bytes, int op, int64_t n, int64_t m, int d, int algo, Workspace* out, bool* tc) {
    const size_t need = ws_bytes_for(op, n, m, d, algo, tc);
    if (!ws || ws_bytes < need)
        return set_error(SOMGB_ERR_WORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes required",
                         ws ? ws_bytes : (size_t)0, need);
    if (((uintptr_t)ws) % 256)
        return set_error(SOMGB_ERR_INVALID, "workspace pointer must be 256-byte aligned");
    char* p = (char*)ws;
    out->counter = (unsigned long long*)p;
    p += WS_HEADER;
    if (op == SOMGB_OP_EPOCH) {
        out->train_bmu = (int32_t*)p;
        p += align_up((size_t)std::max<int64_t>(n, 1) * sizeof(int32_t), 256);
        out->bounds = (float*)p;
        p += 512;
    }
    if (*tc) {
        out->tc = p;
        out->tc_bytes = align_up(tc_workspace_bytes(n, m, d), 256);
    }
    g_last_counter = out->counter;
    return SOMGB_OK;
}

int check_common(const void* x, int64_t n, int d, const void* w, int64_t m, int algo) {
    if (n < 0 || m <= 0 || d <= 0)
        return set_error(SOMGB_ERR_INVALID, "invalid sizes n=%lld m=%lld d=%d", (long long)n, (long long)m, d);
    if (n > 0 && !x) return set_error(SOMGB_ERR_INVALID, "x is NULL");
    if (!w) return set_error(SOMGB_ERR_INVALID, "w is NULL");
    if (m > INT32_MAX) return set_error(SOMGB_ERR_INVALID, "m=%lld exceeds int32 BMU indices", (long long)m);
    if (algo < SOMGB_ALGO_FP32 || algo > SOMGB_ALGO_AUTO) return set_error(SOMGB_ERR_INVALID, "unknown algo %d", algo);
    if (((uintptr_t)x) % 4 || ((uintptr_t)w) % 4) return set_error(SOMGB_ERR_INVALID, "x/w must be 4-byte aligned");
    return SOMGB_OK;
}

int run_pass(PassArgs a, int algo, const Workspace& ws, bool tc, cudaStream_t stream) {
    SOMGB_CUDA_TRY(cudaMemsetAsync(ws.counter, 0, 24, stream));   // recheck counter, status word, sweep-2 tiles
    a.recheck_count = ws.counter;
    a.status = (unsigned int*)(ws.counter + 1);
    a.sweep2_tiles = ws.counter + 2;
    // the tensor-core pass reads sample and unit rows as float4 and topographic coordinates as float2
    const bool aligned = ((uintptr_t)a.x) % 16 == 0 && ((uintptr_t)a.w) % 16 == 0 &&
                         (!(a.outs & OUT_ERR) || ((uintptr_t)a.topo) % 8 == 0);
    if (tc && aligned) return launch_tc_pass(a, ws.tc, ws.tc_bytes, stream);
    if (tc && algo == SOMGB_ALGO_TC)
        return set_error(SOMGB_ERR_INVALID,
                         "the tensor-core pass needs x and w 16-byte aligned and the topography 8-byte aligned");
    if (algo == SOMGB_ALGO_TC)
        return set_error(SOMGB_ERR_UNSUPPORTED, "tensor-core path unsupported for n=%lld m=%lld d=%d on this device",
                         (long long)a.n, (long long)a.m, a.d);
    return launch_k0_pass(a, stream);
}

}  // namespace
}  // namespace somgb

using namespace somgb;

extern "C" {

int somgb_version(void) { return 100; }

size_t somgb_last_error(char* buf, size_t len) {
    const std::string& s = g_last_error;
    if (buf && len) {
        size_t k = std::min(len - 1, s.size());
        memcpy(buf, s.data(), k);
        buf[k] = 0;
    }
    return s.size();
}

size_t somgb_workspace_bytes(int op, int64_t n, int64_t m, int d, int algo) {
    return ws_bytes_for(op, n, m, d, algo, nullptr);
}

int64_t somgb_kernel_launches(void) { return g_launches.load(); }

int somgb_set_kernel_timer(void* start_event, void* stop_event) {
    g_timer_start = (cudaEvent_t)start_event;
    g_timer_stop = (cudaEvent_t)stop_event;
    return SOMGB_OK;
}

int somgb_last_recheck_count(int64_t* count, somgb_stream_t stream) {
    if (!count) return set_error(SOMGB_ERR_INVALID, "count is NULL");
    *count = 0;
    if (!g_last_counter) return SOMGB_OK;
    unsigned long long v = 0;
    SOMGB_CUDA_TRY(cudaMemcpyAsync(&v, g_last_counter, sizeof(v), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    SOMGB_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    *count = (int64_t)v;
    return SOMGB_OK;
}

int somgb_last_sweep2_tiles(int64_t* tiles, somgb_stream_t stream) {
    if (!tiles) return set_error(SOMGB_ERR_INVALID, "tiles is NULL");
    *tiles = 0;
    if (!g_last_counter) return SOMGB_OK;
    unsigned long long v = 0;
    SOMGB_CUDA_TRY(cudaMemcpyAsync(&v, g_last_counter + 2, sizeof(v), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    SOMGB_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    *tiles = (int64_t)v;
    return SOMGB_OK;
}

int somgb_device_status(unsigned int* status, int clear, somgb_stream_t stream) {
    if (!status) return set_error(SOMGB_ERR_INVALID, "status is NULL");
    if (int s = read_device_status(status, clear != 0, (cudaStream_t)stream)) return s;
    return SOMGB_OK;
}

int somgb_algo_supported(int algo, int64_t n, int64_t m, int d) {
    if (algo == SOMGB_ALGO_FP32 || algo == SOMGB_ALGO_AUTO) return 1;
    if (algo == SOMGB_ALGO_TC) return tc_supported(n, m, d, SOMGB_ALGO_TC) ? 1 : 0;
    return 0;
}

int somgb_find_bmus(const float* x, int64_t n, int d, const float* w, int64_t m, int algo, int32_t* bmu_out,
                    void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, algo)) return s;
    if (n > 0 && !bmu_out) return set_error(SOMGB_ERR_INVALID, "bmu_out is NULL");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_FIND_BMUS, n, m, d, algo, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    PassArgs a{};
    a.x = x; a.n = n; a.d = d; a.w = w; a.m = m; a.bmu_out = bmu_out; a.outs = OUT_BMU;
    return run_pass(a, algo, W, tc, (cudaStream_t)stream);
}

int somgb_count_bmus(const float* x, const double* rho, int64_t n, int d, const float* w, int64_t m, int algo,
                     double* hist, void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, algo)) return s;
    if (!hist) return set_error(SOMGB_ERR_INVALID, "hist is NULL");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_COUNT_BMUS, n, m, d, algo, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    PassArgs a{};
    a.x = x; a.rho = rho; a.n = n; a.d = d; a.w = w; a.m = m; a.hist = hist; a.outs = OUT_HIST;
    return run_pass(a, algo, W, tc, (cudaStream_t)stream);
}

int somgb_bmu_histograms(const int32_t* bmu, const double* rho, int64_t n, int64_t m, double* hist_weighted,
                         double* hist_count, somgb_stream_t stream) {
    if (n < 0 || m < 0 || (n > 0 && !bmu)) return set_error(SOMGB_ERR_INVALID, "bad BMU array");
    return launch_bmu_histograms(bmu, rho, n, m, hist_weighted, hist_count, (cudaStream_t)stream);
}

int somgb_footprint_maps(const float* x, const double* rho, int64_t n, int d, const float* w, int64_t m, int algo,
                         int32_t* bmu_out, double* hist_weighted, double* hist_count, void* ws, size_t ws_bytes,
                         somgb_stream_t stream) {
    if (n > 0 && !bmu_out) return set_error(SOMGB_ERR_INVALID, "bmu_out is NULL");
    if (int s = somgb_find_bmus(x, n, d, w, m, algo, bmu_out, ws, ws_bytes, stream)) return s;
    return launch_bmu_histograms(bmu_out, rho, n, m, hist_weighted, hist_count, (cudaStream_t)stream);
}

int somgb_footprint_maps_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                             int32_t* bmu_out, double* hist_weighted, double* hist_count, somgb_stream_t stream) {
    if (n > 0 && !bmu_out) return set_error(SOMGB_ERR_INVALID, "bmu_out is NULL");
    if (int s = somgb_find_bmus_f64(x, n, d, w, m, bmu_out, stream)) return s;
    return launch_bmu_histograms(bmu_out, rho, n, m, hist_weighted, hist_count, (cudaStream_t)stream);
}

int somgb_compute_errors(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                         int64_t m, double penalty, int algo, double* err3, void* ws, size_t ws_bytes,
                         somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, algo)) return s;
    if (!err3 || !topo) return set_error(SOMGB_ERR_INVALID, "err3/topo is NULL");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_ERRORS, n, m, d, algo, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    PassArgs a{};
    a.x = x; a.rho = rho; a.n = n; a.d = d; a.w = w; a.m = m; a.topo = topo; a.penalty = penalty; a.err3 = err3;
    a.outs = OUT_ERR;
    return run_pass(a, algo, W, tc, (cudaStream_t)stream);
}

int somgb_train_epoch_pass(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                           int64_t m, double penalty, int algo, double* S, double* c, double* err3,
                           int32_t* bmu_out, void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, algo)) return s;
    if (!S || !c) return set_error(SOMGB_ERR_INVALID, "S/c is NULL");
    if (err3 && !topo) return set_error(SOMGB_ERR_INVALID, "topo is NULL");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_EPOCH, n, m, d, algo, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    PassArgs a{};
    a.x = x; a.rho = rho; a.n = n; a.d = d; a.w = w; a.m = m; a.topo = topo; a.penalty = penalty;
    a.err3 = err3; a.train_bmu = bmu_out ? bmu_out : W.train_bmu;
    a.outs = OUT_TRAIN | (err3 ? OUT_ERR : 0);
    cudaStream_t st = (cudaStream_t)stream;
    if (d > 64) return set_error(SOMGB_ERR_UNSUPPORTED, "the float32 training pass supports D <= 64");
    if (int s = run_pass(a, algo, W, tc, st)) return s;
    SOMGB_CUDA_TRY(cudaMemsetAsync(W.bounds, 0, (size_t)(d + 1) * 4, st));
    if (int s = launch_feature_bounds(x, rho, n, d, W.bounds, st)) return s;
    return launch_accumulate<float>(x, rho, a.train_bmu, n, d, m, W.bounds, S, c, st);
}

int somgb_train_bmu_pass(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                         int64_t m, double penalty, int algo, int32_t* bmu_out, double* err3, void* ws,
                         size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, algo)) return s;
    if (n > 0 && !bmu_out) return set_error(SOMGB_ERR_INVALID, "bmu_out is NULL");
    if (err3 && !topo) return set_error(SOMGB_ERR_INVALID, "topo is NULL");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_FIND_BMUS, n, m, d, algo, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    PassArgs a{};
    a.x = x; a.rho = rho; a.n = n; a.d = d; a.w = w; a.m = m; a.topo = topo; a.penalty = penalty;
    a.err3 = err3; a.train_bmu = bmu_out;
    a.outs = OUT_TRAIN | (err3 ? OUT_ERR : 0);
    return run_pass(a, algo, W, tc, (cudaStream_t)stream);
}

int somgb_workspace_status(const void* ws, unsigned int* status, int clear, somgb_stream_t stream) {
    if (!ws || !status) return set_error(SOMGB_ERR_INVALID, "ws/status is NULL");
    if (((uintptr_t)ws) % 256) return set_error(SOMGB_ERR_INVALID, "workspace pointer must be 256-byte aligned");
    unsigned int* word = (unsigned int*)((char*)ws + 8);
    SOMGB_CUDA_TRY(cudaMemcpyAsync(status, word, sizeof(unsigned int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    SOMGB_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    if (clear) SOMGB_CUDA_TRY(cudaMemsetAsync(word, 0, sizeof(unsigned int), (cudaStream_t)stream));
    return SOMGB_OK;
}

int somgb_debug_tc_withhold(int64_t row_tile, unsigned int wait_limit) {
    if (row_tile < 0 || wait_limit == 0) return set_error(SOMGB_ERR_INVALID, "row_tile must be >= 0, wait_limit > 0");
    tc_debug_withhold(row_tile, wait_limit);
    return SOMGB_OK;
}

int somgb_debug_iter_withhold(int group, unsigned int wait_limit) {
    if (group < 0 || wait_limit == 0) return set_error(SOMGB_ERR_INVALID, "group must be >= 0, wait_limit > 0");
    iter_tc_debug_withhold(group, wait_limit);
    return SOMGB_OK;
}

int somgb_feature_bounds(const float* x, const double* rho, int64_t n, int d, float* bounds, somgb_stream_t stream) {
    if (n < 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes");
    if ((n > 0 && !x) || !bounds) return set_error(SOMGB_ERR_INVALID, "x/bounds is NULL");
    return launch_feature_bounds(x, rho, n, d, bounds, (cudaStream_t)stream);
}

int somgb_accumulate(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, int64_t m,
                     const float* bounds, double* S, double* c, somgb_stream_t stream) {
    if (n < 0 || m <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes");
    if (d > 64) return set_error(SOMGB_ERR_UNSUPPORTED, "somgb_accumulate supports D <= 64");
    if (n > 0 && (!x || !bmu)) return set_error(SOMGB_ERR_INVALID, "x/bmu is NULL");
    if (!S || !c || !bounds) return set_error(SOMGB_ERR_INVALID, "S/c/bounds is NULL");
    return launch_accumulate<float>(x, rho, bmu, n, d, m, bounds, S, c, (cudaStream_t)stream);
}

int somgb_accumulate_f64(const double* x, const double* rho, const int32_t* bmu, int64_t n, int d, int64_t m,
                         double* S, double* c, somgb_stream_t stream) {
    if (n < 0 || m <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes");
    if (n > 0 && (!x || !bmu)) return set_error(SOMGB_ERR_INVALID, "x/bmu is NULL");
    if (!S || !c) return set_error(SOMGB_ERR_INVALID, "S/c is NULL");
    return launch_accumulate<double>(x, rho, bmu, n, d, m, nullptr, S, c, (cudaStream_t)stream);
}

int somgb_neighbourhood_update(const double* S, const double* c, const float* topo, int64_t m, int d, double sigma,
                               float* w_out, double* num, double* den, somgb_stream_t stream) {
    if (m <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes m=%lld d=%d", (long long)m, d);
    if (!S || !c || !topo || !w_out) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (!(sigma > 0.0)) return set_error(SOMGB_ERR_INVALID, "sigma must be > 0");
    return launch_neighbourhood<float>(S, c, topo, m, d, sigma, w_out, num, den, (cudaStream_t)stream);
}

size_t somgb_sort_rows_workspace_bytes(int64_t m) { return m > 0 ? sort_rows_workspace(m) : 0; }

int somgb_sort_rows(const float* x, const double* rho, const int32_t* key, int64_t n, int d, int64_t m,
                    float* x_out, double* rho_out, void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (n < 0 || m <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes");
    if (n > 0 && (!x || !key || !x_out)) return set_error(SOMGB_ERR_INVALID, "x/key/x_out is NULL");
    if (n > 0 && rho && !rho_out) return set_error(SOMGB_ERR_INVALID, "rho_out is NULL");
    if (n > 0 && x_out == x) return set_error(SOMGB_ERR_INVALID, "x_out must not be x");
    if (!ws) return set_error(SOMGB_ERR_INVALID, "workspace is NULL");
    return launch_sort_rows(x, rho, key, n, d, m, x_out, rho_out, ws, ws_bytes, (cudaStream_t)stream);
}

size_t somgb_neighbourhood_grid_workspace_bytes(int64_t rows, int64_t cols, int d) {
    return rows > 0 && cols > 0 && d > 0 ? grid_neighbourhood_workspace(rows, cols, d) : 0;
}

int somgb_neighbourhood_update_grid(const double* S, const double* c, const float* topo, int64_t rows, int64_t cols,
                                    int d, double sigma, float* w_out, double* num, double* den, void* ws,
                                    size_t ws_bytes, somgb_stream_t stream) {
    if (rows <= 0 || cols <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes");
    if (!S || !c || !topo || !w_out) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (!(sigma > 0.0)) return set_error(SOMGB_ERR_INVALID, "sigma must be > 0");
    return launch_neighbourhood_grid<float>(S, c, topo, rows, cols, d, sigma, w_out, num, den, ws, ws_bytes,
                                            (cudaStream_t)stream);
}

int somgb_neighbourhood_update_grid_f64(const double* S, const double* c, const double* topo, int64_t rows,
                                        int64_t cols, int d, double sigma, double* w_out, double* num, double* den,
                                        void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (rows <= 0 || cols <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes");
    if (!S || !c || !topo || !w_out) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (!(sigma > 0.0)) return set_error(SOMGB_ERR_INVALID, "sigma must be > 0");
    return launch_neighbourhood_grid<double>(S, c, topo, rows, cols, d, sigma, w_out, num, den, ws, ws_bytes,
                                             (cudaStream_t)stream);
}

int somgb_train_iter_pass(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                          int64_t m, double sigma0, int64_t cur_vector, int64_t n_vectors, double* num, double* den,
                          void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, SOMGB_ALGO_FP32)) return s;
    if (!topo || !num || !den) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (n_vectors <= 0) return set_error(SOMGB_ERR_INVALID, "n_vectors must be > 0");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_EPOCH, n, m, d, SOMGB_ALGO_FP32, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    PassArgs a{};
    a.x = x; a.rho = rho; a.n = n; a.d = d; a.w = w; a.m = m; a.train_bmu = W.train_bmu; a.outs = OUT_TRAIN;
    if (int s = run_pass(a, SOMGB_ALGO_FP32, W, false, st)) return s;
    return launch_iter<float>(x, rho, W.train_bmu, n, d, topo, m, sigma0, cur_vector, n_vectors, num, den, st);
}

int somgb_train_iter_pass_grid(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                               int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors,
                               int algo, double* num, double* den, void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (rows <= 0 || cols <= 0) return set_error(SOMGB_ERR_INVALID, "invalid grid %lld x %lld", (long long)rows,
                                                 (long long)cols);
    const int64_t m = rows * cols;
    if (int s = check_common(x, n, d, w, m, algo)) return s;
    if (!topo || !num || !den) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (n_vectors <= 0) return set_error(SOMGB_ERR_INVALID, "n_vectors must be > 0");
    if (d > 64) return set_error(SOMGB_ERR_UNSUPPORTED, "the grid iteration pass supports D <= 64");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_EPOCH, n, m, d, algo, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    PassArgs a{};
    a.x = x; a.rho = rho; a.n = n; a.d = d; a.w = w; a.m = m; a.train_bmu = W.train_bmu; a.outs = OUT_TRAIN;
    if (int s = run_pass(a, algo, W, tc, st)) return s;
    // the tensor-core contraction (K4) for the tensor-core algorithms; AUTO keeps small passes on the CUDA cores
    const bool k4 = algo != SOMGB_ALGO_FP32 && iter_tc_shape_ok(rows, cols, d) && device_has_tc() &&
                    (algo == SOMGB_ALGO_TC || n * m >= ((int64_t)1 << 22));
    if (k4) {
        SOMGB_CUDA_TRY(cudaMemsetAsync(W.bounds, 0, (size_t)(d + 1) * 4, st));
        if (int s = launch_feature_bounds(x, rho, n, d, W.bounds, st)) return s;
        return launch_iter_tc(x, rho, W.train_bmu, n, d, topo, rows, cols, sigma0, cur_vector, n_vectors, W.bounds,
                              num, den, (unsigned int*)(W.counter + 1), st);
    }
    return launch_iter_grid(x, rho, W.train_bmu, n, d, topo, rows, cols, sigma0, cur_vector, n_vectors, num, den, st);
}

int somgb_divide(const double* num, const double* den, int64_t m, int d, float* w_out, somgb_stream_t stream) {
    if (m <= 0 || d <= 0 || !num || !den || !w_out) return set_error(SOMGB_ERR_INVALID, "invalid arguments");
    return launch_divide<float>(num, den, m, d, w_out, (cudaStream_t)stream);
}

// ----- float64 maps -----------------------------------------------------------------------------------------------

int somgb_find_bmus_f64(const double* x, int64_t n, int d, const double* w, int64_t m, int32_t* bmu_out,
                        somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, SOMGB_ALGO_FP32)) return s;
    if (n > 0 && !bmu_out) return set_error(SOMGB_ERR_INVALID, "bmu_out is NULL");
    return launch_exact_pass_f64(x, nullptr, n, d, w, m, nullptr, 0.0, OUT_BMU, bmu_out, nullptr, nullptr, nullptr,
                                 (cudaStream_t)stream);
}

int somgb_count_bmus_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                         double* hist, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, SOMGB_ALGO_FP32)) return s;
    if (!hist) return set_error(SOMGB_ERR_INVALID, "hist is NULL");
    return launch_exact_pass_f64(x, rho, n, d, w, m, nullptr, 0.0, OUT_HIST, nullptr, hist, nullptr, nullptr,
                                 (cudaStream_t)stream);
}

int somgb_compute_errors_f64(const double* x, const double* rho, int64_t n, int d, const double* w,
                             const double* topo, int64_t m, double penalty, double* err3, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, SOMGB_ALGO_FP32)) return s;
    if (!err3 || !topo) return set_error(SOMGB_ERR_INVALID, "err3/topo is NULL");
    return launch_exact_pass_f64(x, rho, n, d, w, m, topo, penalty, OUT_ERR, nullptr, nullptr, err3, nullptr,
                                 (cudaStream_t)stream);
}

int somgb_train_epoch_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w,
                               const double* topo, int64_t m, double penalty, double* S, double* c, double* err3,
                               void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, SOMGB_ALGO_FP32)) return s;
    if (!S || !c) return set_error(SOMGB_ERR_INVALID, "S/c is NULL");
    if (err3 && !topo) return set_error(SOMGB_ERR_INVALID, "topo is NULL");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_EPOCH, n, m, d, SOMGB_ALGO_FP32, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (int s = launch_exact_pass_f64(x, rho, n, d, w, m, topo, penalty, OUT_TRAIN | (err3 ? OUT_ERR : 0), nullptr,
                                      nullptr, err3, W.train_bmu, st))
        return s;
    return launch_accumulate<double>(x, rho, W.train_bmu, n, d, m, nullptr, S, c, st);
}

int somgb_neighbourhood_update_f64(const double* S, const double* c, const double* topo, int64_t m, int d,
                                   double sigma, double* w_out, double* num, double* den, somgb_stream_t stream) {
    if (m <= 0 || d <= 0) return set_error(SOMGB_ERR_INVALID, "invalid sizes m=%lld d=%d", (long long)m, d);
    if (!S || !c || !topo || !w_out) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (!(sigma > 0.0)) return set_error(SOMGB_ERR_INVALID, "sigma must be > 0");
    return launch_neighbourhood<double>(S, c, topo, m, d, sigma, w_out, num, den, (cudaStream_t)stream);
}

int somgb_train_iter_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w,
                              const double* topo, int64_t m, double sigma0, int64_t cur_vector, int64_t n_vectors,
                              double* num, double* den, void* ws, size_t ws_bytes, somgb_stream_t stream) {
    if (int s = check_common(x, n, d, w, m, SOMGB_ALGO_FP32)) return s;
    if (!topo || !num || !den) return set_error(SOMGB_ERR_INVALID, "NULL argument");
    if (n_vectors <= 0) return set_error(SOMGB_ERR_INVALID, "n_vectors must be > 0");
    Workspace W;
    bool tc = false;
    if (int s = carve(ws, ws_bytes, SOMGB_OP_EPOCH, n, m, d, SOMGB_ALGO_FP32, &W, &tc)) return s;
    if (n == 0) return SOMGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (int s = launch_exact_pass_f64(x, rho, n, d, w, m, nullptr, 0.0, OUT_TRAIN, nullptr, nullptr, nullptr,
                                      W.train_bmu, st))
        return s;
    return launch_iter<double>(x, rho, W.train_bmu, n, d, topo, m, sigma0, cur_vector, n_vectors, num, den, st);
}

int somgb_divide_f64(const double* num, const double* den, int64_t m, int d, double* w_out, somgb_stream_t stream) {
    if (m <= 0 || d <= 0 || !num || !den || !w_out) return set_error(SOMGB_ERR_INVALID, "invalid arguments");
    return launch_divide<double>(num, den, m, d, w_out, (cudaStream_t)stream);
}

}  // extern "C"
