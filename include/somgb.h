/*
 * somgb — C ABI of the GB300-native batch self-organising-map hot path.
 *
 * Every entry point takes caller-owned DEVICE pointers (row-major, contiguous),
 * sizes, a CUDA stream, and returns an int status (SOMGB_OK == 0). Work is
 * enqueued on `stream` and is asynchronous with respect to the host; outputs
 * marked "+=" are accumulated into, so callers zero them first (that is how the
 * reference's chunked loops use their device accumulators). No entry point
 * allocates device memory: scratch space is a caller buffer whose size
 * somgb_workspace_bytes() returns. Calls on distinct streams with distinct
 * workspaces may run concurrently.
 *
 * Each entry point names the reference interface it replaces
 * (lpsc-euclid/decontamination 0.0.1, paths inside that project). In the
 * reference these are Numba kernels launched as
 * `kernel[enable_gpu, threads_per_block, n](*arrays, *scalars)`
 * (jit/__init__.py:334-412); results go to caller-allocated device arrays.
 *
 * Arithmetic contract: BMUs are those of the compiled reference for float32
 * maps — distance = float64 sum, in feature order, of float32 squares of
 * float32 differences; argmin by strict '>' (lowest index wins ties); NaN
 * distances skipped. Float64 maps use float64 throughout.
 */
#ifndef SOMGB_H
#define SOMGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* somgb_stream_t; /* == cudaStream_t; NULL = legacy default stream */

/* status codes */
#define SOMGB_OK 0
#define SOMGB_ERR_INVALID 1     /* bad size, null pointer, misaligned pointer */
#define SOMGB_ERR_CUDA 2        /* a CUDA runtime call or launch failed */
#define SOMGB_ERR_WORKSPACE 3   /* workspace smaller than somgb_workspace_bytes() */
#define SOMGB_ERR_UNSUPPORTED 4 /* no device / not an sm_103 device / shape outside a kernel's limits */
#define SOMGB_ERR_TIMEOUT 5     /* a bounded device-side wait gave up (kernel returned early) */

/* distance-search algorithms */
#define SOMGB_ALGO_FP32 0       /* CUDA cores: float32 direct differences, margin-gated float64 recheck */
#define SOMGB_ALGO_TC 1         /* tcgen05 split-FP16 distance GEMM, margin-gated recheck (D in {4, 8, 16, 32},
                                   M <= 16384; somgb_algo_supported tells) */
#define SOMGB_ALGO_AUTO 2       /* TC where its shape limits allow, N*M >= 2^22 and M >= 32; FP32 otherwise */

/* workspace query operations */
#define SOMGB_OP_FIND_BMUS 0
#define SOMGB_OP_COUNT_BMUS 1
#define SOMGB_OP_ERRORS 2
#define SOMGB_OP_EPOCH 3

int somgb_version(void);

/* Copies the calling thread's last error message into buf (NUL-terminated); returns its full length. */
size_t somgb_last_error(char* buf, size_t len);

/* Scratch bytes an entry point needs for these sizes (0 if none). */
size_t somgb_workspace_bytes(int op, int64_t n, int64_t m, int d, int algo);

/* Number of samples the last pass on this thread sent to the exact recheck (diagnostic; synchronises `stream`). */
int somgb_last_recheck_count(int64_t* count, somgb_stream_t stream);

/* Column tiles (256 units each) the second sweeps of the last tensor-core pass on this thread computed, summed over
 * its 128-row tiles; their first sweeps compute every column tile (diagnostic; 0 after a CUDA-core pass;
 * synchronises `stream`). */
int somgb_last_sweep2_tiles(int64_t* tiles, somgb_stream_t stream);

/*
 * Device status word of the current device (synchronises `stream`): 0 while healthy; non-zero once a bounded
 * device-side wait of a tensor-core pass gave up, in which case that pass returned early and its outputs are
 * incomplete. Sticky until read with clear != 0.
 */
int somgb_device_status(unsigned int* status, int clear, somgb_stream_t stream);

/*
 * The status word of the last pass that used workspace `ws` (synchronises `stream`): non-zero when a bounded
 * device-side wait of that pass gave up (its outputs are then incomplete). Each pass clears its workspace's word when
 * it starts, so concurrent calls with their own workspaces each see their own failures. clear != 0 zeroes it.
 */
int somgb_workspace_status(const void* ws, unsigned int* status, int clear, somgb_stream_t stream);

/*
 * Test hook for the bounded waits: the next tensor-core pass on the calling thread never loads the samples of its
 * row tile `row_tile` and bounds its waits by `wait_limit` polls (about 1 us each), so that the wait for those samples
 * runs out: that pass returns early with its status word and the device status word set, and the rows it did not
 * decide keep whatever the outputs held. One-shot; no product call sets it.
 */
int somgb_debug_tc_withhold(int64_t row_tile, unsigned int wait_limit);

/*
 * Test hook for the bounded waits of the tensor-core iteration contraction (somgb_train_iter_pass_grid under
 * SOMGB_ALGO_TC): the next contraction on the calling thread never signals that its accumulator group `group` (of two
 * 32-sample batches per CTA) is complete and bounds its waits by `wait_limit` polls, so that the fold's wait runs out:
 * each CTA stops, drains the MMAs it issued, frees its TMEM and returns with bit 65536 of the workspace's and the
 * device's status words set; its partial sums are not added. One-shot; no product call sets it.
 */
int somgb_debug_iter_withhold(int group, unsigned int wait_limit);

/* 1 if `algo` can run a pass of these sizes on the current device, else 0. */
int somgb_algo_supported(int algo, int64_t n, int64_t m, int d);

/* Kernels this library has launched in this process (diagnostic). */
int64_t somgb_kernel_launches(void);

/*
 * Diagnostic timer: while set (non-NULL cudaEvent_t handles), every BMU pass on the calling thread records
 * `start` on its stream just before its dominant kernel and `stop` just after it. Pass NULLs to clear.
 */
int somgb_set_kernel_timer(void* start_event, void* stop_event);

/*
 * BMU of every sample: bmu_out[i] = argmin_j |x_i - w_j|^2, 0 when every distance is NaN.
 * Replaces _find_bmus_kernel / _find_bmu_xpu (algo/som_abstract.py:736-783), called by get_winners (:670-695).
 */
int somgb_find_bmus(const float* x, int64_t n, int d, const float* w, int64_t m, int algo, int32_t* bmu_out,
                    void* ws, size_t ws_bytes, somgb_stream_t stream);
int somgb_find_bmus_f64(const double* x, int64_t n, int d, const double* w, int64_t m, int32_t* bmu_out,
                        somgb_stream_t stream);

/*
 * Footprint maps in one BMU pass (the fused form of Decontamination_SOM.train's get_winners and compute_gndm's two
 * get_activation_map calls, decontamination/decontamination_som.py:596, 640-641): bmu_out[i] as somgb_find_bmus,
 * hist_weighted[b] += rho_i for rho_i > 0 and hist_count[b] += 1 for every sample (both float64 (m,) "+=", either
 * may be NULL). Workspace: somgb_workspace_bytes(SOMGB_OP_FIND_BMUS, n, m, d, algo).
 */
int somgb_footprint_maps(const float* x, const double* rho, int64_t n, int d, const float* w, int64_t m, int algo,
                         int32_t* bmu_out, double* hist_weighted, double* hist_count, void* ws, size_t ws_bytes,
                         somgb_stream_t stream);
int somgb_footprint_maps_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                             int32_t* bmu_out, double* hist_weighted, double* hist_count, somgb_stream_t stream);
/* The histograms of somgb_footprint_maps from BMUs already computed (bmu[i] outside [0, m) is skipped). */
int somgb_bmu_histograms(const int32_t* bmu, const double* rho, int64_t n, int64_t m, double* hist_weighted,
                         double* hist_count, somgb_stream_t stream);

/*
 * Activation histogram: hist[bmu(x_i)] += rho_i for rho_i > 0 (rho NULL = all ones); hist is float64 (m,) "+=".
 * Replaces _count_bmus_kernel (algo/som_abstract.py:700-732), called by get_activation_map (:605-666).
 */
int somgb_count_bmus(const float* x, const double* rho, int64_t n, int d, const float* w, int64_t m, int algo,
                     double* hist, void* ws, size_t ws_bytes, somgb_stream_t stream);
int somgb_count_bmus_f64(const double* x, const double* rho, int64_t n, int d, const double* w, int64_t m,
                         double* hist, somgb_stream_t stream);

/*
 * Quantisation / topographic error sums, err3 "+=": [sum rho*sqrt(d1), sum rho*[|t_b1-t_b2|^2 > penalty], sum rho]
 * over samples with rho > 0 and two valid units (b1, b2 = the two smallest (distance, index) pairs).
 * Replaces _compute_errors_kernel / _compute_errors_xpu (algo/som_abstract.py:787-878), called by
 * compute_errors (:528-601); penalty is 2.0 for square and 1.0 for hexagonal maps (:575).
 */
int somgb_compute_errors(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                         int64_t m, double penalty, int algo, double* err3, void* ws, size_t ws_bytes,
                         somgb_stream_t stream);
int somgb_compute_errors_f64(const double* x, const double* rho, int64_t n, int d, const double* w,
                             const double* topo, int64_t m, double penalty, double* err3, somgb_stream_t stream);

/*
 * One training pass of epoch mode over a chunk, fused with the error sums of the same weights.
 * For each sample with (float)rho_i > 0 and a valid BMU b_i (training semantics: all-NaN rows are skipped):
 *   S[b_i, :] += (double)(float)rho_i * x_i,  c[b_i] += (double)(float)rho_i      (S: m x d, c: m; float64 "+=")
 * and, when err3 != NULL, the compute_errors sums of `w` as in somgb_compute_errors ("+=").
 * bmu_out (optional, n) receives b_i (-1 when skipped).
 * Replaces the BMU half of _train_step1_epoch_kernel/_train_step2_xpu (algo/som_batch.py:94-150, 509-540) and,
 * fused, the compute_errors pass the reference runs after every epoch (som_batch.py:363). The neighbourhood half
 * (som_batch.py:542-566) is somgb_neighbourhood_update on the per-BMU sums.
 */
int somgb_train_epoch_pass(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                           int64_t m, double penalty, int algo, double* S, double* c, double* err3,
                           int32_t* bmu_out, void* ws, size_t ws_bytes, somgb_stream_t stream);
int somgb_train_epoch_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w,
                               const double* topo, int64_t m, double penalty, double* S, double* c, double* err3,
                               void* ws, size_t ws_bytes, somgb_stream_t stream);

/*
 * The two halves of somgb_train_epoch_pass as separate calls.
 * somgb_train_bmu_pass: bmu_out[i] = training BMU of sample i (-1 when (float)rho_i <= 0 or no unit is valid),
 *   plus the error sums of `w` into err3 when err3 != NULL. Workspace: SOMGB_OP_FIND_BMUS sizing.
 * somgb_feature_bounds: bounds[k] = max(bounds[k], max_i |(float)rho_i * x_ik|) (k < d) and bounds[d] =
 *   max(bounds[d], max_i (float)rho_i) over the samples with finite features and rho_i > 0, as float32 bit patterns
 *   compared as unsigned integers ("max="; zero the d+1 floats first). A dataset's bounds stay valid for every epoch.
 * somgb_accumulate: S[b_i] += (double)(float)rho_i * x_i, c[b_i] += (double)(float)rho_i for b_i >= 0 ("+="), summed
 *   in exact 47-bit fixed point scaled by `bounds`; D <= 64.
 */
int somgb_train_bmu_pass(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                         int64_t m, double penalty, int algo, int32_t* bmu_out, double* err3, void* ws,
                         size_t ws_bytes, somgb_stream_t stream);
int somgb_feature_bounds(const float* x, const double* rho, int64_t n, int d, float* bounds, somgb_stream_t stream);
int somgb_accumulate(const float* x, const double* rho, const int32_t* bmu, int64_t n, int d, int64_t m,
                     const float* bounds, double* S, double* c, somgb_stream_t stream);
int somgb_accumulate_f64(const double* x, const double* rho, const int32_t* bmu, int64_t n, int d, int64_t m,
                         double* S, double* c, somgb_stream_t stream);

/*
 * Row regrouping between epochs (no counterpart in the reference, which visits the catalogue in storage order,
 * algo/som_batch.py:285-376): x_out/rho_out receive the rows of x/rho grouped by key (the rows of key k contiguous,
 * in increasing k; keys outside [0, m) last; the order within a key unspecified). With the keys the BMUs an epoch just
 * found, the 128-row tiles of the next tensor-core pass each meet few column tiles of candidates, and its second
 * sweep recomputes only those; no row's result depends on the order. rho/rho_out may be NULL. Workspace:
 * somgb_sort_rows_workspace_bytes(m).
 */
size_t somgb_sort_rows_workspace_bytes(int64_t m);
int somgb_sort_rows(const float* x, const double* rho, const int32_t* key, int64_t n, int d, int64_t m,
                    float* x_out, double* rho_out, void* ws, size_t ws_bytes, somgb_stream_t stream);

/*
 * Neighbourhood contraction and weight update of one epoch:
 *   num_j = sum_b h_jb S_b, den_j = sum_b h_jb c_b, h_jb = exp(-|t_j - t_b|^2 / (2 sigma^2)),
 *   w_out_j = num_j / den_j if den_j > 1e-12 else 0.
 * `sigma` is the decayed, clamped radius of this epoch (sigma0 * 1/(1+2e/E), >= 1e-12, in float64).
 * Replaces the neighbourhood scatter of _train_step2_xpu (algo/som_batch.py:542-566) and the host divide
 * (som_batch.py:346-359). num/den (optional, m x d and m) receive the float64 numerator and denominator.
 */
int somgb_neighbourhood_update(const double* S, const double* c, const float* topo, int64_t m, int d, double sigma,
                               float* w_out, double* num, double* den, somgb_stream_t stream);
int somgb_neighbourhood_update_f64(const double* S, const double* c, const double* topo, int64_t m, int d,
                                   double sigma, double* w_out, double* num, double* den, somgb_stream_t stream);

/*
 * The same update on a grid topography (unit i*cols + j; x coordinate a function of (i, j mod 2) only and y a function
 * of j only, as on the reference's square and hexagonal grids, algo/som_abstract.py:81-111): the Gaussian factorises
 * into x and y parts and the contraction runs as two one-dimensional ones, rows*cols*(rows + cols) terms instead of
 * (rows*cols)^2. Results equal somgb_neighbourhood_update's to a few float64 ulps. ws: device scratch of
 * somgb_neighbourhood_grid_workspace_bytes(rows, cols, d) bytes (8-byte aligned).
 */
size_t somgb_neighbourhood_grid_workspace_bytes(int64_t rows, int64_t cols, int d);
int somgb_neighbourhood_update_grid(const double* S, const double* c, const float* topo, int64_t rows, int64_t cols,
                                    int d, double sigma, float* w_out, double* num, double* den, void* ws,
                                    size_t ws_bytes, somgb_stream_t stream);
int somgb_neighbourhood_update_grid_f64(const double* S, const double* c, const double* topo, int64_t rows,
                                        int64_t cols, int d, double sigma, double* w_out, double* num, double* den,
                                        void* ws, size_t ws_bytes, somgb_stream_t stream);

/*
 * Iteration ("n_vectors") mode over a chunk: sample i of the chunk has sigma_i = sigma0 * 1/(1+2(cur+i)/n_vectors)
 * (clamped >= 1e-12) and adds rho_i * h_j(i) * x_i to num[j] and rho_i * h_j(i) to den[j] for every unit j
 * (float64 "+="). Replaces _train_step1_iter_kernel (algo/som_batch.py:154-210). sigma0 is the map dtype's value.
 * Workspace: somgb_workspace_bytes(SOMGB_OP_EPOCH, n, m, d, SOMGB_ALGO_FP32).
 */
int somgb_train_iter_pass(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                          int64_t m, double sigma0, int64_t cur_vector, int64_t n_vectors, double* num, double* den,
                          void* ws, size_t ws_bytes, somgb_stream_t stream);
/*
 * The same on the reference's square and hexagonal grids (unit i * cols + j of a rows x cols map, topography as the
 * reference builds it), with the neighbourhood factor split by grid axis; BMUs by `algo` (workspace:
 * somgb_workspace_bytes(SOMGB_OP_EPOCH, n, m, d, algo)). D <= 64. SOMGB_ALGO_TC, and SOMGB_ALGO_AUTO when n * m >=
 * 2^22, contract on the tensor cores for D <= 47 (split-FP16 products, float32 accumulation of 64 samples, folded
 * into compensated float32 sums, then float64); otherwise the sums are float32 per batch of 32 samples on the CUDA
 * cores, folded into float64. Both agree with somgb_train_iter_pass to ~1e-6 relative. A bounded wait of the
 * tensor-core contraction that gives up sets bit 65536 of the workspace's and the device's status words.
 */
int somgb_train_iter_pass_grid(const float* x, const double* rho, int64_t n, int d, const float* w, const float* topo,
                               int64_t rows, int64_t cols, double sigma0, int64_t cur_vector, int64_t n_vectors,
                               int algo, double* num, double* den, void* ws, size_t ws_bytes, somgb_stream_t stream);
int somgb_train_iter_pass_f64(const double* x, const double* rho, int64_t n, int d, const double* w,
                              const double* topo, int64_t m, double sigma0, int64_t cur_vector, int64_t n_vectors,
                              double* num, double* den, void* ws, size_t ws_bytes, somgb_stream_t stream);

/*
 * somgb_find_bmus for callers that cannot allocate device memory: a host framework that hands out a fixed
 * device-memory budget up front and owns every allocation, or a pipeline that only holds the input and output buffers
 * it passes in and has no allocator to call. It has no counterpart in the reference: it is the same computation as
 * somgb_find_bmus, but its scratch is one static device array of somgb_find_bmus_noalloc_scratch_bytes() bytes
 * (4 MiB) inside the library, held by every GPU that loads it until the process exits. Inputs with more rows than fit
 * are processed in chunks; a map whose unit operand does not fit is refused with SOMGB_ERR_WORKSPACE. The first call
 * on a device, with that device current, looks up the array's address (a failed lookup is retried by the next call);
 * make that first call before any stream capture: during a capture it is refused with SOMGB_ERR_INVALID. Every call
 * on a device shares the array: calls that overlap on the GPU (on different streams) race; calls in stream order do
 * not. Nothing is allocated or freed.
 */
int somgb_find_bmus_noalloc(const float* x, int64_t n, int d, const float* w, int64_t m, int algo, int32_t* bmu_out,
                            somgb_stream_t stream);
size_t somgb_find_bmus_noalloc_scratch_bytes(void);

/*
 * Weighted moments of a catalogue, the sums behind the covariance of the PCA initialisation (replaces Welford's
 * update Covariance._update_welford_cov_sums, algo/covariance.py:24-44, used by SOM_PCA.train, algo/som_pca.py:181):
 *   out[0] = W = sum w_i, out[1 .. d] = mean = sum w_i x_i / W,
 *   out[1 + d .. 1 + d + d*d) = M2 = sum w_i (x_i - mean)(x_i - mean)^T (row-major, symmetric),
 * over the samples whose features are all finite and whose weight w_i = rho[i] (1 when rho is NULL) is finite and
 * positive; float64 sums ("="; out is overwritten). The covariance is M2 / (W - ddof); chunks combine on the host.
 * 1 <= d <= 64. No workspace.
 */
int somgb_weighted_moments(const float* x, const double* rho, int64_t n, int d, double* out, somgb_stream_t stream);
int somgb_weighted_moments_f64(const double* x, const double* rho, int64_t n, int d, double* out,
                               somgb_stream_t stream);

/* w_out_j = num_j / den_j where den_j > 1e-12, else 0 (algo/som_batch.py:481-486). */
int somgb_divide(const double* num, const double* den, int64_t m, int d, float* w_out, somgb_stream_t stream);
int somgb_divide_f64(const double* num, const double* den, int64_t m, int d, double* w_out, somgb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SOMGB_H */
