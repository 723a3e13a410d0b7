// somref — CPU restatement of the reference's batch-SOM kernels.
//
// TEST INFRASTRUCTURE ONLY. This library is the parity oracle and the timed
// CPU baseline. Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
// load it, and only to check or to time against; the product path
// (decontamination_gb300) never calls it.
//
// Parity is pinned: tests/test_oracle.py checks the `pyref` mode of this file
// bit-for-bit (BMUs, counts) and to float32 rounding (weights) against
// fixtures produced by the reference's own pure-Python code path
// (tests/golden/make_golden.py).
//
// Reference functions restated (lpsc-euclid/decontamination 0.0.1):
//   sqdist            algo/__init__.py:89-98          square_distance_xpu
//   decay             algo/__init__.py:64-74          asymptotic_decay_{cpu,gpu}
//   find_bmu          algo/som_abstract.py:764-783    _find_bmu_xpu (min_index starts at 0)
//   count_bmus        algo/som_abstract.py:700-732    _count_bmus_kernel
//   compute_errors    algo/som_abstract.py:787-878    _compute_errors_kernel/_xpu
//   train_step2       algo/som_batch.py:509-566       _train_step2_xpu (min_index starts at -1)
//   epoch kernel      algo/som_batch.py:94-150        _train_step1_epoch_kernel
//   iter kernel       algo/som_batch.py:154-210       _train_step1_iter_kernel
//
// Arithmetic modes (the reference's arithmetic depends on how it is run):
//   MODE_NUMBA (0): the Numba-compiled reference. For float32 data a distance
//     term is (float)(w-x) squared in float32 and summed into a float64
//     accumulator that starts at the literal 0.0; sigma and the neighbourhood
//     factor are float64; each atomic add casts its float64 value to the
//     accumulator's dtype.
//   MODE_PYREF (1): the reference's pure-Python path under NumPy 2 (NEP 50):
//     Python-float literals are weak, so distance sums, sigma, 1/(2 sigma^2)
//     and the neighbourhood factor all stay float32 (math.exp itself runs in
//     float64 and is rounded back).
//   MODE_EXACT (2): float64 everywhere (differences, squares, sums); the
//     tie-adjudication oracle. For float64 data every mode is float64.
//
// Build: oracle/build.sh (g++ -O2 -fopenmp -ffp-contract=off; contraction is
// disabled so x86 and Arm hosts round identically).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

constexpr int MODE_NUMBA = 0;
constexpr int MODE_PYREF = 1;
constexpr int MODE_EXACT = 2;
constexpr double FLOAT_EPS = 1.0e-12;   // algo/som_batch.py:24

// The C library's powf, called through a volatile pointer so that the compiler cannot fold powf(t, 2) into t*t.
float (*volatile libc_powf)(float, float) = powf;

// square_distance_xpu (algo/__init__.py:89-98) for float32 operands.
inline double sqdist_f32(const float* a, const float* b, int d, int mode) {
    if (mode == MODE_PYREF) {
        // NumPy evaluates np.float32 ** 2 with the C library's powf, which is not always the correctly
        // rounded t*t; the pure-Python reference inherits that.
        float acc = 0.0f;
        for (int k = 0; k < d; ++k) {
            float t = a[k] - b[k];
            acc = acc + libc_powf(t, 2.0f);
        }
        return (double)acc;
    }
    if (mode == MODE_EXACT) {
        double acc = 0.0;
        for (int k = 0; k < d; ++k) {
            double t = (double)a[k] - (double)b[k];
            acc += t * t;
        }
        return acc;
    }
    double acc = 0.0;
    for (int k = 0; k < d; ++k) {
        float t = a[k] - b[k];
        float s = t * t;
        acc += (double)s;
    }
    return acc;
}

// The same for float64 operands: every mode is float64.
inline double sqdist_f64(const double* a, const double* b, int d, int /*mode*/) {
    double acc = 0.0;
    for (int k = 0; k < d; ++k) {
        double t = a[k] - b[k];
        acc += t * t;
    }
    return acc;
}

inline double sqdist(const float* a, const float* b, int d, int mode) { return sqdist_f32(a, b, d, mode); }
inline double sqdist(const double* a, const double* b, int d, int mode) { return sqdist_f64(a, b, d, mode); }

// asymptotic_decay_cpu (algo/__init__.py:64-67): 1 / (1 + 2 e / E) in float64.
inline double decay(int64_t e, int64_t total) { return 1.0 / (1.0 + 2.0 * (double)e / (double)total); }

// _find_bmu_xpu (algo/som_abstract.py:764-783) when first_index == 0, and the
// BMU loop of _train_step2_xpu (algo/som_batch.py:520-540) when first_index == -1.
// Strict '>' keeps the lowest index on ties; NaN distances are skipped.
template <typename T>
inline int64_t find_bmu(const T* w, int64_t m, int d, const T* x, int mode, int64_t first_index, double* dmin) {
    double best = 1.0e99;
    int64_t idx = first_index;
    for (int64_t j = 0; j < m; ++j) {
        double dist = sqdist(w + j * d, x, d, mode);
        if (dist != dist) continue;
        if (mode == MODE_PYREF && sizeof(T) == 4) {
            // float32 comparison against the float64 literal 1e99 (cast to +inf in float32)
            if ((float)best > (float)dist) { best = dist; idx = j; }
        } else if (best > dist) {
            best = dist;
            idx = j;
        }
    }
    if (dmin) *dmin = best;
    return idx;
}

// Top-2 selection of _compute_errors_xpu (algo/som_abstract.py:822-850).
template <typename T>
inline void find_top2(const T* w, int64_t m, int d, const T* x, int mode, int64_t* i1, int64_t* i2, double* d1,
                      double* d2) {
    double md2 = 1.0e99, md1 = 1.0e99;
    int64_t mi2 = -1, mi1 = -1;
    for (int64_t j = 0; j < m; ++j) {
        double d0 = sqdist(w + j * d, x, d, mode);
        if (d0 != d0) continue;
        if (md1 > d0) {
            if (j != mi1) { md2 = md1; mi2 = mi1; }
            md1 = d0;
            mi1 = j;
        } else if (j != mi1 && md2 > d0) {
            md2 = d0;
            mi2 = j;
        }
    }
    *i1 = mi1; *i2 = mi2; *d1 = md1; *d2 = md2;
}

inline int nthreads_or_default(int threads) { return threads > 0 ? threads : omp_get_max_threads(); }

// Neighbourhood factors and accumulation of one sample, _train_step2_xpu
// (algo/som_batch.py:548-566). `sigma` is already decayed and clamped.
template <typename T>
inline void scatter_sample(T* num, T* den, const T* topo, const T* x, int64_t m, int d, int64_t bmu, double rho,
                           double sigma, int mode, bool atomic) {
    const T* tb = topo + 2 * bmu;
    if (mode == MODE_PYREF && sizeof(T) == 4) {
        float s = (float)sigma;
        float inv = 1.0f / ((2.0f * s) * s);
        for (int64_t j = 0; j < m; ++j) {
            float sq = (float)sqdist(topo + 2 * j, tb, 2, mode);
            float arg = (-sq) * inv;
            float h = (float)rho * (float)std::exp((double)arg);
            for (int k = 0; k < d; ++k) {
                float v = h * (float)x[k];
                if (atomic) {
#pragma omp atomic
                    num[j * d + k] += (T)v;
                } else {
                    num[j * d + k] += (T)v;
                }
            }
            if (atomic) {
#pragma omp atomic
                den[j] += (T)h;
            } else {
                den[j] += (T)h;
            }
        }
        return;
    }
    double inv = 1.0 / (2.0 * sigma * sigma);
    for (int64_t j = 0; j < m; ++j) {
        double h = rho * std::exp(-sqdist(topo + 2 * j, tb, 2, mode) * inv);
        for (int k = 0; k < d; ++k) {
            T v = (T)(h * (double)x[k]);
            if (atomic) {
#pragma omp atomic
                num[j * d + k] += v;
            } else {
                num[j * d + k] += v;
            }
        }
        T hv = (T)(h * 1.0);
        if (atomic) {
#pragma omp atomic
            den[j] += hv;
        } else {
            den[j] += hv;
        }
    }
}

// sigma of _train_step1_*_kernel (algo/som_batch.py:107-110, 133-136, 167-170, 195-198).
inline double kernel_sigma(double sigma0_dtype, int64_t e, int64_t total, int mode, bool f32) {
    if (mode == MODE_PYREF && f32) {
        float s = (float)sigma0_dtype * (float)decay(e, total);
        double sd = (double)s;
        return sd < FLOAT_EPS ? FLOAT_EPS : sd;
    }
    double s = sigma0_dtype * decay(e, total);
    return s < FLOAT_EPS ? FLOAT_EPS : s;
}

template <typename T>
void train_epoch_scatter(T* num, T* den, const T* w, const T* topo, const T* x, const T* rho, int64_t n, int64_t m,
                         int d, double sigma0, int64_t epoch, int64_t n_epochs, int mode, int threads) {
    double sigma = kernel_sigma((double)(T)sigma0, epoch, n_epochs, mode, sizeof(T) == 4);
    if (threads == 1) {
        for (int64_t i = 0; i < n; ++i) {
            double r = (double)rho[i];
            if (!(r > 0.0)) continue;
            int64_t b = find_bmu(w, m, d, x + i * d, mode, -1, nullptr);
            if (b < 0) continue;
            scatter_sample(num, den, topo, x + i * d, m, d, b, r, sigma, mode, false);
        }
        return;
    }
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_or_default(threads))
    for (int64_t i = 0; i < n; ++i) {
        double r = (double)rho[i];
        if (!(r > 0.0)) continue;
        int64_t b = find_bmu(w, m, d, x + i * d, mode, -1, nullptr);
        if (b < 0) continue;
        scatter_sample(num, den, topo, x + i * d, m, d, b, r, sigma, mode, true);
    }
}

template <typename T>
void train_iter_scatter(T* num, T* den, const T* w, const T* topo, const T* x, const T* rho, int64_t n, int64_t m,
                        int d, double sigma0, int64_t cur_vector, int64_t n_vectors, int mode, int threads) {
    auto body = [&](int64_t i, bool atomic) {
        double r = (double)rho[i];
        if (!(r > 0.0)) return;
        double sigma = kernel_sigma((double)(T)sigma0, cur_vector + i, n_vectors, mode, sizeof(T) == 4);
        int64_t b = find_bmu(w, m, d, x + i * d, mode, -1, nullptr);
        if (b < 0) return;
        scatter_sample(num, den, topo, x + i * d, m, d, b, r, sigma, mode, atomic);
    };
    if (threads == 1) {
        for (int64_t i = 0; i < n; ++i) body(i, false);
        return;
    }
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_or_default(threads))
    for (int64_t i = 0; i < n; ++i) body(i, true);
}

template <typename T>
void find_bmus(const T* w, int64_t m, int d, const T* x, int64_t n, int mode, int32_t* out, int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(threads))
    for (int64_t i = 0; i < n; ++i) out[i] = (int32_t)find_bmu(w, m, d, x + i * d, mode, 0, nullptr);
}

// _count_bmus_kernel (algo/som_abstract.py:700-732): hist[bmu] += density for density > 0.
// Partial histograms per thread are combined in thread order (deterministic for a given thread count).
template <typename T>
void count_bmus(const T* w, int64_t m, int d, const T* x, const double* rho, int64_t n, int mode, double* hist,
                int threads) {
    int nt = threads == 1 ? 1 : nthreads_or_default(threads);
    std::vector<double> part((size_t)nt * m, 0.0);
#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double* h = part.data() + (size_t)t * m;
        for (int64_t i = lo; i < hi; ++i) {
            double r = rho ? rho[i] : 1.0;
            if (r > 0.0) h[find_bmu(w, m, d, x + i * d, mode, 0, nullptr)] += r;
        }
    }
    for (int t = 0; t < nt; ++t)
        for (int64_t j = 0; j < m; ++j) hist[j] += part[(size_t)t * m + j];
}

// _compute_errors_xpu (algo/som_abstract.py:815-878): errors[0] += rho*sqrt(d1),
// errors[1] += rho if |t(b1)-t(b2)|^2 > penalty, errors[2] += rho.
template <typename T>
void compute_errors(const T* w, const T* topo, int64_t m, int d, const T* x, const double* rho, int64_t n,
                    double penalty, int mode, double* out3, int threads) {
    int nt = threads == 1 ? 1 : nthreads_or_default(threads);
    std::vector<double> part((size_t)nt * 3, 0.0);
#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double e0 = 0, e1 = 0, e2 = 0;
        for (int64_t i = lo; i < hi; ++i) {
            double r = rho ? rho[i] : 1.0;
            if (!(r > 0.0)) continue;
            int64_t i1, i2;
            double d1, d2;
            find_top2(w, m, d, x + i * d, mode, &i1, &i2, &d1, &d2);
            if (i1 < 0 || i2 < 0 || i1 == i2) continue;
            e0 += r * std::sqrt(d1);
            double tsq = sqdist(topo + 2 * i1, topo + 2 * i2, 2, mode);
            bool far = (mode == MODE_PYREF && sizeof(T) == 4) ? ((float)tsq > (float)penalty) : (tsq > penalty);
            if (far) e1 += r;
            e2 += r;
        }
        part[t * 3 + 0] = e0; part[t * 3 + 1] = e1; part[t * 3 + 2] = e2;
    }
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k) out3[k] += part[t * 3 + k];
}

// FP64 factored epoch: the same update as train_epoch_scatter in exact
// arithmetic, reorganised as num = H.S, den = H.c with S_b = sum rho_i x_i and
// c_b = sum rho_i over the samples whose BMU is b. BMUs follow `mode`.
template <typename T>
void train_epoch_fp64(double* num, double* den, const T* w, const T* topo, const T* x, const T* rho, int64_t n,
                      int64_t m, int d, double sigma0, int64_t epoch, int64_t n_epochs, int mode,
                      int32_t* bmus_out, int threads) {
    int nt = threads == 1 ? 1 : nthreads_or_default(threads);
    std::vector<double> S((size_t)nt * m * d, 0.0), C((size_t)nt * m, 0.0);
#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double* s = S.data() + (size_t)t * m * d;
        double* c = C.data() + (size_t)t * m;
        for (int64_t i = lo; i < hi; ++i) {
            double r = (double)rho[i];
            int64_t b = -1;
            if (r > 0.0) b = find_bmu(w, m, d, x + i * d, mode, -1, nullptr);
            if (bmus_out) bmus_out[i] = (int32_t)b;
            if (b < 0) continue;
            for (int k = 0; k < d; ++k) s[b * d + k] += r * (double)x[i * d + k];
            c[b] += r;
        }
    }
    for (int t = 1; t < nt; ++t) {
        for (int64_t q = 0; q < m * d; ++q) S[q] += S[(size_t)t * m * d + q];
        for (int64_t q = 0; q < m; ++q) C[q] += C[(size_t)t * m + q];
    }
    double sigma = kernel_sigma((double)(T)sigma0, epoch, n_epochs, MODE_NUMBA, sizeof(T) == 4);
    double inv = 1.0 / (2.0 * sigma * sigma);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t j = 0; j < m; ++j) {
        double dn = 0.0;
        for (int k = 0; k < d; ++k) num[j * d + k] = 0.0;
        for (int64_t b = 0; b < m; ++b) {
            if (C[b] == 0.0) continue;
            double h = std::exp(-sqdist(topo + 2 * j, topo + 2 * b, 2, MODE_NUMBA) * inv);
            for (int k = 0; k < d; ++k) num[j * d + k] += h * S[b * d + k];
            dn += h * C[b];
        }
        den[j] = dn;
    }
}

}  // namespace

extern "C" {

int somref_version(void) { return 1; }

void somref_find_bmus_f32(const float* w, int64_t m, int d, const float* x, int64_t n, int mode, int32_t* out,
                          int threads) {
    find_bmus(w, m, d, x, n, mode, out, threads);
}
void somref_find_bmus_f64(const double* w, int64_t m, int d, const double* x, int64_t n, int mode, int32_t* out,
                          int threads) {
    find_bmus(w, m, d, x, n, mode, out, threads);
}

// BMU (first_index = -1 semantics) plus exact top-2 for every sample; used by the
// parity tests to check per-sample outputs (bmu1, bmu2, d1, d2).
void somref_top2_f32(const float* w, int64_t m, int d, const float* x, int64_t n, int mode, int32_t* i1,
                     int32_t* i2, double* d1, double* d2, int threads) {
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(threads))
    for (int64_t i = 0; i < n; ++i) {
        int64_t a, b;
        double da, db;
        find_top2(w, m, d, x + i * d, mode, &a, &b, &da, &db);
        i1[i] = (int32_t)a; i2[i] = (int32_t)b; d1[i] = da; d2[i] = db;
    }
}

void somref_count_bmus_f32(const float* w, int64_t m, int d, const float* x, const double* rho, int64_t n, int mode,
                           double* hist, int threads) {
    count_bmus(w, m, d, x, rho, n, mode, hist, threads);
}
void somref_count_bmus_f64(const double* w, int64_t m, int d, const double* x, const double* rho, int64_t n,
                           int mode, double* hist, int threads) {
    count_bmus(w, m, d, x, rho, n, mode, hist, threads);
}

void somref_compute_errors_f32(const float* w, const float* topo, int64_t m, int d, const float* x, const double* rho,
                               int64_t n, double penalty, int mode, double* out3, int threads) {
    compute_errors(w, topo, m, d, x, rho, n, penalty, mode, out3, threads);
}
void somref_compute_errors_f64(const double* w, const double* topo, int64_t m, int d, const double* x,
                               const double* rho, int64_t n, double penalty, int mode, double* out3, int threads) {
    compute_errors(w, topo, m, d, x, rho, n, penalty, mode, out3, threads);
}

void somref_train_epoch_scatter_f32(float* num, float* den, const float* w, const float* topo, const float* x,
                                    const float* rho, int64_t n, int64_t m, int d, double sigma0, int64_t epoch,
                                    int64_t n_epochs, int mode, int threads) {
    train_epoch_scatter(num, den, w, topo, x, rho, n, m, d, sigma0, epoch, n_epochs, mode, threads);
}
void somref_train_epoch_scatter_f64(double* num, double* den, const double* w, const double* topo, const double* x,
                                    const double* rho, int64_t n, int64_t m, int d, double sigma0, int64_t epoch,
                                    int64_t n_epochs, int mode, int threads) {
    train_epoch_scatter(num, den, w, topo, x, rho, n, m, d, sigma0, epoch, n_epochs, mode, threads);
}

void somref_train_iter_scatter_f32(float* num, float* den, const float* w, const float* topo, const float* x,
                                   const float* rho, int64_t n, int64_t m, int d, double sigma0, int64_t cur_vector,
                                   int64_t n_vectors, int mode, int threads) {
    train_iter_scatter(num, den, w, topo, x, rho, n, m, d, sigma0, cur_vector, n_vectors, mode, threads);
}
void somref_train_iter_scatter_f64(double* num, double* den, const double* w, const double* topo, const double* x,
                                   const double* rho, int64_t n, int64_t m, int d, double sigma0, int64_t cur_vector,
                                   int64_t n_vectors, int mode, int threads) {
    train_iter_scatter(num, den, w, topo, x, rho, n, m, d, sigma0, cur_vector, n_vectors, mode, threads);
}

void somref_train_epoch_fp64_f32(double* num, double* den, const float* w, const float* topo, const float* x,
                                 const float* rho, int64_t n, int64_t m, int d, double sigma0, int64_t epoch,
                                 int64_t n_epochs, int mode, int32_t* bmus_out, int threads) {
    train_epoch_fp64(num, den, w, topo, x, rho, n, m, d, sigma0, epoch, n_epochs, mode, bmus_out, threads);
}

}  // extern "C"
