"""CPU oracle for the batch-SOM hot path (ctypes front end of libsomref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, as the checker or as the timed CPU baseline. The
product package never imports it.

`OracleSOM` restates the host-side control flow of the reference's
`SOM_Batch` (algo/som_batch.py:214-505) and `SOM_Abstract`
(algo/som_abstract.py:81-111, 528-695) on top of the C restatements of its
kernels in somref.cpp. Arithmetic modes: 'numba' (the compiled reference),
'pyref' (the reference's pure-Python path under NumPy 2), 'exact' (float64).

Accumulation for training:
  'scatter'  the reference formulation (per sample, for every unit, float32
             adds of h*x in sample order; OpenMP atomics when threads > 1);
  'fp64'     the same update in float64, factored as num = H.S, den = H.c
             (the float64 oracle the GPU weights are measured against).
"""

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libsomref.so')

MODES = {'numba': 0, 'pyref': 1, 'exact': 2}
FLOAT_EPS = 1.0e-12          # algo/som_batch.py:24

_lib = None


def build():
    subprocess.check_call(['sh', os.path.join(HERE, 'build.sh')])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        P, I64, I32, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        sig = {
            'somref_find_bmus_f32': [P, I64, I32, P, I64, I32, P, I32],
            'somref_find_bmus_f64': [P, I64, I32, P, I64, I32, P, I32],
            'somref_top2_f32': [P, I64, I32, P, I64, I32, P, P, P, P, I32],
            'somref_count_bmus_f32': [P, I64, I32, P, P, I64, I32, P, I32],
            'somref_count_bmus_f64': [P, I64, I32, P, P, I64, I32, P, I32],
            'somref_compute_errors_f32': [P, P, I64, I32, P, P, I64, D, I32, P, I32],
            'somref_compute_errors_f64': [P, P, I64, I32, P, P, I64, D, I32, P, I32],
            'somref_train_epoch_scatter_f32': [P, P, P, P, P, P, I64, I64, I32, D, I64, I64, I32, I32],
            'somref_train_epoch_scatter_f64': [P, P, P, P, P, P, I64, I64, I32, D, I64, I64, I32, I32],
            'somref_train_iter_scatter_f32': [P, P, P, P, P, P, I64, I64, I32, D, I64, I64, I32, I32],
            'somref_train_iter_scatter_f64': [P, P, P, P, P, P, I64, I64, I32, D, I64, I64, I32, I32],
            'somref_train_epoch_fp64_f32': [P, P, P, P, P, P, I64, I64, I32, D, I64, I64, I32, P, I32],
        }
        for name, argtypes in sig.items():
            fn = getattr(_lib, name)
            fn.argtypes = argtypes
            fn.restype = None
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _sfx(dtype):
    return 'f32' if np.dtype(dtype) == np.float32 else 'f64'


def topography(m, n, topology, dtype=np.float32):
    """Unit coordinates, algo/som_abstract.py:81-111 (square [i, j]; hexagonal [i + (j&1)/2, j*sqrt(3)/2])."""
    if topology == 'square':
        pts = [[i, j] for i in range(m) for j in range(n)]
    else:
        pts = [[i + (j & 1) * 0.5, j * 0.8660254037844386] for i in range(m) for j in range(n)]
    return np.array(pts, dtype=dtype)


def decay(epoch, epochs):
    """asymptotic_decay_cpu, algo/__init__.py:64-67."""
    return 1.0 / (1.0 + 2.0 * epoch / epochs)


def sqdist_exact(a, b):
    """|a - b|^2 in float64 (the tie-adjudication distance)."""
    t = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return float(np.dot(t, t))


def to_builder(dataset):
    """dataset_to_generator_builder, algo/__init__.py:21-27."""
    if dataset is None:
        return None
    return dataset if callable(dataset) else (lambda: lambda: (dataset,))


# ---------------------------------------------------------------------------------------------------------------------
# kernel wrappers
# ---------------------------------------------------------------------------------------------------------------------

def find_bmus(w, x, mode='numba', threads=0):
    x = np.ascontiguousarray(x, dtype=w.dtype)
    out = np.empty(x.shape[0], dtype=np.int32)
    getattr(lib(), f'somref_find_bmus_{_sfx(w.dtype)}')(_p(w), w.shape[0], w.shape[1], _p(x), x.shape[0],
                                                       MODES[mode], _p(out), threads)
    return out


def top2(w, x, mode='numba', threads=0):
    """Per-sample (bmu1, bmu2, d1, d2) with the selection rule of _compute_errors_xpu."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.shape[0]
    i1 = np.empty(n, np.int32); i2 = np.empty(n, np.int32)
    d1 = np.empty(n, np.float64); d2 = np.empty(n, np.float64)
    lib().somref_top2_f32(_p(w), w.shape[0], w.shape[1], _p(x), n, MODES[mode], _p(i1), _p(i2), _p(d1), _p(d2),
                          threads)
    return i1, i2, d1, d2


def count_bmus(w, x, rho=None, mode='numba', threads=0, hist=None):
    x = np.ascontiguousarray(x, dtype=w.dtype)
    rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
    if hist is None:
        hist = np.zeros(w.shape[0], dtype=np.float64)
    getattr(lib(), f'somref_count_bmus_{_sfx(w.dtype)}')(_p(w), w.shape[0], w.shape[1], _p(x), _p(rho), x.shape[0],
                                                        MODES[mode], _p(hist), threads)
    return hist


def compute_errors_raw(w, topo, x, rho=None, penalty=2.0, mode='numba', threads=0, out=None):
    x = np.ascontiguousarray(x, dtype=w.dtype)
    rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
    if out is None:
        out = np.zeros(3, dtype=np.float64)
    getattr(lib(), f'somref_compute_errors_{_sfx(w.dtype)}')(_p(w), _p(topo), w.shape[0], w.shape[1], _p(x), _p(rho),
                                                            x.shape[0], penalty, MODES[mode], _p(out), threads)
    return out


def train_epoch_scatter(num, den, w, topo, x, rho, sigma0, epoch, n_epochs, mode='numba', threads=1):
    x = np.ascontiguousarray(x, dtype=w.dtype)
    rho = np.ascontiguousarray(rho, dtype=w.dtype)
    getattr(lib(), f'somref_train_epoch_scatter_{_sfx(w.dtype)}')(
        _p(num), _p(den), _p(w), _p(topo), _p(x), _p(rho), x.shape[0], w.shape[0], w.shape[1], float(sigma0),
        epoch, n_epochs, MODES[mode], threads)


def train_iter_scatter(num, den, w, topo, x, rho, sigma0, cur_vector, n_vectors, mode='numba', threads=1):
    x = np.ascontiguousarray(x, dtype=w.dtype)
    rho = np.ascontiguousarray(rho, dtype=w.dtype)
    getattr(lib(), f'somref_train_iter_scatter_{_sfx(w.dtype)}')(
        _p(num), _p(den), _p(w), _p(topo), _p(x), _p(rho), x.shape[0], w.shape[0], w.shape[1], float(sigma0),
        cur_vector, n_vectors, MODES[mode], threads)


def train_epoch_fp64(num, den, w, topo, x, rho, sigma0, epoch, n_epochs, mode='numba', threads=0, bmus=None):
    x = np.ascontiguousarray(x, dtype=np.float32)
    rho = np.ascontiguousarray(rho, dtype=np.float32)
    lib().somref_train_epoch_fp64_f32(_p(num), _p(den), _p(w), _p(topo), _p(x), _p(rho), x.shape[0], w.shape[0],
                                      w.shape[1], float(sigma0), epoch, n_epochs, MODES[mode], _p(bmus), threads)


# ---------------------------------------------------------------------------------------------------------------------
# SOM_Batch restatement
# ---------------------------------------------------------------------------------------------------------------------

class OracleSOM:
    """Host-side control flow of the reference's SOM_Batch over the C kernels."""

    def __init__(self, m, n, dim, dtype=np.float32, topology=None, sigma=None, mode='numba', threads=1,
                 accumulate='scatter'):
        self.m, self.n, self.dim = int(m), int(n), int(dim)
        self.dtype = np.dtype(dtype).type
        self.topology = topology or 'hexagonal'
        self.sigma = max(m, n) / 2.0 if sigma is None else float(sigma)
        self.mode, self.threads, self.accumulate = mode, threads, accumulate
        self.topo = topography(self.m, self.n, self.topology, self.dtype)
        self.weights = np.zeros((self.m * self.n, self.dim), dtype=self.dtype)
        self.history = np.empty((0, self.m * self.n, self.dim), dtype=self.dtype)
        self.quantization_errors = np.empty(0)
        self.topographic_errors = np.empty(0)

    @property
    def penalty(self):
        return 2.0 if self.topology == 'square' else 1.0

    def get_winners(self, x):
        return find_bmus(self.weights, x, self.mode, self.threads)

    def get_activation_map(self, dataset, dataset_weights=None):
        hist = np.zeros(self.m * self.n, dtype=np.float64)
        for xc, rc in self._chunks(dataset, dataset_weights):
            count_bmus(self.weights, xc, rc, self.mode, self.threads, hist)
        return hist.astype(self.dtype).reshape(self.m, self.n)

    def compute_errors(self, dataset, dataset_weights=None):
        if self.m * self.n < 2:
            return math.nan, math.nan
        out = np.zeros(3)
        for xc, rc in self._chunks(dataset, dataset_weights):
            compute_errors_raw(self.weights, self.topo, xc, rc, self.penalty, self.mode, self.threads, out)
        return (out[0] / out[2], out[1] / out[2]) if out[2] > 0.0 else (math.nan, math.nan)

    @staticmethod
    def _chunks(dataset, dataset_weights):
        db, wb = to_builder(dataset), to_builder(dataset_weights)
        if wb is None:
            for xc in db()():
                yield xc, None
        else:
            for xc, rc in zip(db()(), wb()()):
                if xc.shape[0] != rc.shape[0]:
                    raise ValueError('`dataset` and `dataset_weights` chunks must be aligned')
                yield xc, rc

    def _divide(self, num, den):
        den2 = den[:, None]
        return np.divide(num, den2, out=np.zeros_like(num), where=den2 > FLOAT_EPS).astype(self.dtype)

    def train(self, dataset, dataset_weights=None, n_epochs=None, n_vectors=None, use_best_epoch=True,
              stop_quantization_error=None, stop_topographic_error=None):
        sq = -1.0e6 if stop_quantization_error is None else stop_quantization_error
        st = -1.0e6 if stop_topographic_error is None else stop_topographic_error
        M, D = self.m * self.n, self.dim
        if n_epochs is not None and n_vectors is None:
            self.history = np.empty((n_epochs, M, D), dtype=self.dtype)
            self.quantization_errors = np.full(n_epochs, np.nan)
            self.topographic_errors = np.full(n_epochs, np.nan)
            for e in range(n_epochs):
                if self.accumulate == 'fp64':
                    num = np.zeros((M, D)); den = np.zeros(M)
                else:
                    num = np.zeros((M, D), self.dtype); den = np.zeros(M, self.dtype)
                for xc, rc in self._chunks(dataset, dataset_weights):
                    rc = np.ones(xc.shape[0], self.dtype) if rc is None else rc
                    if self.accumulate == 'fp64':
                        n_ = np.zeros((M, D)); d_ = np.zeros(M)
                        train_epoch_fp64(n_, d_, self.weights, self.topo, xc, rc, self.sigma, e, n_epochs,
                                         self.mode, self.threads)
                        num += n_; den += d_
                    else:
                        train_epoch_scatter(num, den, self.weights, self.topo, xc, rc, self.sigma, e, n_epochs,
                                            self.mode, self.threads)
                self.weights = self._divide(num, den)
                self.history[e] = self.weights
                qe, te = self.compute_errors(dataset, dataset_weights)
                self.quantization_errors[e] = qe
                self.topographic_errors[e] = te
                if qe <= sq and te <= st:
                    break
        elif n_epochs is None and n_vectors is not None:
            self.history = np.empty((1, M, D), dtype=self.dtype)
            self.quantization_errors = np.zeros(1)
            self.topographic_errors = np.zeros(1)
            num = np.zeros((M, D), self.dtype); den = np.zeros(M, self.dtype)
            cur = 0
            for xc, rc in self._chunks(dataset, dataset_weights):
                count = min(xc.shape[0], n_vectors - cur)
                rc = np.ones(count, self.dtype) if rc is None else rc[:count]
                train_iter_scatter(num, den, self.weights, self.topo, xc[:count], rc, self.sigma, cur, n_vectors,
                                   self.mode, self.threads)
                cur += count
                if cur >= n_vectors:
                    break
            self.weights = self._divide(num, den)
            self.history[0] = self.weights
            qe, te = self.compute_errors(dataset, dataset_weights)
            self.quantization_errors[0] = qe
            self.topographic_errors[0] = te
        else:
            raise ValueError('Invalid training method, specify either `n_epochs` or `n_vectors`')
        if use_best_epoch:
            self.weights = self.history[np.nanargmin(self.quantization_errors)].copy()
