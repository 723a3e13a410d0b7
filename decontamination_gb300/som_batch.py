"""SOM_Batch: batch self-organising map training on GB300.

Drop-in for the reference's ``decontamination.algo.som_batch.SOM_Batch``
(algo/som_batch.py:29-505): same constructor, ``train`` signature, attributes
(``_weights``, ``_history``, ``_quantization_errors``,
``_topographic_errors``, ``_sigma``, ``_n_epochs``, ``_n_vectors``) and HDF5
header. ``enable_gpu`` / ``threads_per_blocks`` are accepted and ignored.

Epoch mode, per epoch e (reference: :285-374):
  1. one fused device pass over the data with the weights w(e): BMUs (training
     semantics), per-BMU sums S and c in float64, and the compute_errors sums
     of w(e) — which are the errors the reference computes at the end of epoch
     e-1 (the weights of both passes are identical), so E epochs take E+1
     passes over the data instead of 2E;
  2. the neighbourhood contraction w(e+1) = (H.S)/(H.c) on the device.
The data stay resident on the device for all epochs when they are an array.
The host synchronises once per epoch only when a stop threshold is set.
"""

import math
import typing

import numpy as np
import torch

from . import _device, _native
from ._dataset import device_pieces, is_array, iterate_chunks, raw_chunks
from .som_abstract import SOM_Abstract

FLOAT_EPS = 1.0e-12   # algo/som_batch.py:24


def asymptotic_decay(epoch: int, epochs: int) -> float:
    """algo/__init__.py:64-74."""
    return 1.0 / (1.0 + 2.0 * epoch / epochs)


class SOM_Batch(SOM_Abstract):
    """Self Organizing Maps (standard batch implementation) with constant memory usage.

    Parameters
    ----------
    m, n : int
        Number of neuron rows / columns.
    dim : int
        Dimensionality of the input data.
    dtype : np.float32 (default) or np.float64
        Neural network data type.
    topology : str, default None == 'hexagonal'
        Neural network topology, either 'square' or 'hexagonal'.
    sigma : float, default None == max(m, n) / 2
        Starting value of the neighborhood radius.
    """

    __MODE__ = 'batch'

    def __init__(self, m: int, n: int, dim: int, dtype=np.float32, topology: typing.Optional[str] = None,
                 sigma: float = None):
        super().__init__(m, n, dim, dtype, topology)
        self._sigma = max(m, n) / 2.0 if sigma is None else float(sigma)
        self._n_epochs = 0
        self._n_vectors = 0
        self._header_extra = {'mode': '__MODE__', 'sigma': '_sigma', 'n_epochs': '_n_epochs',
                              'n_vectors': '_n_vectors'}

    @property
    def sigma(self) -> float:
        """Starting value of the neighborhood radius."""
        return self._sigma

    # ------------------------------------------------------------------------------------------------------------------

    def _epoch_sigma(self, epoch, total):
        # sigma0 is passed to the reference kernel in the map dtype and multiplied in float64 (som_batch.py:107-110)
        s = float(self._dtype(self._sigma)) * asymptotic_decay(epoch, total)
        return FLOAT_EPS if s < FLOAT_EPS else s

    def _with_bounds(self, xc, rc, device):
        """A chunk plus the per-feature bounds of its fixed-point sums (float32 maps), valid for every epoch."""
        if self._is_f64:
            return xc, rc, None
        bounds = torch.zeros(self._dim + 1, dtype=torch.float32, device=device)
        _native.call('somgb_feature_bounds', xc.data_ptr(), _device.ptr(rc), _device.rows(xc), self._dim,
                     bounds.data_ptr(), _device.stream())
        return xc, rc, bounds

    def _chunk_source(self, dataset, dataset_weights, device):
        """Chunks for the epoch loop, as (x, rho, bounds, pieces). Arrays are uploaded once and reused by every epoch:
        the first epoch gets them with the row pieces of their upload (its passes overlap the copy, and the bounds
        are accumulated piece by piece), later epochs whole (pieces None, bounds complete). Generator datasets are
        uploaded every epoch, as the reference does."""
        if (dataset is None or is_array(dataset)) and (dataset_weights is None or is_array(dataset_weights)):
            resident = self._resident = []
            self._regroup_bufs = {}

            def first():
                for xr, rr in raw_chunks(dataset, dataset_weights):
                    xd, rd, pieces = device_pieces(xr, rr, self._dtype, device)
                    bounds = None if self._is_f64 else torch.zeros(self._dim + 1, dtype=torch.float32, device=device)
                    resident.append((xd, rd, bounds, None))
                    yield xd, rd, bounds, pieces

            return lambda: first() if not resident else iter(list(resident))
        self._resident = None
        return lambda: ((*self._with_bounds(xc, rc, device), None)
                        for xc, rc in iterate_chunks(dataset, dataset_weights, self._dtype, device))

    def _bmu_buffer(self, n, device):
        buf = getattr(self, '_bmu_buf', None)
        if buf is None or buf.numel() < n or buf.device != device:
            buf = self._bmu_buf = torch.empty(max(n, 1), dtype=torch.int32, device=device)
        return buf

    def _piece_pass(self, xd, rd, a, b, last, with_errors, w, topo, err, e, device):
        """Rows a..b of a resident chunk: the training pass (BMUs; error sums of the previous epoch's map when e > 0)
        or, after the last epoch, the error pass. Float64 maps train in one call per chunk (_accumulate)."""
        M, D = self._m * self._n, self._dim
        xc, rc = xd[a:b], (None if rd is None else rd[a:b])
        n = b - a
        status = self._status
        if last:
            if not with_errors:
                return
            if self._is_f64:
                _native.call('somgb_compute_errors_f64', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(),
                             topo.data_ptr(), M, self._penalty, err.data_ptr(), _device.stream())
            else:
                wsp, wsb = self._ws.for_op(_native.OP_ERRORS, n, M, D, self._algo, device)
                _native.call('somgb_compute_errors', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(),
                             topo.data_ptr(), M, self._penalty, self._algo, err.data_ptr(), wsp, wsb,
                             _device.stream())
                status.note(self._ws)
            return
        if self._is_f64:
            return
        bmu = self._bmu_buffer(_device.rows(xd), device)[a:b]
        wsp, wsb = self._ws.for_op(_native.OP_FIND_BMUS, n, M, D, self._algo, device)
        _native.call('somgb_train_bmu_pass', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(), topo.data_ptr(), M,
                     self._penalty, self._algo, bmu.data_ptr(), _device.ptr(err if e > 0 else None), wsp, wsb,
                     _device.stream())
        status.note(self._ws)

    def _accumulate(self, xd, rd, bounds, S, c, w, topo, err):
        """The per-BMU sums of a whole chunk after its BMU passes (float64 maps: the fused float64 epoch pass, with
        the error sums `err` of the previous epoch's map)."""
        n = _device.rows(xd)
        M, D = self._m * self._n, self._dim
        if self._is_f64:
            wsp, wsb = self._ws.for_op(_native.OP_EPOCH, n, M, D, _native.ALGO_FP32, xd.device)
            _native.call('somgb_train_epoch_pass_f64', xd.data_ptr(), _device.ptr(rd), n, D, w.data_ptr(),
                         topo.data_ptr(), M, self._penalty, S.data_ptr(), c.data_ptr(), _device.ptr(err), wsp, wsb,
                         _device.stream())
            return
        _native.call('somgb_accumulate', xd.data_ptr(), _device.ptr(rd), self._bmu_buffer(n, xd.device).data_ptr(),
                     n, D, M, bounds.data_ptr(), S.data_ptr(), c.data_ptr(), _device.stream())

    def _regroups(self, n):
        """Whether the rows of a resident chunk of n rows are regrouped by BMU between training epochs (not after the
        last one: the final error pass keeps the grouping of the epoch before): when its passes take the tensor-core
        path, whose second sweep then recomputes only the column tiles holding candidates, and the map has more than
        one column tile (256 units)."""
        M = self._m * self._n
        if self._is_f64 or M <= 256 or n < 1024:
            return False
        algo = self._algo
        if algo == _native.ALGO_FP32 or (algo == _native.ALGO_AUTO and n * M < (1 << 22)):
            return False   # the CUDA-core form (AUTO takes it below 2^22 sample-units) has no second sweep to spare
        return bool(_native.lib().somgb_algo_supported(_native.ALGO_TC, n, M, self._dim))

    def _regroup(self, k, xd, rd, bounds, device):
        """Replaces resident chunk k by its rows regrouped by the BMUs the epoch just found (somgb_sort_rows): each
        row keeps its values and weight, so every result is unchanged. The rows go to one of two buffers allocated
        here for the chunk, the one that is not the source; the caller's own tensors are never written."""
        n, D, M = _device.rows(xd), self._dim, self._m * self._n
        bufs = self._regroup_bufs.setdefault(k, [])
        target = next((b for b in bufs if b[0] is not xd), None)
        if target is None:
            target = (torch.empty_like(xd), None if rd is None else torch.empty_like(rd))
            bufs.append(target)
        xs, rs = target
        if getattr(self, '_sort_ws', None) is None:
            self._sort_ws = _device.Workspace()
        wsp, wsb = self._sort_ws.get(int(_native.lib().somgb_sort_rows_workspace_bytes(M)), device)
        _native.call('somgb_sort_rows', xd.data_ptr(), _device.ptr(rd), self._bmu_buffer(n, device).data_ptr(), n, D,
                     M, xs.data_ptr(), _device.ptr(rs), wsp, wsb, _device.stream())
        self._resident[k] = (xs, rs, bounds, None)

    def _update(self, S, c, topo, sigma, w_out):
        """num = H S, den = H c, w = num / den, with the map's grid topography factorised by axis."""
        D = self._dim
        nbytes = int(_native.lib().somgb_neighbourhood_grid_workspace_bytes(self._m, self._n, D))
        if getattr(self, '_upd_ws', None) is None:
            self._upd_ws = _device.Workspace()
        wsp, wsb = self._upd_ws.get(nbytes, w_out.device)
        name = 'somgb_neighbourhood_update_grid_f64' if self._is_f64 else 'somgb_neighbourhood_update_grid'
        _native.call(name, S.data_ptr(), c.data_ptr(), topo.data_ptr(), self._m, self._n, D, sigma,
                     w_out.data_ptr(), None, None, wsp, wsb, _device.stream())

    @staticmethod
    def _errors_of(err_host):
        return (err_host[0] / err_host[2], err_host[1] / err_host[2]) if err_host[2] > 0.0 else (np.nan, np.nan)

    # ------------------------------------------------------------------------------------------------------------------

    def train(self, dataset, dataset_weights=None, n_epochs: typing.Optional[int] = None,
              n_vectors: typing.Optional[int] = None, use_best_epoch: bool = True,
              stop_quantization_error: typing.Optional[float] = None,
              stop_topographic_error: typing.Optional[float] = None, show_progress_bar: bool = False,
              enable_gpu: bool = True, threads_per_blocks: typing.Optional[int] = None) -> None:
        """Trains the neural network with `n_epochs` epochs or on `n_vectors` vectors (algo/som_batch.py:214-505).

        w_j(e+1) = sum_i h_ji x_i / sum_i h_ji, h_ji = rho_i exp(-|t_j - t_bmu(x_i)|^2 / (2 sigma(e)^2)),
        sigma(e) = sigma / (1 + 2 e / e_tot).
        """
        self._n_epochs = n_epochs
        self._n_vectors = n_vectors
        if n_epochs is not None and n_vectors is None:
            self._train_epochs(dataset, dataset_weights, n_epochs, stop_quantization_error, stop_topographic_error)
        elif n_epochs is None and n_vectors is not None:
            self._train_vectors(dataset, dataset_weights, n_vectors)
        else:
            raise ValueError('Invalid training method, specify either `n_epochs` or `n_vectors`')
        if use_best_epoch:
            self._weights[:] = self._history[np.nanargmin(self._quantization_errors)]

    def _train_epochs(self, dataset, dataset_weights, n_epochs, stop_qe, stop_te):
        device = _device.require_cuda()
        sq = -1.0e6 if stop_qe is None else stop_qe
        st = -1.0e6 if stop_te is None else stop_te
        check_stop = stop_qe is not None or stop_te is not None
        M, D = self._m * self._n, self._dim
        td = _device.torch_dtype(self._dtype)
        with_errors = M >= 2   # compute_errors returns (nan, nan) below two units (som_abstract.py:547-549)

        chunks = self._chunk_source(dataset, dataset_weights, device)
        self._status = _device.StatusCheck(device)
        topo = self._device_topography()
        w = self._device_weights()
        history = torch.empty((n_epochs, M, D), dtype=td, device=device)
        S = torch.empty((M, D), dtype=torch.float64, device=device)
        c = torch.empty(M, dtype=torch.float64, device=device)
        errs = torch.zeros((n_epochs + 1, 3), dtype=torch.float64, device=device)

        done = n_epochs            # epochs whose update was kept
        for e in range(n_epochs + 1):
            S.zero_()
            c.zero_()
            err = errs[e] if with_errors else None
            last = e == n_epochs
            for k, (xd, rd, bounds, pieces) in enumerate(chunks()):
                if pieces is None:
                    pieces = [(0, _device.rows(xd))]
                elif bounds is not None:
                    # the first sight of an uploaded chunk: its fixed-point bounds, piece by piece
                    for a, b in pieces:
                        _native.call('somgb_feature_bounds', xd[a:b].data_ptr(), _device.ptr(rd[a:b] if rd is not None
                                     else None), b - a, D, bounds.data_ptr(), _device.stream())
                        self._piece_pass(xd, rd, a, b, last, with_errors, w, topo, err, e, device)
                    if not last:
                        self._accumulate(xd, rd, bounds, S, c, w, topo, err if e > 0 else None)
                        if self._resident is not None and e + 1 < n_epochs and self._regroups(_device.rows(xd)):
                            self._regroup(k, xd, rd, bounds, device)
                    continue
                for a, b in pieces:
                    self._piece_pass(xd, rd, a, b, last, with_errors, w, topo, err, e, device)
                if not last:
                    self._accumulate(xd, rd, bounds, S, c, w, topo, err if e > 0 else None)
                    if self._resident is not None and e + 1 < n_epochs and self._regroups(_device.rows(xd)):
                        self._regroup(k, xd, rd, bounds, device)
            if check_stop and e > 0 and with_errors:
                qe, te = self._errors_of(errs[e].cpu().numpy())
                if qe <= sq and te <= st:
                    done = e          # the reference stops after epoch e-1 (som_batch.py:368-374)
                    break
            if last:
                break
            w_next = torch.empty_like(w)
            self._update(S, c, topo, self._epoch_sigma(e, n_epochs), w_next)
            history[e].copy_(w_next)
            w = w_next

        self._history = np.empty((n_epochs, M, D), dtype=self._dtype)
        self._history[:done] = history[:done].cpu().numpy()
        self._quantization_errors = np.full(n_epochs, np.nan, dtype=np.float64)
        self._topographic_errors = np.full(n_epochs, np.nan, dtype=np.float64)
        if with_errors:
            eh = errs.cpu().numpy()
            for e in range(done):
                self._quantization_errors[e], self._topographic_errors[e] = self._errors_of(eh[e + 1])
        self._weights[:] = history[done - 1].cpu().numpy() if done > 0 else self._weights
        self._resident, self._regroup_bufs = None, {}   # the catalogue's device copies go with this call
        self._status.check()

    def _train_vectors(self, dataset, dataset_weights, n_vectors):
        device = _device.require_cuda()
        M, D = self._m * self._n, self._dim
        td = _device.torch_dtype(self._dtype)
        topo = self._device_topography()
        w = self._device_weights()
        num = torch.zeros((M, D), dtype=torch.float64, device=device)
        den = torch.zeros(M, dtype=torch.float64, device=device)
        sigma0 = float(self._dtype(self._sigma))
        cur = 0
        grid = not self._is_f64 and D <= 64   # float32 maps: the grid-factorised pass, BMUs by bmu_algo
        status = _device.StatusCheck(device)
        for xc, rc in iterate_chunks(dataset, dataset_weights, self._dtype, device):
            count = min(_device.rows(xc), n_vectors - cur)
            xk = xc[:count]
            rk = None if rc is None else rc[:count]
            if grid:
                wsp, wsb = self._ws.for_op(_native.OP_EPOCH, count, M, D, self._algo, device)
                _native.call('somgb_train_iter_pass_grid', xk.data_ptr(), _device.ptr(rk), count, D, w.data_ptr(),
                             topo.data_ptr(), self._m, self._n, sigma0, cur, n_vectors, self._algo, num.data_ptr(),
                             den.data_ptr(), wsp, wsb, _device.stream())
                status.note(self._ws)
            else:
                name = 'somgb_train_iter_pass_f64' if self._is_f64 else 'somgb_train_iter_pass'
                wsp, wsb = self._ws.for_op(_native.OP_EPOCH, count, M, D, _native.ALGO_FP32, device)
                _native.call(name, xk.data_ptr(), _device.ptr(rk), count, D, w.data_ptr(), topo.data_ptr(), M,
                             sigma0, cur, n_vectors, num.data_ptr(), den.data_ptr(), wsp, wsb, _device.stream())
            cur += count
            if cur >= n_vectors:
                break
        status.check()   # a bounded wait that gave up fails the call before its sums are used
        w_new = torch.empty((M, D), dtype=td, device=device)
        _native.call('somgb_divide_f64' if self._is_f64 else 'somgb_divide', num.data_ptr(), den.data_ptr(), M, D,
                     w_new.data_ptr(), _device.stream())
        self._history = np.empty((1, M, D), dtype=self._dtype)
        self._history[0] = w_new.cpu().numpy()
        self._weights[:] = self._history[0]
        self._quantization_errors = np.zeros(1, dtype=np.float64)
        self._topographic_errors = np.zeros(1, dtype=np.float64)
        errors = self.compute_errors(dataset, dataset_weights)
        self._quantization_errors[0] = errors[0]
        self._topographic_errors[0] = errors[1]
