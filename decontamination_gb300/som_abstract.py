"""SOM_Abstract: map state, topography, I/O and the projection calls (BMUs, activation map, errors).

Same constructor, attributes, properties and call signatures as the
reference's ``decontamination.algo.som_abstract.SOM_Abstract``
(algo/som_abstract.py:23-695). The projection calls run the libsomgb kernels
on the current CUDA device; ``enable_gpu`` and ``threads_per_blocks`` are
accepted for compatibility and ignored (there is no CPU path).
"""

import ctypes
import math
import typing

import numpy as np
import torch

from . import _device, _native
from ._dataset import dataset_to_generator_builder, device_pieces, iterate_chunks, iterate_pieces

ALGO_DEFAULT = 'auto'


class SOM_Abstract(object):
    """Self Organizing Maps (abstract class).

    Parameters
    ----------
    m : int
        Number of neuron rows.
    n : int
        Number of neuron columns.
    dim : int
        Dimensionality of the input data.
    dtype : np.float32 (default) or np.float64
        Neural network data type.
    topology : str, default None == 'hexagonal'
        Neural network topology, either 'square' or 'hexagonal'.
    """

    __MODE__ = 'abstract'

    def __init__(self, m: int, n: int, dim: int, dtype=np.float32, topology: typing.Optional[str] = None):
        self._m = int(m)
        self._n = int(n)
        self._dim = int(dim)
        self._dtype = dtype.type if hasattr(dtype, 'type') else dtype
        self._topology = topology or 'hexagonal'
        self._rebuild_topography()
        self._weights = np.empty((self._m * self._n, self._dim), dtype=self._dtype)
        self._history = np.empty((0, self._m * self._n, self._dim), dtype=self._dtype)
        self._quantization_errors = np.empty(0, dtype=np.float64)
        self._topographic_errors = np.empty(0, dtype=np.float64)
        self._header_extra = {'mode': '__MODE__'}
        self._dataset_extra = {}
        # distance-search algorithm of the projection and training passes: 'auto', 'tc' or 'fp32'
        self.bmu_algo = ALGO_DEFAULT
        self._ws = _device.Workspace()
        self._last_recheck_count = 0

    # -- topography (algo/som_abstract.py:81-111) ----------------------------------------------------------------------

    @staticmethod
    def _neuron_locations_square(m: int, n: int):
        for i in range(m):
            for j in range(n):
                yield [i, j]

    @staticmethod
    def _neuron_locations_hexagonal(m: int, n: int):
        for i in range(m):
            for j in range(n):
                yield [i + (j & 1) * 0.5, j * 0.8660254037844386]

    def _rebuild_topography(self):
        if self._topology == 'square':
            self._topography = np.array(list(SOM_Abstract._neuron_locations_square(self._m, self._n)),
                                        dtype=self._dtype)
        else:
            self._topography = np.array(list(SOM_Abstract._neuron_locations_hexagonal(self._m, self._n)),
                                        dtype=self._dtype)

    # -- initialisation (algo/som_abstract.py:115-159) -------------------------------------------------------------------

    def init_rand(self, seed: typing.Optional[int] = None) -> None:
        """Initializes the neural network randomly (U[0, 1), numpy PCG64 stream of `seed`)."""
        rng = np.random.default_rng(seed=seed)
        self._weights[...] = rng.random((self._m * self._n, self._dim), dtype=self._dtype)

    def init_from(self, other: 'SOM_Abstract') -> None:
        """Initializes the neural network from another one (same shape, dtype and topology)."""
        if self._m != other._m or self._n != other._n or self._dim != other._dim \
                or self._dtype != other._dtype or self._topology != other._topology:
            raise TypeError('Incompatible shapes, dtypes or topologies')
        self._weights[...] = other._weights

    # -- HDF5 I/O (algo/som_abstract.py:163-319; same group, attribute and dataset names) ------------------------------

    def _init_hdf5_extra(self):
        header_extra = dict(self._header_extra)
        dataset_extra = dict(self._dataset_extra)
        header_extra['m'] = '_m'
        header_extra['n'] = '_n'
        header_extra['dim'] = '_dim'
        header_extra['topology'] = '_topology'
        dataset_extra['weights'] = '_weights'
        dataset_extra['quantization_errors'] = '_quantization_errors'
        dataset_extra['topographic_errors'] = '_topographic_errors'
        return header_extra, dataset_extra

    def save(self, filename: str) -> None:
        """Saves the trained neural network to a HDF5 file (needs h5py)."""
        import h5py
        header_extra, dataset_extra = self._init_hdf5_extra()
        with h5py.File(filename, mode='w') as file:
            model_group = file.create_group('model', track_order=True)
            for name, field in header_extra.items():
                data = getattr(self, field)
                if data is not None:
                    model_group.attrs[name] = data
            for name, field in dataset_extra.items():
                data = getattr(self, field)
                if data is not None:
                    model_group.create_dataset(name, data=data, shape=data.shape, dtype=data.dtype)
        self._rebuild_topography()

    def load(self, filename: str) -> None:
        """Loads the trained neural network from a HDF5 file (needs h5py)."""
        import h5py
        header_extra, dataset_extra = self._init_hdf5_extra()
        with h5py.File(filename, mode='r') as file:
            model_group = file['model']
            for name, field in header_extra.items():
                try:
                    value = model_group.attrs[name]
                    if isinstance(value, (np.int32, np.int64)):
                        setattr(self, field, int(value))
                    elif isinstance(value, (np.float32, np.float64)):
                        setattr(self, field, float(value))
                    else:
                        setattr(self, field, value)
                except KeyError:
                    pass
            for name, field in dataset_extra.items():
                try:
                    setattr(self, field, np.array(model_group[name]).astype(self._dtype))
                except KeyError:
                    pass
        self._rebuild_topography()

    # -- properties (algo/som_abstract.py:323-447) ------------------------------------------------------------------------

    @property
    def m(self) -> int:
        """Number of neuron rows."""
        return self._m

    @property
    def n(self) -> int:
        """Number of neuron columns."""
        return self._n

    @property
    def dim(self) -> int:
        """Dimensionality of the input data."""
        return self._dim

    @property
    def dtype(self):
        """Neural network data type."""
        return self._dtype

    @property
    def topology(self) -> str:
        """Neural network topology, either 'square' or 'hexagonal'."""
        return self._topology

    @property
    def weights(self) -> np.ndarray:
        """Neural network weights with the shape [m*n, dim]."""
        return self._weights.reshape((self._m * self._n, self._dim))

    @property
    def centroids(self) -> np.ndarray:
        """Neural network weights with the shape [m, n, dim]."""
        return self._weights.reshape((self._m, self._n, self._dim))

    @property
    def quantization_errors(self) -> np.ndarray:
        """Quantization error per epoch: mean distance to the best matching unit."""
        return self._quantization_errors

    @property
    def topographic_errors(self) -> np.ndarray:
        """Topographic error per epoch: fraction of samples whose two best units are not grid neighbours."""
        return self._topographic_errors

    @property
    def last_recheck_count(self) -> int:
        """Samples the last get_winners call sent to the exact recheck (diagnostic; for a host catalogue copied in
        pieces, those of its last piece)."""
        return self._last_recheck_count

    # -- device helpers ---------------------------------------------------------------------------------------------------

    @property
    def _is_f64(self):
        return np.dtype(self._dtype) == np.float64

    @property
    def _algo(self):
        return _native.ALGOS[self.bmu_algo]

    @property
    def _penalty(self):
        # algo/som_abstract.py:575
        return 2.0 if self._topology == 'square' else 1.0

    def _device_weights(self):
        return _device.to_device(self._weights, self._dtype)

    def _device_topography(self):
        return _device.to_device(self._topography, self._dtype)

    def _record_recheck(self):
        cnt = np.zeros(1, dtype=np.int64)
        _native.call('somgb_last_recheck_count', cnt.ctypes.data, _device.stream())
        self._last_recheck_count = int(cnt[0])

    # -- projection calls -------------------------------------------------------------------------------------------------

    def compute_errors(self, dataset, dataset_weights=None, show_progress_bar: bool = False, enable_gpu: bool = True,
                       threads_per_blocks: typing.Optional[int] = None) -> typing.Tuple[float, float]:
        """Quantization and topographic errors of `dataset` (algo/som_abstract.py:528-601)."""
        if self._m * self._n < 2:
            return np.nan, np.nan
        device = _device.require_cuda()
        out = torch.zeros(3, dtype=torch.float64, device=device)
        w = self._device_weights()
        topo = self._device_topography()
        M, D = self._m * self._n, self._dim
        status = _device.StatusCheck(device)
        for xc, rc in iterate_pieces(dataset, dataset_weights, self._dtype, device):
            n = _device.rows(xc)
            if self._is_f64:
                _native.call('somgb_compute_errors_f64', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(),
                             topo.data_ptr(), M, self._penalty, out.data_ptr(), _device.stream())
            else:
                wsp, wsb = self._ws.for_op(_native.OP_ERRORS, n, M, D, self._algo, device)
                _native.call('somgb_compute_errors', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(),
                             topo.data_ptr(), M, self._penalty, self._algo, out.data_ptr(), wsp, wsb,
                             _device.stream())
                status.note(self._ws)
        o = out.cpu().numpy()
        status.check()
        return (o[0] / o[2], o[1] / o[2]) if o[2] > 0.0 else (np.nan, np.nan)

    def get_activation_map(self, dataset, dataset_weights=None, show_progress_bar: bool = False,
                           enable_gpu: bool = True, threads_per_blocks: typing.Optional[int] = None) -> np.ndarray:
        """Per-unit sum of the weights of the samples it wins, shape (m, n) (algo/som_abstract.py:605-666)."""
        device = _device.require_cuda()
        M, D = self._m * self._n, self._dim
        hist = torch.zeros(M, dtype=torch.float64, device=device)
        w = self._device_weights()
        status = _device.StatusCheck(device)
        for xc, rc in iterate_pieces(dataset, dataset_weights, self._dtype, device):
            n = _device.rows(xc)
            if self._is_f64:
                _native.call('somgb_count_bmus_f64', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(), M,
                             hist.data_ptr(), _device.stream())
            else:
                wsp, wsb = self._ws.for_op(_native.OP_COUNT_BMUS, n, M, D, self._algo, device)
                _native.call('somgb_count_bmus', xc.data_ptr(), _device.ptr(rc), n, D, w.data_ptr(), M, self._algo,
                             hist.data_ptr(), wsp, wsb, _device.stream())
                status.note(self._ws)
        h = hist.cpu().numpy()
        status.check()
        return h.astype(self._dtype).reshape((self._m, self._n))

    def get_footprint_maps(self, dataset, dataset_weights=None) -> typing.Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(weighted activation map, unweighted activation map, winners) of one array in a single BMU pass: the fused
        form of ``get_activation_map(dataset, dataset_weights)``, ``get_activation_map(dataset)`` and
        ``get_winners(dataset)`` that Decontamination_SOM calls on its footprint (decontamination_som.py:596,
        640-641). Same values as the three calls."""
        device = _device.require_cuda()
        M, D = self._m * self._n, self._dim
        x, rho, pieces = device_pieces(dataset, dataset_weights, self._dtype, device)
        n = _device.rows(x)
        winners = torch.empty(n, dtype=torch.int32, device=device)
        hist_w = torch.zeros(M, dtype=torch.float64, device=device)
        hist_c = torch.zeros(M, dtype=torch.float64, device=device)
        w = self._device_weights()
        status = _device.StatusCheck(device)
        for a, b in pieces:
            xp, op = x[a:b], winners[a:b]
            rp = None if rho is None else rho[a:b]
            if self._is_f64:
                _native.call('somgb_footprint_maps_f64', xp.data_ptr(), _device.ptr(rp), b - a, D, w.data_ptr(), M,
                             op.data_ptr(), hist_w.data_ptr(), hist_c.data_ptr(), _device.stream())
            else:
                wsp, wsb = self._ws.for_op(_native.OP_FIND_BMUS, b - a, M, D, self._algo, device)
                _native.call('somgb_footprint_maps', xp.data_ptr(), _device.ptr(rp), b - a, D, w.data_ptr(), M,
                             self._algo, op.data_ptr(), hist_w.data_ptr(), hist_c.data_ptr(), wsp, wsb,
                             _device.stream())
                status.note(self._ws)
        cat = hist_w.cpu().numpy().astype(self._dtype).reshape((self._m, self._n))
        foot = hist_c.cpu().numpy().astype(self._dtype).reshape((self._m, self._n))
        res = winners.cpu().numpy()
        status.check()
        return cat, foot, res

    def get_winners(self, dataset, enable_gpu: bool = True,
                    threads_per_blocks: typing.Optional[int] = None) -> np.ndarray:
        """Best matching unit index of every row of `dataset`, int32 (algo/som_abstract.py:670-695)."""
        device = _device.require_cuda()
        M, D = self._m * self._n, self._dim
        x, _, pieces = device_pieces(dataset, None, self._dtype, device)
        out = torch.empty(_device.rows(x), dtype=torch.int32, device=device)
        w = self._device_weights()
        status = _device.StatusCheck(device)
        for a, b in pieces:
            xp, op = x[a:b], out[a:b]
            if self._is_f64:
                _native.call('somgb_find_bmus_f64', xp.data_ptr(), b - a, D, w.data_ptr(), M, op.data_ptr(),
                             _device.stream())
            else:
                wsp, wsb = self._ws.for_op(_native.OP_FIND_BMUS, b - a, M, D, self._algo, device)
                _native.call('somgb_find_bmus', xp.data_ptr(), b - a, D, w.data_ptr(), M, self._algo, op.data_ptr(),
                             wsp, wsb, _device.stream())
                status.note(self._ws)
        if not self._is_f64:
            self._record_recheck()
        res = out.cpu().numpy()
        status.check()
        return res
