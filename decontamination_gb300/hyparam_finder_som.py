"""HypParamFinder_SOM: the grid search over map size and neighbourhood radius, on the GPU.

Same API and result as the reference's ``decontamination.algo.hyparam_finder_som.HypParamFinder_SOM`` (batch mode,
algo/hyparam_finder_som.py:20-222): with m_ref = sqrt(5 sqrt(N)) (N the number of rows, or the sum of the weights),
8 map sizes from 1.5 m_ref down to 0.5 m_ref and, for each size m, 8 radii m / linspace(8, 1); every grid point is a
PCA-initialised ``SOM_Batch`` trained for ``n_epochs``; the point with the lowest quantization error (at its best
epoch with ``use_best_epoch``) wins. ``find`` returns (m, alpha, sigma, epoch index, QEs, TEs) of that point.

GB300 form of the same search: the catalogue is uploaded once and stays resident for all the grid points (the
reference re-reads it for every covariance and every epoch of every training), and the covariance is computed once
(it depends on the dataset only; the reference recomputes it for every grid point). Online-SOM grids (batch=False)
need ``SOM_Online``, which this package does not provide.
"""

import math
import typing

import numpy as np
import torch

from . import _device
from ._dataset import dataset_to_generator_builder, is_array
from .covariance import Covariance
from .som_batch import SOM_Batch
from .som_pca import SOM_PCA

__all__ = ['HypParamFinder_SOM']


class HypParamFinder_SOM(object):
    """Estimates the best hyperparameters (giving the best quantization error) using a grid."""

    M_MIN = 0.5
    M_MAX = 1.5
    M_NB_OF_STEPS = 8

    Σ_MIN = 1.0
    Σ_MAX = 8.0
    Σ_NB_OF_STEPS = 8

    ALPHA_LIST = [0.05, 0.1, 0.2, 0.3, 0.4]

    def __init__(self, dataset, dataset_weights=None, topology: typing.Optional[str] = None, batch: bool = True,
                 use_best_epoch: bool = True, show_progress_bar: bool = True, enable_gpu: bool = True,
                 threads_per_blocks: typing.Optional[int] = None):
        self._dataset = dataset
        self._dataset_weights = dataset_weights
        self._topology = topology
        self._batch = batch
        self._use_best_epoch = use_best_epoch
        self._show_progress_bar = show_progress_bar
        self._enable_gpu = enable_gpu
        self._threads_per_blocks = threads_per_blocks

    def grid(self) -> typing.List[typing.Tuple[int, float]]:
        """The (m, sigma) points in the reference's scan order (hyparam_finder_som.py:140-160)."""
        size = 0.0
        if self._dataset_weights is None:
            for vectors in dataset_to_generator_builder(self._dataset)()():
                size += vectors.shape[0]
        else:
            for weights in dataset_to_generator_builder(self._dataset_weights)()():
                size += float(np.sum(np.asarray(weights.cpu() if isinstance(weights, torch.Tensor) else weights)))
        m_ref = np.sqrt(5.0 * np.sqrt(size))
        points = []
        m_list = np.unique(np.linspace(self.M_MAX * m_ref, self.M_MIN * m_ref, num=self.M_NB_OF_STEPS, dtype=float))
        for m in m_list:
            sigma_list = np.unique(m / np.linspace(self.Σ_MAX, self.Σ_MIN, num=self.Σ_NB_OF_STEPS, dtype=float))
            for sigma in sigma_list:
                points.append((round(m), float(sigma)))
        return points

    def find(self, n_epochs):
        """Finds the best hyperparameters: (m, alpha, sigma, epoch index, quantization errors, topographic errors)."""
        if not self._batch:
            raise NotImplementedError('the online-SOM grid needs SOM_Online, which decontamination_gb300 does not '
                                      'provide; use batch=True')
        dataset, weights = self._dataset, self._dataset_weights
        dim = int(dataset.shape[1])
        dtype = dataset.dtype if isinstance(dataset, np.ndarray) else np.float32
        if isinstance(dataset, torch.Tensor):
            dtype = np.float64 if dataset.dtype == torch.float64 else np.float32
        # resident copies for every grid point (arrays only; generator datasets are re-read as the reference does)
        if is_array(dataset) and (weights is None or is_array(weights)):
            device = _device.require_cuda()
            dataset = _device.to_device(dataset, dtype, device)
            if weights is not None:
                weights = _device.to_device(weights, np.float64, device)
        cov = Covariance.compute(dim, dataset, weights, ddof=1)

        result = (0, math.nan, math.nan, -1, np.empty(0, dtype=np.float64), np.empty(0, dtype=np.float64))
        min_qe = math.inf
        for m, sigma in self.grid():
            pca = SOM_PCA(m, m, dim, dtype=dtype, topology=self._topology)
            pca.train_from_cov_matrix(cov, min_weight=0.0, max_weight=1.0)
            som = SOM_Batch(m, m, dim, dtype=dtype, topology=self._topology, sigma=sigma)
            som.init_from(pca)
            som.train(dataset, dataset_weights=weights, n_epochs=n_epochs, n_vectors=None,
                      use_best_epoch=self._use_best_epoch)
            qes, tes = som.quantization_errors, som.topographic_errors
            idx = int(np.argmin(qes)) if self._use_best_epoch else qes.shape[0] - 1
            if min_qe > qes[idx]:
                min_qe = qes[idx]
                result = (m, None, sigma, idx, qes, tes)
        return result
