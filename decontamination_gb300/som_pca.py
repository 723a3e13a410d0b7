"""SOM_PCA: a map laid out on the plane of the first two principal components.

Same API as the reference's ``decontamination.algo.som_pca.SOM_PCA`` (algo/som_pca.py:20-283): the constructor,
``train`` (covariance of the dataset, then ``train_from_cov_matrix``), the options ``min_weight``, ``max_weight``,
``scale_by_variance``, ``apply_cdf``, ``cdf_gain`` and the properties ``cov_matrix``, ``eigenvalues``,
``eigenvectors``. The covariance is computed on the GPU (``Covariance``); the eigen-decomposition of the D x D matrix
and the M x D grid of weights are host work, as in the reference. It is the initialisation that ``HypParamFinder_SOM``
gives every map of its grid (``SOM_Batch.init_from``).
"""

import math
import typing

import numpy as np

from .covariance import Covariance
from .som_abstract import SOM_Abstract

__all__ = ['SOM_PCA']


class SOM_PCA(SOM_Abstract):
    """Self Organizing Map spanning the first two principal components of a dataset."""

    __MODE__ = 'pca'

    def __init__(self, m: int, n: int, dim: int, dtype=np.float32, topology: typing.Optional[str] = None):
        if dim < 2:
            raise ValueError('SOM_PCA requires dim >= 2.')
        super().__init__(m, n, dim, dtype, topology)
        self._scale_by_variance = False
        self._apply_cdf = False
        self._cdf_gain = 1.0
        self._cov_matrix = np.zeros((dim, dim), dtype=np.float64)
        self._eigenvalues = np.zeros((dim,), dtype=np.float64)
        self._eigenvectors = np.zeros((dim, dim), dtype=np.float64)
        self._header_extra = {
            'mode': '__MODE__',
            'scale_by_variance': '_scale_by_variance',
            'apply_cdf': '_apply_cdf',
            'cdf_gain': '_cdf_gain',
        }

    @property
    def cov_matrix(self) -> np.ndarray:
        """Covariance matrix of the training dataset."""
        return self._cov_matrix

    @property
    def eigenvalues(self) -> np.ndarray:
        """Eigenvalues of the covariance matrix."""
        return self._eigenvalues

    @property
    def eigenvectors(self) -> np.ndarray:
        """Eigenvectors of the covariance matrix."""
        return self._eigenvectors

    @staticmethod
    def _grid_weights(cov_matrix, min_weight, max_weight, m, n, dim, scale_by_variance, apply_cdf, cdf_gain):
        """(eigenvalues, eigenvectors, weights (m, n, dim) float64): unit (i, j) at c1_i v0 + c2_j v1, the c's evenly
        spaced over [min_weight, max_weight] (or [-1, 1] before the optional Gaussian-CDF map), algo/som_pca.py:116-177.
        """
        eigenvalues, eigenvectors = Covariance.diagonalize(cov_matrix, sort=True)
        v0 = eigenvectors[:, 0]
        v1 = eigenvectors[:, 1]
        if scale_by_variance:
            if eigenvalues[0] > 0.0:
                v0 = v0 * np.sqrt(eigenvalues[0])
            if eigenvalues[1] > 0.0:
                v1 = v1 * np.sqrt(eigenvalues[1])
        lo, hi = (-1.0, 1.0) if apply_cdf else (min_weight, max_weight)
        c1 = np.linspace(lo, hi, m)
        c2 = np.linspace(lo, hi, n)
        # w[i, j, d] = v0[d] * c1[i] + v1[d] * c2[j], each term rounded as the reference's scalar loop rounds it
        w = v0[None, None, :] * c1[:, None, None] + v1[None, None, :] * c2[None, :, None]
        if apply_cdf:
            sigma = np.sqrt(v0 * v0 + v1 * v1)
            sigma[sigma == 0.0] = 1.0
            scale = cdf_gain / (math.sqrt(2.0) * sigma)
            erf = np.vectorize(math.erf, otypes=[np.float64])
            w = min_weight + (max_weight - min_weight) * 0.5 * (1.0 + erf(w * scale[None, None, :]))
        return eigenvalues, eigenvectors, w

    def train(self, dataset, dataset_weights=None, min_weight: float = 0.0, max_weight: float = 1.0,
              scale_by_variance: bool = False, apply_cdf: bool = False, cdf_gain: float = 1.0,
              show_progress_bar: bool = False) -> None:
        """Trains the map from the dataset: its covariance (ddof 1), then ``train_from_cov_matrix``."""
        cov_matrix = Covariance.compute(self._dim, dataset, dataset_weights, ddof=1)
        self.train_from_cov_matrix(cov_matrix, min_weight=min_weight, max_weight=max_weight,
                                   scale_by_variance=scale_by_variance, apply_cdf=apply_cdf, cdf_gain=cdf_gain)

    def train_from_cov_matrix(self, cov_matrix: np.ndarray, min_weight: float = 0.0, max_weight: float = 1.0,
                              scale_by_variance: bool = False, apply_cdf: bool = False, cdf_gain: float = 1.0,
                              show_progress_bar: bool = False) -> None:
        """Trains the map from a covariance matrix (algo/som_pca.py:226-283)."""
        if max_weight <= min_weight:
            raise ValueError('max_weight must be > min_weight.')
        if apply_cdf and cdf_gain <= 0.0:
            raise ValueError('cdf_gain must be > 0 when apply_cdf is True.')
        eigenvalues, eigenvectors, weights = SOM_PCA._grid_weights(
            np.asarray(cov_matrix).astype(np.float64, copy=False), min_weight, max_weight, self._m, self._n,
            self._dim, scale_by_variance, apply_cdf, cdf_gain)
        # the header fields _scale_by_variance, _apply_cdf and _cdf_gain keep their constructor values, as in the
        # reference (som_pca.py:270-283 does not record the options)
        self._cov_matrix[:] = np.asarray(cov_matrix).astype(self._dtype, copy=False)
        self._eigenvalues[:] = eigenvalues.astype(self._dtype, copy=False)
        self._eigenvectors[:] = eigenvectors.astype(self._dtype, copy=False)
        self._weights[:] = weights.astype(self._dtype, copy=False).reshape(self._weights.shape)
