"""Covariance of a catalogue on the GPU (the PCA initialisation's input).

Same API as the reference's ``decontamination.algo.covariance.Covariance`` (algo/covariance.py:20-258): ``compute``,
``diagonalize``, ``project_pca``. The reference runs Welford's update sample by sample on the host; here every chunk
goes through ``somgb_weighted_moments`` (weight sum, mean and centred second moments in float64 on the device) and
chunks are combined on the host with Chan's pairwise update. The samples that count are the reference's: all
features finite, weight finite and positive (covariance.py:33-38).
"""

import typing

import numpy as np
import torch

from . import _device, _native
from ._dataset import dataset_to_generator_builder, device_pieces

__all__ = ['Covariance']


class Covariance(object):
    """Covariance calculation with constant device memory per chunk."""

    @staticmethod
    def moments(dim: int, dataset, dataset_weights=None) -> typing.Tuple[float, np.ndarray, np.ndarray]:
        """(W, mean, M2): weight sum, weighted mean and sum of weighted centred outer products, float64."""
        device = _device.require_cuda()
        db = dataset_to_generator_builder(dataset)
        wb = dataset_to_generator_builder(dataset_weights)
        chunks = zip(db()(), wb()()) if wb is not None else ((xc, None) for xc in db()())
        W, mean, M2 = 0.0, np.zeros(dim, dtype=np.float64), np.zeros((dim, dim), dtype=np.float64)
        out = torch.empty(1 + dim + dim * dim, dtype=torch.float64, device=device)
        for xc, rc in chunks:
            if rc is not None and _len(xc) != _len(rc):
                raise ValueError('`dataset` and `dataset_weights` chunks must be aligned')
            # float32 chunks are read as they are (exact in float64); any other type as float64, as the reference casts
            f64 = not (xc.dtype == torch.float32 if isinstance(xc, torch.Tensor)
                       else np.dtype(getattr(xc, 'dtype', np.float64)) == np.float32)
            xd, rd, pieces = device_pieces(xc, rc, np.float64 if f64 else np.float32, device)
            for _ in pieces:   # the whole chunk is used below; this waits for every piece's copy
                pass
            name = 'somgb_weighted_moments_f64' if f64 else 'somgb_weighted_moments'
            _native.call(name, xd.data_ptr(), _device.ptr(rd), _device.rows(xd), dim, out.data_ptr(), _device.stream())
            o = out.cpu().numpy()
            W, mean, M2 = combine_moments(W, mean, M2, float(o[0]), o[1:1 + dim], o[1 + dim:].reshape(dim, dim))
        return W, mean, M2

    @staticmethod
    def compute(dim: int, dataset, dataset_weights=None, ddof: int = 1, show_progress_bar: bool = False) -> np.ndarray:
        """Covariance matrix of the dataset, M2 / (W - ddof) (algo/covariance.py:124-204)."""
        if ddof < 0:
            raise ValueError('ddof must be greater than or equal to zero.')
        W, _, M2 = Covariance.moments(dim, dataset, dataset_weights)
        norm = W - ddof
        if norm <= 0.0:
            raise ValueError('Empty dataset or degrees of freedom <= 0.')
        return M2 / norm

    @staticmethod
    def diagonalize(cov_matrix: np.ndarray, sort: bool = True) -> typing.Tuple[np.ndarray, np.ndarray]:
        """Eigenvalues and eigenvectors (by decreasing eigenvalue when `sort`), algo/covariance.py:208-239."""
        if cov_matrix.shape[0] != cov_matrix.shape[1]:
            raise ValueError('Input covariance matrix is not square.')
        eigenvalues, eigenvectors = np.linalg.eigh(cov_matrix)
        if sort:
            eigenvalues = np.flip(eigenvalues, axis=0)
            eigenvectors = np.flip(eigenvectors, axis=1)
        return eigenvalues, eigenvectors

    @staticmethod
    def project_pca(dataset: np.ndarray, eigenvectors: np.ndarray) -> np.ndarray:
        """The dataset in the PCA basis, dataset . eigenvectors (algo/covariance.py:243-258)."""
        return np.dot(dataset, eigenvectors)


def combine_moments(W, mean, M2, wc, mc, m2c):
    """Moments (weight sum, mean, centred second moments) of two sample sets from each set's (Chan et al.'s pairwise
    update): M2 = M2_a + M2_b + d d^T W_a W_b / (W_a + W_b), d = mean_b - mean_a."""
    if wc <= 0.0:
        return W, mean, M2
    if W == 0.0:
        return wc, np.array(mc, dtype=np.float64), np.array(m2c, dtype=np.float64)
    delta = mc - mean
    tot = W + wc
    return tot, mean + delta * (wc / tot), M2 + m2c + np.outer(delta, delta) * (W * wc / tot)


def _len(a):
    return int(a.shape[0]) if isinstance(a, (np.ndarray, torch.Tensor)) else len(a)
