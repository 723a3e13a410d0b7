"""The reference's dataset protocol: an array, or a generator builder () -> (() -> iterable of chunks).

Restates ``dataset_to_generator_builder`` (algo/__init__.py:21-27) and the
chunk loops of the reference (algo/som_batch.py:295-342,
algo/som_abstract.py:557-597): chunks of `dataset` and `dataset_weights` are
zipped and must have the same length. Arrays (numpy or torch, host or device)
are accepted wherever the reference accepts a numpy array.
"""

import typing

import numpy as np
import torch

from . import _device


def dataset_to_generator_builder(dataset) -> typing.Optional[typing.Callable]:
    if dataset is None:
        return None
    return dataset if callable(dataset) else (lambda: lambda: (dataset,))


def iterate_chunks(dataset, dataset_weights, dtype, device, weight_dtype=np.float64):
    """Yields (x, rho) device tensors per chunk; rho is None when there are no weights.

    x has the map dtype (the reference casts chunks with astype(dtype)); rho is float64, the type the reference uses
    for densities in compute_errors / get_activation_map (training casts it to the map dtype on the device).
    """
    db = dataset_to_generator_builder(dataset)
    wb = dataset_to_generator_builder(dataset_weights)
    if wb is None:
        for xc in db()():
            yield _device.to_device(xc, dtype, device), None
        return
    for xc, rc in zip(db()(), wb()()):
        if _len(xc) != _len(rc):
            raise ValueError('`dataset` and `dataset_weights` chunks must be aligned')
        yield _device.to_device(xc, dtype, device), _device.to_device(rc, weight_dtype, device)


def _len(a):
    return int(a.shape[0]) if isinstance(a, (np.ndarray, torch.Tensor)) else len(a)


def is_array(a):
    return isinstance(a, (np.ndarray, torch.Tensor))
