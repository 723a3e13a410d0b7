#!/usr/bin/env python3
"""Generate the golden fixtures for the batch-SOM hot path from the reference itself.

This script is test infrastructure. It imports the reference package
(lpsc-euclid/decontamination 0.0.1) from a source checkout, runs its own
``SOM_Batch`` / ``SOM_Abstract`` code on small seeded inputs and stores the
outputs in ``tests/golden/*.npz``. Only the fixtures are used at test time;
the reference is not needed on the machine that runs the tests.

Numba is not installed here, so the reference runs in the mode its own CI uses
(``NUMBA_DISABLE_JIT=1``, reference ``Makefile:21-22``): the jit layer rewrites
each kernel into plain Python (``jit/processor.py:112-123``). A minimal
``numba`` stand-in module (identity decorators, ``prange = range``,
``cuda.is_available() == False``) satisfies the reference's imports. The
package ``__init__`` (which pulls in healpy, matplotlib, ...) is bypassed by
registering a bare package object and importing only ``decontamination.jit``,
``decontamination.logging`` and ``decontamination.algo.som_*``.

Arithmetic note: in this pure-Python mode NumPy 2 (NEP 50) keeps every
intermediate in float32 (distance sums, sigma, neighbourhood factors), whereas
the Numba-compiled reference sums distances in float64. The oracle exposes both
semantics; the fixtures pin its ``pyref`` mode.

Usage::

    python tests/golden/make_golden.py [--reference /path/to/reference]
"""

import argparse
import hashlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


########################################################################################################################
# numba stand-in (only what the reference's hot-path modules touch at import time)
########################################################################################################################

def _install_numba_standin():
    def _decorator_factory(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    nb = types.ModuleType('numba')
    nb.njit = _decorator_factory
    nb.jit = _decorator_factory
    nb.prange = range
    nb.get_num_threads = lambda: 1
    nb.set_num_threads = lambda n: None

    nb_types = types.ModuleType('numba.types')
    nb_types.Buffer = object
    nb_types.Any = object
    nb_types.Float = float
    nb_types.Integer = int
    nb.types = nb_types

    extending = types.ModuleType('numba.extending')
    extending.lower_builtin = lambda *a, **k: (lambda f: f)
    extending.type_callable = lambda *a, **k: (lambda f: f)
    nb.extending = extending

    np_mod = types.ModuleType('numba.np')
    arrayobj = types.ModuleType('numba.np.arrayobj')
    arrayobj.make_array = None
    arrayobj.basic_indexing = None
    arrayobj.normalize_indices = None
    np_mod.arrayobj = arrayobj
    nb.np = np_mod

    core = types.ModuleType('numba.core')
    typing_mod = types.ModuleType('numba.core.typing')
    arraydecl = types.ModuleType('numba.core.typing.arraydecl')
    arraydecl.get_array_index_type = None
    typing_mod.arraydecl = arraydecl
    core.typing = typing_mod
    nb.core = core

    cuda = types.ModuleType('numba.cuda')
    cuda.is_available = lambda: False
    cuda.jit = _decorator_factory
    cuda.is_cuda_array = lambda a: False
    nb.cuda = cuda

    for name, mod in {
        'numba': nb, 'numba.types': nb_types, 'numba.extending': extending, 'numba.np': np_mod,
        'numba.np.arrayobj': arrayobj, 'numba.core': core, 'numba.core.typing': typing_mod,
        'numba.core.typing.arraydecl': arraydecl, 'numba.cuda': cuda,
    }.items():
        sys.modules[name] = mod


def load_reference(reference_root):
    """Import the reference's SOM_Batch in pure-Python mode, bypassing its package __init__."""
    os.environ['NUMBA_DISABLE_JIT'] = '1'
    _install_numba_standin()
    pkg_dir = os.path.join(reference_root, 'decontamination')
    pkg = types.ModuleType('decontamination')
    pkg.__path__ = [pkg_dir]
    sys.modules['decontamination'] = pkg
    import importlib
    jit_mod = importlib.import_module('decontamination.jit')
    for name in ('jit', 'DeviceArray', 'device_array_from', 'device_array_empty', 'device_array_zeros',
                 'device_array_full'):
        setattr(pkg, name, getattr(jit_mod, name))
    som_batch = importlib.import_module('decontamination.algo.som_batch')
    return som_batch.SOM_Batch


########################################################################################################################
# seeded inputs
########################################################################################################################

def gaussian_mixture(rng, n, dim, k=5, spread=3.0, sigma=0.5):
    means = rng.uniform(-spread, spread, size=(k, dim))
    labels = rng.integers(0, k, size=n)
    return (means[labels] + sigma * rng.standard_normal((n, dim))).astype(np.float32)


def make_cases(SOM_Batch):
    cases = {}

    # --- the reference's own known-answer tests, re-run (inputs from test/test_som_batch.py:19-23,
    #     test/test_som_abstract.py:110-164; SOM_PCA's init_rand is SOM_Abstract.init_rand) -----------------------
    data = np.random.default_rng(seed=0).random((1_000, 4), np.float32)
    som = SOM_Batch(4, 4, 4, dtype=np.float32, topology='square')
    som.init_rand(seed=0)
    w0 = som.weights.copy()
    som.train(data, n_epochs=1, enable_gpu=False)
    cases['kat_epoch'] = dict(m=4, n=4, dim=4, topology='square', sigma=som.sigma, n_epochs=1, x=data, w0=w0,
                              weights=som.weights.copy(), qe=som.quantization_errors.copy(),
                              te=som.topographic_errors.copy())

    som.init_rand(seed=0)
    som.train(data, n_vectors=data.shape[0], enable_gpu=False)
    cases['kat_iter'] = dict(m=4, n=4, dim=4, topology='square', sigma=som.sigma, n_vectors=1000, x=data, w0=w0,
                             weights=som.weights.copy(), qe=som.quantization_errors.copy(),
                             te=som.topographic_errors.copy())

    som.init_rand(seed=0)
    act_x = np.random.default_rng(seed=0).random((25_000, 4), np.float32)
    # the 25 000-row input is regenerated from its seed at test time; only its digest is stored
    cases['kat_activation'] = dict(m=4, n=4, dim=4, topology='square', w0=w0, x_seed=0, x_shape=act_x.shape,
                                   x_sha256=hashlib.sha256(act_x.tobytes()).hexdigest(),
                                   activation=som.get_activation_map(act_x, enable_gpu=False))
    win_x = np.random.default_rng(seed=0).random((8, 4), np.float32)
    cases['kat_winners'] = dict(m=4, n=4, dim=4, topology='square', w0=w0, x=win_x,
                                winners=som.get_winners(win_x, enable_gpu=False))
    cases['kat_errors'] = dict(m=4, n=4, dim=4, topology='square', w0=w0, x=win_x,
                               errors=np.array(som.compute_errors(win_x, enable_gpu=False)))

    # --- wider coverage on small seeded inputs -------------------------------------------------------------------
    rng = np.random.default_rng(11)
    x = gaussian_mixture(rng, 600, 7)
    rho = rng.random(600).astype(np.float32)
    rho[rng.random(600) < 0.1] = 0.0          # zero-weight rows are skipped (som_batch.py:512-514)
    som = SOM_Batch(6, 5, 7, dtype=np.float32, topology='hexagonal', sigma=2.5)
    w0 = rng.uniform(-1, 1, size=(30, 7)).astype(np.float32)
    som._weights[...] = w0
    som.train(x, dataset_weights=rho, n_epochs=3, use_best_epoch=True, enable_gpu=False)
    cases['hex_weighted_epochs'] = dict(m=6, n=5, dim=7, topology='hexagonal', sigma=2.5, n_epochs=3, x=x, rho=rho,
                                        w0=w0, weights=som.weights.copy(), history=som._history.copy(),
                                        qe=som.quantization_errors.copy(), te=som.topographic_errors.copy())

    rng = np.random.default_rng(12)
    x = gaussian_mixture(rng, 500, 3)
    chunks = [x[0:170], x[170:171], x[171:500]]
    som = SOM_Batch(5, 7, 3, dtype=np.float32, topology='square')
    w0 = rng.uniform(-1, 1, size=(35, 3)).astype(np.float32)
    som._weights[...] = w0
    som.train(lambda: lambda: iter(chunks), n_epochs=2, use_best_epoch=False, enable_gpu=False)
    cases['square_chunked_epochs'] = dict(m=5, n=7, dim=3, topology='square', sigma=som.sigma, n_epochs=2, x=x,
                                          chunk_bounds=np.array([0, 170, 171, 500]), w0=w0,
                                          weights=som.weights.copy(), history=som._history.copy(),
                                          qe=som.quantization_errors.copy(), te=som.topographic_errors.copy())

    rng = np.random.default_rng(13)
    x = gaussian_mixture(rng, 400, 5)
    rho = (rng.random(400) * 2.0).astype(np.float32)
    som = SOM_Batch(4, 6, 5, dtype=np.float32, topology='hexagonal', sigma=3.0)
    w0 = rng.uniform(-1, 1, size=(24, 5)).astype(np.float32)
    som._weights[...] = w0
    som.train(x, dataset_weights=rho, n_vectors=300, enable_gpu=False)
    cases['hex_weighted_iter'] = dict(m=4, n=6, dim=5, topology='hexagonal', sigma=3.0, n_vectors=300, x=x,
                                      rho=rho, w0=w0, weights=som.weights.copy(), qe=som.quantization_errors.copy(),
                                      te=som.topographic_errors.copy())

    # edge cases for the projection calls: NaN features, all-NaN rows, duplicated units (exact ties),
    # zero / negative densities
    rng = np.random.default_rng(14)
    w0 = rng.uniform(-1, 1, size=(20, 6)).astype(np.float32)
    w0[7] = w0[3]                               # exact tie: the lower index must win
    w0[15] = w0[3]
    w0[11, 2] = np.nan                          # a NaN unit is never selected
    x = gaussian_mixture(rng, 300, 6, spread=1.0)
    x[5] = w0[3]
    x[6] = w0[3]
    x[10, 4] = np.nan                           # a NaN feature makes every distance NaN
    x[11, :] = np.nan
    rho = rng.standard_normal(300)
    som = SOM_Batch(4, 5, 6, dtype=np.float32, topology='square')
    som._weights[...] = w0
    cases['edge_projection'] = dict(m=4, n=5, dim=6, topology='square', w0=w0, x=x, rho=rho,
                                    winners=som.get_winners(x, enable_gpu=False),
                                    activation=som.get_activation_map(x, enable_gpu=False),
                                    activation_weighted=som.get_activation_map(x, dataset_weights=rho,
                                                                               enable_gpu=False),
                                    errors=np.array(som.compute_errors(x, enable_gpu=False)),
                                    errors_weighted=np.array(som.compute_errors(x, dataset_weights=rho,
                                                                                enable_gpu=False)))

    rng = np.random.default_rng(15)
    x64 = gaussian_mixture(rng, 300, 4).astype(np.float64)
    som = SOM_Batch(3, 4, 4, dtype=np.float64, topology='hexagonal')
    w0 = rng.uniform(-1, 1, size=(12, 4))
    som._weights[...] = w0
    som.train(x64, n_epochs=2, use_best_epoch=False, enable_gpu=False)
    cases['float64_epoch'] = dict(m=3, n=4, dim=4, topology='hexagonal', sigma=som.sigma, n_epochs=2, x=x64, w0=w0,
                                  weights=som.weights.copy(), qe=som.quantization_errors.copy(),
                                  te=som.topographic_errors.copy())
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('DECONTAMINATION_REFERENCE'), required=not os.environ.get('DECONTAMINATION_REFERENCE'),
                    help='checkout of lpsc-euclid/decontamination 0.0.1 (or set DECONTAMINATION_REFERENCE)')
    ap.add_argument('--out', default=HERE)
    args = ap.parse_args()
    SOM_Batch = load_reference(args.reference)
    cases = make_cases(SOM_Batch)
    for name, payload in cases.items():
        arrays = {k: (np.asarray(v) if not isinstance(v, str) else np.array(v)) for k, v in payload.items()}
        np.savez_compressed(os.path.join(args.out, f'{name}.npz'), **arrays)
        print(f'wrote {name}.npz: ' + ', '.join(f'{k}{tuple(np.shape(v))}' for k, v in arrays.items()))


if __name__ == '__main__':
    main()
