"""The CPU oracle, pinned against fixtures produced by the reference itself (tests/golden/make_golden.py).

`pyref` mode restates the reference's pure-Python arithmetic and must reproduce
the fixtures bit for bit. `numba` mode (the compiled reference's typing, the
mode the GPU path is checked against) may differ from it only where two
distances tie within float32 rounding; such samples are adjudicated in float64.
"""

import hashlib

import numpy as np
import pytest

from conftest import golden

TRAIN_CASES = ['kat_epoch', 'kat_iter', 'hex_weighted_epochs', 'square_chunked_epochs', 'hex_weighted_iter',
               'float64_epoch']
BEST_EPOCH = {'kat_epoch': True, 'hex_weighted_epochs': True, 'square_chunked_epochs': False,
              'float64_epoch': False}


def _train_oracle(somref, g, mode, name):
    som = somref.OracleSOM(int(g['m']), int(g['n']), int(g['dim']), dtype=g['w0'].dtype,
                           topology=str(g['topology']), sigma=float(g['sigma']), mode=mode, threads=1)
    som.weights = g['w0'].copy()
    x = g['x']
    if 'chunk_bounds' in g:
        b = g['chunk_bounds']
        chunks = [x[b[i]:b[i + 1]] for i in range(len(b) - 1)]
        ds = lambda: lambda: iter(chunks)
    else:
        ds = x
    rho = g.get('rho')
    if 'n_epochs' in g:
        som.train(ds, rho, n_epochs=int(g['n_epochs']), use_best_epoch=BEST_EPOCH[name])
    else:
        som.train(ds, rho, n_vectors=int(g['n_vectors']))
    return som


@pytest.mark.parametrize('name', TRAIN_CASES)
def test_pyref_training_is_bit_exact(oracle, name):
    g = golden(name)
    som = _train_oracle(oracle, g, 'pyref', name)
    assert np.array_equal(som.weights, g['weights'])
    np.testing.assert_allclose(som.quantization_errors, g['qe'], rtol=1e-12)
    np.testing.assert_allclose(som.topographic_errors, g['te'], rtol=1e-12)
    if 'history' in g:
        assert np.array_equal(som.history, g['history'])


@pytest.mark.parametrize('name', TRAIN_CASES)
def test_numba_mode_training_close(oracle, name):
    g = golden(name)
    som = _train_oracle(oracle, g, 'numba', name)
    # the reference's own known-answer tolerance (test/test_som_batch.py:56)
    np.testing.assert_allclose(som.weights, g['weights'], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(som.quantization_errors, g['qe'], rtol=1e-5)


def test_kat_activation_and_winners(oracle):
    g = golden('kat_activation')
    x = np.random.default_rng(int(g['x_seed'])).random(tuple(g['x_shape']), np.float32)
    assert hashlib.sha256(x.tobytes()).hexdigest() == str(g['x_sha256'])
    for mode in ('pyref', 'numba'):
        assert np.array_equal(oracle.count_bmus(g['w0'], x, mode=mode).reshape(4, 4), g['activation'])
    gw = golden('kat_winners')
    for mode in ('pyref', 'numba'):
        assert np.array_equal(oracle.find_bmus(gw['w0'], gw['x'], mode), gw['winners'])
    ge = golden('kat_errors')
    topo = oracle.topography(4, 4, 'square')
    o = oracle.compute_errors_raw(ge['w0'], topo, ge['x'], None, 2.0, 'pyref')
    np.testing.assert_allclose(o[:2] / o[2], ge['errors'], rtol=1e-12)


@pytest.mark.parametrize('mode', ['pyref', 'numba'])
def test_edge_projection(oracle, mode):
    g = golden('edge_projection')
    w, x, rho = g['w0'], g['x'], g['rho']
    assert np.array_equal(oracle.find_bmus(w, x, mode), g['winners'])
    assert np.array_equal(oracle.count_bmus(w, x, None, mode).reshape(4, 5).astype(np.float32), g['activation'])
    assert np.array_equal(oracle.count_bmus(w, x, rho, mode).reshape(4, 5).astype(np.float32),
                          g['activation_weighted'])
    topo = oracle.topography(4, 5, 'square')
    # distances (hence sqrt(d1)) are float32 sums in pyref mode and float64 sums in numba mode
    rtol = 1e-12 if mode == 'pyref' else 1e-6
    o = oracle.compute_errors_raw(w, topo, x, None, 2.0, mode)
    np.testing.assert_allclose(o[:2] / o[2], g['errors'], rtol=rtol)
    o = oracle.compute_errors_raw(w, topo, x, rho, 2.0, mode)
    np.testing.assert_allclose(o[:2] / o[2], g['errors_weighted'], rtol=rtol)


def test_numba_vs_pyref_bmus_differ_only_at_ties(oracle):
    rng = np.random.default_rng(5)
    w = rng.random((256, 8), dtype=np.float32)
    x = rng.random((20000, 8), dtype=np.float32)
    b_numba = oracle.find_bmus(w, x, 'numba')
    b_py = oracle.find_bmus(w, x, 'pyref')
    diff = np.nonzero(b_numba != b_py)[0]
    for i in diff:
        d = [oracle.sqdist_exact(w[b], x[i]) for b in (b_numba[i], b_py[i])]
        assert abs(d[0] - d[1]) <= 8 * 2.0 ** -24 * max(d), 'a non-tied BMU differs between the two typings'


def test_factored_fp64_matches_scatter(oracle):
    rng = np.random.default_rng(7)
    M, D, N = 30, 5, 700
    w = rng.random((M, D), dtype=np.float32)
    x = rng.random((N, D), dtype=np.float32)
    rho = rng.random(N).astype(np.float32)
    topo = oracle.topography(5, 6, 'hexagonal')
    num32 = np.zeros((M, D), np.float32); den32 = np.zeros(M, np.float32)
    oracle.train_epoch_scatter(num32, den32, w, topo, x, rho, 3.0, 1, 4, 'numba', threads=1)
    num64 = np.zeros((M, D)); den64 = np.zeros(M)
    bmus = np.empty(N, np.int32)
    oracle.train_epoch_fp64(num64, den64, w, topo, x, rho, 3.0, 1, 4, 'numba', threads=1, bmus=bmus)
    assert np.array_equal(bmus, oracle.find_bmus(w, x, 'numba'))
    np.testing.assert_allclose(num32, num64, rtol=2e-5)
    np.testing.assert_allclose(den32, den64, rtol=2e-5)


def test_parallel_oracle_deterministic(oracle):
    rng = np.random.default_rng(9)
    w = rng.random((64, 6), dtype=np.float32)
    x = rng.random((5000, 6), dtype=np.float32)
    rho = rng.random(5000)
    h1 = oracle.count_bmus(w, x, rho, 'numba', threads=1)
    h4 = oracle.count_bmus(w, x, rho, 'numba', threads=4)
    np.testing.assert_allclose(h1, h4, rtol=1e-13)
    assert np.array_equal(oracle.find_bmus(w, x, 'numba', 1), oracle.find_bmus(w, x, 'numba', 4))
