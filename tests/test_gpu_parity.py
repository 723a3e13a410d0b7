"""GPU parity: the libsomgb kernels (through the C ABI) against the CPU oracle.

BMUs must be bit-identical to the oracle's `numba` mode (the compiled
reference's arithmetic); activation counts exact; error sums within float64
summation-order rounding; trained weights within 1e-5 relative of the float64
oracle (the bar the path is held to) and within the reference's own 1e-4
known-answer tolerance of its fixtures.
"""

import zlib

import numpy as np
import pytest
import torch

import decontamination_gb300 as dg
from decontamination_gb300 import _native
from conftest import golden

pytestmark = pytest.mark.gpu

ALGOS = ['fp32', 'auto', 'tc']
W_RTOL = 1e-5          # trained weights vs the float64 oracle
ERR_RTOL = 1e-9        # error sums: float64, summation order differs


def _rand(rng, n, d, kind='uniform'):
    if kind == 'uniform':
        return rng.random((n, d), dtype=np.float32)
    if kind == 'mixture':
        means = rng.uniform(-3, 3, size=(5, d))
        return (means[rng.integers(0, 5, n)] + 0.5 * rng.standard_normal((n, d))).astype(np.float32)
    z = rng.standard_normal((n, d))
    return np.exp(0.3 * z).astype(np.float32)


def _som(m, n, d, w, topology='square', algo='auto', sigma=None, dtype=np.float32):
    som = dg.SOM_Batch(m, n, d, dtype=dtype, topology=topology, sigma=sigma)
    som._weights[...] = w
    som.bmu_algo = algo
    return som


def _tc_ok(native, n, m, d):
    return bool(native.lib().somgb_algo_supported(native.ALGO_TC, n, m, d))


def _skip_unsupported_tc(native, algo, n, m, d, call):
    """For algo 'tc' on a shape outside the tensor-core limits the call must fail loudly (no silent fallback)."""
    if algo == 'tc' and not _tc_ok(native, n, m, d):
        with pytest.raises(native.SomgbError) as ei:
            call()
        assert ei.value.status == native.SOMGB_ERR_UNSUPPORTED
        pytest.skip('shape outside the tensor-core limits (checked that it is refused)')


# ----------------------------------------------------------------------------------------------------------------------
# projection calls
# ----------------------------------------------------------------------------------------------------------------------

SHAPES = [(1, 1, 3, 50), (1, 2, 4, 300), (4, 4, 4, 25_000), (10, 10, 4, 20_000), (8, 9, 7, 5000),
          (32, 32, 16, 40_000), (16, 16, 17, 8000), (8, 16, 32, 10_000), (5, 7, 64, 3000), (4, 5, 100, 2000),
          (64, 64, 16, 6000), (80, 80, 32, 5000), (3, 3, 1, 500)]


@pytest.mark.parametrize('algo', ALGOS)
@pytest.mark.parametrize('m,n,d,N', SHAPES)
def test_winners_bit_exact(cuda, native, oracle, algo, m, n, d, N):
    rng = np.random.default_rng(m * 1000 + n * 10 + d)
    x = _rand(rng, N, d, 'lognormal' if d >= 16 else 'uniform')
    w = x[rng.integers(0, N, m * n)] + 0.01 * rng.standard_normal((m * n, d)).astype(np.float32)
    som = _som(m, n, d, w, algo=algo)
    _skip_unsupported_tc(native, algo, N, m * n, d, lambda: som.get_winners(x))
    got = som.get_winners(x)
    want = oracle.find_bmus(w.astype(np.float32), x, 'numba')
    assert got.dtype == np.int32
    assert np.array_equal(got, want), f'{np.sum(got != want)} BMU mismatches'


@pytest.mark.parametrize('algo', ALGOS)
def test_kat_activation_map_exact(cuda, native, algo):
    g = golden('kat_activation')
    x = np.random.default_rng(int(g['x_seed'])).random(tuple(g['x_shape']), np.float32)
    som = _som(4, 4, 4, g['w0'], algo=algo)
    assert np.array_equal(som.get_activation_map(x), g['activation'])
    gw = golden('kat_winners')
    assert np.array_equal(_som(4, 4, 4, gw['w0'], algo=algo).get_winners(gw['x']), gw['winners'])


@pytest.mark.parametrize('algo', ALGOS)
@pytest.mark.parametrize('topology', ['square', 'hexagonal'])
def test_errors_and_activation_vs_oracle(cuda, native, oracle, algo, topology):
    rng = np.random.default_rng(3)
    m, n, d, N = 12, 10, 8, 30_000
    x = _rand(rng, N, d, 'mixture')
    w = x[rng.integers(0, N, m * n)].copy()
    rho = rng.standard_normal(N)
    som = _som(m, n, d, w, topology=topology, algo=algo)
    topo = oracle.topography(m, n, topology)
    pen = 2.0 if topology == 'square' else 1.0
    for r in (None, rho):
        o = oracle.compute_errors_raw(w, topo, x, r, pen, 'numba')
        np.testing.assert_allclose(som.compute_errors(x, r), o[:2] / o[2], rtol=ERR_RTOL)
        h = oracle.count_bmus(w, x, r, 'numba')
        np.testing.assert_allclose(som.get_activation_map(x, r).ravel(), h.astype(np.float32), rtol=1e-6)


@pytest.mark.parametrize('algo', ALGOS)
def test_edge_cases_golden(cuda, native, algo):
    """NaN features and rows, a NaN unit, exact ties between duplicated units, zero and negative densities."""
    g = golden('edge_projection')
    if algo == 'tc':
        pytest.skip('D=6 is outside the tensor-core limits; the padded variant below covers the same cases')
    som = _som(4, 5, 6, g['w0'], algo=algo)
    assert np.array_equal(som.get_winners(g['x']), g['winners'])
    assert np.array_equal(som.get_activation_map(g['x']), g['activation'])
    assert np.array_equal(som.get_activation_map(g['x'], g['rho']), g['activation_weighted'])
    np.testing.assert_allclose(som.compute_errors(g['x']), g['errors'], rtol=1e-6)
    np.testing.assert_allclose(som.compute_errors(g['x'], g['rho']), g['errors_weighted'], rtol=1e-6)


@pytest.mark.parametrize('algo', ALGOS)
def test_infinities_and_empty(cuda, native, oracle, algo):
    rng = np.random.default_rng(4)
    w = rng.random((9, 3), dtype=np.float32)
    x = rng.random((64, 3), dtype=np.float32)
    x[3, 1] = np.inf
    x[4] = [1e20, -1e20, 3e19]          # float32 squares overflow
    w[2, 0] = np.inf
    if algo == 'tc':
        w = np.concatenate([w, np.zeros((9, 1), np.float32)], axis=1)   # the tensor-core pass needs D % 4 == 0
        x = np.concatenate([x, np.zeros((64, 1), np.float32)], axis=1)
    som = _som(3, 3, w.shape[1], w, algo=algo)
    assert np.array_equal(som.get_winners(x), oracle.find_bmus(w, x, 'numba'))
    assert som.get_winners(np.zeros((0, w.shape[1]), np.float32)).shape == (0,)
    assert np.all(som.get_activation_map(np.zeros((0, w.shape[1]), np.float32)) == 0)


# ----------------------------------------------------------------------------------------------------------------------
# training
# ----------------------------------------------------------------------------------------------------------------------

def _oracle_train(oracle, m, n, d, w0, topology, sigma, x, rho=None, **kw):
    osom = oracle.OracleSOM(m, n, d, topology=topology, sigma=sigma, mode='numba', threads=0, accumulate='fp64')
    osom.weights = w0.copy()
    osom.train(x, rho, **kw)
    return osom


@pytest.mark.parametrize('algo', ALGOS)
def test_kat_training(cuda, native, oracle, algo):
    for name, kw in (('kat_epoch', dict(n_epochs=1)), ('kat_iter', dict(n_vectors=1000))):
        g = golden(name)
        som = _som(4, 4, 4, g['w0'], algo=algo)
        som.train(g['x'], **kw)
        # the reference's own known-answer tolerance (test/test_som_batch.py:56)
        np.testing.assert_allclose(som.weights, g['weights'], rtol=1e-4)
        np.testing.assert_allclose(som.quantization_errors, g['qe'], rtol=1e-5)


@pytest.mark.parametrize('algo', ALGOS)
@pytest.mark.parametrize('topology', ['square', 'hexagonal'])
def test_epoch_training_vs_fp64_oracle(cuda, native, oracle, algo, topology):
    rng = np.random.default_rng(21)
    m, n, d, N, E = 10, 12, 8, 40_000, 4
    x = _rand(rng, N, d, 'mixture')
    rho = rng.random(N).astype(np.float32)
    rho[rng.random(N) < 0.05] = 0.0
    w0 = rng.uniform(-1, 1, (m * n, d)).astype(np.float32)
    som = _som(m, n, d, w0, topology=topology, algo=algo, sigma=4.0)
    som.train(x, rho, n_epochs=E, use_best_epoch=False)
    ref = _oracle_train(oracle, m, n, d, w0, topology, 4.0, x, rho, n_epochs=E, use_best_epoch=False)
    np.testing.assert_allclose(som.weights, ref.weights, rtol=W_RTOL, atol=1e-6)
    np.testing.assert_allclose(som._history, ref.history, rtol=W_RTOL, atol=1e-6)
    np.testing.assert_allclose(som.quantization_errors, ref.quantization_errors, rtol=1e-6)
    np.testing.assert_allclose(som.topographic_errors, ref.topographic_errors, rtol=1e-6)


def test_chunked_generator_and_best_epoch(cuda, native, oracle):
    g = golden('square_chunked_epochs')
    x, b = g['x'], g['chunk_bounds']
    chunks = [x[b[i]:b[i + 1]] for i in range(len(b) - 1)]
    som = _som(5, 7, 3, g['w0'])
    som.train(lambda: lambda: iter(chunks), n_epochs=2, use_best_epoch=False)
    np.testing.assert_allclose(som.weights, g['weights'], rtol=1e-4, atol=1e-6)
    ref = _oracle_train(oracle, 5, 7, 3, g['w0'], 'square', float(g['sigma']), x, n_epochs=2, use_best_epoch=False)
    np.testing.assert_allclose(som.weights, ref.weights, rtol=W_RTOL, atol=1e-6)

    gh = golden('hex_weighted_epochs')
    som = _som(6, 5, 7, gh['w0'], topology='hexagonal', sigma=2.5)
    som.train(gh['x'], gh['rho'], n_epochs=3, use_best_epoch=True)
    ref = _oracle_train(oracle, 6, 5, 7, gh['w0'], 'hexagonal', 2.5, gh['x'], gh['rho'], n_epochs=3,
                        use_best_epoch=True)
    np.testing.assert_allclose(som.weights, ref.weights, rtol=W_RTOL, atol=1e-6)
    np.testing.assert_allclose(som.quantization_errors, ref.quantization_errors, rtol=1e-6)
    np.testing.assert_allclose(som.topographic_errors, ref.topographic_errors, rtol=1e-6)


def test_early_stop(cuda, native, oracle):
    rng = np.random.default_rng(8)
    x = _rand(rng, 5000, 4, 'mixture')
    w0 = rng.uniform(-1, 1, (36, 4)).astype(np.float32)
    free = _som(6, 6, 4, w0)
    free.train(x, n_epochs=6, use_best_epoch=False)
    stop_at = free.quantization_errors[2] * (1 + 1e-9)
    som = _som(6, 6, 4, w0)
    som.train(x, n_epochs=6, use_best_epoch=False, stop_quantization_error=stop_at, stop_topographic_error=1.0)
    first = int(np.argmax(free.quantization_errors <= stop_at))
    assert np.all(np.isnan(som.quantization_errors[first + 1:]))
    # float64 atomics make runs differ at the last bit at most
    np.testing.assert_allclose(som.quantization_errors[:first + 1], free.quantization_errors[:first + 1], rtol=1e-6)
    np.testing.assert_allclose(som.weights, free._history[first], rtol=1e-6, atol=1e-7)


def test_iter_mode_vs_oracle(cuda, native, oracle):
    g = golden('hex_weighted_iter')
    som = _som(4, 6, 5, g['w0'], topology='hexagonal', sigma=3.0)
    som.train(g['x'], g['rho'], n_vectors=300)
    np.testing.assert_allclose(som.weights, g['weights'], rtol=1e-4, atol=1e-6)
    ref = oracle.OracleSOM(4, 6, 5, topology='hexagonal', sigma=3.0, mode='numba', threads=1)
    ref.weights = g['w0'].copy()
    ref.train(g['x'], g['rho'], n_vectors=300)
    np.testing.assert_allclose(som.weights, ref.weights, rtol=1e-5, atol=1e-6)


def test_float64_map(cuda, native, oracle):
    g = golden('float64_epoch')
    som = _som(3, 4, 4, g['w0'], topology='hexagonal', dtype=np.float64)
    som.train(g['x'], n_epochs=2, use_best_epoch=False)
    np.testing.assert_allclose(som.weights, g['weights'], rtol=1e-10)
    np.testing.assert_allclose(som.quantization_errors, g['qe'], rtol=1e-10)
    np.testing.assert_allclose(som.topographic_errors, g['te'], rtol=1e-12)
    assert np.array_equal(som.get_winners(g['x']), oracle.find_bmus(g['weights'], g['x'], 'numba'))


# ----------------------------------------------------------------------------------------------------------------------
# direct C ABI use with caller-owned device buffers
# ----------------------------------------------------------------------------------------------------------------------

def test_c_abi_epoch_pass_accumulators(cuda, native, oracle):
    rng = np.random.default_rng(30)
    M, D, N = 64, 16, 50_000
    x = _rand(rng, N, D, 'lognormal')
    w = x[rng.integers(0, N, M)].copy()
    topo = oracle.topography(8, 8, 'square')
    xd, wd, td = (torch.from_numpy(a).to(cuda) for a in (x, w, topo))
    S = torch.zeros((M, D), dtype=torch.float64, device=cuda)
    c = torch.zeros(M, dtype=torch.float64, device=cuda)
    err = torch.zeros(3, dtype=torch.float64, device=cuda)
    bmu = torch.empty(N, dtype=torch.int32, device=cuda)
    nbytes = native.workspace_bytes(native.OP_EPOCH, N, M, D, native.ALGO_AUTO)
    ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=cuda)
    wsp = ws.data_ptr() + (-ws.data_ptr()) % 256
    s = torch.cuda.current_stream().cuda_stream
    native.call('somgb_train_epoch_pass', xd.data_ptr(), None, N, D, wd.data_ptr(), td.data_ptr(), M, 2.0,
                native.ALGO_AUTO, S.data_ptr(), c.data_ptr(), err.data_ptr(), bmu.data_ptr(), wsp, nbytes, s)
    torch.cuda.synchronize()
    b = oracle.find_bmus(w, x, 'numba')
    assert np.array_equal(bmu.cpu().numpy(), b)
    S_ref = np.zeros((M, D)); np.add.at(S_ref, b, x.astype(np.float64))
    c_ref = np.bincount(b, minlength=M).astype(np.float64)
    np.testing.assert_allclose(S.cpu().numpy(), S_ref, rtol=1e-12)   # fixed-point sums are exact to ~1e-14
    assert np.array_equal(c.cpu().numpy(), c_ref)
    o = oracle.compute_errors_raw(w, topo, x, None, 2.0, 'numba')
    np.testing.assert_allclose(err.cpu().numpy(), o, rtol=ERR_RTOL)
    # a workspace one byte short is refused before any launch
    with pytest.raises(native.SomgbError) as ei:
        native.call('somgb_train_epoch_pass', xd.data_ptr(), None, N, D, wd.data_ptr(), td.data_ptr(), M, 2.0,
                    native.ALGO_AUTO, S.data_ptr(), c.data_ptr(), None, None, wsp, nbytes - 1, s)
    assert ei.value.status == native.SOMGB_ERR_WORKSPACE


ACCUMULATE_CASES = [
    # (M, D, N, weighted, bmu pattern): one unit range; several (64x64 at D = 32: 8 ranges; 48x48 at D = 24); every
    # sample on one unit (more than the limbs' 2^15-add headroom per flush decision); BMUs of -1; a BMU array that
    # is not 16-byte aligned (scalar loads)
    (1024, 16, 300_000, False, 'uniform'),
    (4096, 32, 400_000, False, 'uniform'),
    (2304, 24, 200_000, True, 'uniform'),
    (4096, 32, 200_000, True, 'clustered'),
    (64, 3, 500_000, False, 'one-unit'),
    (4096, 32, 300_000, False, 'one-unit'),   # several unit ranges: the unit's sums held in registers
    (300, 7, 100_000, True, 'with-negatives'),
    (4096, 32, 150_001, False, 'unaligned'),
]


@pytest.mark.parametrize('M,D,N,weighted,pattern', ACCUMULATE_CASES)
def test_accumulate_segmented_sums(cuda, native, M, D, N, weighted, pattern):
    rng = np.random.default_rng(M + D + N)
    x = _rand(rng, N, D, 'lognormal')
    if pattern == 'one-unit':
        b = np.full(N, 17 % M, dtype=np.int32)
    elif pattern == 'clustered':
        b = np.minimum(rng.geometric(0.01, N) - 1, M - 1).astype(np.int32)
    else:
        b = rng.integers(0, M, N).astype(np.int32)
    if pattern == 'with-negatives':
        b[rng.random(N) < 0.2] = -1
    rho = rng.random(N) * 3.0 if weighted else None
    xd = torch.from_numpy(x).to(cuda)
    if pattern == 'unaligned':
        bd_full = torch.from_numpy(np.concatenate([[0], b]).astype(np.int32)).to(cuda)
        bd = bd_full[1:]
        assert bd.data_ptr() % 16 != 0
    else:
        bd = torch.from_numpy(b).to(cuda)
    rd = torch.from_numpy(rho).to(cuda) if weighted else None
    bounds = torch.zeros(D + 1, dtype=torch.float32, device=cuda)
    S = torch.zeros((M, D), dtype=torch.float64, device=cuda)
    c = torch.zeros(M, dtype=torch.float64, device=cuda)
    s = torch.cuda.current_stream().cuda_stream
    native.call('somgb_feature_bounds', xd.data_ptr(), rd.data_ptr() if weighted else None, N, D, bounds.data_ptr(), s)
    native.call('somgb_accumulate', xd.data_ptr(), rd.data_ptr() if weighted else None, bd.data_ptr(), N, D, M,
                bounds.data_ptr(), S.data_ptr(), c.data_ptr(), s)
    torch.cuda.synchronize()
    keep = b >= 0
    r32 = rho.astype(np.float32).astype(np.float64) if weighted else np.ones(N)
    S_ref = np.zeros((M, D))
    np.add.at(S_ref, b[keep], x[keep].astype(np.float64) * r32[keep, None])
    c_ref = np.bincount(b[keep], weights=r32[keep], minlength=M)
    np.testing.assert_allclose(S.cpu().numpy(), S_ref, rtol=1e-12, atol=1e-9)
    if weighted:
        np.testing.assert_allclose(c.cpu().numpy(), c_ref, rtol=1e-12)
    else:
        assert np.array_equal(c.cpu().numpy(), c_ref)


@pytest.mark.parametrize('D,weighted,dtype', [(16, False, np.float32), (3, True, np.float32), (5, True, np.float64)])
def test_host_catalogue_in_pieces(cuda, D, weighted, dtype):
    """A host catalogue above two pieces is copied in pieces whose passes overlap the copy: every output equals the
    one computed from the same catalogue already on the device (one piece)."""
    from decontamination_gb300 import _dataset
    rng = np.random.default_rng(D)
    N = 2 * _dataset.PIECE_ROWS + 12_345
    x = _rand(rng, N, D, 'lognormal').astype(dtype)
    x[rng.integers(0, N, 50)] = np.nan                  # rows that never win
    rho = rng.random(N) if weighted else None
    xd = torch.from_numpy(x).to(cuda)
    rd = torch.from_numpy(rho).to(cuda) if weighted else None
    xh = torch.from_numpy(x).pin_memory()
    w0 = x[rng.integers(0, N, 48)].copy()
    w0[np.isnan(w0)] = 0.0
    soms = []
    for data, wts in ((xh, rho), (xd, rd)):
        som = dg.SOM_Batch(6, 8, D, dtype=dtype, topology='hexagonal')
        som._weights[...] = w0.reshape(som._weights.shape)
        som.train(data, dataset_weights=wts, n_epochs=2, use_best_epoch=False)
        soms.append(som)
    a, b = soms
    # BMUs and fixed-point sums are exact; float64 error sums differ only in the order of their atomic additions
    np.testing.assert_allclose(a.weights, b.weights, rtol=1e-6)
    np.testing.assert_allclose(a.quantization_errors, b.quantization_errors, rtol=ERR_RTOL)
    np.testing.assert_allclose(a.topographic_errors, b.topographic_errors, rtol=ERR_RTOL)
    assert np.array_equal(a.get_winners(x), a.get_winners(xd))
    np.testing.assert_allclose(a.get_activation_map(x, rho), a.get_activation_map(xd, rd), rtol=1e-12)
    np.testing.assert_allclose(a.compute_errors(xh, rho), a.compute_errors(xd, rd), rtol=ERR_RTOL)


@pytest.mark.parametrize('m,n,topology,dtype', [(32, 32, 'hexagonal', np.float32), (64, 64, 'square', np.float32),
                                                 (7, 1, 'hexagonal', np.float32), (5, 9, 'hexagonal', np.float64),
                                                 (12, 10, 'square', np.float64)])
def test_grid_neighbourhood_update_matches_the_pairwise_one(cuda, native, m, n, topology, dtype):
    """The axis-factorised contraction gives the pairwise num = H S, den = H c to a few float64 ulps, and the
    same weights."""
    rng = np.random.default_rng(m * 100 + n)
    M, D = m * n, 6
    som = dg.SOM_Batch(m, n, D, dtype=dtype, topology=topology)
    topo = torch.from_numpy(som._topography).to(cuda)
    c = np.where(rng.random(M) < 0.3, 0.0, rng.integers(1, 500, M)).astype(np.float64)
    S = rng.standard_normal((M, D)) * c[:, None]
    Sd, cd = torch.from_numpy(S).to(cuda), torch.from_numpy(c).to(cuda)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    sfx = '_f64' if dtype == np.float64 else ''
    s = torch.cuda.current_stream().cuda_stream
    for sigma in (0.7, 3.0, 40.0):
        w1, w2 = (torch.empty((M, D), dtype=tdt, device=cuda) for _ in range(2))
        n1, n2 = (torch.empty((M, D), dtype=torch.float64, device=cuda) for _ in range(2))
        d1, d2 = (torch.empty(M, dtype=torch.float64, device=cuda) for _ in range(2))
        native.call('somgb_neighbourhood_update' + sfx, Sd.data_ptr(), cd.data_ptr(), topo.data_ptr(), M, D, sigma,
                    w1.data_ptr(), n1.data_ptr(), d1.data_ptr(), s)
        nb = int(native.lib().somgb_neighbourhood_grid_workspace_bytes(m, n, D))
        ws = torch.empty(nb, dtype=torch.uint8, device=cuda)
        native.call('somgb_neighbourhood_update_grid' + sfx, Sd.data_ptr(), cd.data_ptr(), topo.data_ptr(), m, n, D,
                    sigma, w2.data_ptr(), n2.data_ptr(), d2.data_ptr(), ws.data_ptr(), nb, s)
        torch.cuda.synchronize()
        np.testing.assert_allclose(n2.cpu().numpy(), n1.cpu().numpy(), rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(d2.cpu().numpy(), d1.cpu().numpy(), rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(w2.cpu().numpy(), w1.cpu().numpy(), rtol=1e-6 if dtype == np.float32 else 1e-12,
                                   atol=1e-7)
    with pytest.raises(native.SomgbError):
        native.call('somgb_neighbourhood_update_grid' + sfx, Sd.data_ptr(), cd.data_ptr(), topo.data_ptr(), m, n, D,
                    1.0, w2.data_ptr(), None, None, ws.data_ptr(), nb - 8, s)


def test_edge_cases_tc_padded(cuda, native):
    """The golden edge cases through the tensor-core pass: two zero features pad D=6 to 8 without changing any
    distance, so every output must equal the reference's."""
    g = golden('edge_projection')
    pad = lambda a: np.concatenate([a, np.zeros((a.shape[0], 2), a.dtype)], axis=1)
    som = _som(4, 5, 8, pad(g['w0']), algo='tc')
    x = pad(g['x'])
    assert np.array_equal(som.get_winners(x), g['winners'])
    assert np.array_equal(som.get_activation_map(x), g['activation'])
    assert np.array_equal(som.get_activation_map(x, g['rho']), g['activation_weighted'])
    np.testing.assert_allclose(som.compute_errors(x), g['errors'], rtol=1e-6)
    np.testing.assert_allclose(som.compute_errors(x, g['rho']), g['errors_weighted'], rtol=1e-6)


TC_STRESS = [
    ('lognormal-outliers', 16, 32, 32, 200_000),
    ('mixture', 8, 16, 16, 150_000),
    ('near-ties', 16, 16, 16, 100_000),
    ('far-offset', 4, 20, 20, 100_000),
    ('uniform', 32, 8, 16, 60_000),
    ('duplicates', 8, 10, 10, 50_000),
    # maps whose unit operand streams through shared memory (64x64 at D = 8 and 16: rings of 4 column tiles; D = 32:
    # 3 tiles), more than 8 column tiles with a resident operand (64x64 at D = 4), and 9 column tiles (48x48)
    ('large-streamed', 16, 64, 64, 30_000),
    ('large-streamed', 32, 64, 64, 20_000),
    ('large-streamed', 8, 64, 64, 30_000),
    ('large-streamed', 16, 32, 64, 30_000),
    ('large-streamed', 4, 64, 64, 30_000),
    ('large-streamed', 16, 48, 48, 30_000),
    # more than 16 column tiles: the 80x80 grids of the mixed-training configuration (25 tiles) and 128x128 (64)
    ('large-streamed', 16, 80, 80, 30_000),
    ('large-streamed', 32, 80, 80, 20_000),
    ('large-streamed', 8, 128, 128, 10_000),
]


@pytest.mark.parametrize('kind,d,m,n,N', TC_STRESS)
def test_tc_stress_vs_oracle(cuda, native, oracle, kind, d, m, n, N):
    """BMUs, second BMUs (through the error sums) and activation counts of the tensor-core pass on inputs built to
    stress its error bound: outliers, near-tied units, data far from the origin, duplicated units."""
    from decontamination_gb300 import synthetic
    rng = np.random.default_rng(zlib.crc32(kind.encode()))
    M = m * n
    if kind == 'lognormal-outliers':
        x = synthetic.correlated_lognormal(N, d, 7)
        w = x[rng.integers(0, N, M)] * (1 + 0.01 * rng.standard_normal((M, d))).astype(np.float32)
    elif kind == 'mixture':
        x = synthetic.gaussian_mixture(N, d, 8)
        w = x[rng.integers(0, N, M)].copy()
    elif kind == 'near-ties':
        x = rng.random((N, d), dtype=np.float32)
        base = rng.random((M // 2, d), dtype=np.float32)
        w = np.concatenate([base, base * (1 + 1e-6 * rng.standard_normal(base.shape)).astype(np.float32)])
    elif kind == 'far-offset':
        x = (1.0e4 + rng.standard_normal((N, d))).astype(np.float32)
        w = (1.0e4 + 0.7 * rng.standard_normal((M, d))).astype(np.float32)
    elif kind == 'large-streamed':
        x = synthetic.correlated_lognormal(N, d, 11)
        w = x[rng.integers(0, N, M)] * (1 + 0.02 * rng.standard_normal((M, d))).astype(np.float32)
    elif kind == 'uniform':
        x = rng.random((N, d), dtype=np.float32)
        w = rng.random((M, d), dtype=np.float32)
    else:
        x = synthetic.gaussian_mixture(N, d, 9)
        w = x[rng.integers(0, N, M)].copy()
        w[M // 2:] = w[:M - M // 2]
    w = np.ascontiguousarray(w, dtype=np.float32)
    som = _som(m, n, d, w, algo='tc')
    assert np.array_equal(som.get_winners(x), oracle.find_bmus(w, x, 'numba'))
    h = oracle.count_bmus(w, x, None, 'numba')
    assert np.array_equal(som.get_activation_map(x).ravel(), h.astype(np.float32))
    topo = oracle.topography(m, n, 'square')
    o = oracle.compute_errors_raw(w, topo, x, None, 2.0, 'numba')
    np.testing.assert_allclose(som.compute_errors(x), o[:2] / o[2], rtol=ERR_RTOL)


@pytest.mark.parametrize('algo', ALGOS)
def test_near_tied_best_two_units(cuda, native, oracle, algo):
    """Rows of the benchmark catalogue whose two nearest units are closer than float32 rounding (the third well
    apart), against the benchmark's initial map. The BMU must be the reference's in both the BMU-only pass and the
    pass that also produces the error sums (which ranks the best two), and the error sums must match."""
    from decontamination_gb300 import synthetic
    g = golden('near_ties')
    x = np.ascontiguousarray(np.tile(g['x'], (64, 1)))
    w = synthetic.uniform_weights(1024, 16, 2)
    b = oracle.find_bmus(w, x, 'numba')
    assert np.array_equal(b[:len(g['x'])], g['oracle_bmu'])
    som = _som(32, 32, 16, w, topology='hexagonal', algo=algo)
    assert np.array_equal(som.get_winners(x), b)
    topo = oracle.topography(32, 32, 'hexagonal')
    N, M, D = x.shape[0], 1024, 16
    xd, wd, td = (torch.from_numpy(a).to(cuda) for a in (x, w, topo))
    bmu = torch.empty(N, dtype=torch.int32, device=cuda)
    err = torch.zeros(3, dtype=torch.float64, device=cuda)
    A = native.ALGOS[algo]
    nbytes = native.workspace_bytes(native.OP_FIND_BMUS, N, M, D, A)
    ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=cuda)
    wsp = ws.data_ptr() + (-ws.data_ptr()) % 256
    native.call('somgb_train_bmu_pass', xd.data_ptr(), None, N, D, wd.data_ptr(), td.data_ptr(), M, 1.0, A,
                bmu.data_ptr(), err.data_ptr(), wsp, nbytes, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(bmu.cpu().numpy(), b)
    o = oracle.compute_errors_raw(w, topo, x, None, 1.0, 'numba')
    np.testing.assert_allclose(err.cpu().numpy(), o, rtol=ERR_RTOL)
