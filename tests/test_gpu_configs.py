"""GPU parity at the benchmark configurations, against the CPU oracle.

* The 10x10, D = 4 configuration trained end to end as stated (100,000 rows of the 5-component Gaussian mixture,
  weights U[-1, 1], sigma0 = 5, 10 epochs), with the tensor-core pass and with the plain FP32 form: every epoch's map
  within 1e-5 of the float64 oracle's training, its quantization and topographic errors within 1e-6, and the BMUs
  the GPU computes on each epoch's map identical to the oracle's on that same map.
* Maps of real trainings (the initial map, early epochs while the map contracts, and the last) of the 32x32 hexagonal
  D = 16, 64x64 D = 16 and 64x64 D = 32 configurations, each checked on 1,000,000 catalogue rows: BMUs identical to
  the oracle's, error sums within float64 summation-order rounding.
"""

import numpy as np
import pytest

import decontamination_gb300 as dg
from decontamination_gb300 import synthetic

pytestmark = pytest.mark.gpu

W_RTOL = 1e-5
ERR_RTOL = 1e-9


def _oracle_errors(oracle, w, topo, x, penalty):
    """The compute_errors sums of the oracle from its exact top-2 (reference typing): [sum sqrt(d1), sum of
    topographically distant pairs, rows counted], and its BMUs."""
    i1, i2, d1, _ = oracle.top2(w, x, 'numba')
    ok = (i1 >= 0) & (i2 >= 0) & (i1 != i2)
    t = topo.astype(np.float32)
    dt = (t[i1[ok]] - t[i2[ok]]).astype(np.float32)
    far = (dt * dt).astype(np.float64).sum(1) > penalty
    return np.array([np.sqrt(d1[ok]).sum(), far.sum(), ok.sum()], dtype=np.float64), i1


@pytest.mark.parametrize('algo', ['tc', 'fp32'])
def test_ten_by_ten_configuration_end_to_end(cuda, native, oracle, algo):
    m = n = 10
    d, N, E, sigma0 = 4, 100_000, 10, 5.0
    x = synthetic.gaussian_mixture(N, d, 1)
    w0 = synthetic.uniform_weights(m * n, d, 1)
    som = dg.SOM_Batch(m, n, d, topology='square', sigma=sigma0)
    som._weights[...] = w0.reshape(som._weights.shape)
    som.bmu_algo = algo
    som.train(x, n_epochs=E, use_best_epoch=False)
    ref = oracle.OracleSOM(m, n, d, topology='square', sigma=sigma0, mode='numba', threads=0, accumulate='fp64')
    ref.weights = w0.copy()
    ref.train(x, n_epochs=E, use_best_epoch=False)
    np.testing.assert_allclose(som._history.reshape(E, m * n, d), ref.history, rtol=W_RTOL, atol=1e-6)
    np.testing.assert_allclose(som.quantization_errors, ref.quantization_errors, rtol=1e-6)
    np.testing.assert_allclose(som.topographic_errors, ref.topographic_errors, rtol=1e-6)
    probe = dg.SOM_Batch(m, n, d, topology='square')
    probe.bmu_algo = algo
    for e, wmap in enumerate([w0] + [som._history[k].reshape(m * n, d) for k in range(E)]):
        probe._weights[...] = wmap.reshape(probe._weights.shape)
        got = probe.get_winners(x)
        want = oracle.find_bmus(np.ascontiguousarray(wmap, dtype=np.float32), x, 'numba')
        assert np.array_equal(got, want), f'map {e}: {int(np.sum(got != want))} BMU mismatches'


TRAINED = [   # (m, n, d, topology, sigma0, training rows, epochs of the schedule, maps checked)
    (32, 32, 16, 'hexagonal', 16.0, 1_000_000, 8, (0, 1, 2, 5, 8)),
    (64, 64, 16, 'square', 32.0, 1_000_000, 6, (0, 1, 2, 6)),
    (64, 64, 32, 'square', 32.0, 1_000_000, 4, (0, 1, 4)),
]


@pytest.mark.parametrize('m,n,d,topology,sigma0,N,E,check', TRAINED)
def test_trained_map_states(cuda, native, oracle, m, n, d, topology, sigma0, N, E, check):
    M = m * n
    x = synthetic.correlated_lognormal(N, d, 2 if d == 16 else 3)
    w0 = synthetic.uniform_weights(M, d, 2 if d == 16 else 3)
    som = dg.SOM_Batch(m, n, d, topology=topology, sigma=sigma0)
    som._weights[...] = w0.reshape(som._weights.shape)
    som.bmu_algo = 'tc'
    som.train(x, n_epochs=E, use_best_epoch=False)
    topo = oracle.topography(m, n, topology)
    penalty = 2.0 if topology == 'square' else 1.0
    probe = dg.SOM_Batch(m, n, d, topology=topology)
    probe.bmu_algo = 'tc'
    for e in check:
        wmap = w0 if e == 0 else som._history[e - 1].reshape(M, d)
        wmap = np.ascontiguousarray(wmap, dtype=np.float32)
        probe._weights[...] = wmap.reshape(probe._weights.shape)
        want_err, want_bmu = _oracle_errors(oracle, wmap, topo, x, penalty)
        got = probe.get_winners(x)
        assert np.array_equal(got, want_bmu), f'map {e}: {int(np.sum(got != want_bmu))} BMU mismatches'
        qe, te = probe.compute_errors(x)
        np.testing.assert_allclose([qe, te], want_err[:2] / want_err[2], rtol=ERR_RTOL, err_msg=f'map {e}')
