"""PCA initialisation, covariance and the hyper-parameter grid search against the reference's own outputs
(tests/golden/pca_*.npz and hyparam_search.npz, written by tests/golden/make_pca_golden.py)."""

import numpy as np
import pytest
import torch

from conftest import golden


def test_pca_grid_weights_from_the_reference_covariance():
    """The host half of SOM_PCA (eigen-decomposition and grid) reproduces the reference's weights from the same
    covariance (the reference's own Welford result), without a GPU."""
    from decontamination_gb300.som_pca import SOM_PCA
    g = golden('pca_init')
    c = golden('pca_covariance')
    cov = c['cov_plain']
    for tag, m, n, kw in [('plain', 5, 7, {}), ('scaled', 6, 4, dict(scale_by_variance=True, min_weight=-1.0)),
                          ('cdf', 4, 4, dict(apply_cdf=True, cdf_gain=1.5))]:
        ev, _, w = SOM_PCA._grid_weights(cov, kw.get('min_weight', 0.0), kw.get('max_weight', 1.0), m, n, 6,
                                         kw.get('scale_by_variance', False), kw.get('apply_cdf', False),
                                         kw.get('cdf_gain', 1.0))
        np.testing.assert_allclose(w.astype(np.float32).reshape(m * n, 6), g[f'{tag}_weights'], rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(ev.astype(np.float32), g[f'{tag}_eigenvalues'], rtol=1e-6)


def test_chunk_moments_combine_to_the_whole():
    """The host-side pairwise update of chunk moments gives the moments of the whole weighted catalogue."""
    from decontamination_gb300.covariance import combine_moments
    rng = np.random.default_rng(3)
    x = rng.standard_normal((5000, 5)) * [1.0, 3.0, 0.5, 2.0, 1.0] + 7.0
    w = rng.random(5000)

    def moments(xs, ws):
        W = ws.sum()
        mu = (ws[:, None] * xs).sum(0) / W
        c = xs - mu
        return W, mu, (ws[:, None] * c).T @ c

    W, mu, M2 = 0.0, np.zeros(5), np.zeros((5, 5))
    for a in range(0, 5000, 1300):
        W, mu, M2 = combine_moments(W, mu, M2, *moments(x[a:a + 1300], w[a:a + 1300]))
    W0, mu0, M20 = moments(x, w)
    assert W == pytest.approx(W0, rel=1e-14)
    np.testing.assert_allclose(mu, mu0, rtol=1e-13)
    np.testing.assert_allclose(M2, M20, rtol=1e-12)
    assert combine_moments(W, mu, M2, 0.0, mu * 0, M2 * 0)[0] == W   # an empty chunk changes nothing


def test_grid_points_follow_the_reference():
    from decontamination_gb300.hyparam_finder_som import HypParamFinder_SOM
    g = golden('hyparam_search')
    pts = HypParamFinder_SOM(g['x']).grid()
    assert len(pts) == 64
    assert (int(g['m']), float(g['sigma'])) in pts
    assert all(isinstance(m, int) for m, _ in pts)
    with pytest.raises(NotImplementedError):
        HypParamFinder_SOM(g['x'], batch=False).find(1)


def test_argument_errors_are_the_reference_ones():
    """The reference's ValueErrors (algo/covariance.py:152,239, algo/som_pca.py:54,253,257), raised before any
    device work; online grids are not provided."""
    from decontamination_gb300 import Covariance, HypParamFinder_SOM, SOM_PCA
    with pytest.raises(ValueError):
        Covariance.compute(3, np.zeros((4, 3), dtype=np.float32), ddof=-1)
    with pytest.raises(ValueError):
        Covariance.diagonalize(np.zeros((3, 2)))
    with pytest.raises(ValueError):
        SOM_PCA(4, 4, 1)
    pca = SOM_PCA(4, 4, 3)
    with pytest.raises(ValueError):
        pca.train_from_cov_matrix(np.eye(3), min_weight=1.0, max_weight=1.0)
    with pytest.raises(ValueError):
        pca.train_from_cov_matrix(np.eye(3), apply_cdf=True, cdf_gain=0.0)
    with pytest.raises(NotImplementedError):
        HypParamFinder_SOM(np.zeros((100, 3), dtype=np.float32), batch=False).find(2)


def test_gndm_arithmetic_follows_the_reference():
    """compute_gndm's densities from given maps (decontamination_som.py:603-626): n_gal and n_pix are the map sums,
    gnd = catalogue / footprint where the footprint map is positive and NaN elsewhere, gndm = gnd at each winner."""
    from decontamination_gb300.gndm import compute_gndm

    class Som:
        m, n, dtype = 2, 3, np.float32

        def get_footprint_maps(self, x, rho):
            cat = np.array([[4.0, 0.0, 3.0], [1.5, 2.0, 0.0]], dtype=np.float32)
            foot = np.array([[2.0, 0.0, 3.0], [3.0, 0.0, 1.0]], dtype=np.float32)
            return cat, foot, np.array([0, 2, 3, 1, 5, 0], dtype=np.int32)

    r = compute_gndm(Som(), None, None)
    assert r['n_gal'] == np.float32(10.5) and r['n_pix'] == np.float32(9.0)
    want = np.array([[2.0, np.nan, 1.0], [0.5, np.nan, 0.0]], dtype=np.float32)
    assert r['gnd'].dtype == np.float32
    np.testing.assert_array_equal(r['gnd'], want)
    np.testing.assert_array_equal(r['gndm'], want.ravel()[[0, 2, 3, 1, 5, 0]])


@pytest.mark.gpu
def test_covariance_on_the_gpu(cuda):
    import decontamination_gb300 as dg
    c = golden('pca_covariance')
    x, w = c['x'], c['w']
    np.testing.assert_allclose(dg.Covariance.compute(6, x), c['cov_plain'], rtol=1e-10, atol=1e-13)
    chunks = lambda: (lambda: (x[a:a + 700] for a in range(0, 3000, 700)))
    wchunks = lambda: (lambda: (w[a:a + 700] for a in range(0, 3000, 700)))
    np.testing.assert_allclose(dg.Covariance.compute(6, chunks, wchunks, ddof=0), c['cov_weighted_ddof0'],
                               rtol=1e-10, atol=1e-13)
    # device tensors, float64 data, a large catalogue against numpy's float64 two-pass result
    rng = np.random.default_rng(7)
    big = rng.standard_normal((3_000_000, 16)).astype(np.float32) * rng.random(16).astype(np.float32) + 3.0
    ref = np.cov(big.astype(np.float64), rowvar=False, ddof=1)
    np.testing.assert_allclose(dg.Covariance.compute(16, torch.from_numpy(big).to(cuda)), ref, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(dg.Covariance.compute(6, x.astype(np.float64)), c['cov_plain'], rtol=1e-10, atol=1e-13)
    with pytest.raises(ValueError):
        dg.Covariance.compute(6, x[:1])


@pytest.mark.gpu
def test_som_pca_train(cuda):
    import decontamination_gb300 as dg
    g = golden('pca_init')
    for tag, m, n, topo, kw in [('plain', 5, 7, 'hexagonal', {}),
                                ('scaled', 6, 4, 'square', dict(scale_by_variance=True, min_weight=-1.0)),
                                ('cdf', 4, 4, 'hexagonal', dict(apply_cdf=True, cdf_gain=1.5))]:
        som = dg.SOM_PCA(m, n, 6, topology=topo)
        som.train(g['x'], **kw)
        np.testing.assert_allclose(som.weights, g[f'{tag}_weights'].reshape(som.weights.shape), rtol=1e-5,
                                   atol=1e-6)


@pytest.mark.gpu
def test_hyparam_search_matches_the_reference(cuda):
    import decontamination_gb300 as dg
    g = golden('hyparam_search')
    m, alpha, sigma, idx, qes, tes = dg.HypParamFinder_SOM(g['x'], topology='hexagonal').find(2)
    assert (m, idx) == (int(g['m']), int(g['idx'])) and alpha is None
    assert sigma == pytest.approx(float(g['sigma']), rel=1e-12)
    # the reference's pure-Python mode sums distances in float32 (the GPU follows the compiled reference's float64):
    # the quantization errors agree to float32 rounding, the topographic errors do not on a hexagonal map, whose
    # nearest neighbours sit at squared topographic distance 1.0, the penalty itself
    np.testing.assert_allclose(qes, g['qes'], rtol=1e-5)
    # the winning grid point trained directly gives the same errors
    x = g['x']
    pca = dg.SOM_PCA(m, m, 4, topology='hexagonal')
    pca.train(x)
    som = dg.SOM_Batch(m, m, 4, topology='hexagonal', sigma=sigma)
    som.init_from(pca)
    som.train(x, n_epochs=2)
    np.testing.assert_allclose(som.quantization_errors, qes, rtol=1e-12)
    np.testing.assert_allclose(som.topographic_errors, tes, rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize('N,dtype', [(50_000, np.float32), (2 * (1 << 20) + 777, np.float32), (40_000, np.float64)])
def test_footprint_maps_fuse_the_three_calls(cuda, N, dtype):
    """get_footprint_maps (one BMU pass + one histogram kernel) equals get_activation_map weighted and unweighted and
    get_winners; compute_gndm follows the reference's _compute_gndm arithmetic on them."""
    import decontamination_gb300 as dg
    from decontamination_gb300.gndm import compute_gndm
    rng = np.random.default_rng(N)
    x = (rng.standard_normal((N, 8)) * 2.0).astype(dtype)
    x[rng.integers(0, N, 20)] = np.nan
    rho = rng.random(N) * 3.0
    rho[rng.integers(0, N, 100)] = 0.0
    som = dg.SOM_Batch(12, 10, 8, dtype=dtype, topology='square')
    som.init_rand(seed=5)
    som._weights[...] = som._weights * 4.0 - 2.0
    cat, foot, win = som.get_footprint_maps(x, rho)
    assert np.array_equal(win, som.get_winners(x))
    np.testing.assert_allclose(cat, som.get_activation_map(x, rho), rtol=1e-12)
    assert np.array_equal(foot, som.get_activation_map(x))
    out = compute_gndm(som, x, rho)
    gnd = np.full(cat.shape, np.nan, dtype=dtype)
    np.divide(cat, foot, out=gnd, where=foot > 0.0)
    np.testing.assert_allclose(out['gnd'], gnd, rtol=1e-12)
    np.testing.assert_allclose(out['gndm'], gnd.reshape(-1)[win], rtol=1e-12)
    assert out['n_pix'] == N
