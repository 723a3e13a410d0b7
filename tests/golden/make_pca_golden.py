#!/usr/bin/env python3
"""Generate golden fixtures for the PCA initialisation and the hyper-parameter grid search from the reference itself.

Test infrastructure, like make_golden.py (whose reference loader it reuses): the reference's own
``Covariance.compute`` (algo/covariance.py), ``SOM_PCA.train`` (algo/som_pca.py) and
``HypParamFinder_SOM.find`` (algo/hyparam_finder_som.py, batch mode) run in the reference's pure-Python mode on
small seeded inputs; the outputs are stored in ``tests/golden/pca_*.npz`` and ``tests/golden/hyparam_*.npz``.

Usage::

    python tests/golden/make_pca_golden.py [--reference /path/to/reference]
"""

import argparse
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import gaussian_mixture, load_reference   # noqa: E402


def make_cases():
    cov = importlib.import_module('decontamination.algo.covariance')
    pca = importlib.import_module('decontamination.algo.som_pca')
    hyp = importlib.import_module('decontamination.algo.hyparam_finder_som')
    cases = {}

    # covariance: unweighted array, weighted chunked generator with non-finite rows and non-positive weights
    rng = np.random.default_rng(101)
    x = gaussian_mixture(rng, 3000, 6)
    x[[5, 77]] = np.nan
    w = rng.random(3000)
    w[[3, 9]] = 0.0
    w[11] = -1.0
    c_plain = cov.Covariance.compute(6, x)
    chunks = lambda: (lambda: (x[a:a + 700] for a in range(0, 3000, 700)))
    wchunks = lambda: (lambda: (w[a:a + 700] for a in range(0, 3000, 700)))
    c_weighted = cov.Covariance.compute(6, chunks, wchunks, ddof=0)
    cases['pca_covariance'] = dict(x=x, w=w, cov_plain=c_plain, cov_weighted_ddof0=c_weighted)

    # SOM_PCA initial weights: plain, scaled by variance, CDF-mapped; hexagonal and square
    out = dict(x=x)
    for tag, m, n, topo, kw in [('plain', 5, 7, 'hexagonal', {}),
                                ('scaled', 6, 4, 'square', dict(scale_by_variance=True, min_weight=-1.0)),
                                ('cdf', 4, 4, 'hexagonal', dict(apply_cdf=True, cdf_gain=1.5))]:
        som = pca.SOM_PCA(m, n, 6, topology=topo)
        som.train(x, **kw)
        out[f'{tag}_weights'] = som.weights.copy()
        out[f'{tag}_eigenvalues'] = som.eigenvalues.copy()
    cases['pca_init'] = out

    # hyper-parameter grid search (batch SOM): a small catalogue, two epochs per grid point
    rng = np.random.default_rng(102)
    xh = gaussian_mixture(rng, 400, 4)
    finder = hyp.HypParamFinder_SOM(xh, topology='hexagonal', batch=True, use_best_epoch=True,
                                    show_progress_bar=False, enable_gpu=False)
    m, alpha, sigma, idx, qes, tes = finder.find(2)
    cases['hyparam_search'] = dict(x=xh, m=m, sigma=sigma, idx=idx, qes=qes, tes=tes)
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('DECONTAMINATION_REFERENCE'), required=not os.environ.get('DECONTAMINATION_REFERENCE'),
                    help='checkout of lpsc-euclid/decontamination 0.0.1 (or set DECONTAMINATION_REFERENCE)')
    ap.add_argument('--out', default=HERE)
    args = ap.parse_args()
    load_reference(args.reference)
    for name, payload in make_cases().items():
        arrays = {k: np.asarray(v) for k, v in payload.items()}
        np.savez_compressed(os.path.join(args.out, f'{name}.npz'), **arrays)
        print(f'wrote {name}.npz: ' + ', '.join(f'{k}{tuple(np.shape(v))}' for k, v in arrays.items()))


if __name__ == '__main__':
    main()
