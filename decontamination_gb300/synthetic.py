"""Seeded synthetic catalogues with the shapes and value distributions of the benchmark workloads.

No real survey systematics maps are available, so these generators stand in for them:

* ``gaussian_mixture`` — k equal-weight isotropic Gaussians in D dimensions, means U[-3, 3]^D, sigma 0.5
  (the 10x10, D=4 workload and the serving catalogues);
* ``correlated_lognormal`` — systematics-like features: z = L eps with eps ~ N(0, I) and L the Cholesky factor of a
  seeded correlation matrix Q diag(lambda) Q^T (Q Haar-orthogonal, lambda log-spaced with condition number 100,
  rescaled to unit diagonal); x = exp(0.3 z); 2 % of the rows (seeded) are scaled by 10.

Both use numpy's PCG64 streams seeded by (seed, stream, chunk index) and produce the same values on every host,
whatever the number of threads used to fill the chunks.
"""

import concurrent.futures
import os

import numpy as np

CHUNK = 1 << 20


def _fill(out, fn, threads=None):
    n = out.shape[0]
    starts = list(range(0, n, CHUNK))

    def work(ci):
        s = starts[ci]
        e = min(n, s + CHUNK)
        out[s:e] = fn(ci, e - s)

    with concurrent.futures.ThreadPoolExecutor(threads or min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(work, range(len(starts))))
    return out


def gaussian_mixture(n, d, seed, k=5, spread=3.0, sigma=0.5):
    means = np.random.default_rng(seed).uniform(-spread, spread, size=(k, d))

    def chunk(ci, rows):
        rng = np.random.default_rng([seed, 1, ci])
        return means[rng.integers(0, k, rows)] + sigma * rng.standard_normal((rows, d))

    return _fill(np.empty((n, d), dtype=np.float32), chunk)


def correlation_cholesky(d, seed, cond=100.0):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((d, d))
    q, r = np.linalg.qr(a)
    q = q * np.sign(np.diag(r))              # Haar-distributed orthogonal matrix
    lam = np.logspace(0.0, np.log10(cond), d)
    c = (q * lam) @ q.T
    s = 1.0 / np.sqrt(np.diag(c))
    c = c * s[:, None] * s[None, :]
    return np.linalg.cholesky(c)


def correlated_lognormal(n, d, seed, scale=0.3, outlier_frac=0.02, outlier_scale=10.0):
    L = correlation_cholesky(d, seed)

    def chunk(ci, rows):
        rng = np.random.default_rng([seed, 1, ci])
        x = np.exp(scale * (rng.standard_normal((rows, d)) @ L.T))
        x[rng.random(rows) < outlier_frac] *= outlier_scale
        return x

    return _fill(np.empty((n, d), dtype=np.float32), chunk)


def uniform_weights(m, d, seed, low=-1.0, high=1.0):
    return np.random.default_rng([seed, 3]).uniform(low, high, size=(m, d)).astype(np.float32)


def correlated_lognormal_device(n, d, seed, device, scale=0.3, outlier_frac=0.02, outlier_scale=10.0,
                                chunk=1 << 22):
    """The recipe of ``correlated_lognormal`` generated on the device (a torch float32 tensor), for catalogues too
    large to generate and copy from the host in a benchmark's time: the same correlation factor L, the same
    log-normal transform and outlier fraction, with torch's seeded generator in place of numpy's streams (so the
    values differ from ``correlated_lognormal``'s, the distribution does not)."""
    import torch
    L = torch.from_numpy(correlation_cholesky(d, seed).T.copy()).to(device=device, dtype=torch.float32)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed) * 1000003 + 17)
    out = torch.empty((n, d), dtype=torch.float32, device=device)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        z = torch.randn((e - s, d), generator=g, device=device, dtype=torch.float32) @ L
        x = torch.exp(scale * z)
        mask = torch.rand(e - s, generator=g, device=device) < outlier_frac
        x[mask] *= outlier_scale
        out[s:e] = x
    return out


def gaussian_mixture_device(n, d, seed, device, k=5, spread=3.0, sigma=0.5):
    """The recipe of ``gaussian_mixture`` generated on the device (torch's seeded generator; same means, values
    differ from the host generator's)."""
    import torch
    means = torch.from_numpy(np.random.default_rng(seed).uniform(-spread, spread, size=(k, d))).to(
        device=device, dtype=torch.float32)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed) * 1000003 + 29)
    idx = torch.randint(0, k, (n,), generator=g, device=device)
    return (means[idx] + sigma * torch.randn((n, d), generator=g, device=device)).contiguous()
