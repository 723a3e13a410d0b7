#!/usr/bin/env python3
"""Generate tests/golden/near_ties.npz: catalogue rows whose two nearest units are closer than float32 rounding.

The rows come from the benchmark catalogue (decontamination_gb300.synthetic.correlated_lognormal with N = 12582912,
D = 16, seed 2) against its initial map (uniform_weights(1024, 16, 2)): for each of them the float32 distance chain
cannot order the best two units while the third is well separated. They pin the tensor-core pass's decision rule in
its error-sum mode, where both the order of the best two and the identity of the second matter. The oracle's BMUs
and error sums are recomputed at test time; the fixture holds the rows only.

Usage::

    python tests/golden/make_near_ties.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ROWS = [629180, 1266837, 1684150, 2202612, 7236927, 8341309, 8667712, 9792349, 10148774, 11970629, 12480606]


def main():
    from decontamination_gb300 import synthetic
    from oracle import somref
    x = synthetic.correlated_lognormal(12_582_912, 16, 2)[ROWS].copy()
    w = synthetic.uniform_weights(1024, 16, 2)
    fac = 1.0 + 8.0 * 18 * 2.0 ** -24
    keep = []
    for i in range(len(ROWS)):
        xr = x[i]
        df = np.zeros(1024, np.float32)   # float32 FMA chain in feature order
        for k in range(16):
            t = (w[:, k] - xr[k]).astype(np.float32)
            df = (np.longdouble(t) * t + np.longdouble(df)).astype(np.float32)
        o = np.argsort(df, kind='stable')[:3]
        f = df[o]
        if not f[1] > f[0] * fac and f[2] > f[1] * fac:
            keep.append(i)
    x = x[keep]
    b = somref.find_bmus(w, x, 'numba')
    np.savez(os.path.join(HERE, 'near_ties.npz'), x=x, rows=np.array(ROWS)[keep], oracle_bmu=b)
    print(f'{len(keep)} rows kept')


if __name__ == '__main__':
    main()
