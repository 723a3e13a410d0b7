"""GPU tests of the row regrouping between epochs (somgb_sort_rows) and of the tensor-core pass on regrouped rows.

* somgb_sort_rows groups the rows by key in increasing order, keys outside [0, m) last, each row with its values and
  its weight.
* On rows grouped by BMU the tensor-core pass recomputes in its second sweeps only the column tiles where a row of the
  128-row tile has a candidate: its BMUs and error sums stay the oracle's, and it computes far fewer column tiles.
* SOM_Batch.train regroups a resident catalogue between epochs: every epoch's map is bit-identical to a training that
  keeps the storage order, and the errors agree to float64 summation order.
"""

import numpy as np
import pytest
import torch

import decontamination_gb300 as dg
from decontamination_gb300 import synthetic

pytestmark = pytest.mark.gpu

ERR_RTOL = 1e-9


def _ws(native, op, n, m, d, algo, device):
    nbytes = native.workspace_bytes(op, n, m, d, algo)
    buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
    return buf, buf.data_ptr() + (-buf.data_ptr()) % 256, nbytes


def _sort(native, cuda, x, key, m, rho=None):
    n, d = x.shape
    xd = torch.from_numpy(np.ascontiguousarray(x)).to(cuda)
    kd = torch.from_numpy(np.ascontiguousarray(key, dtype=np.int32)).to(cuda)
    rd = None if rho is None else torch.from_numpy(np.ascontiguousarray(rho)).to(cuda)
    xs = torch.full_like(xd, float('nan'))
    rs = None if rho is None else torch.full_like(rd, -1.0)
    ws = torch.empty(int(native.lib().somgb_sort_rows_workspace_bytes(m)), dtype=torch.uint8, device=cuda)
    native.call('somgb_sort_rows', xd.data_ptr(), None if rd is None else rd.data_ptr(), kd.data_ptr(), n, d, m,
                xs.data_ptr(), None if rs is None else rs.data_ptr(), ws.data_ptr(), ws.numel(),
                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return xs.cpu().numpy(), None if rs is None else rs.cpu().numpy()


@pytest.mark.parametrize('n,d,with_rho', [(100_003, 16, True), (70_001, 3, False), (50_000, 32, False), (5, 4, True),
                                          (0, 8, False)])
def test_sort_rows_groups_rows_by_key(cuda, native, n, d, with_rho):
    rng = np.random.default_rng(n + d)
    m = 777
    x = rng.standard_normal((n, d)).astype(np.float32)   # rows are distinct, so each output row names its input row
    key = rng.integers(-3, m + 3, n).astype(np.int32)
    key[: n // 3] = 5                                     # a long run of one key (warp-aggregated counts and slots)
    rho = rng.random(n) if with_rho else None
    xs, rs = _sort(native, cuda, x, key, m, rho)
    index = {r.tobytes(): i for i, r in enumerate(x)}
    perm = np.array([index[r.tobytes()] for r in xs], dtype=np.int64)
    assert np.array_equal(np.sort(perm), np.arange(n)), 'a permutation of the rows'
    bucket = np.where((key >= 0) & (key < m), key, m)
    assert np.all(np.diff(bucket[perm]) >= 0), 'grouped by key, in increasing order, out-of-range keys last'
    if with_rho:
        assert np.array_equal(rs, rho[perm])


def _pass(native, cuda, x, w, topo, pen, with_err):
    N, d = x.shape
    M = w.shape[0]
    xd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w, topo))
    s = torch.cuda.current_stream().cuda_stream
    bmu = torch.full((N,), -7, dtype=torch.int32, device=cuda)
    err = torch.zeros(3, dtype=torch.float64, device=cuda)
    buf, wsp, nbytes = _ws(native, native.OP_FIND_BMUS, N, M, d, native.ALGO_TC, cuda)
    if with_err:
        native.call('somgb_train_bmu_pass', xd.data_ptr(), None, N, d, wd.data_ptr(), td.data_ptr(), M, pen,
                    native.ALGO_TC, bmu.data_ptr(), err.data_ptr(), wsp, nbytes, s)
    else:
        native.call('somgb_find_bmus', xd.data_ptr(), N, d, wd.data_ptr(), M, native.ALGO_TC, bmu.data_ptr(), wsp,
                    nbytes, s)
    tiles = np.zeros(1, dtype=np.int64)
    native.call('somgb_last_sweep2_tiles', tiles.ctypes.data, s)
    return bmu.cpu().numpy(), err.cpu().numpy(), int(tiles[0])


def _smooth_map(m, n, d, rng):
    """Units on a smooth 2-D sheet in d dimensions, ordered along the grid like a trained map."""
    gi, gj = np.divmod(np.arange(m * n), n)
    g = np.stack([gi / m, gj / n], 1)
    return np.tanh(g @ rng.standard_normal((2, d)) * 2.0 + rng.standard_normal(d)).astype(np.float32)


@pytest.mark.parametrize('kind,d', [('random', 16), ('smooth', 16), ('clustered', 16), ('smooth', 4), ('smooth', 8),
                                    ('smooth', 32)])
@pytest.mark.parametrize('with_err', [False, True])
def test_tc_pass_on_rows_grouped_by_bmu(cuda, native, oracle, kind, d, with_err):
    """A 64x64 map (16 column tiles of 256 units), D = 4 to 32, rows grouped by their BMU. Random: units are catalogue rows, so a
    row's candidates lie anywhere in the map and every column tile is recomputed. Smooth: the units lie on a sheet
    ordered along the grid, as in a trained map, and the rows near it, so a row tile's candidates lie in a few column
    tiles. Clustered: the rows lie near 40 units only. A few rows are not finite (they go to the exact recheck)."""
    rng = np.random.default_rng(41 + len(kind))
    m = n = 64
    M, N = m * n, 60_000
    if kind == 'random':
        x = synthetic.correlated_lognormal(N, d, 12)
        w = (x[rng.integers(0, N, M)] * (1 + 0.02 * rng.standard_normal((M, d)))).astype(np.float32)
    else:
        w = _smooth_map(m, n, d, rng)
        pick = rng.integers(0, M, N) if kind == 'smooth' else rng.choice(M, 40, replace=False)[rng.integers(0, 40, N)]
        x = (w[pick] + 0.01 * rng.standard_normal((N, d))).astype(np.float32)
    x[rng.choice(N, 7, replace=False), d - 1] = np.nan
    topo = oracle.topography(m, n, 'square')
    order = np.argsort(oracle.find_bmus(w, x, 'numba'), kind='stable')
    xs = np.ascontiguousarray(x[order])
    bmu, err, tiles = _pass(native, cuda, xs, w, topo, 2.0, with_err)
    want = oracle.find_bmus(w, xs, 'numba')
    if with_err:   # training BMUs: -1 for rows without a valid unit (not finite)
        want = np.where(np.isfinite(xs).all(1), want, -1)
    np.testing.assert_array_equal(bmu, want)
    if with_err:
        np.testing.assert_allclose(err, oracle.compute_errors_raw(w, topo, xs, None, 2.0, 'numba'), rtol=ERR_RTOL)
    full = 16 * ((N + 127) // 128)
    assert 0 < tiles <= full
    if kind != 'random':
        assert tiles < (0.35 if kind == 'smooth' else 0.2) * full, (tiles, full)


def test_training_regroups_rows_without_changing_results(cuda, native):
    """SOM_Batch.train on a resident 64x64 catalogue with the rows regrouped between epochs, and with the storage order
    kept: every epoch's map is bit-identical (order-free fixed-point sums) and the errors agree to rounding."""
    m = n = 64
    d, N, E = 16, 200_000, 4
    x = torch.from_numpy(synthetic.correlated_lognormal(N, d, 3)).to(cuda)
    x0 = x.clone()
    w0 = synthetic.uniform_weights(m * n, d, 3)
    runs = []
    for regroup in (True, False):
        som = dg.SOM_Batch(m, n, d, topology='square', sigma=16.0)
        som._weights[...] = w0.reshape(som._weights.shape)
        som.bmu_algo = 'tc'
        calls = []
        if not regroup:
            som._regroups = lambda rows: False
        else:
            inner = som._regroup
            som._regroup = lambda *a: (calls.append(1), inner(*a))
        som.train(x, n_epochs=E, use_best_epoch=False)
        assert len(calls) == (E - 1 if regroup else 0)   # between training epochs
        runs.append((som._history.copy(), som.quantization_errors.copy(), som.topographic_errors.copy()))
    assert np.array_equal(runs[0][0], runs[1][0])
    np.testing.assert_allclose(runs[0][1], runs[1][1], rtol=1e-12)
    np.testing.assert_allclose(runs[0][2], runs[1][2], rtol=1e-12)
    assert torch.equal(x, x0), "the caller's tensor is left as it was"


def test_row_tiles_with_no_candidates_and_with_one_tile(cuda, native, oracle):
    """Whole 128-row tiles whose rows are all non-finite (every row flagged: an empty tile set for sweep 2, every row
    to the exact recheck), and whole tiles of one repeated row (a single column tile), between ordinary rows."""
    rng = np.random.default_rng(77)
    m = n = 64
    M, d, N = m * n, 16, 20_000
    w = _smooth_map(m, n, d, rng)
    x = (w[rng.integers(0, M, N)] + 0.01 * rng.standard_normal((N, d))).astype(np.float32)
    x[128:384] = np.nan                 # row tiles 1 and 2
    x[640:1024] = x[5000]               # row tiles 5 to 7: one row
    topo = oracle.topography(m, n, 'square')
    for with_err in (False, True):
        bmu, err, tiles = _pass(native, cuda, x, w, topo, 2.0, with_err)
        want = oracle.find_bmus(w, x, 'numba')
        if with_err:
            want = np.where(np.isfinite(x).all(1), want, -1)
            np.testing.assert_allclose(err, oracle.compute_errors_raw(w, topo, x, None, 2.0, 'numba'), rtol=ERR_RTOL)
        np.testing.assert_array_equal(bmu, want)
