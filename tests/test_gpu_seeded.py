"""GPU tests of the seeded tensor-core pass, its larger maps and its bounded waits (through the C ABI).

The seeded training pass (somgb_train_bmu_pass_seeded) takes each row's best two units under an earlier map. They
only bound the search, so every output must be the unseeded pass's, bit for bit, whatever the pairs hold: the true
previous units, random units, duplicates, -1 or indices out of range. Its pairs output must be the oracle's best two
units, also when it started without seeds (the first pass of a training). Maps above 4096 units (80x80, as in the
mixed-training configuration) take the tensor-core path and must match the oracle. A row tile whose samples are
withheld (the test hook) makes a bounded wait run out: the pass reports it in its own workspace's status word and in
the device status word, and the next call is exact again.
"""

import ctypes

import numpy as np
import pytest
import torch

from decontamination_gb300 import synthetic

pytestmark = pytest.mark.gpu

ERR_RTOL = 1e-9


def _ws(native, op, n, m, d, algo, device):
    nbytes = native.workspace_bytes(op, n, m, d, algo)
    buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
    return buf, buf.data_ptr() + (-buf.data_ptr()) % 256, nbytes


def _pass(native, xd, wd, td, penalty, algo, pairs=None, with_bmu=True, with_err=True, pairs_in=1):
    """One training BMU pass (with pairs when given; seeded by them when pairs_in): (bmu or None, err3 or None)."""
    n, d = xd.shape
    m = wd.shape[0]
    s = torch.cuda.current_stream().cuda_stream
    bmu = torch.full((n,), -7, dtype=torch.int32, device=xd.device) if with_bmu else None
    err = torch.zeros(3, dtype=torch.float64, device=xd.device) if with_err else None
    buf, wsp, nbytes = _ws(native, native.OP_FIND_BMUS, n, m, d, algo, xd.device)
    ptr = lambda t: None if t is None else t.data_ptr()
    if pairs is None:
        native.call('somgb_train_bmu_pass', xd.data_ptr(), None, n, d, wd.data_ptr(), td.data_ptr(), m, penalty, algo,
                    ptr(bmu), ptr(err), wsp, nbytes, s)
    else:
        native.call('somgb_train_bmu_pass_seeded', xd.data_ptr(), None, n, d, wd.data_ptr(), td.data_ptr(), m,
                    penalty, algo, ptr(bmu), ptr(err), pairs.data_ptr(), pairs_in, wsp, nbytes, s)
    torch.cuda.synchronize()
    return (None if bmu is None else bmu.cpu().numpy()), (None if err is None else err.cpu().numpy())


SEED_SHAPES = [   # (m, n, d, N, topology)
    (32, 32, 16, 60_000, 'hexagonal'),
    (64, 64, 16, 40_000, 'square'),
    (64, 64, 32, 30_000, 'square'),
    (80, 80, 16, 30_000, 'square'),
    (80, 80, 32, 20_000, 'hexagonal'),
    (12, 10, 8, 50_000, 'square'),
    (10, 10, 4, 100_000, 'square'),
]


@pytest.mark.parametrize('m,n,d,N,topology', SEED_SHAPES)
def test_seeded_pass_is_the_unseeded_pass(cuda, native, oracle, m, n, d, N, topology):
    rng = np.random.default_rng(m * 7 + d)
    M = m * n
    x = synthetic.correlated_lognormal(N, d, 5)
    w_prev = x[rng.integers(0, N, M)] * (1 + 0.02 * rng.standard_normal((M, d))).astype(np.float32)
    w = (w_prev * (1 + 0.003 * rng.standard_normal((M, d)))).astype(np.float32)   # the next epoch's map, nearby
    topo = oracle.topography(m, n, topology)
    pen = 2.0 if topology == 'square' else 1.0
    xd, wpd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w_prev, w, topo))
    tc = native.ALGO_TC
    if not native.lib().somgb_algo_supported(tc, N, M, d):
        pytest.fail(f'{m}x{n}, D={d} must take the tensor-core path')
    b_ref, e_ref = _pass(native, xd, wd, td, pen, tc)                    # unseeded
    np.testing.assert_array_equal(b_ref, oracle.find_bmus(w, x, 'numba'))
    np.testing.assert_allclose(e_ref, oracle.compute_errors_raw(w, topo, x, None, pen, 'numba'), rtol=ERR_RTOL)
    # the training flow: pairs filled by a pass on the earlier map, then the seeded pass on this one
    pairs = torch.full((N, 2), -1, dtype=torch.int32, device=cuda)
    _pass(native, xd, wpd, td, pen, tc, pairs, pairs_in=0)
    kinds = {'previous map': pairs.clone()}
    kinds['random units'] = torch.from_numpy(rng.integers(0, M, (N, 2)).astype(np.int32)).to(cuda)
    dup = rng.integers(0, M, N).astype(np.int32)
    kinds['duplicated unit'] = torch.from_numpy(np.stack([dup, dup], 1)).to(cuda)
    kinds['unknown'] = torch.full((N, 2), -1, dtype=torch.int32, device=cuda)
    kinds['out of range'] = torch.from_numpy(rng.choice([M, M + 5, -3, 1 << 30], (N, 2)).astype(np.int32)).to(cuda)
    for name, p in kinds.items():
        for with_err in (True, False):
            b, e = _pass(native, xd, wd, td, pen, tc, p.clone(), with_err=with_err)
            assert np.array_equal(b, b_ref), f'{name}, err={with_err}: {int(np.sum(b != b_ref))} BMU mismatches'
            if with_err:
                np.testing.assert_allclose(e, e_ref, rtol=ERR_RTOL, err_msg=name)
        # the error pass alone (no BMU output)
        _, e = _pass(native, xd, wd, td, pen, tc, p.clone(), with_bmu=False)
        np.testing.assert_allclose(e, e_ref, rtol=ERR_RTOL, err_msg=f'{name}, errors only')


@pytest.mark.parametrize('m,n,d,N', [(32, 32, 16, 60_000), (80, 80, 32, 20_000)])
def test_seeded_pass_reports_the_best_two_units(cuda, native, oracle, m, n, d, N):
    rng = np.random.default_rng(11)
    M = m * n
    x = synthetic.correlated_lognormal(N, d, 6)
    w = x[rng.integers(0, N, M)] * (1 + 0.02 * rng.standard_normal((M, d))).astype(np.float32)
    topo = oracle.topography(m, n, 'square')
    xd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w, topo))
    i1, i2, _, _ = oracle.top2(w, x, 'numba')
    pairs = torch.full((N, 2), -1, dtype=torch.int32, device=cuda)
    _pass(native, xd, wd, td, 2.0, native.ALGO_TC, pairs, pairs_in=0)   # error sums: both units ranked exactly
    p = pairs.cpu().numpy()
    assert np.array_equal(p[:, 0], i1) and np.array_equal(p[:, 1], i2)
    pairs.fill_(-1)
    _pass(native, xd, wd, td, 2.0, native.ALGO_TC, pairs, with_err=False, pairs_in=0)   # BMU only: the best unit
    p = pairs.cpu().numpy()
    assert np.array_equal(p[:, 0], i1)
    assert np.all(p[:, 1] != p[:, 0])


def test_fp32_form_leaves_pairs_unchanged(cuda, native, oracle):
    rng = np.random.default_rng(12)
    N, M, d = 20_000, 256, 16
    x = synthetic.correlated_lognormal(N, d, 7)
    w = x[rng.integers(0, N, M)].copy()
    topo = oracle.topography(16, 16, 'square')
    xd, wd, td = (torch.from_numpy(a).to(cuda) for a in (x, w, topo))
    seeds = torch.from_numpy(rng.integers(0, M, (N, 2)).astype(np.int32)).to(cuda)
    p = seeds.clone()
    b, e = _pass(native, xd, wd, td, 2.0, native.ALGO_FP32, p)
    assert torch.equal(p, seeds)
    np.testing.assert_array_equal(b, oracle.find_bmus(w, x, 'numba'))
    np.testing.assert_allclose(e, oracle.compute_errors_raw(w, topo, x, None, 2.0, 'numba'), rtol=ERR_RTOL)


def test_bounded_wait_runs_out_and_the_next_call_is_exact(cuda, native):
    """The producer never loads one row tile's samples (test hook, short wait limit): the pass returns with its
    status set instead of hanging, and a normal call afterwards gives exactly the BMUs of a normal call before."""
    rng = np.random.default_rng(13)
    N, M, d = 200_000, 1024, 16
    x = synthetic.correlated_lognormal(N, d, 8)
    w = x[rng.integers(0, N, M)].copy()
    xd, wd = torch.from_numpy(x).to(cuda), torch.from_numpy(w).to(cuda)
    s = torch.cuda.current_stream().cuda_stream
    buf, wsp, nbytes = _ws(native, native.OP_FIND_BMUS, N, M, d, native.ALGO_TC, cuda)
    buf2, wsp2, _ = _ws(native, native.OP_FIND_BMUS, N, M, d, native.ALGO_TC, cuda)
    st = ctypes.c_uint(0)
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    assert st.value == 0

    def find(ws_ptr):
        out = torch.full((N,), -7, dtype=torch.int32, device=cuda)
        native.call('somgb_find_bmus', xd.data_ptr(), N, d, wd.data_ptr(), M, native.ALGO_TC, out.data_ptr(), ws_ptr,
                    nbytes, s)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    before = find(wsp)
    native.call('somgb_workspace_status', wsp, ctypes.addressof(st), 0, s)
    assert st.value == 0
    native.call('somgb_debug_tc_withhold', 5, 20_000)
    find(wsp)                                          # returns early on the GPU; the C call itself succeeds
    native.call('somgb_workspace_status', wsp, ctypes.addressof(st), 0, s)
    assert st.value != 0, 'the call whose wait ran out reports it in its own workspace'
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    assert st.value != 0
    native.call('somgb_device_status', ctypes.addressof(st), 0, s)
    assert st.value == 0, 'reading with clear resets the device status'
    after = find(wsp2)                                 # the hook is one-shot
    assert np.array_equal(after, before)
    native.call('somgb_workspace_status', wsp2, ctypes.addressof(st), 0, s)
    assert st.value == 0
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    assert st.value == 0


def test_debug_hook_arguments_are_checked(native):
    with pytest.raises(native.SomgbError):
        native.call('somgb_debug_tc_withhold', -1, 100)
    with pytest.raises(native.SomgbError):
        native.call('somgb_debug_tc_withhold', 0, 0)
