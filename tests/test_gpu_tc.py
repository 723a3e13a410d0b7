"""GPU tests of the tensor-core pass's training entry point on large maps and of its bounded waits (C ABI).

Maps above 4096 units (80x80, as in the mixed-training configuration, and 128x128) take the tensor-core path, and the
training pass must give the oracle's BMUs and error sums. A row tile whose samples are withheld (the test hook) makes a
bounded wait run out: the pass reports it in its own workspace's status word and in the device status word instead of
hanging, and the next call is exact again.
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


@pytest.mark.parametrize('m,n,d,N,topology', [(80, 80, 16, 30_000, 'square'), (80, 80, 32, 20_000, 'hexagonal'),
                                               (128, 128, 8, 10_000, 'square'), (64, 64, 16, 40_000, 'square')])
def test_training_pass_on_large_maps(cuda, native, oracle, m, n, d, N, topology):
    rng = np.random.default_rng(m * 7 + d)
    M = m * n
    x = synthetic.correlated_lognormal(N, d, 5)
    w = x[rng.integers(0, N, M)] * (1 + 0.02 * rng.standard_normal((M, d))).astype(np.float32)
    topo = oracle.topography(m, n, topology)
    pen = 2.0 if topology == 'square' else 1.0
    assert native.lib().somgb_algo_supported(native.ALGO_TC, N, M, d), 'must take the tensor-core path'
    xd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w, topo))
    s = torch.cuda.current_stream().cuda_stream
    bmu = torch.full((N,), -7, dtype=torch.int32, device=cuda)
    err = torch.zeros(3, dtype=torch.float64, device=cuda)
    buf, wsp, nbytes = _ws(native, native.OP_FIND_BMUS, N, M, d, native.ALGO_TC, cuda)
    native.call('somgb_train_bmu_pass', xd.data_ptr(), None, N, d, wd.data_ptr(), td.data_ptr(), M, pen,
                native.ALGO_TC, bmu.data_ptr(), err.data_ptr(), wsp, nbytes, s)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bmu.cpu().numpy(), oracle.find_bmus(w, x, 'numba'))
    np.testing.assert_allclose(err.cpu().numpy(), oracle.compute_errors_raw(w, topo, x, None, pen, 'numba'),
                               rtol=ERR_RTOL)
    st = ctypes.c_uint(1)
    native.call('somgb_workspace_status', wsp, ctypes.addressof(st), 0, s)
    assert st.value == 0


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
    with pytest.raises(native.SomgbError):
        native.call('somgb_debug_iter_withhold', -1, 100)
    with pytest.raises(native.SomgbError):
        native.call('somgb_debug_iter_withhold', 0, 0)


def test_a_wait_that_runs_out_fails_only_its_own_call(cuda, native):
    """The serving executor and the API methods read the status word of their own workspace: the pass whose wait ran
    out raises, the same request on the other worker's slot and the next calls give the normal results."""
    import decontamination_gb300 as dg
    from decontamination_gb300.serve import GpuExecutor
    rng = np.random.default_rng(14)
    N, d = 200_000, 16
    x = synthetic.correlated_lognormal(N, d, 9)
    som = dg.SOM_Batch(32, 32, d, topology='square')
    som._weights[...] = x[rng.integers(0, N, 1024)].reshape(som._weights.shape)
    som.bmu_algo = 'tc'
    ex = GpuExecutor(workers=2)
    entry = ex.load(som)
    want = ex.run_bmu(entry, [x], slot=1)[0]
    native.call('somgb_debug_tc_withhold', 3, 20_000)
    with pytest.raises(native.SomgbError) as ei:
        ex.run_bmu(entry, [x], slot=0)
    assert ei.value.status == native.SOMGB_ERR_TIMEOUT
    assert np.array_equal(ex.run_bmu(entry, [x], slot=1)[0], want)
    assert np.array_equal(ex.run_bmu(entry, [x], slot=0)[0], want)
    native.call('somgb_debug_tc_withhold', 2, 20_000)
    with pytest.raises(native.SomgbError):
        som.get_winners(x)
    assert np.array_equal(som.get_winners(x), want)
    st = ctypes.c_uint(0)
    native.call('somgb_device_status', ctypes.addressof(st), 1, torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize('m,n,d,topology,algo,N', [
    # the tensor-core contraction (K4): the 64x64 D = 16 map, one partial 512-unit tile, a single grid row, tiles that
    # end inside a grid row, a tile across two long grid rows and one inside a row, the largest D, a batch or two
    # (AUTO where D has no tensor-core BMU search: BMUs on the CUDA cores, the contraction on the tensor cores)
    (64, 64, 16, 'square', 'tc', 15_000), (32, 32, 16, 'hexagonal', 'tc', 60_000),
    (20, 17, 5, 'square', 'auto', 60_000), (1, 300, 3, 'hexagonal', 'auto', 20_000),
    (80, 80, 8, 'hexagonal', 'tc', 8_000), (2, 300, 4, 'square', 'tc', 10_000), (64, 64, 31, 'square', 'auto', 10_000),
    (32, 32, 16, 'square', 'tc', 37), (32, 32, 4, 'square', 'tc', 64), (40, 40, 20, 'square', 'auto', 10_000),
    # a single grid column
    (100, 1, 4, 'square', 'tc', 20_000),
    # D = 32 to 47: three M tiles per CTA
    (64, 64, 32, 'square', 'tc', 15_000), (30, 30, 40, 'hexagonal', 'auto', 8_000),
    # the float32 CUDA-core pass: the FP32 algorithm, D above the tensor-core contraction's limit of 47, and grid rows
    # too long for the tensor-core contraction's tables
    (32, 32, 16, 'hexagonal', 'fp32', 60_000), (20, 17, 5, 'square', 'fp32', 60_000),
    (32, 32, 32, 'square', 'fp32', 20_000), (20, 20, 50, 'square', 'auto', 8_000),
    (1, 9, 3, 'hexagonal', 'fp32', 60_000), (3, 700, 4, 'square', 'tc', 10_000)])
def test_grid_iteration_pass_matches_the_float64_pass(cuda, native, oracle, m, n, d, topology, algo, N):
    """Iteration mode: the grid-factorised pass (somgb_train_iter_pass_grid; the tensor-core contraction for the TC
    algorithm, the float32 CUDA-core pass otherwise) against the float64 pass over an arbitrary topography
    (somgb_train_iter_pass) on the same rows: the same numerators and denominators to 2e-6."""
    rng = np.random.default_rng(m * n + d)
    M = m * n
    x = synthetic.correlated_lognormal(N, d, 9) if d >= 4 else rng.standard_normal((N, d)).astype(np.float32)
    w = x[rng.integers(0, N, M)].copy()
    rho = rng.random(N)
    rho[rng.random(N) < 0.05] = 0.0
    topo = oracle.topography(m, n, topology)
    xd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w, topo))
    rd = torch.from_numpy(rho).to(cuda)
    s = torch.cuda.current_stream().cuda_stream
    out = []
    for grid in (True, False):
        num = torch.zeros((M, d), dtype=torch.float64, device=cuda)
        den = torch.zeros(M, dtype=torch.float64, device=cuda)
        A = native.ALGOS[algo] if grid else native.ALGO_FP32
        buf, wsp, nbytes = _ws(native, native.OP_EPOCH, N, M, d, A, cuda)
        if grid:
            native.call('somgb_train_iter_pass_grid', xd.data_ptr(), rd.data_ptr(), N, d, wd.data_ptr(), td.data_ptr(),
                        m, n, 6.0, 1000, 2 * N, A, num.data_ptr(), den.data_ptr(), wsp, nbytes, s)
        else:
            native.call('somgb_train_iter_pass', xd.data_ptr(), rd.data_ptr(), N, d, wd.data_ptr(), td.data_ptr(), M,
                        6.0, 1000, 2 * N, num.data_ptr(), den.data_ptr(), wsp, nbytes, s)
        torch.cuda.synchronize()
        out.append((num.cpu().numpy(), den.cpu().numpy()))
    (n_g, d_g), (n_r, d_r) = out
    np.testing.assert_allclose(d_g, d_r, rtol=2e-6, atol=1e-9 * d_r.max())
    np.testing.assert_allclose(n_g, n_r, rtol=2e-6, atol=2e-6 * np.abs(n_r).max())
    st = ctypes.c_uint(0)
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    assert st.value == 0, 'no bounded wait ran out'


def _iter_pass(native, cuda, xd, rd, wd, td, m, n, sigma0, algo, ws=None):
    N, d = xd.shape
    M = m * n
    num = torch.zeros((M, d), dtype=torch.float64, device=cuda)
    den = torch.zeros(M, dtype=torch.float64, device=cuda)
    buf, wsp, nbytes = ws if ws is not None else _ws(native, native.OP_EPOCH, N, M, d, algo, cuda)
    s = torch.cuda.current_stream().cuda_stream
    if algo is None:
        native.call('somgb_train_iter_pass', xd.data_ptr(), None if rd is None else rd.data_ptr(), N, d, wd.data_ptr(),
                    td.data_ptr(), M, sigma0, 500, 2 * N, num.data_ptr(), den.data_ptr(), wsp, nbytes, s)
    else:
        native.call('somgb_train_iter_pass_grid', xd.data_ptr(), None if rd is None else rd.data_ptr(), N, d,
                    wd.data_ptr(), td.data_ptr(), m, n, sigma0, 500, 2 * N, algo, num.data_ptr(), den.data_ptr(), wsp,
                    nbytes, s)
    torch.cuda.synchronize()
    return num.cpu().numpy(), den.cpu().numpy()


@pytest.mark.parametrize('sigma0', [6.0, 1e-13])
@pytest.mark.parametrize('algo', ['tc', 'fp32'])
def test_iteration_pass_edge_cases(cuda, native, oracle, sigma0, algo):
    """Non-finite rows (no training BMU: they add nothing), zero weights (likewise), and sigma clamped at 1e-12 (every
    factor 0 but the BMU's own, 1): both grid forms against the float64 pass."""
    rng = np.random.default_rng(int(sigma0 > 1) + 2 * (algo == 'tc'))
    m = n = 32
    d, N, M = 16, 30_000, 1024
    x = synthetic.correlated_lognormal(N, d, 4)
    w = x[rng.integers(0, N, M)].copy()
    x[rng.choice(N, N // 50, replace=False), rng.integers(0, d)] = np.nan
    rho = rng.random(N)
    rho[rng.random(N) < 0.05] = 0.0
    topo = oracle.topography(m, n, 'hexagonal')
    xd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w, topo))
    rd = torch.from_numpy(rho).to(cuda)
    n_g, d_g = _iter_pass(native, cuda, xd, rd, wd, td, m, n, sigma0, native.ALGOS[algo])
    n_r, d_r = _iter_pass(native, cuda, xd, rd, wd, td, m, n, sigma0, None, _ws(native, native.OP_EPOCH, N, M, d,
                                                                                   native.ALGO_FP32, cuda))
    assert np.isfinite(n_g).all() and np.isfinite(d_g).all()
    np.testing.assert_allclose(d_g, d_r, rtol=2e-6, atol=1e-9 * d_r.max())
    np.testing.assert_allclose(n_g, n_r, rtol=2e-6, atol=2e-6 * np.abs(n_r).max())


def test_a_wait_of_the_iteration_contraction_that_runs_out(cuda, native, oracle):
    """The test hook withholds the completion of the first accumulator group: every CTA's fold wait runs out, the call
    reports bit 65536 in its workspace's and the device's status words instead of hanging, and the next call gives the
    normal sums."""
    rng = np.random.default_rng(23)
    m = n = 32
    d, N, M = 16, 50_000, 1024
    x = synthetic.correlated_lognormal(N, d, 6)
    w = x[rng.integers(0, N, M)].copy()
    topo = oracle.topography(m, n, 'square')
    xd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (x, w, topo))
    s = torch.cuda.current_stream().cuda_stream
    ws1 = _ws(native, native.OP_EPOCH, N, M, d, native.ALGO_TC, cuda)
    ws2 = _ws(native, native.OP_EPOCH, N, M, d, native.ALGO_TC, cuda)
    st = ctypes.c_uint(0)
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    before = _iter_pass(native, cuda, xd, None, wd, td, m, n, 8.0, native.ALGO_TC, ws1)
    native.call('somgb_debug_iter_withhold', 0, 20_000)
    _iter_pass(native, cuda, xd, None, wd, td, m, n, 8.0, native.ALGO_TC, ws1)
    native.call('somgb_workspace_status', ws1[1], ctypes.addressof(st), 0, s)
    assert st.value & 65536, 'the call whose wait ran out reports it in its own workspace'
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    assert st.value & 65536
    after = _iter_pass(native, cuda, xd, None, wd, td, m, n, 8.0, native.ALGO_TC, ws2)   # the hook is one-shot
    np.testing.assert_allclose(after[0], before[0], rtol=1e-12, atol=1e-12 * np.abs(before[0]).max())
    np.testing.assert_allclose(after[1], before[1], rtol=1e-12)
    native.call('somgb_workspace_status', ws2[1], ctypes.addressof(st), 0, s)
    assert st.value == 0
    native.call('somgb_device_status', ctypes.addressof(st), 1, s)
    assert st.value == 0


def test_iteration_training_through_the_api_on_the_tensor_cores(cuda, native):
    """SOM_Batch.train(n_vectors=...) with the tensor-core algorithm (BMU pass and contraction on the tensor cores) and
    with the FP32 algorithm (both on the CUDA cores) give the same map; a wait of the contraction that runs out fails
    the call with SOMGB_ERR_TIMEOUT, and the next call trains normally."""
    import decontamination_gb300 as dg
    m = n = 32
    d, N = 16, 300_000
    x = torch.from_numpy(synthetic.correlated_lognormal(N, d, 8)).to(cuda)
    w0 = synthetic.uniform_weights(m * n, d, 8)
    maps = {}
    for algo in ('tc', 'fp32'):
        som = dg.SOM_Batch(m, n, d, topology='hexagonal', sigma=8.0)
        som._weights[...] = w0.reshape(som._weights.shape)
        som.bmu_algo = algo
        som.train(x, n_vectors=N)
        maps[algo] = (som.weights.copy(), som.quantization_errors.copy())
    np.testing.assert_allclose(maps['tc'][0], maps['fp32'][0], rtol=2e-5, atol=2e-6)
    np.testing.assert_allclose(maps['tc'][1], maps['fp32'][1], rtol=1e-5)
    som = dg.SOM_Batch(m, n, d, topology='hexagonal', sigma=8.0)
    som._weights[...] = w0.reshape(som._weights.shape)
    som.bmu_algo = 'tc'
    native.call('somgb_debug_iter_withhold', 0, 20_000)
    with pytest.raises(native.SomgbError) as ei:
        som.train(x, n_vectors=N)
    assert ei.value.status == native.SOMGB_ERR_TIMEOUT
    som._weights[...] = w0.reshape(som._weights.shape)
    som.train(x, n_vectors=N)
    np.testing.assert_allclose(som.weights, maps['tc'][0], rtol=1e-9, atol=1e-12)
    st = ctypes.c_uint(0)
    native.call('somgb_device_status', ctypes.addressof(st), 1, torch.cuda.current_stream().cuda_stream)
