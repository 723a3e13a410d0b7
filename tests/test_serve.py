"""The serving loop: queueing, packing, admission and failure isolation on CPU with a fake executor; results against
the direct API calls on the GPU."""

import threading
import time

import numpy as np
import pytest

from decontamination_gb300.serve import SomServer


class FakeExecutor:
    """Records the batches it is given; BMU i of a request is its first value; a row of NaN makes a pass raise."""

    def __init__(self, free=10 ** 9, block_first=False):
        self.free = free
        self.release = threading.Event()
        if not block_first:
            self.release.set()
        self.bmu_batches = []
        self.trained = []

    def free_bytes(self):
        return self.free

    def load(self, som):
        return {'M': 4, 'D': 2, 'name': som}

    def footprint(self, entry, kind, n, weighted):
        return 100 * n + (50 if weighted else 0)

    def run_bmu(self, entry, xs, slot=0, hist=None):
        self.release.wait(5)
        self.bmu_batches.append([len(x) for x in xs])
        for x in xs:
            if np.isnan(np.asarray(x)).any():
                raise ValueError('poisoned request')
        out = [np.full(len(x), int(np.asarray(x)[0, 0]), dtype=np.int32) for x in xs]
        return [(o, np.bincount(o, minlength=4).astype(np.float64)) if h else o
                for o, h in zip(out, hist or [False] * len(xs))]

    def run_activation(self, entry, x, rho, slot=0):
        return ('activation', entry['name'], len(x))

    def run_errors(self, entry, x, rho, slot=0):
        return (0.5, 0.25)

    def run_train(self, som, dataset, rho, kwargs, slot=0):
        time.sleep(0.05)
        self.trained.append((som, len(dataset), kwargs))
        return som


def _req(v, n=10):
    return np.full((n, 2), float(v), dtype=np.float32)


def test_small_requests_on_one_map_are_packed():
    ex = FakeExecutor(block_first=True)
    srv = SomServer(ex, max_batch_rows=1000, workers=1)
    m0, m1 = srv.add_map('a'), srv.add_map('b')
    first = srv.submit_bmu(m0, _req(0))
    time.sleep(0.1)   # the loop now holds the first request inside the executor
    futs = [srv.submit_bmu(m0, _req(i)) for i in range(1, 6)] + [srv.submit_bmu(m1, _req(9))] + \
           [srv.submit_bmu(m0, _req(7))]
    ex.release.set()
    assert first.result(5)[0] == 0
    got = [f.result(5) for f in futs]
    assert [g[0] for g in got] == [1, 2, 3, 4, 5, 9, 7]
    srv.close()
    # the five queued requests on map 0 share a pass; the map-1 request breaks the run
    assert ex.bmu_batches == [[10], [10] * 5, [10], [10]]
    assert srv.batch_sizes() == [1, 5, 1, 1]


def test_row_cap_splits_packs():
    ex = FakeExecutor(block_first=True)
    srv = SomServer(ex, max_batch_rows=100, workers=1)
    m = srv.add_map('a')
    f0 = srv.submit_bmu(m, _req(0, 40))
    time.sleep(0.1)
    futs = [srv.submit_bmu(m, _req(i, 40)) for i in range(5)]
    ex.release.set()
    f0.result(5)
    for f in futs:
        assert len(f.result(5)) == 40
    srv.close()
    assert ex.bmu_batches == [[40], [40, 40], [40, 40], [40]]
    # a request above the cap is served alone
    ex2 = FakeExecutor()
    with SomServer(ex2, max_batch_rows=100, workers=1) as srv2:
        assert len(srv2.submit_bmu(srv2.add_map('a'), _req(3, 150)).result(5)) == 150
    assert ex2.bmu_batches == [[150]]


def test_admission_rejects_what_can_never_fit_and_serves_the_rest():
    ex = FakeExecutor()
    with SomServer(ex, hbm_budget=5000) as srv:
        m = srv.add_map('a')
        big = srv.submit_bmu(m, _req(1, 60))       # 6000 bytes > budget
        small = srv.submit_bmu(m, _req(2, 10))
        with pytest.raises(MemoryError):
            big.result(5)
        assert small.result(5)[0] == 2


def test_a_failing_request_fails_alone():
    ex = FakeExecutor(block_first=True)
    srv = SomServer(ex, max_batch_rows=10, workers=1)
    m = srv.add_map('a')
    f0 = srv.submit_bmu(m, _req(0))
    time.sleep(0.1)
    bad = np.full((10, 2), np.nan, dtype=np.float32)
    fb = srv.submit_bmu(m, bad)
    f1 = srv.submit_bmu(m, _req(1))
    ex.release.set()
    assert f0.result(5)[0] == 0
    with pytest.raises(ValueError):
        fb.result(5)
    assert f1.result(5)[0] == 1
    srv.close()
    assert 'bmu' in srv.stats() and srv.stats()['bmu']['count'] == 2


def test_a_device_timeout_fails_only_its_own_request():
    """An executor pass whose device-side wait ran out raises a timeout status (the executor reads its own
    workspace's status word): that request's future gets the error, the others their results."""
    from decontamination_gb300 import _native

    class TimingOut(FakeExecutor):
        def run_bmu(self, entry, xs, slot=0, hist=None):
            if any(np.asarray(x)[0, 0] == 13 for x in xs):
                raise _native.SomgbError(_native.SOMGB_ERR_TIMEOUT, 'a device-side wait gave up')
            return super().run_bmu(entry, xs, slot, hist)

    with SomServer(executor=TimingOut(), max_batch_rows=10, workers=1) as srv:
        mid = srv.add_map('m')
        futs = [srv.submit_bmu(mid, _req(v)) for v in (1, 13, 2)]
        assert np.all(futs[0].result(5) == 1) and np.all(futs[2].result(5) == 2)
        with pytest.raises(_native.SomgbError) as ei:
            futs[1].result(5)
        assert ei.value.status == _native.SOMGB_ERR_TIMEOUT


def test_other_kinds_training_and_stats():
    ex = FakeExecutor()
    with SomServer(ex) as srv:
        m = srv.add_map('a')
        fa = srv.submit_activation(m, _req(0, 7))
        fe = srv.submit_errors(m, _req(0, 7), rho=np.ones(7))
        assert fa.result(5) == ('activation', 'a', 7)
        assert fe.result(5) == (0.5, 0.25)
    st = srv.stats()
    assert st['activation']['count'] == 1 and st['errors']['count'] == 1
    assert st['errors']['p99_ms'] >= st['errors']['p50_ms'] >= 0.0
    with pytest.raises(RuntimeError):
        srv.submit_bmu(m, _req(0))


class BarrierExecutor(FakeExecutor):
    """run_bmu returns only once two calls are in it at the same time (or after 5 s, flagging the timeout)."""

    def __init__(self):
        super().__init__()
        self.barrier = threading.Barrier(2, timeout=5)
        self.timed_out = False

    def run_bmu(self, entry, xs, slot=0, hist=None):
        try:
            self.barrier.wait()
        except threading.BrokenBarrierError:
            self.timed_out = True
        return super().run_bmu(entry, xs, slot=slot, hist=hist)


def test_two_workers_run_batches_at_the_same_time():
    ex = BarrierExecutor()
    with SomServer(ex, max_batch_rows=10, workers=2) as srv:
        m = srv.add_map('a')
        f1, f2 = srv.submit_bmu(m, _req(1)), srv.submit_bmu(m, _req(2, 10))
        assert f1.result(10)[0] == 1 and f2.result(10)[0] == 2
    assert not ex.timed_out


class SlowLargeExecutor(FakeExecutor):
    """Batches of more than 10 rows wait for `release`; small ones return at once."""

    def run_bmu(self, entry, xs, slot=0, hist=None):
        if sum(len(x) for x in xs) > 10:
            self.release.wait(5)
        self.bmu_batches.append([len(x) for x in xs])
        return [np.full(len(x), int(np.asarray(x)[0, 0]), dtype=np.int32) for x in xs]


def test_small_requests_pass_large_ones_on_the_second_worker():
    ex = SlowLargeExecutor(block_first=True)
    with SomServer(ex, max_batch_rows=10, workers=2) as srv:
        m = srv.add_map('a')
        big1 = srv.submit_bmu(m, _req(1, 50))
        time.sleep(0.1)                       # the first worker holds it
        big2 = srv.submit_bmu(m, _req(2, 50))
        small = srv.submit_bmu(m, _req(3, 5))
        assert small.result(2)[0] == 3        # served beside big1, ahead of big2
        assert not big1.done() and not big2.done()
        ex.release.set()
        assert big1.result(5)[0] == 1 and big2.result(5)[0] == 2


def test_bmu_requests_with_histograms():
    ex = FakeExecutor()
    with SomServer(ex, workers=1) as srv:
        m = srv.add_map('a')
        b, h = srv.submit_bmu(m, _req(3), histogram=True).result(5)
        assert b[0] == 3 and h[3] == 10 and h.sum() == 10
        assert srv.submit_bmu(m, _req(2)).result(5)[0] == 2


class _Som:
    dim, m, n = 2, 2, 2


def test_training_runs_on_its_own_loop_while_assignments_continue():
    ex = FakeExecutor()
    with SomServer(ex) as srv:
        m = srv.add_map('a')
        ft = srv.submit_train(_Som(), _req(0, 12), n_epochs=3)
        fb = srv.submit_bmu(m, _req(4))
        assert fb.result(5)[0] == 4
        assert isinstance(ft.result(5), _Som)
    assert ex.trained[0][1:] == (12, {'n_epochs': 3})
    assert srv.stats()['train']['count'] == 1


class CountingExecutor(FakeExecutor):
    """Records how many run_bmu calls were inside it at once."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.inside = 0
        self.most = 0
        self.lock = threading.Lock()

    def run_bmu(self, entry, xs, slot=0, hist=None):
        with self.lock:
            self.inside += 1
            self.most = max(self.most, self.inside)
        try:
            return super().run_bmu(entry, xs, slot=slot, hist=hist)
        finally:
            with self.lock:
                self.inside -= 1


def test_in_flight_bytes_hold_back_a_request_until_it_fits():
    """Two 2000-byte requests under a 2500-byte budget: the second worker may not start the second one while the
    first is on the device, however idle it is; it runs once the first has finished."""
    ex = CountingExecutor(block_first=True)
    with SomServer(ex, hbm_budget=2500, max_batch_rows=10, workers=2) as srv:
        m = srv.add_map('a')
        f0 = srv.submit_bmu(m, _req(0, 20))
        time.sleep(0.1)
        f1 = srv.submit_bmu(m, _req(1, 20))
        time.sleep(0.2)
        assert not f1.done()
        ex.release.set()
        assert f0.result(5)[0] == 0 and f1.result(5)[0] == 1
    assert ex.most == 1


def test_unknown_map_and_oversized_training_are_refused():
    ex = FakeExecutor()
    with SomServer(ex, hbm_budget=10_000) as srv:
        with pytest.raises(KeyError):
            srv.submit_bmu(3, _req(0))
        big = srv.submit_train(_Som(), _req(0, 10_000), n_epochs=1)
        with pytest.raises(MemoryError):
            big.result(5)
        small = srv.submit_train(_Som(), _req(0, 12), n_epochs=1)
        assert isinstance(small.result(5), _Som)


class FailingTrainExecutor(FakeExecutor):
    def run_train(self, som, dataset, rho, kwargs, slot=0):
        if kwargs.get('n_epochs') == 0:
            raise ValueError('no epochs')
        return super().run_train(som, dataset, rho, kwargs, slot=slot)


def test_a_failing_training_fails_alone():
    ex = FailingTrainExecutor()
    with SomServer(ex) as srv:
        m = srv.add_map('a')
        bad = srv.submit_train(_Som(), _req(0, 5), n_epochs=0)
        good = srv.submit_train(_Som(), _req(0, 5), n_epochs=2)
        fb = srv.submit_bmu(m, _req(3))
        with pytest.raises(ValueError):
            bad.result(5)
        assert isinstance(good.result(5), _Som)
        assert fb.result(5)[0] == 3
    assert srv.stats()['train']['count'] == 1


def test_close_serves_what_is_queued():
    ex = FakeExecutor(block_first=True)
    srv = SomServer(ex, workers=1)
    m = srv.add_map('a')
    futs = [srv.submit_bmu(m, _req(i)) for i in range(4)]
    t = threading.Thread(target=srv.close)
    t.start()
    time.sleep(0.05)
    ex.release.set()
    t.join(5)
    assert [f.result(0)[0] for f in futs] == [0, 1, 2, 3]


@pytest.mark.gpu
def test_served_results_match_the_direct_calls(cuda):
    import decontamination_gb300 as dg
    from decontamination_gb300 import synthetic
    x = synthetic.gaussian_mixture(300_000, 16, 4)
    som = dg.SOM_Batch(16, 16, 16, topology='hexagonal')
    som._weights[...] = x[np.random.default_rng(1).integers(0, len(x), 256)].reshape(som._weights.shape)
    rho = np.random.default_rng(2).random(len(x))
    sizes = [1000, 37, 250_000, 5000, 20_000, 1]
    parts, r = [], 0
    for s in sizes:
        parts.append(np.ascontiguousarray(x[r:r + s]))
        r += s
    with SomServer(max_batch_rows=1 << 16) as srv:
        mid = srv.add_map(som)
        fb = [srv.submit_bmu(mid, p) for p in parts]
        fa = srv.submit_activation(mid, x, rho)
        fe = srv.submit_errors(mid, x)
        fh = [srv.submit_bmu(mid, p, histogram=True) for p in parts]
        for p, f in zip(parts, fb):
            assert np.array_equal(f.result(120), som.get_winners(p))
        for p, f in zip(parts, fh):
            b, h = f.result(120)
            assert np.array_equal(b, som.get_winners(p))
            assert np.array_equal(h, som.get_activation_map(p).reshape(-1).astype(np.float64))
        assert np.array_equal(fa.result(120), som.get_activation_map(x, rho))
        np.testing.assert_allclose(fe.result(120), som.compute_errors(x), rtol=1e-12)
        # mixed training jobs (grid sizes, topologies, feature counts, catalogue sizes) served together give the maps
        # of the same trainings run alone
        jobs = [(8, 8, 4, 'square', 20_000, 6), (16, 16, 8, 'hexagonal', 120_000, 4), (32, 32, 16, 'hexagonal',
                200_000, 3), (12, 12, 32, 'square', 60_000, 5)]
        futs, alone = [], []
        for i, (mm, nn, dd, topo, nrow, ep) in enumerate(jobs):
            xj = np.ascontiguousarray(synthetic.gaussian_mixture(nrow, dd, 10 + i))
            for target in (futs, alone):
                s_ = dg.SOM_Batch(mm, nn, dd, topology=topo)
                s_.init_rand(seed=i)
                if target is futs:
                    target.append(srv.submit_train(s_, xj, n_epochs=ep))
                else:
                    s_.train(xj, n_epochs=ep)
                    target.append(s_)
        for f, s_ in zip(futs, alone):
            t_ = f.result(300)
            # BMUs and fixed-point sums are exact; the float64 flush order may move a weight by a float32 ulp
            np.testing.assert_allclose(t_.weights, s_.weights, rtol=1e-6, atol=1e-7)
            np.testing.assert_allclose(t_.quantization_errors, s_.quantization_errors, rtol=1e-9)
        # a training request gives the same map as training directly
        a = dg.SOM_Batch(8, 8, 16, topology='square')
        b = dg.SOM_Batch(8, 8, 16, topology='square')
        a.init_rand(seed=3)
        b.init_rand(seed=3)
        ft = srv.submit_train(a, x[:50_000], n_epochs=3)
        b.train(x[:50_000], n_epochs=3)
        assert np.array_equal(ft.result(120).weights, b.weights)


@pytest.mark.gpu
def test_a_large_pinned_request_is_served_in_pieces(cuda):
    """A request of pinned host rows above serve.PIECE_MIN is uploaded in pieces, each piece's BMU pass running as soon
    as it has landed: the BMUs and the histogram equal the direct calls, and a bounded wait that runs out in the first
    piece's pass fails the request although the later passes clear their workspace's status word."""
    import ctypes
    import torch
    import decontamination_gb300 as dg
    from decontamination_gb300 import synthetic, serve, _native
    from decontamination_gb300.serve import GpuExecutor
    n = serve.PIECE_MIN + 300_001
    x = synthetic.gaussian_mixture(n, 16, 7)
    som = dg.SOM_Batch(32, 32, 16, topology='square')
    som._weights[...] = x[np.random.default_rng(3).integers(0, n, 1024)].reshape(som._weights.shape)
    som.bmu_algo = 'tc'
    xp = torch.from_numpy(x).pin_memory()
    want = som.get_winners(x)
    ex = GpuExecutor(workers=2)
    entry = ex.load(som)
    b, h = ex.run_bmu(entry, [xp], slot=1, hist=[True])[0]
    assert np.array_equal(b, want)
    assert np.array_equal(h, np.bincount(want, minlength=1024).astype(np.float64))
    _native.call('somgb_debug_tc_withhold', 3, 20_000)   # this thread's next pass: the first piece's
    with pytest.raises(_native.SomgbError) as ei:
        ex.run_bmu(entry, [xp], slot=0)
    assert ei.value.status == _native.SOMGB_ERR_TIMEOUT
    assert np.array_equal(ex.run_bmu(entry, [xp], slot=0)[0], want)
    with SomServer() as srv:   # and through the request loop
        mid = srv.add_map(som)
        assert np.array_equal(srv.submit_bmu(mid, xp).result(120), want)
    st = ctypes.c_uint(0)
    _native.call('somgb_device_status', ctypes.addressof(st), 1, torch.cuda.current_stream().cuda_stream)
