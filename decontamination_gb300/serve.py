"""Serving loop: BMU-assignment, activation-map, error and training requests on one GPU.

The reference has no server; its callers (``Decontamination_SOM``, ``HypParamFinder_SOM``) call ``get_winners``,
``get_activation_map``, ``compute_errors`` and ``SOM_Batch.train`` one after another. ``SomServer`` takes the same
requests as they arrive, from any thread, and returns futures:

* maps are registered once (``add_map``) and stay resident on the device;
* requests are admitted in arrival order when their device-memory footprint (catalogue, outputs, workspace) fits the
  budget; a request that can never fit is rejected with ``MemoryError``;
* consecutive small BMU-assignment requests on the same map are packed into one pinned host buffer and served by one
  upload, one BMU pass and one download; a BMU request can also return its M-bin activation histogram;
* ``workers`` serving threads (default 2) take admitted batches as they free up, each on its own stream with its own
  staging buffers and workspaces, so that a request arriving while another is on the GPU overlaps it on the device;
  the first worker takes requests in arrival order, the others only packable BMU requests (ahead of larger ones), so
  that small requests run beside a large one rather than behind it;
  training requests run on their own threads and streams (``train_workers``, default 2), so that a long training
  does not hold up assignments and small trainings overlap;
* a request whose computation raises fails alone: its future carries the exception and the loop goes on;
* latency (submit to result on the host) is recorded per kind; ``stats()`` gives count, p50 and p99.
"""

import collections
import concurrent.futures
import threading
import time

import numpy as np

__all__ = ['SomServer', 'GpuExecutor']

KINDS = ('bmu', 'activation', 'errors', 'train')


class _Request:
    __slots__ = ('kind', 'map_id', 'x', 'rho', 'n', 'footprint', 'future', 't_submit', 'kwargs')

    def __init__(self, kind, map_id, x, rho, n, footprint, kwargs=None):
        self.kind, self.map_id, self.x, self.rho, self.n = kind, map_id, x, rho, n
        self.footprint = int(footprint)
        self.future = concurrent.futures.Future()
        self.t_submit = time.perf_counter()
        self.kwargs = kwargs or {}


def _rows(x):
    return int(x.shape[0])


class _Slot:
    """One serving worker's device resources: its stream and pinned host buffers."""

    def __init__(self, torch, device):
        self.stream = torch.cuda.Stream(device=device)
        self.copy_stream = torch.cuda.Stream(device=device)   # uploads of large requests, piece by piece
        self.stage = None   # pinned host staging buffer for packed requests
        self.out = None     # pinned host buffer for packed results


# A single request from pinned host memory of at least PIECE_MIN rows is uploaded in PIECES pieces on the worker's copy
# stream, and the BMU pass of piece p runs while piece p + 1 is copied.
PIECE_MIN = 1 << 21
PIECES = 4


class GpuExecutor:
    """Runs the requests through libsomgb on a CUDA device (float32 maps). `slot` (0 .. workers - 1) selects the
    calling worker's stream, buffers and per-map workspace and map object, so that workers never share scratch."""

    def __init__(self, device=None, workers=2, train_workers=2):
        import torch
        from . import _device, _native
        self._torch, self._dev_mod, self._nat = torch, _device, _native
        self.device = device if device is not None else _device.require_cuda()
        self.slots = [_Slot(torch, self.device) for _ in range(max(1, workers))]
        self.stream = self.slots[0].stream
        self.train_streams = [torch.cuda.Stream(device=self.device) for _ in range(max(1, train_workers))]

    def free_bytes(self):
        free, _ = self._torch.cuda.mem_get_info(self.device)
        return int(free)

    # --- resident maps -------------------------------------------------------------------------------------------------
    def load(self, som):
        """Resident copy of `som`: its weights on the device and a private map object (own workspace), so that later
        changes to `som`, or calls on it from other threads, do not touch what the server uses."""
        from .som_abstract import SOM_Abstract
        if som.dtype != np.float32:
            raise TypeError('the serving loop holds float32 maps')
        owns = []
        for _ in self.slots:
            own = SOM_Abstract(som.m, som.n, som.dim, som.dtype, som.topology)
            own._weights[...] = som._weights
            own.bmu_algo = som.bmu_algo
            owns.append(own)
        torch = self._torch
        with torch.cuda.stream(self.stream):
            w = torch.from_numpy(np.ascontiguousarray(owns[0].weights.reshape(-1, owns[0].dim))).to(self.device)
        self.stream.synchronize()
        return {'soms': owns, 'w': w, 'M': owns[0].m * owns[0].n, 'D': owns[0].dim, 'algo': owns[0]._algo,
                'ws': [self._dev_mod.Workspace() for _ in self.slots]}

    def footprint(self, entry, kind, n, weighted):
        nat = self._nat
        M, D = entry['M'], entry['D']
        op = {'bmu': nat.OP_FIND_BMUS, 'activation': nat.OP_COUNT_BMUS, 'errors': nat.OP_ERRORS}[kind]
        b = n * D * 4 + n * 4 + (n * 8 if weighted else 0)
        return b + nat.workspace_bytes(op, max(n, 1), M, D, entry['algo'])

    # --- requests ------------------------------------------------------------------------------------------------------
    def _pinned(self, sl, attr, nbytes):
        torch = self._torch
        buf = getattr(sl, attr)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8).pin_memory()
            setattr(sl, attr, buf)
        return buf

    def run_bmu(self, entry, xs, slot=0, hist=None):
        """BMUs of every request in `xs` (host arrays or device tensors), packed into one pass; request i also gets
        its activation histogram (unweighted, float64 (M,)) when hist[i], as a (bmu, histogram) pair."""
        torch, nat = self._torch, self._nat
        sl = self.slots[slot]
        M, D = entry['M'], entry['D']
        counts = [_rows(x) for x in xs]
        n = sum(counts)
        hist = hist or [False] * len(xs)
        pieces = None
        with torch.cuda.stream(sl.stream):
            one = xs[0] if len(xs) == 1 and isinstance(xs[0], torch.Tensor) else None
            if one is not None and not one.is_cuda and one.is_pinned() and one.dtype == torch.float32 and \
                    one.is_contiguous() and n >= PIECE_MIN:
                # pinned host rows: copied in pieces on the copy stream, each piece's pass as soon as it has landed
                xd = torch.empty((n, D), dtype=torch.float32, device=self.device)
                bounds = [n * p // PIECES for p in range(PIECES + 1)]
                pieces = []
                for p in range(PIECES):
                    r0, r1 = bounds[p], bounds[p + 1]
                    done = torch.cuda.Event()
                    with torch.cuda.stream(sl.copy_stream):
                        sl.copy_stream.wait_stream(sl.stream)   # xd is allocated on the worker's stream
                        xd[r0:r1].copy_(one[r0:r1], non_blocking=True)
                        done.record(sl.copy_stream)
                    pieces.append((r0, r1, done))
            elif one is not None and (one.is_cuda or one.is_pinned()):
                # device tensor, or pinned host memory: no staging copy
                xd = one.to(device=self.device, dtype=torch.float32, non_blocking=True).contiguous()
            else:
                stage = self._pinned(sl, 'stage', n * D * 4)
                host = stage[:n * D * 4].view(torch.float32).view(n, D)
                hv = host.numpy()
                r = 0
                for x, c in zip(xs, counts):
                    hv[r:r + c] = x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x, dtype=np.float32)
                    r += c
                xd = host.to(self.device, non_blocking=True)
            out = torch.empty(n, dtype=torch.int32, device=self.device)
            nh = sum(1 for h in hist if h)
            hd = torch.zeros((max(nh, 1), M), dtype=torch.float64, device=self.device) if nh else None
            status = torch.zeros(1, dtype=torch.int32, device=self.device)
            if n:
                ws = entry['ws'][slot]
                if pieces is None:
                    pieces = [(0, n, None)]
                wsp, wsb = ws.for_op(nat.OP_FIND_BMUS, max(r1 - r0 for r0, r1, _ in pieces), M, D, entry['algo'],
                                     self.device)
                for r0, r1, done in pieces:
                    if done is not None:
                        sl.stream.wait_event(done)
                    nat.call('somgb_find_bmus', xd[r0:].data_ptr(), r1 - r0, D, entry['w'].data_ptr(), M,
                             entry['algo'], out[r0:].data_ptr(), wsp, wsb, sl.stream.cuda_stream)
                    ws.note_status(status)   # each pass clears the word when it starts
                r, k = 0, 0
                for c, h in zip(counts, hist):
                    if h:
                        nat.call('somgb_bmu_histograms', out[r:].data_ptr(), None, c, M, None, hd[k].data_ptr(),
                                 sl.stream.cuda_stream)
                        k += 1
                    r += c
            ob = self._pinned(sl, 'out', n * 4 + 8 + nh * M * 8)
            oh = ob[:n * 4].view(torch.int32)
            oh.copy_(out, non_blocking=True)
            if nh:
                hh = ob[n * 4 + (-(n * 4)) % 8:][:nh * M * 8].view(torch.float64).view(nh, M)
                hh.copy_(hd[:nh], non_blocking=True)
        sl.stream.synchronize()
        if n and int(status.item()):
            # a bounded wait of this pass gave up: this batch fails, and no other (the word is this workspace's)
            raise nat.SomgbError(nat.SOMGB_ERR_TIMEOUT, 'a device-side wait gave up; the pass returned early')
        res = oh.numpy().copy()
        hres = hh.numpy().copy() if nh else None
        parts, r, k = [], 0, 0
        for c, h in zip(counts, hist):
            if h:
                parts.append((res[r:r + c], hres[k]))
                k += 1
            else:
                parts.append(res[r:r + c])
            r += c
        return parts

    def run_activation(self, entry, x, rho, slot=0):
        with self._torch.cuda.stream(self.slots[slot].stream):
            return entry['soms'][slot].get_activation_map(x, rho)

    def run_errors(self, entry, x, rho, slot=0):
        with self._torch.cuda.stream(self.slots[slot].stream):
            return entry['soms'][slot].compute_errors(x, rho)

    def run_train(self, som, dataset, rho, kwargs, slot=0):
        st = self.train_streams[slot]
        with self._torch.cuda.stream(st):
            som.train(dataset, rho, **kwargs)
        st.synchronize()
        return som


class SomServer:
    """Request loop over resident maps (see the module docstring).

    executor: the object that runs requests (default: ``GpuExecutor`` on the current CUDA device).
    hbm_budget: device bytes that admitted requests may hold at once (default: 80 % of the free memory at start).
    max_batch_rows: BMU requests with at most this many rows are packed together, up to this many rows per pass.
    workers: serving threads taking admitted batches (the executor keeps a stream and buffers per worker).
    train_workers: training threads (each on its own stream), so that small trainings overlap on the device.
    """

    def __init__(self, executor=None, hbm_budget=None, max_batch_rows=1 << 20, workers=2, train_workers=2):
        self.workers = max(1, int(workers))
        self.train_workers = max(1, int(train_workers))
        self._ex = executor if executor is not None else GpuExecutor(workers=self.workers,
                                                                     train_workers=self.train_workers)
        self.hbm_budget = int(hbm_budget if hbm_budget is not None else 0.8 * self._ex.free_bytes())
        self.max_batch_rows = int(max_batch_rows)
        self._maps = {}
        self._queue = collections.deque()
        self._train_queue = collections.deque()
        self._cv = threading.Condition()
        self._in_flight = 0
        self._closing = False
        self._lat = {k: [] for k in KINDS}
        self._batches = []
        self._threads = [threading.Thread(target=self._serve_loop, args=(i,), name=f'somgb-serve-{i}', daemon=True)
                         for i in range(self.workers)]
        self._threads += [threading.Thread(target=self._train_loop, args=(i,), name=f'somgb-train-{i}', daemon=True)
                          for i in range(self.train_workers)]
        for t in self._threads:
            t.start()

    # --- public API ----------------------------------------------------------------------------------------------------
    def add_map(self, som):
        """Registers `som` (its current weights) as a resident map; returns its id."""
        entry = self._ex.load(som)
        with self._cv:
            mid = len(self._maps)
            self._maps[mid] = entry
        return mid

    def submit_bmu(self, map_id, x, histogram=False):
        """Future of the int32 BMU of every row of `x` (``get_winners``); with `histogram`, of (BMUs, M-bin
        activation histogram) (the unweighted ``get_activation_map`` of `x`, flattened, float64)."""
        return self._submit('bmu', map_id, x, None, {'histogram': bool(histogram)})

    def submit_activation(self, map_id, x, rho=None):
        """Future of the activation map of `x` (``get_activation_map``)."""
        return self._submit('activation', map_id, x, rho)

    def submit_errors(self, map_id, x, rho=None):
        """Future of (QE, TE) of `x` (``compute_errors``)."""
        return self._submit('errors', map_id, x, rho)

    def submit_train(self, som, dataset, dataset_weights=None, **train_kwargs):
        """Future of `som` after ``som.train(dataset, dataset_weights, **train_kwargs)`` (runs on its own stream)."""
        n = _rows(dataset) if hasattr(dataset, 'shape') else 0
        fp = n * som.dim * 4 * 2 + som.m * som.n * som.dim * 8 * 4
        req = _Request('train', None, dataset, dataset_weights, n, fp, train_kwargs)
        req.x = (som, dataset)
        with self._cv:
            self._check_open()
            if req.footprint > self.hbm_budget:
                req.future.set_exception(MemoryError(f'training request needs {req.footprint} device bytes, '
                                                     f'over the {self.hbm_budget}-byte budget'))
                return req.future
            self._train_queue.append(req)
            self._cv.notify_all()
        return req.future

    def stats(self):
        """Per kind: number of completed requests and their p50 / p99 latency in milliseconds."""
        with self._cv:
            out = {}
            for k, v in self._lat.items():
                if v:
                    a = np.asarray(v) * 1e3
                    out[k] = {'count': len(v), 'p50_ms': float(np.percentile(a, 50)),
                              'p99_ms': float(np.percentile(a, 99))}
            return out

    def latencies(self, kind):
        """Latencies (seconds, completion order) of the completed requests of `kind`."""
        with self._cv:
            return list(self._lat[kind])

    def batch_sizes(self):
        """Requests packed into each BMU pass so far."""
        with self._cv:
            return list(self._batches)

    def close(self, wait=True):
        """Stops accepting requests; with `wait`, serves what is queued and joins the loops."""
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        if wait:
            for t in self._threads:
                t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- internals -----------------------------------------------------------------------------------------------------
    def _check_open(self):
        if self._closing:
            raise RuntimeError('the server is closed')

    def _submit(self, kind, map_id, x, rho, kwargs=None):
        n = _rows(x)
        with self._cv:
            self._check_open()
            if map_id not in self._maps:
                raise KeyError(f'unknown map {map_id}')
            entry = self._maps[map_id]
        req = _Request(kind, map_id, x, rho, n, self._ex.footprint(entry, kind, n, rho is not None), kwargs)
        with self._cv:
            if req.footprint > self.hbm_budget:
                req.future.set_exception(MemoryError(f'request needs {req.footprint} device bytes, over the '
                                                     f'{self.hbm_budget}-byte budget'))
                return req.future
            self._queue.append(req)
            self._cv.notify_all()
        return req.future

    def _admit(self, q, small_only=False):
        """Pops the next batch from `q` once its footprint fits the budget (lock held); None when closing and there
        is nothing left for this worker. `small_only` (the extra workers): the first packable BMU request in the
        queue, ahead of any larger one, so that small requests run beside a large one instead of behind it."""
        while True:
            idx = None
            if q:
                if not small_only:
                    idx = 0
                else:
                    idx = next((i for i, r in enumerate(q) if r.kind == 'bmu' and r.n <= self.max_batch_rows), None)
            if idx is not None:
                head = q[idx]
                if self._in_flight + head.footprint <= self.hbm_budget:
                    del q[idx]
                    batch = [head]
                    total_rows, total_fp = head.n, head.footprint
                    if head.kind == 'bmu' and head.n <= self.max_batch_rows:
                        while idx < len(q) and q[idx].kind == 'bmu' and q[idx].map_id == head.map_id and \
                                total_rows + q[idx].n <= self.max_batch_rows and \
                                self._in_flight + total_fp + q[idx].footprint <= self.hbm_budget:
                            nxt = q[idx]
                            del q[idx]
                            batch.append(nxt)
                            total_rows += nxt.n
                            total_fp += nxt.footprint
                    self._in_flight += total_fp
                    return batch, total_fp
            elif self._closing:
                return None, 0
            self._cv.wait(0.05)

    def _finish(self, batch, fp, results=None, exc=None):
        t = time.perf_counter()
        for i, req in enumerate(batch):
            if exc is not None:
                req.future.set_exception(exc)
            else:
                req.future.set_result(results[i])
        with self._cv:
            self._in_flight -= fp
            if exc is None:
                for req in batch:
                    self._lat[req.kind].append(t - req.t_submit)
            self._cv.notify_all()

    def _serve_loop(self, slot):
        while True:
            with self._cv:
                batch, fp = self._admit(self._queue, small_only=slot > 0)
            if batch is None:
                return
            head = batch[0]
            try:
                entry = self._maps[head.map_id]
                if head.kind == 'bmu':
                    res = self._ex.run_bmu(entry, [r.x for r in batch], slot=slot,
                                           hist=[r.kwargs.get('histogram', False) for r in batch])
                    with self._cv:
                        self._batches.append(len(batch))
                elif head.kind == 'activation':
                    res = [self._ex.run_activation(entry, head.x, head.rho, slot=slot)]
                else:
                    res = [self._ex.run_errors(entry, head.x, head.rho, slot=slot)]
            except Exception as e:   # the request fails alone
                self._finish(batch, fp, exc=e)
                continue
            self._finish(batch, fp, results=res)

    def _train_loop(self, slot):
        while True:
            with self._cv:
                batch, fp = self._admit(self._train_queue)
            if batch is None:
                return
            req = batch[0]
            som, dataset = req.x
            try:
                res = self._ex.run_train(som, dataset, req.rho, req.kwargs, slot=slot)
            except Exception as e:
                self._finish(batch, fp, exc=e)
                continue
            self._finish(batch, fp, results=[res])
