"""The reference's dataset protocol: an array, or a generator builder () -> (() -> iterable of chunks).

Restates ``dataset_to_generator_builder`` (algo/__init__.py:21-27) and the
chunk loops of the reference (algo/som_batch.py:295-342,
algo/som_abstract.py:557-597): chunks of `dataset` and `dataset_weights` are
zipped and must have the same length. Arrays (numpy or torch, host or device)
are accepted wherever the reference accepts a numpy array.
"""

import typing

import numpy as np
import torch

from . import _device


def dataset_to_generator_builder(dataset) -> typing.Optional[typing.Callable]:
    if dataset is None:
        return None
    return dataset if callable(dataset) else (lambda: lambda: (dataset,))


# Host chunks of at least two pieces' rows are copied to the device in pieces on a side stream, so that the work on
# piece p overlaps the copy of piece p + 1. Piece edges are multiples of 16 rows (16-byte aligned rows for any D).
PIECE_ROWS = 1 << 20
MAX_PIECES = 4
_COPY_STREAMS = {}


def _copy_stream(device):
    s = _COPY_STREAMS.get(device.index)
    if s is None:
        s = _COPY_STREAMS[device.index] = torch.cuda.Stream(device=device)
    return s


def _host_tensor(a, np_dtype):
    """A contiguous CPU tensor of `np_dtype` holding the host array `a` (no copy when it already is one)."""
    td = _device.torch_dtype(np_dtype)
    if isinstance(a, torch.Tensor):
        t = a if a.dtype == td else a.to(td)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(np_dtype, copy=False)))
    return t.contiguous()


def piece_edges(n):
    """Row edges [0, e1, ..., n] of the pieces of an n-row host chunk (n >= 2 * PIECE_ROWS): between 2 and
    MAX_PIECES pieces of about equal size, interior edges rounded up to multiples of 16 rows."""
    k = max(2, min(MAX_PIECES, n // PIECE_ROWS))
    return [min(n, (n * p // k + 15) // 16 * 16) for p in range(k)] + [n]


def device_pieces(x, rho, dtype, device, weight_dtype=np.float64):
    """(x_dev, rho_dev, pieces): one chunk as device tensors, and an iterable of row ranges (a, b) that yields each
    range once its rows are on the device for the current stream (rho_dev is None without weights).

    Device inputs give one range. A host chunk of n >= 2 * PIECE_ROWS rows is copied in up to MAX_PIECES pieces on a
    side stream, piece p + 1 issued before piece p is handed out, so the caller's work on p overlaps that copy (from
    pinned memory; a pageable copy blocks the host instead, which still overlaps the device work already queued).
    Every range must be consumed before the tensors are used whole.
    """
    on_host = not (isinstance(x, torch.Tensor) and x.device.type == 'cuda')
    n = _len(x)
    if not on_host or n < 2 * PIECE_ROWS:
        xd = _device.to_device(x, dtype, device)
        rd = None if rho is None else _device.to_device(rho, weight_dtype, device)
        return xd, rd, [(0, int(xd.shape[0]))]
    xt = _host_tensor(x, dtype)
    rt = None if rho is None else _host_tensor(rho, weight_dtype)
    xd = torch.empty(xt.shape, dtype=xt.dtype, device=device)
    rd = None if rt is None else torch.empty(rt.shape, dtype=rt.dtype, device=device)
    cs = _copy_stream(device)
    cs.wait_stream(torch.cuda.current_stream(device))   # the buffers were allocated on the current stream
    xd.record_stream(cs)
    if rd is not None:
        rd.record_stream(cs)
    edges = piece_edges(n)
    k = len(edges) - 1

    def gen():
        events = []

        def issue(p):
            a, b = edges[p], edges[p + 1]
            with torch.cuda.stream(cs):
                xd[a:b].copy_(xt[a:b], non_blocking=True)
                if rd is not None:
                    rd[a:b].copy_(rt[a:b], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
            events.append(ev)

        issue(0)
        for p in range(k):
            if p + 1 < k:
                issue(p + 1)
            torch.cuda.current_stream(device).wait_event(events[p])
            if edges[p + 1] > edges[p]:
                yield edges[p], edges[p + 1]

    return xd, rd, gen()


def raw_chunks(dataset, dataset_weights):
    """(x, rho) chunk pairs of the dataset protocol as given (host or device), rho None without weights."""
    db = dataset_to_generator_builder(dataset)
    wb = dataset_to_generator_builder(dataset_weights)
    if wb is None:
        for xc in db()():
            yield xc, None
        return
    for xc, rc in zip(db()(), wb()()):
        if _len(xc) != _len(rc):
            raise ValueError('`dataset` and `dataset_weights` chunks must be aligned')
        yield xc, rc


def iterate_pieces(dataset, dataset_weights, dtype, device, weight_dtype=np.float64):
    """Yields (x, rho) device views per piece of every chunk (see device_pieces)."""
    for xc, rc in raw_chunks(dataset, dataset_weights):
        xd, rd, pieces = device_pieces(xc, rc, dtype, device, weight_dtype)
        for a, b in pieces:
            yield xd[a:b], (None if rd is None else rd[a:b])


def iterate_chunks(dataset, dataset_weights, dtype, device, weight_dtype=np.float64):
    """Yields (x, rho) device tensors per chunk; rho is None when there are no weights.

    x has the map dtype (the reference casts chunks with astype(dtype)); rho is float64, the type the reference uses
    for densities in compute_errors / get_activation_map (training casts it to the map dtype on the device).
    """
    db = dataset_to_generator_builder(dataset)
    wb = dataset_to_generator_builder(dataset_weights)
    if wb is None:
        for xc in db()():
            yield _device.to_device(xc, dtype, device), None
        return
    for xc, rc in zip(db()(), wb()()):
        if _len(xc) != _len(rc):
            raise ValueError('`dataset` and `dataset_weights` chunks must be aligned')
        yield _device.to_device(xc, dtype, device), _device.to_device(rc, weight_dtype, device)


def _len(a):
    return int(a.shape[0]) if isinstance(a, (np.ndarray, torch.Tensor)) else len(a)


def is_array(a):
    return isinstance(a, (np.ndarray, torch.Tensor))
