"""The allocation-free BMU entry point (somgb_find_bmus_noalloc) against somgb_find_bmus.

Callers that cannot allocate device memory (a framework that owns a fixed device-memory budget, or a pipeline that
holds only its own input and output buffers) use this entry point; its scratch is a static array inside the library
that every call shares. This file is collected last so that a failure here does not hide any other test, and it passes both
alone in a fresh process and after the rest of the suite: each call must give exactly the BMUs of the workspace-based
entry point, whatever an earlier call left in the shared array.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bmus(native, fn, x, w, algo, use_ws):
    n, d = x.shape
    m = w.shape[0]
    out = torch.full((n,), -7, dtype=torch.int32, device=x.device)
    s = torch.cuda.current_stream().cuda_stream
    if use_ws:
        nbytes = native.workspace_bytes(native.OP_FIND_BMUS, n, m, d, algo)
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=x.device)
        wsp = ws.data_ptr() + (-ws.data_ptr()) % 256
        native.call(fn, x.data_ptr(), n, d, w.data_ptr(), m, algo, out.data_ptr(), wsp, nbytes, s)
    else:
        native.call(fn, x.data_ptr(), n, d, w.data_ptr(), m, algo, out.data_ptr(), s)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize('algo_name', ['auto', 'fp32'])
def test_noalloc_matches_workspace_entry_point_twice(cuda, native, algo_name):
    algo = native.ALGOS[algo_name]
    assert native.lib().somgb_find_bmus_noalloc_scratch_bytes() == 4 << 20
    rng = np.random.default_rng(1234)
    cases = []
    # the second needs two chunks of the 4 MiB array; the third leaves a last chunk of one row
    for n, m, d in ((300_000, 256, 16), (1_300_000, 1024, 8), (1_300_001, 1024, 8)):
        x = np.exp(0.3 * rng.standard_normal((n, d))).astype(np.float32)
        w = x[rng.integers(0, n, m)] * (1 + 0.01 * rng.standard_normal((m, d))).astype(np.float32)
        cases.append((torch.from_numpy(x).to(cuda), torch.from_numpy(np.ascontiguousarray(w)).to(cuda)))
    # two calls in a row on different inputs: the second must not see the first's scratch contents
    for xd, wd in cases:
        want = _bmus(native, 'somgb_find_bmus', xd, wd, algo, use_ws=True)
        got = _bmus(native, 'somgb_find_bmus_noalloc', xd, wd, algo, use_ws=False)
        assert np.array_equal(got, want), f'{int(np.sum(got != want))} BMU mismatches'
        assert got.min() >= 0


def test_noalloc_fails_loudly_outside_limits(cuda, native):
    # a request the tensor-core pass cannot serve is refused with a status, never handled silently
    m, d = 1 << 20, 32
    x = torch.zeros((128, d), dtype=torch.float32, device=cuda)
    w = torch.zeros((m, d), dtype=torch.float32, device=cuda)
    out = torch.empty(128, dtype=torch.int32, device=cuda)
    status = native.lib().somgb_find_bmus_noalloc(x.data_ptr(), 128, d, w.data_ptr(), m, native.ALGO_TC,
                                                  out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert status in (native.SOMGB_ERR_WORKSPACE, native.SOMGB_ERR_UNSUPPORTED)
