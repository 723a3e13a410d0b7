"""Device plumbing on top of PyTorch: tensors as device buffers, the current stream, workspaces.

PyTorch provides device memory and streams only; all compute goes through
libsomgb (decontamination_gb300/_native.py).
"""

import numpy as np
import torch

from . import _native

_NP_TO_TORCH = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
                np.dtype(np.int32): torch.int32}


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError('decontamination_gb300 needs a CUDA device (sm_103); there is no CPU fallback')
    return torch.device('cuda', torch.cuda.current_device())


def torch_dtype(np_dtype):
    return _NP_TO_TORCH[np.dtype(np_dtype)]


def to_device(a, np_dtype, device=None):
    """Contiguous device tensor of dtype `np_dtype` holding `a` (ndarray, tensor or array-like)."""
    device = device or require_cuda()
    td = torch_dtype(np_dtype)
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=td)
    else:
        arr = np.ascontiguousarray(np.asarray(a).astype(np_dtype, copy=False))
        t = torch.from_numpy(arr).to(device)
    return t.contiguous()


def ptr(t):
    return None if t is None else t.data_ptr()


def stream():
    return torch.cuda.current_stream().cuda_stream


class Workspace:
    """A growable device scratch buffer for libsomgb calls (256-byte aligned)."""

    def __init__(self):
        self._buf = None
        self._off = 0

    def get(self, nbytes, device=None):
        device = device or require_cuda()
        nbytes = max(int(nbytes), 256)
        if self._buf is None or self._buf.numel() < nbytes or self._buf.device != device:
            self._buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
        base = self._buf.data_ptr()
        self._off = (-base) % 256
        return base + self._off, self._buf.numel() - self._off

    def for_op(self, op, n, m, d, algo, device=None):
        return self.get(_native.workspace_bytes(op, n, m, d, algo), device)

    def status_word(self):
        """The status word of the last pass that used this workspace (a one-element int32 device tensor; non-zero
        when a bounded device-side wait of that pass gave up). Each pass clears it when it starts."""
        return self._buf[self._off + 8:self._off + 12].view(torch.int32)

    def note_status(self, acc):
        """ORs the last pass's status word into `acc` on the device, in stream order (no synchronisation)."""
        if self._buf is not None:
            acc.bitwise_or_(self.status_word())


class StatusCheck:
    """The status words of every pass of one API call, OR-ed on the device and checked once at its end, so that a
    wait that gave up in this call fails this call and no other (concurrent calls use their own workspaces)."""

    def __init__(self, device):
        self.acc = torch.zeros(1, dtype=torch.int32, device=device)

    def note(self, ws):
        ws.note_status(self.acc)

    def check(self):
        v = int(self.acc.item())
        if v:
            raise _native.SomgbError(_native.SOMGB_ERR_TIMEOUT,
                                     f'a device-side wait gave up (status {v:#x}); results are incomplete')


def rows(x):
    return int(x.shape[0])
