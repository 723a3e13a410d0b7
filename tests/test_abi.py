"""The C ABI: libsomgb.so builds, loads without a GPU and exports exactly what include/somgb.h declares.

Argument checks run on the host before any CUDA call, so they are exercised here too.
"""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, 'include', 'somgb.h')


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'^\s*(?:int|size_t|int64_t)\s+(somgb_\w+)\s*\(', text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert 'somgb_train_epoch_pass' in names and 'somgb_find_bmus' in names
    assert len(names) >= 18


def test_library_exports_every_declared_symbol(native):
    lib = native.lib()
    for name in declared_functions():
        assert hasattr(lib, name), f'{name} declared in somgb.h but not exported'
        assert name in native.SIGNATURES, f'{name} has no ctypes signature in _native.py'


def test_version_and_workspace_query(native):
    lib = native.lib()
    assert lib.somgb_version() >= 100
    for op in (native.OP_FIND_BMUS, native.OP_COUNT_BMUS, native.OP_ERRORS):
        assert native.workspace_bytes(op, 1000, 64, 16, native.ALGO_FP32) >= 256
    # the epoch pass keeps one int32 BMU per sample in the workspace
    assert native.workspace_bytes(native.OP_EPOCH, 10**6, 64, 16, native.ALGO_FP32) >= 4 * 10**6


def test_host_side_argument_checks(native):
    lib = native.lib()
    buf = (ctypes.c_char * 512)()
    addr = ctypes.addressof(buf)
    ws = addr + (-addr) % 256
    # invalid sizes
    assert lib.somgb_find_bmus(ws, -1, 4, ws, 16, 0, ws, ws, 256, None) == native.SOMGB_ERR_INVALID
    assert 'invalid sizes' in native.last_error()
    assert lib.somgb_find_bmus(ws, 10, 0, ws, 16, 0, ws, ws, 256, None) == native.SOMGB_ERR_INVALID
    # unknown algorithm
    assert lib.somgb_find_bmus(ws, 10, 4, ws, 16, 7, ws, ws, 256, None) == native.SOMGB_ERR_INVALID
    # workspace too small
    assert lib.somgb_find_bmus(ws, 10, 4, ws, 16, 0, ws, ws, 16, None) == native.SOMGB_ERR_WORKSPACE
    assert 'workspace' in native.last_error()
    # misaligned workspace
    assert lib.somgb_find_bmus(ws, 10, 4, ws, 16, 0, ws, ws + 4, 400, None) == native.SOMGB_ERR_INVALID
    # non-positive sigma
    assert lib.somgb_neighbourhood_update(ws, ws, ws, 16, 4, 0.0, ws, None, None, None) == native.SOMGB_ERR_INVALID


def test_python_raises_on_status(native):
    with pytest.raises(native.SomgbError) as ei:
        native.call('somgb_divide', None, None, 0, 0, None, None)
    assert ei.value.status == native.SOMGB_ERR_INVALID
