"""oct_sort_keys_noalloc: the sort for callers that cannot call cudaMalloc
(device memory owned by another allocator or a fixed pool; frame loops where
an allocation would stall the device). Its scratch is a fixed __device__
array inside the library, so the caller passes only keys and keys_alt.

Checked through the C ABI against the workspace-based oct_sort_keys on two
calls in a row (the second call must not see the first call's leftover
counters and flags), bit for bit, as every sort test here is. Collected last
(file name) so a failure here leaves every other test already run; it also
passes alone in a fresh process, where its first call sets the array up.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from pipeline_gb300 import _lib

pytestmark = pytest.mark.gpu


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sort_with_workspace(lib, a: np.ndarray, bits: int) -> np.ndarray:
    n = len(a)
    keys = torch.from_numpy(a.view(np.int32).copy()).cuda()
    alt = torch.empty(n, dtype=torch.int32, device="cuda")
    ws_bytes = lib.oct_sort_workspace_bytes(n, bits)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    rc = lib.oct_sort_keys(C.c_void_p(keys.data_ptr()), C.c_void_p(alt.data_ptr()), n, bits,
                           C.c_void_p(ws.data_ptr()), ws_bytes, None, _stream())
    _lib.check(rc, "oct_sort_keys")
    return keys.cpu().numpy().view(np.uint32)


def _sort_noalloc(lib, a: np.ndarray, bits: int):
    n = len(a)
    keys = torch.from_numpy(a.view(np.int32).copy()).cuda()
    alt = torch.empty(n, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.oct_sort_keys_noalloc(C.c_void_p(keys.data_ptr()), C.c_void_p(alt.data_ptr()), n,
                                   bits, C.c_void_p(status.data_ptr()), _stream())
    _lib.check(rc, "oct_sort_keys_noalloc")
    return keys.cpu().numpy().view(np.uint32), int(status.item())


@pytest.mark.parametrize("bits", [30, 32])
def test_noalloc_sort_matches_workspace_sort_twice(bits):
    lib = _lib.load()
    rng = np.random.default_rng(bits)
    # Two calls in a row with different sizes and key mixes.
    n_max = 1 << 22  # the largest size the fixed scratch accepts
    first = rng.integers(0, 1 << bits, n_max, dtype=np.uint64).astype(np.uint32)
    second = (rng.integers(0, 4, 300_007) << (bits - 3)).astype(np.uint32)
    for a in (first, second):
        got, status = _sort_noalloc(lib, a, bits)
        want = _sort_with_workspace(lib, a, bits)
        assert status == 0
        assert got.tobytes() == want.tobytes()
        assert got.tobytes() == np.sort(a).tobytes()


def test_noalloc_sort_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    n = (1 << 22) + 1
    dummy = torch.empty(1, dtype=torch.int32, device="cuda")
    rc = lib.oct_sort_keys_noalloc(C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()), n,
                                   30, None, _stream())
    assert rc == _lib.OCT_ERR_TOO_LARGE
    assert b"4194304" in lib.oct_last_error()
