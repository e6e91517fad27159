"""The sort entry point that allocates nothing, for callers that cannot call
cudaMalloc (an engine owning the GPU's memory through its own pool, a frame
loop that may not stall on an allocation, a binding that only holds raw
device pointers). Its scratch is a fixed array inside libvsim.

Checked through the C ABI against the allocating entry point, on two calls in
a row (the array keeps the first call's contents when the second runs).
Permutations are integers, so agreement must be exact. This file is named
to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20


def allocating_sort(lib, torch, keys_dev, n, bits):
    order = torch.empty(n, dtype=torch.int32, device=keys_dev.device)
    need = C.c_size_t()
    assert lib.vsim_radix_sort_u32(keys_dev.data_ptr(), order.data_ptr(), n, bits, None, C.byref(need), None) == 0
    temp = torch.empty(max(need.value, 1), dtype=torch.uint8, device=keys_dev.device)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.vsim_radix_sort_u32(keys_dev.data_ptr(), order.data_ptr(), n, bits, temp.data_ptr(), C.byref(need),
                                   stream) == 0
    torch.cuda.synchronize()
    return order.cpu().numpy().view(np.uint32)


def test_no_alloc_sort_matches_allocating_sort(vsimlib, gpu):
    import torch

    lib = vsimlib.lib()
    rng = np.random.default_rng(20261203)
    # two multi-pass sorts in a row, then a single 8-bit pass (keys straight
    # to the order, no ping-pong through the scratch's key buffers)
    cases = [(MAX_KEYS, 32), (300_001, 24), (4097, 8)]
    for call, (n, bits) in enumerate(cases):
        keys = rng.integers(0, 2 ** bits, n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 4] = keys[n // 2]  # a long run of equal keys: stability matters
        keys_dev = torch.from_numpy(keys.view(np.int32)).to(gpu)
        expected = allocating_sort(lib, torch, keys_dev, n, bits)
        order = torch.full((n,), -1, dtype=torch.int32, device=gpu)
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.vsim_radix_sort_u32_noalloc(keys_dev.data_ptr(), order.data_ptr(), n, bits, stream)
        assert rc == 0, lib.vsim_last_error()
        torch.cuda.synchronize()
        got = order.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, expected), f"call {call}: differs from the allocating sort"
        assert np.array_equal(keys_dev.cpu().numpy().view(np.uint32), keys)


def test_no_alloc_sort_rejects_oversize(vsimlib, gpu):
    lib = vsimlib.lib()
    rc = lib.vsim_radix_sort_u32_noalloc(None, None, MAX_KEYS + 1, 32, None)
    assert rc == vsimlib.VSIM_ERR_CAPACITY
    assert b"1048576" in lib.vsim_last_error()
