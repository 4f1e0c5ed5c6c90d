"""The forward's own radix sort and prefix sums (sgr_sort.cu) against the
stable sort of the same keys (numpy's, and PyTorch's on the GPU) and
numpy's cumulative sums: identical keys and values, in the same order, for
every size around the sort's 4096-key tiles and the scans' 2048-element
tiles, heavy ties, all-equal keys, and partial key widths."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 31, 2047, 2048, 2049, 4095, 4096, 4097, 6143, 12_289, 100_003, 1_048_576 + 17]


def _sort(lib, keys, vals, key_bytes, end_bit):
    n = keys.numel()
    ko = torch.empty_like(keys)
    vo = torch.empty_like(vals)
    tb = lib.sgr_radix_sort_temp_bytes(n, key_bytes)
    tmp = torch.empty(max(1, tb), dtype=torch.uint8, device="cuda")
    rc = lib.sgr_radix_sort_pairs(keys.data_ptr(), ko.data_ptr(), vals.data_ptr(), vo.data_ptr(), n, key_bytes,
                                  end_bit, tmp.data_ptr(), tb, torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return ko, vo


def _expect(keys_np, end_bit, dtype):
    mask = np.array((1 << end_bit) - 1 if end_bit < 64 else (1 << 64) - 1, dtype=np.uint64).astype(dtype)
    k = keys_np & mask
    order = np.argsort(k, kind="stable")
    return order


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("end_bit", [36, 64])
def test_sort_u64(sgr_lib, n, end_bit):
    g = np.random.default_rng(n + end_bit)
    view = g.integers(0, 16, n, dtype=np.uint64)
    depth = g.random(n).astype(np.float32) * 5 + 0.2
    bits = depth.view(np.uint32).astype(np.uint64)
    bits[g.random(n) < 0.2] = 0xffffffff                         # culled records sort last in their view
    bits[g.random(n) < 0.3] = bits[0]                            # ties
    keys_np = (view << np.uint64(32)) | bits
    if end_bit == 64:
        keys_np |= g.integers(0, 1 << 20, n, dtype=np.uint64) << np.uint64(40)
    vals_np = np.arange(n, dtype=np.uint32)[::-1].copy()
    keys = torch.from_numpy(keys_np.view(np.int64)).cuda()
    vals = torch.from_numpy(vals_np.view(np.int32)).cuda()
    ko, vo = _sort(sgr_lib, keys, vals, 8, end_bit)
    order = _expect(keys_np, end_bit, np.uint64)
    np.testing.assert_array_equal(ko.cpu().numpy().view(np.uint64), keys_np[order])
    np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), vals_np[order])
    # the inputs are untouched
    np.testing.assert_array_equal(keys.cpu().numpy().view(np.uint64), keys_np)
    if end_bit < 63:   # PyTorch's stable GPU sort of the same (non-negative) keys
        _, idx = torch.sort(keys, stable=True)
        np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), vals_np[idx.cpu().numpy()])


@pytest.mark.parametrize("n", [1, 2049, 300_001])
@pytest.mark.parametrize("end_bit", [0, 7, 32])
def test_sort_u32(sgr_lib, n, end_bit):
    g = np.random.default_rng(7 * n + end_bit)
    keys_np = g.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys_np[g.random(n) < 0.5] = 12345
    vals_np = g.integers(0, 1 << 31, n, dtype=np.uint32)
    keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
    vals = torch.from_numpy(vals_np.view(np.int32)).cuda()
    ko, vo = _sort(sgr_lib, keys, vals, 4, end_bit)
    mask = np.uint32((1 << end_bit) - 1) if end_bit < 32 else np.uint32(0xffffffff)
    order = np.argsort(keys_np & mask, kind="stable")
    np.testing.assert_array_equal(ko.cpu().numpy().view(np.uint32), keys_np[order])
    np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), vals_np[order])


def test_sort_all_equal_and_empty(sgr_lib):
    n = 50_000
    keys = torch.full((n,), 7, dtype=torch.int64, device="cuda")
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    ko, vo = _sort(sgr_lib, keys, vals, 8, 36)
    assert torch.equal(vo, vals) and torch.equal(ko, keys)
    e = torch.empty(0, dtype=torch.int64, device="cuda")
    ei = torch.empty(0, dtype=torch.int32, device="cuda")
    assert sgr_lib.sgr_radix_sort_pairs(e.data_ptr(), e.data_ptr(), ei.data_ptr(), ei.data_ptr(), 0, 8, 36, None, 0,
                                        None) == 0


@pytest.mark.parametrize("n", SIZES)
def test_prefix_sums(sgr_lib, n):
    g = np.random.default_rng(n)
    a64 = g.integers(0, 1 << 20, n, dtype=np.uint64)
    a32 = g.integers(0, 1000, n, dtype=np.uint32)
    st = torch.cuda.current_stream().cuda_stream
    t64 = torch.from_numpy(a64.view(np.int64)).cuda()
    tb = sgr_lib.sgr_prefix_sum_temp_bytes(n, 8)
    tmp = torch.empty(max(1, tb), dtype=torch.uint8, device="cuda")
    assert sgr_lib.sgr_inclusive_sum_u64(t64.data_ptr(), t64.data_ptr(), n, tmp.data_ptr(), tb, st) == 0   # in place
    t32 = torch.from_numpy(a32.view(np.int32)).cuda()
    o32 = torch.empty_like(t32)
    tb = sgr_lib.sgr_prefix_sum_temp_bytes(n, 4)
    tmp = torch.empty(max(1, tb), dtype=torch.uint8, device="cuda")
    assert sgr_lib.sgr_exclusive_sum_u32(t32.data_ptr(), o32.data_ptr(), n, tmp.data_ptr(), tb, st) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t64.cpu().numpy().view(np.uint64), np.cumsum(a64, dtype=np.uint64))
    ex = np.concatenate([[0], np.cumsum(a32, dtype=np.uint64)[:-1]]).astype(np.uint32)
    np.testing.assert_array_equal(o32.cpu().numpy().view(np.uint32), ex)


def test_argument_checks(sgr_lib):
    INVALID = 1
    assert sgr_lib.sgr_radix_sort_pairs(None, None, None, None, 10, 8, 36, None, 0, None) == INVALID
    assert sgr_lib.sgr_radix_sort_pairs(None, None, None, None, 10, 3, 8, None, 0, None) == INVALID
    assert sgr_lib.sgr_radix_sort_pairs(None, None, None, None, -1, 8, 8, None, 0, None) == INVALID
    assert sgr_lib.sgr_inclusive_sum_u64(None, None, 5, None, 0, None) == INVALID
    assert sgr_lib.sgr_exclusive_sum_u32(None, None, -2, None, 0, None) == INVALID
    assert sgr_lib.sgr_radix_sort_temp_bytes(100, 3) == 0
    assert C.c_size_t(sgr_lib.sgr_prefix_sum_temp_bytes(0, 8)).value == 0
