"""tq_nest_sum_noalloc: the block-offset scan for callers that cannot allocate
device memory (a fixed arena owns it all, or an allocation could stall a
latency-critical loop).  Called through the C ABI and compared with the
allocating tq_nest_sum on the same inputs, on two calls in a row; integer
results, so the comparison is exact.  Kept in a file collected last."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_nest_sum_matches_allocating_entry_point(tq):
    import torch
    lib = tq.load()
    g = torch.Generator(device="cuda")
    g.manual_seed(17)
    # multi-tile calls in a row (each reuses the shared static scratch): two
    # large ones, then smaller ones (2 and 3 tiles of 2048 counts) that must
    # not read tile sums a larger earlier call left behind, then a single-tile one
    for n in (3_000_001, 4_194_304, 2049, 4097, 1000):
        x = torch.randint(0, 100_000, (n,), dtype=torch.int64, device="cuda", generator=g)
        ref_o = torch.empty(n, dtype=torch.int64, device="cuda")
        ref_t = torch.empty(1, dtype=torch.int64, device="cuda")
        assert lib.tq_nest_sum(_p(x), n, _p(ref_o), _p(ref_t), None) == 0
        o = torch.full((n,), -1, dtype=torch.int64, device="cuda")
        t = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        # every library allocation is refused meanwhile: the call must not need one
        lib.tq_debug_fail_alloc_after(0)
        try:
            st = lib.tq_nest_sum_noalloc(_p(x), n, _p(o), _p(t), None)
        finally:
            lib.tq_debug_fail_alloc_after(-1)
        assert st == 0, lib.tq_last_error_string()
        torch.cuda.synchronize()
        assert torch.equal(o, ref_o)
        assert torch.equal(t, ref_t)
        assert int(t.item()) == int(x.sum().item())


def test_noalloc_nest_sum_rejects_sizes_beyond_its_limit(tq):
    import torch
    lib = tq.load()
    n = 4_194_305
    x = torch.zeros(n, dtype=torch.int64, device="cuda")
    o = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    t = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    assert lib.tq_nest_sum_noalloc(_p(x), n, _p(o), _p(t), None) == 1
    assert b"4194304" in lib.tq_last_error_string()
    torch.cuda.synchronize()
    assert int(t.item()) == -1 and int(o[0].item()) == -1
