"""Failure paths of the CUDA path that need no GPU fault: a bounded
device-side wait made to run out (the onesweep look-back of the sort, on a
status that nothing sets), and the host-memory ray API refusing in-place
access to a host range with an unmapped gap.  Nothing here faults, traps or
hangs a GPU: the timeout comes from the library's own poll limit, and the gap
is only inspected on the host."""
from __future__ import annotations

import ctypes as C
import mmap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sort_lookback_timeout_is_reported(ctx):
    """The first tile of each pass withholds its status (a flag that nothing
    sets), so the look-back of the tile after it polls until its limit runs
    out: rt_sync reports RT_ERR_TIMEOUT, every kernel returns (no write
    leaves the output) and the context stays usable -- the next sort with
    normal settings is correct."""
    import torch
    import rtcore
    n = 1 << 20
    rng = np.random.default_rng(11)
    keys = rng.integers(0, 2**63, n, dtype=np.uint64)
    vals = np.arange(n, dtype=np.uint32)
    out = C.c_uint64()
    assert rtcore.load().rt_get_sort_scratch_bytes(n, 64, C.byref(out)) == 0
    nb = out.value
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    dv = torch.from_numpy(vals.view(np.int32)).cuda()
    codes = []
    ctx.set_sort_spin_limit(1 << 12)
    ctx.set_sort_withhold(True)
    try:
        for _ in range(2):
            k, v = dk.clone(), dv.clone()
            ctx.sort_pairs(k, v, n, 64, scratch, nb)
            try:
                ctx.sync()
                codes.append(0)
            except rtcore.RtError as e:
                codes.append(e.code)
    finally:
        ctx.set_sort_withhold(False)
        ctx.set_sort_spin_limit(0)
    print(f"statuses with the first tile's status withheld: {codes}")
    assert codes == [rtcore.RT_ERR_TIMEOUT] * 2, codes
    k, v = dk.clone(), dv.clone()
    ctx.sort_pairs(k, v, n, 64, scratch, nb)
    ctx.sync()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k.cpu().numpy().view(np.uint64), keys[order])
    assert np.array_equal(v.cpu().numpy().view(np.uint32), vals[order])
    assert rtcore.load().rt_debug_set_sort_spin_limit(None, 1) == rtcore.RT_ERR_INVALID_ARG
    assert rtcore.load().rt_debug_set_sort_withhold(None, 1) == rtcore.RT_ERR_INVALID_ARG


def test_host_range_with_unmapped_gap_is_staged(ctx):
    """A host range whose middle page is unmapped is never read in place (the
    traversal would fault on the gap): rt_debug_host_in_place answers 0 for
    it.  The range's bytes are not touched by the query.  Pinned buffers are
    read in place."""
    import torch
    libc = C.CDLL(None, use_errno=True)
    libc.mmap.restype = C.c_void_p
    libc.mmap.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_long]
    libc.munmap.argtypes = [C.c_void_p, C.c_size_t]
    pg = mmap.PAGESIZE
    base = libc.mmap(None, 3 * pg, mmap.PROT_READ | mmap.PROT_WRITE, mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS, -1, 0)
    assert base not in (None, C.c_void_p(-1).value)
    try:
        assert libc.munmap(base + pg, pg) == 0
        assert not ctx.host_in_place(base, 3 * pg), "a range over an unmapped page was accepted for in-place access"
        assert not ctx.host_in_place(base + pg - 32, 64)
    finally:
        libc.munmap(base, pg)
        libc.munmap(base + 2 * pg, pg)
    pinned = torch.zeros(1 << 20, dtype=torch.uint8).pin_memory()
    assert ctx.host_in_place(pinned.data_ptr(), pinned.numel())
    dev = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
    assert ctx.host_in_place(dev.data_ptr(), dev.numel())
