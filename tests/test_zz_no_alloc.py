"""The allocation-free respond entry point, checked against the allocating one.

ig_respond_seeded_batch_noalloc exists for embedders that cannot let a library allocate
device memory while it serves: servers that size every device buffer once at start-up and
refuse growth later, and GPUs shared with other jobs under a memory cap, where a late
allocation can fail. Its scratch is one fixed device array inside the library. This test
calls it through the C ABI twice in a row (the array keeps the previous call's contents
between calls) and requires the bytes of ig_respond_seeded_batch_device, exactly: the
arithmetic is integer mod q, so the tolerance is zero. Around each call the context's
allocation injector is armed, so any device allocation the call made would refuse it. It
lives in its own file so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

Q = 1152921504606830593
N = 2048
GAMMA = 256


def _bind(lib):
    f = lib.ig_respond_seeded_batch_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                  ctypes.c_void_p]
    return f


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    import torch

    pkg = load_package()
    ctx = pkg.Context.default()
    noalloc = _bind(ctx._lib)
    rng = np.random.default_rng(20261203)
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), rng.bytes(32), GAMMA)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase(cache, 4)
    for s in range(4):
        db.set_shard(s, rng.integers(0, 1 << 16, (GAMMA, N), dtype=np.uint64))
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(ctx)
    handle = store.register_server_side(
        pkg.ClientPackingKeys(rng.integers(0, Q, (3, N), dtype=np.uint64), GAMMA), cache)
    for call, (count, ms) in enumerate([(8, pkg.MOD_SWITCH_TARGET_36BIT), (5, 0)]):
        shard_ids = np.ascontiguousarray(rng.integers(0, 4, count), dtype=np.uint32)
        seeds = torch.from_numpy(rng.integers(0, 256, (count, 32), dtype=np.uint8)).cuda()
        bs = torch.from_numpy(rng.integers(0, Q, (count, N), dtype=np.uint64).view(np.int64)).cuda()
        a_ref = torch.empty((count, N), dtype=torch.int64, device="cuda")
        b_ref = torch.empty_like(a_ref)
        a_new = torch.full_like(a_ref, -1)
        b_new = torch.full_like(a_ref, -1)
        status = torch.zeros(count, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        ctx.check(ctx._lib.ig_respond_seeded_batch_device(
            ctx.h, db.h, store.h, int(handle), count, shard_ids.ctypes.data, seeds.data_ptr(), bs.data_ptr(), ms,
            a_ref.data_ptr(), b_ref.data_ptr(), status.data_ptr()))
        torch.cuda.synchronize()
        # The next device allocation of this context fails: the call must not make one.
        ctx.check(ctx._lib.ig_debug_fail_alloc_at(ctx.h, 1))
        try:
            ctx.check(noalloc(ctx.h, db.h, store.h, int(handle), count, shard_ids.ctypes.data, seeds.data_ptr(),
                              bs.data_ptr(), ms, a_new.data_ptr(), b_new.data_ptr()))
        finally:
            ctx.check(ctx._lib.ig_debug_fail_alloc_at(ctx.h, 0))
        torch.cuda.synchronize()
        assert int(status.abs().sum()) == 0
        assert torch.equal(a_new, a_ref), f"call {call}: a differs"
        assert torch.equal(b_new, b_ref), f"call {call}: b differs"
    # With the injector disarmed, the allocating path still serves (it grows a new scratch).
    more = np.ascontiguousarray(rng.integers(0, 4, 80), dtype=np.uint32)
    seeds = torch.from_numpy(rng.integers(0, 256, (80, 32), dtype=np.uint8)).cuda()
    bs = torch.from_numpy(rng.integers(0, Q, (80, N), dtype=np.uint64).view(np.int64)).cuda()
    a_big = torch.empty((80, N), dtype=torch.int64, device="cuda")
    b_big = torch.empty_like(a_big)
    status = torch.zeros(80, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.check(ctx._lib.ig_respond_seeded_batch_device(
        ctx.h, db.h, store.h, int(handle), 80, more.ctypes.data, seeds.data_ptr(), bs.data_ptr(), 0,
        a_big.data_ptr(), b_big.data_ptr(), status.data_ptr()))
    torch.cuda.synchronize()
    assert int(status.abs().sum()) == 0


def test_noalloc_refuses_batches_beyond_its_fixed_scratch():
    import torch

    pkg = load_package()
    ctx = pkg.Context.default()
    noalloc = _bind(ctx._lib)
    rng = np.random.default_rng(7)
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), rng.bytes(32), 16)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase(cache, 1)
    db.set_shard(0, np.zeros((16, N), dtype=np.uint64))
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(ctx)
    handle = store.register_server_side(pkg.ClientPackingKeys(np.zeros((3, N), dtype=np.uint64), 16), cache)
    shard_ids = np.zeros(65, dtype=np.uint32)
    # Real device buffers sized for the 65 queries: should the size check ever stop refusing,
    # the call computes into them instead of touching memory it does not own.
    seeds = torch.zeros((65, 32), dtype=torch.uint8, device="cuda")
    bs = torch.zeros((65, N), dtype=torch.int64, device="cuda")
    a_out = torch.zeros((65, N), dtype=torch.int64, device="cuda")
    b_out = torch.zeros((65, N), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = noalloc(ctx.h, db.h, store.h, int(handle), 65, shard_ids.ctypes.data, seeds.data_ptr(), bs.data_ptr(), 0,
                 a_out.data_ptr(), b_out.data_ptr())
    torch.cuda.synchronize()
    assert rc == 1
    with pytest.raises(pkg.PirError, match="at most 64 queries"):
        ctx.check(rc)
