"""Device-resident serving pieces: batches over several lanes (ig_ctx_set_lanes), whose
responses must equal the host-buffer respond_seeded_batch answers for one lane and for
three, and the device-side response wire (ig_response_encode_device) and RIMS frames
(ig_response_encode_rims_device), whose bytes must equal the host encoders'."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    return load_package()


@pytest.mark.parametrize("batch", [8, 32])  # 8 x 3 lanes: two CTAs per query; 32 x 3: one
def test_lanes_give_the_same_responses(pkg, oracle, batch):
    torch = pytest.importorskip("torch")
    ctx = pkg.Context.default()
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 256, 0x1A2E)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(ctx)
    h = store.register_server_side(pkg.ClientPackingKeys(cell.keys(), cell.gamma), cache)
    n, nbatches = P.n, 6
    total = cell.num_shards * n
    qs = [[pkg.SeededBatchQuery(*cell.next_query((j * batch + k) * 389 % total)) for k in range(batch)]
          for j in range(nbatches)]
    ms = pkg.MOD_SWITCH_TARGET_36BIT
    want = []
    for j in range(nbatches):
        out = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), qs[j]),
                                       cache, store, mod_switch_target=ms)
        want.append((np.stack([r.a for r in out]), np.stack([r.b for r in out])))
    sids = [np.ascontiguousarray([q.shard_id for q in qs[j]], dtype=np.uint32) for j in range(nbatches)]
    seeds = torch.from_numpy(np.stack([np.frombuffer(b"".join(q.seed for q in qs[j]), dtype=np.uint8)
                                       for j in range(nbatches)]).copy()).cuda()
    bs = torch.from_numpy(np.stack([np.stack([q.b for q in qs[j]]) for j in range(nbatches)]).view(np.int64)).cuda()
    for lanes in (1, 3):
        a = torch.zeros((nbatches, batch, n), dtype=torch.int64, device="cuda")
        b = torch.zeros_like(a)
        st = torch.ones((nbatches, batch), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        ctx.set_lanes(lanes)
        try:
            for j in range(nbatches):
                ctx.check(ctx._lib.ig_respond_seeded_batch_device(
                    ctx.h, db.h, store.h, int(h), batch, sids[j].ctypes.data, seeds[j].data_ptr(), bs[j].data_ptr(),
                    ms, a[j].data_ptr(), b[j].data_ptr(), st[j].data_ptr()))
            ctx.join()
            torch.cuda.ExternalStream(ctx.stream).synchronize()
        finally:
            ctx.set_lanes(1)
        assert int(st.abs().sum().item()) == 0
        got_a = a.cpu().numpy().view(np.uint64)
        got_b = b.cpu().numpy().view(np.uint64)
        for j in range(nbatches):
            assert (got_a[j] == want[j][0]).all() and (got_b[j] == want[j][1]).all(), (lanes, j)


def test_device_wire_matches_host_bytes(pkg, oracle):
    """ig_response_encode_device builds the ServerResponse bytes next to the responses; they
    equal the host encoder's (and so the reference's) bytes, unswitched and 36-bit."""
    torch = pytest.importorskip("torch")
    ctx = pkg.Context.default()
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 512, 0x3A7E)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(ctx)
    h = store.register_server_side(pkg.ClientPackingKeys(cell.keys(), cell.gamma), cache)
    n, count = P.n, 5
    qs = [pkg.SeededBatchQuery(*cell.next_query(k * 1201 % (cell.num_shards * n))) for k in range(count)]
    for ms in (0, pkg.MOD_SWITCH_TARGET_36BIT):
        out = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), qs), cache,
                                       store, mod_switch_target=ms)
        want = [r.to_binary() for r in out]
        a = torch.from_numpy(np.stack([r.a for r in out]).view(np.int64)).cuda()
        b = torch.from_numpy(np.stack([r.b for r in out]).view(np.int64)).cuda()
        modulus = ms or P.q
        length = ctx.response_wire_len(n, cell.gamma, modulus)
        d_out = torch.zeros(count * length, dtype=torch.uint8, device="cuda")
        st = torch.ones(count, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        assert ctx.response_wire_device(count, a.data_ptr(), b.data_ptr(), n, cell.gamma, modulus, d_out.data_ptr(),
                                        st.data_ptr()) == length
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        got = d_out.cpu().numpy().tobytes()
        assert int(st.abs().sum().item()) == 0
        for r in range(count):
            assert got[r * length:(r + 1) * length] == want[r], (ms, r)
        # The RIMS frames (mod_switch.rs:254-345) of the same responses, built on the device.
        rlen = ctx.response_rims_device(count, 0, 0, n, cell.gamma, modulus, 0, 0)
        d_rims = torch.zeros(count * rlen, dtype=torch.uint8, device="cuda")
        st.fill_(1)
        torch.cuda.synchronize()
        assert ctx.response_rims_device(count, a.data_ptr(), b.data_ptr(), n, cell.gamma, modulus, d_rims.data_ptr(),
                                        st.data_ptr()) == rlen
        torch.cuda.ExternalStream(ctx.stream).synchronize()
        got = d_rims.cpu().numpy().tobytes()
        assert int(st.abs().sum().item()) == 0
        for r in range(count):
            assert got[r * rlen:(r + 1) * rlen] == out[r].to_rims(), (ms, r)


def test_concurrent_host_calls_over_lanes(pkg, oracle):
    """respond_seeded_batch from three threads with three lanes: each call holds a lane
    while its batch runs, the context lock only while it launches; every answer equals the
    one-lane answer, including inline-key calls, whose seats live in their caller's lane."""
    import threading
    ctx = pkg.Context.default()
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 256, 0x7A4E)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(ctx)
    keys = pkg.ClientPackingKeys(cell.keys(), cell.gamma)
    other = pkg.ClientPackingKeys(np.random.default_rng(3).integers(0, pkg.DEFAULT_Q, cell.keys().shape,
                                                                   dtype=np.uint64), cell.gamma)
    h = store.register_server_side(keys, cache)
    total = cell.num_shards * P.n
    batches = []
    for j in range(9):
        qs = [pkg.SeededBatchQuery(*cell.next_query((j * 13 + k) * 577 % total)) for k in range(6)]
        src = [pkg.PackingKeySource.Registered(h), pkg.PackingKeySource.Inline(keys),
               pkg.PackingKeySource.Inline(other)][j % 3]
        batches.append(pkg.SeededQueryBatch(src, qs))
    want = [[r.to_binary() for r in pkg.respond_seeded_batch(crs, db, b, cache, store)] for b in batches]
    got = [None] * len(batches)
    errors = []
    ctx.set_lanes(3)
    try:
        def caller(t):
            try:
                for j in range(t, len(batches), 3):
                    got[j] = [r.to_binary() for r in pkg.respond_seeded_batch(crs, db, batches[j], cache, store)]
            except Exception as e:
                errors.append(e)
        threads = [threading.Thread(target=caller, args=(t,)) for t in range(3)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
    finally:
        ctx.set_lanes(1)
    assert not errors, errors
    assert got == want
