"""Mixed databases side by side (the shapes of the reference's multi-database serving
case, shrunk to three shards each): 32 B, 512 B and 2048 B records (gamma 16, 256 and
1024), each under the exact and the approximate gadget, so six parameter sets; two seats
per set (the cell's client key, which decodes, and a second key); batch sizes 1, 7, 33 and
128, which run both launch shapes (two CTAs per query up to half the SMs, one above).
Every response is checked against the oracle's bytes or by decoding, and the serving loop
must return the same bytes for the same queries interleaved across all six sets."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

ENTRIES = [(32, 0x3001), (512, 0x4001), (2048, 0x5001)]
BATCHES = [1, 7, 33, 128]
WAIT_MS = 120_000


@pytest.fixture(scope="module")
def pkg():
    return load_package()


@pytest.fixture(scope="module")
def ctx(pkg):
    return pkg.Context.default()


class Set:
    def __init__(self, pkg, oracle, ctx, store, entry, seed, approx):
        self.P = oracle.Params.d2048_approximate_gadget() if approx else oracle.Params.d2048()
        self.cell = oracle.Cell(self.P, entry, seed)
        params = pkg.InspireParams(ring_dim=self.P.n, p=self.P.p, approximate_packing_gadget=approx)
        self.crs = pkg.ServerCrs(params, self.cell.w_seed, self.cell.gamma)
        self.cache = pkg.ServerInspiringCache.new(self.crs, ctx=ctx)
        self.db = pkg.EncodedDatabase.from_columns(
            self.cache, [self.cell.columns(s) for s in range(self.cell.num_shards)])
        self.db.precompute_packing_all()
        self.keys = self.cell.keys()
        rng = np.random.default_rng(seed)
        self.other_keys = rng.integers(0, pkg.DEFAULT_Q, size=self.keys.shape, dtype=np.uint64)
        self.h_real = store.register_server_side(pkg.ClientPackingKeys(self.keys, self.cell.gamma), self.cache)
        self.h_other = store.register_server_side(pkg.ClientPackingKeys(self.other_keys, self.cell.gamma),
                                                  self.cache)
        self.ocache = oracle.Cache(self.P, self.cell.gamma, self.cell.w_seed)
        self.ostores = {}

    def queries(self, pkg, count, salt):
        total = self.cell.num_shards * self.P.n
        idx = [(salt * 7919 + k * 104729) % total for k in range(count)]
        return idx, [pkg.SeededBatchQuery(*self.cell.next_query(i)) for i in idx]

    def oracle_bytes(self, oracle, q, keys):
        cols = self.cell.columns(q.shard_id)
        if q.shard_id not in self.ostores:
            self.ostores[q.shard_id] = oracle.Store(self.ocache, cols)
        ao, bo = self.ostores[q.shard_id].respond(cols, oracle.expand_seed(q.seed, self.P.n), q.b, keys)
        return oracle.response_bytes(ao, bo, self.cell.gamma)


@pytest.fixture(scope="module")
def world(pkg, oracle, ctx):
    store = pkg.ServerSessionStore.new(ctx)
    sets = [Set(pkg, oracle, ctx, store, entry, seed + 16 * approx, approx)
            for entry, seed in ENTRIES for approx in (False, True)]
    return store, sets


@pytest.mark.parametrize("batch", BATCHES)
def test_every_set_and_batch_size(pkg, oracle, ctx, world, batch):
    store, sets = world
    for k, s in enumerate(sets):
        idx, qs = s.queries(pkg, batch, salt=batch + 31 * k)
        real = pkg.respond_seeded_batch(s.crs, s.db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(s.h_real),
                                                                           qs), s.cache, store)
        other = pkg.respond_seeded_batch(s.crs, s.db,
                                         pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(s.h_other), qs),
                                         s.cache, store)
        assert len(real) == len(other) == batch
        for i, r in zip(idx, real):
            assert s.cell.decode(i, r.a, r.b)[0], f"set {k} batch {batch}: index {i} decoded to another record"
        # Oracle bytes for the first and last query under both seats.
        for j in sorted({0, batch - 1}):
            assert real[j].to_binary() == s.oracle_bytes(oracle, qs[j], s.keys)
            assert other[j].to_binary() == s.oracle_bytes(oracle, qs[j], s.other_keys)


def test_serving_loop_across_all_sets(pkg, oracle, ctx, world):
    store, sets = world
    reqs = []
    for k, s in enumerate(sets):
        idx, qs = s.queries(pkg, 12, salt=977 + k)
        for j, q in enumerate(qs):
            reqs.append((s, q, s.h_real if j % 2 == 0 else s.h_other))
    order = np.random.default_rng(5).permutation(len(reqs))
    reqs = [reqs[i] for i in order]
    alone = [pkg.respond_seeded_batch(s.crs, s.db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), [q]),
                                      s.cache, store)[0].to_binary() for s, q, h in reqs]
    with pkg.ServingLoop(ctx, slots=3, max_batch=32) as loop:
        tickets = [loop.submit(s.crs, s.db, q, store, h) for s, q, h in reqs]
        got = [loop.wait(t, WAIT_MS).to_binary() for t in tickets]
        st = loop.stats()
    assert got == alone
    # Batches span parameter sets (one launch serves several), so 72 requests of up to 32 a
    # batch take at least three batches, and may take fewer than the six sets.
    assert st["served"] == len(reqs) and st["batches"] >= 3


@pytest.mark.parametrize("shape", ["pair", "single", "quad"])
def test_one_launch_across_all_sets(pkg, oracle, ctx, world, shape):
    """One scan and one respond launch over queries of all six sets, both seats of each and
    two switch targets: every response is the one its query gets alone, under both launch
    shapes (the launch orders its queries by gamma, so rows must come back in place)."""
    store, sets = world
    items = []
    for k, s in enumerate(sets):
        idx, qs = s.queries(pkg, 5, salt=4001 + 13 * k)
        for j, q in enumerate(qs):
            ms = pkg.MOD_SWITCH_TARGET_36BIT if (j + k) % 2 else 0
            items.append((s, q, s.h_real if j % 2 == 0 else s.h_other, ms))
    order = np.random.default_rng(11).permutation(len(items))
    items = [items[i] for i in order]
    alone = [pkg.respond_seeded_batch(s.crs, s.db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), [q]),
                                      s.cache, store, mod_switch_target=ms)[0].to_binary() for s, q, h, ms in items]
    ctx.set_launch_shape({"pair": 2, "single": 1, "quad": 4}[shape])
    try:
        got = pkg.respond_mixed_batch([pkg.MixedQuery(s.db, store, h, q, ms) for s, q, h, ms in items])
    finally:
        ctx.set_launch_shape(0)
    assert [r.to_binary() for r in got] == alone
    # The first query of the mix against the oracle directly.
    s, q, h, ms = items[0]
    want = s.oracle_bytes(oracle, q, s.keys if h == s.h_real else s.other_keys)
    if not ms:
        assert got[0].to_binary() == want


def test_mixed_launch_device_buffers_and_refusals(pkg, oracle, ctx, world):
    import torch

    store, sets = world
    items = []
    for k, s in enumerate(sets):
        _, qs = s.queries(pkg, 3, salt=5003 + k)
        items += [(s, q, s.h_real) for q in qs]
    n = 2048
    count = len(items)
    dbs = np.array([s.db.h for s, _, _ in items], dtype=np.uint64)
    stores = np.full(count, store.h, dtype=np.uint64)
    handles = np.array([int(h) for _, _, h in items], dtype=np.uint64)
    sids = np.array([q.shard_id for _, q, _ in items], dtype=np.uint32)
    ms = np.zeros(count, dtype=np.uint64)
    seeds = torch.from_numpy(np.stack([np.frombuffer(q.seed, dtype=np.uint8) for _, q, _ in items]).copy()).cuda()
    bs = torch.from_numpy(np.stack([np.asarray(q.b, dtype=np.uint64) for _, q, _ in items]).view(np.int64)).cuda()
    a = torch.zeros((count, n), dtype=torch.int64, device="cuda")
    b = torch.zeros_like(a)
    status = torch.full((count,), 7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.check(ctx._lib.ig_respond_mixed_batch_device(
        ctx.h, count, dbs.ctypes.data, stores.ctypes.data, handles.ctypes.data, sids.ctypes.data, seeds.data_ptr(),
        bs.data_ptr(), ms.ctypes.data, a.data_ptr(), b.data_ptr(), status.data_ptr()))
    ctx.join()
    torch.cuda.synchronize()
    assert int(status.abs().sum()) == 0
    host = pkg.respond_mixed_batch([pkg.MixedQuery(s.db, store, h, q) for s, q, h in items])
    a_h, b_h = a.cpu().numpy().view(np.uint64), b.cpu().numpy().view(np.uint64)
    for i, r in enumerate(host):
        assert np.array_equal(a_h[i], r.a) and np.array_equal(b_h[i], r.b)
    # An unknown seat refuses the whole launch.
    bad = [pkg.MixedQuery(s.db, store, h, q) for s, q, h in items]
    bad[4] = pkg.MixedQuery(bad[4].db, store, 1 << 60, bad[4].query)
    with pytest.raises(pkg.PirError, match="no entry for session_handle"):
        pkg.respond_mixed_batch(bad)
    # A shard whose columns changed after its store was built refuses the whole launch.
    s0 = sets[0]
    edited = s0.cell.columns(0)
    edited[0, 0] ^= 1
    s0.db.set_shard(0, edited)
    try:
        q_edit = pkg.SeededBatchQuery(*s0.cell.next_query(3))
        mix = [pkg.MixedQuery(s.db, store, h, q) for s, q, h in items[-4:]] + [
            pkg.MixedQuery(s0.db, store, s0.h_real, q_edit)]
        with pytest.raises(pkg.PirError, match="packing store refused") as e:
            pkg.respond_mixed_batch(mix)
        assert e.value.code == 5
    finally:
        s0.db.set_shard(0, s0.cell.columns(0))  # the original words: the store serves again


def test_seats_of_either_gadget_share_one_database(pkg, oracle, ctx):
    """A packing store depends only on the ring and the width, so one resident database
    serves seats of the exact and the approximate gadget side by side (the reference takes
    the CRS apart from the EncodedDatabase, respond.rs:1189-1202): a mixed launch and the
    serving loop answer approximate-gadget seats on an exact-gadget database with the bytes
    the approximate set's own database gives, and the single-set batch call still refuses
    the foreign seat as the reference does."""
    Pe, Pa = oracle.Params.d2048(), oracle.Params.d2048_approximate_gadget()
    ce, ca = oracle.Cell(Pe, 64, 0x6A11), oracle.Cell(Pa, 64, 0x6A11)
    assert all((ce.columns(s) == ca.columns(s)).all() for s in range(ce.num_shards))
    sets = []
    for cell, P, approx in ((ce, Pe, False), (ca, Pa, True)):
        crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p, approximate_packing_gadget=approx), cell.w_seed,
                            cell.gamma)
        cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
        db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
        db.precompute_packing_all()
        sets.append((crs, cache, db))
    (crs_e, cache_e, db_e), (crs_a, cache_a, db_a) = sets
    store = pkg.ServerSessionStore.new(ctx)
    h_e = store.register_server_side(pkg.ClientPackingKeys(ce.keys(), ce.gamma), cache_e)
    h_a = store.register_server_side(pkg.ClientPackingKeys(ca.keys(), ca.gamma), cache_a)
    idx_a, idx_e = [5, 2048 + 7, 2 * 2048 + 100], [9, 4000]
    qa = [pkg.SeededBatchQuery(*ca.next_query(i)) for i in idx_a]
    qe = [pkg.SeededBatchQuery(*ce.next_query(i)) for i in idx_e]
    alone_a = pkg.respond_seeded_batch(crs_a, db_a, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h_a), qa),
                                       cache_a, store)
    alone_e = pkg.respond_seeded_batch(crs_e, db_e, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h_e), qe),
                                       cache_e, store)
    mix = pkg.respond_mixed_batch([pkg.MixedQuery(db_e, store, h_a, q) for q in qa] +
                                  [pkg.MixedQuery(db_e, store, h_e, q) for q in qe])
    assert [r.to_binary() for r in mix] == [r.to_binary() for r in alone_a + alone_e]
    for i, r in zip(idx_a, mix[:3]):
        assert ca.decode(i, r.a, r.b)[0]
    with pkg.ServingLoop(ctx, slots=2, max_batch=8) as loop:
        tickets = [loop.submit(crs_a, db_e, q, store, h_a) for q in qa]
        served = [loop.wait(t, WAIT_MS).to_binary() for t in tickets]
    assert served == [r.to_binary() for r in alone_a]
    with pytest.raises(pkg.PirError, match="another ring or gadget"):
        pkg.respond_seeded_batch(crs_e, db_e, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h_a), qa[:1]),
                                 cache_e, store)
