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
    assert st["served"] == len(reqs) and st["batches"] >= len(sets)
