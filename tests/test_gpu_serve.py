"""The serving loop (continuous batching, ig_serve_*): every request's response is the one
the same query gets alone through respond_seeded_batch, byte for byte, while requests of
two parameter sets (exact and approximate gadget), two mod-switch targets and several
shards arrive interleaved; a refused request finishes alone without touching the others;
latency percentiles are reported."""
import threading

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

WAIT_MS = 120_000  # a host-side stall surfaces as an error, never as a hung test


@pytest.fixture(scope="module")
def pkg():
    return load_package()


@pytest.fixture(scope="module")
def ctx(pkg):
    return pkg.Context.default()


class ParamSet:
    """One parameter set served from stores: the cell's database, its seat and its queries."""

    def __init__(self, pkg, oracle, P, entry, seed, approx, store):
        self.P = P
        self.cell = oracle.Cell(P, entry, seed)
        params = pkg.InspireParams(ring_dim=P.n, p=P.p, approximate_packing_gadget=approx)
        self.crs = pkg.ServerCrs(params, self.cell.w_seed, self.cell.gamma)
        self.cache = pkg.ServerInspiringCache.new(self.crs)
        self.db = pkg.EncodedDatabase.from_columns(
            self.cache, [self.cell.columns(s) for s in range(self.cell.num_shards)])
        self.db.precompute_packing_all()
        self.keys = pkg.ClientPackingKeys(self.cell.keys(), self.cell.gamma)
        self.handle = store.register_server_side(self.keys, self.cache)

    def query(self, pkg, idx):
        sid, qseed, b = self.cell.next_query(idx)
        return pkg.SeededBatchQuery(sid, qseed, b)

    def alone(self, pkg, store, q, ms=0):
        batch = pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(self.handle), [q])
        return pkg.respond_seeded_batch(self.crs, self.db, batch, self.cache, store, mod_switch_target=ms)[0]


@pytest.fixture(scope="module")
def sets(pkg, oracle, ctx):
    store = pkg.ServerSessionStore.new()
    exact = ParamSet(pkg, oracle, oracle.Params.d2048(), 256, 0x5E2E, False, store)
    approx = ParamSet(pkg, oracle, oracle.Params.d2048_approximate_gadget(), 64, 0x5E2F, True, store)
    return store, exact, approx


def mixed_requests(pkg, sets, count):
    """Interleaved (set, query, target, index) requests over every shard of both sets."""
    store, exact, approx = sets
    ms36 = pkg.MOD_SWITCH_TARGET_36BIT
    out = []
    for k in range(count):
        ps = exact if k % 3 != 2 else approx
        total = ps.cell.num_shards * ps.P.n
        idx = (k * 7919 + 13) % total
        ms = ms36 if (ps is exact and k % 2 == 1) else 0
        out.append((ps, ps.query(pkg, idx), ms, idx))
    return out


def test_mixed_stream_matches_each_query_alone(pkg, oracle, ctx, sets):
    store = sets[0]
    reqs = mixed_requests(pkg, sets, 36)
    alone = [ps.alone(pkg, store, q, ms).to_binary() for ps, q, ms, _ in reqs]
    with pkg.ServingLoop(ctx, slots=3, max_batch=8) as loop:
        tickets = [loop.submit(ps.crs, ps.db, q, store, ps.handle, mod_switch_target=ms) for ps, q, ms, _ in reqs]
        served = [loop.wait(t, WAIT_MS) for t in tickets]
        st = loop.stats()
    assert [r.to_binary() for r in served] == alone
    # The unswitched responses decode to the requested record.
    for (ps, q, ms, idx), r in zip(reqs, served):
        if not ms:
            assert ps.cell.decode(idx, r.a, r.b)[0], f"index {idx} decoded to another record"
    assert st["served"] == len(reqs) and st["refused"] == 0
    # 36 requests in batches of at most 8 (a batch may mix sets and switch targets).
    assert st["batches"] >= 5
    assert 1.0 <= st["mean_batch"] <= 8.0
    assert 0.0 < st["p50_us"] <= st["p99_us"] <= st["max_us"]
    assert all(t.latency_us and t.latency_us > 0 for t in tickets)


def test_mixed_stream_against_oracle(pkg, oracle, ctx, sets):
    """Two requests of the mix, checked against the oracle's bytes directly."""
    store, exact, approx = sets
    ms36 = pkg.MOD_SWITCH_TARGET_36BIT
    picks = [(exact, 2048 + 5, ms36), (approx, 77, 0)]
    with pkg.ServingLoop(ctx, slots=2, max_batch=4) as loop:
        tickets = []
        for ps, idx, ms in picks:
            q = ps.query(pkg, idx)
            tickets.append((ps, q, ms, loop.submit(ps.crs, ps.db, q, store, ps.handle, mod_switch_target=ms)))
        for ps, q, ms, t in tickets:
            r = loop.wait(t, WAIT_MS)
            ocache = oracle.Cache(ps.P, ps.cell.gamma, ps.cell.w_seed)
            ao, bo = ocache.respond_per_query(ps.cell.columns(q.shard_id), oracle.expand_seed(q.seed, ps.P.n), q.b,
                                              ps.cell.keys())
            if ms:
                ao, bo = oracle.mod_switch(ao, ps.P.q, ms), oracle.mod_switch(bo, ps.P.q, ms)
            assert r.to_binary() == oracle.response_bytes(ao, bo, ps.cell.gamma, ms or ps.P.q)


def test_concurrent_submitters(pkg, oracle, ctx, sets):
    store = sets[0]
    reqs = mixed_requests(pkg, sets, 48)
    alone = [ps.alone(pkg, store, q, ms).to_binary() for ps, q, ms, _ in reqs]
    results = [None] * len(reqs)
    errors = []
    with pkg.ServingLoop(ctx, slots=2, max_batch=16) as loop:
        def worker(part):
            try:
                for i in part:
                    ps, q, ms, _ = reqs[i]
                    t = loop.submit(ps.crs, ps.db, q, store, ps.handle, mod_switch_target=ms)
                    results[i] = loop.wait(t, WAIT_MS).to_binary()
            except Exception as e:  # reported below
                errors.append(e)
        threads = [threading.Thread(target=worker, args=(range(k, len(reqs), 4),)) for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
    assert not errors, errors
    assert results == alone


def test_refusals_finish_alone(pkg, oracle, ctx, sets):
    store, exact, approx = sets
    last = exact.cell.num_shards - 1
    assert last >= 1
    good = [exact.query(pkg, i) for i in (1, 700, 2000)]  # shard 0
    alone = [exact.alone(pkg, store, q).to_binary() for q in good]
    # A shard without a store, an unknown seat, a shard past the database.
    exact.db.shards[last].drop_packing_store()
    try:
        with pkg.ServingLoop(ctx, slots=2, max_batch=8) as loop:
            t0 = loop.submit(exact.crs, exact.db, good[0], store, exact.handle)
            bad_store = loop.submit(exact.crs, exact.db, exact.query(pkg, last * exact.P.n + 3), store,
                                    exact.handle)
            bad_seat = loop.submit(exact.crs, exact.db, good[1], store, 0xDEAD_BEEF)
            q = exact.query(pkg, 5)
            q.shard_id = exact.cell.num_shards + 3
            bad_shard = loop.submit(exact.crs, exact.db, q, store, exact.handle)
            t1 = loop.submit(exact.crs, exact.db, good[1], store, exact.handle)
            t2 = loop.submit(exact.crs, exact.db, good[2], store, exact.handle)
            with pytest.raises(pkg.PirError, match="has no packing store"):
                loop.wait(bad_store, WAIT_MS)
            with pytest.raises(pkg.PirError, match="no entry for session_handle") as e:
                loop.wait(bad_seat, WAIT_MS)
            assert e.value.code == 4
            with pytest.raises(pkg.PirError, match="not found"):
                loop.wait(bad_shard, WAIT_MS)
            got = [loop.wait(t, WAIT_MS).to_binary() for t in (t0, t1, t2)]
            st = loop.stats()
    finally:
        exact.db.shards[last].precompute_packing()
    assert got == alone
    assert st["served"] == 3 and st["refused"] == 3


def test_admission_by_request_memory(pkg, ctx, sets):
    """A budget that holds only a few requests' keys and buffers: every request is served with
    its alone bytes, the bytes in flight never pass the budget, and batches stay small; a
    budget below one request's key and buffers refuses that request (IG_ERR_NOMEM)."""
    store, exact, approx = sets
    # One gamma-256 request at ring 2048: about 51 KB of buffers, 48 KiB for its key.
    budget = 400_000
    reqs = [(exact, exact.query(pkg, (k * 104729 + 5) % (exact.cell.num_shards * 2048)),
             pkg.MOD_SWITCH_TARGET_36BIT if k % 2 else 0) for k in range(24)]
    alone = [ps.alone(pkg, store, q, ms).to_binary() for ps, q, ms in reqs]
    with pkg.ServingLoop(ctx, slots=3, max_batch=64, hbm_budget_bytes=budget) as loop:
        tickets = [loop.submit(ps.crs, ps.db, q, store, ps.handle, mod_switch_target=ms) for ps, q, ms in reqs]
        got = [loop.wait(t, WAIT_MS).to_binary() for t in tickets]
        st = loop.stats()
    assert got == alone
    assert st["budget_bytes"] == budget and st["device_bytes"] == budget
    assert 0 < st["peak_inflight_bytes"] <= budget
    assert st["mean_batch"] <= 7  # 64 would fit the slots; memory holds a batch to a handful
    assert st["inflight_bytes"] == 0
    with pkg.ServingLoop(ctx, slots=1, max_batch=4, hbm_budget_bytes=60_000) as loop:
        t = loop.submit(exact.crs, exact.db, reqs[0][1], store, exact.handle)
        with pytest.raises(pkg.PirError, match="admission refused") as e:
            loop.wait(t, WAIT_MS)
        assert e.value.code == 8
    with pytest.raises(pkg.PirError, match="cannot be allocated") as e:
        pkg.ServingLoop(ctx, slots=1, max_batch=4, hbm_budget_bytes=1 << 50)
    assert e.value.code == 8


def test_native_replay_matches_alone(pkg, oracle, ctx, sets):
    """ig_serve_replay drives the loop from native code, closed loop (a window of
    outstanding requests) and open loop (arrival times); the responses equal the same
    queries answered alone."""
    store, exact, approx = sets
    count = 40
    rng = np.random.default_rng(11)
    total = exact.cell.num_shards * exact.P.n
    idx = [int(i) for i in rng.integers(0, total, count)]
    qs = [exact.query(pkg, i) for i in idx]
    alone = [exact.alone(pkg, store, q) for q in qs]
    shard_ids = [q.shard_id for q in qs]
    handles = [exact.handle] * count
    seeds = np.stack([np.frombuffer(q.seed, dtype=np.uint8) for q in qs])
    bs = np.stack([q.b for q in qs])
    with pkg.ServingLoop(ctx, slots=2, max_batch=16) as loop:
        a, b, lat, el = loop.replay(exact.db, store, shard_ids, handles, seeds, bs, window=24)
        assert el > 0 and (lat > 0).all()
        for k in range(count):
            assert (a[k] == alone[k].a).all() and (b[k] == alone[k].b).all()
        arrivals = np.cumsum(rng.exponential(50_000, count)).astype(np.uint64)  # ~20k/s offered
        a, b, lat, el = loop.replay(exact.db, store, shard_ids, handles, seeds, bs, arrival_ns=arrivals)
        assert el * 1e9 >= float(arrivals[-1])
        for k in range(count):
            assert (a[k] == alone[k].a).all() and (b[k] == alone[k].b).all()


def test_wire_requests_return_reference_bytes(pkg, oracle, ctx, sets):
    """Requests submitted for wire bytes get the ServerResponse built on the GPU: the same
    bytes as the host encoder's for the same query answered alone, mixed in one loop with
    requests for coefficient words."""
    store, exact, approx = sets
    reqs = mixed_requests(pkg, sets, 18)
    alone = [ps.alone(pkg, store, q, ms).to_binary() for ps, q, ms, _ in reqs]
    with pkg.ServingLoop(ctx, slots=2, max_batch=8) as loop:
        tickets = [loop.submit(ps.crs, ps.db, q, store, ps.handle, mod_switch_target=ms, wire=(k % 3 != 1))
                   for k, (ps, q, ms, _) in enumerate(reqs)]
        got = [loop.wait(t, WAIT_MS) for t in tickets]
    for k, g in enumerate(got):
        assert (g if isinstance(g, bytes) else g.to_binary()) == alone[k], k
