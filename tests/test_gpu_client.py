"""The client side on the GPU (DeviceClient: ClientSession::query_batch, session.rs:377-434;
extract_inspiring / extract_packed / extract_inspiring_mod_switched, extract.rs:184-263 and
mod_switch.rs:573-640). The query batch must reproduce, word for word, the queries the
oracle's session draws one after another from the same sampler stream (and leave the
sampler at the same position); extraction must recover the records of the server's
responses, unswitched, switched to 36 bits and tree-packed."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def session(pkg, oracle, P, entry, seed, galois=False):
    cell = oracle.Cell(P, entry, seed)
    keys = cell.galois_keys(bytes(range(32))) if galois else None
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma, galois_keys=keys)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    return cell, crs, cache, db, pkg.DeviceClient(cache, cell.secret(), P.sigma)


@pytest.mark.parametrize("n,count", [(2048, 5), (2048, 64), (256, 40)])
def test_query_batch_equals_the_sessions_queries(pkg, oracle, n, count):
    P = oracle.Params(n=n)
    cell, crs, cache, db, client = session(pkg, oracle, P, 32, 0xC11E + n)
    key, pos = cell.sampler_state()
    total = cell.num_shards * n
    idx = [(k * 7919 + 3) % total for k in range(count)]
    want = [cell.next_query(i) for i in idx]
    _, pos_after = cell.sampler_state()
    qs, new_pos = client.query_batch(idx, [w[1] for w in want], key, pos)
    assert new_pos == pos_after
    for (sid, seed, b), q in zip(want, qs):
        assert q.shard_id == sid and q.seed == seed and (q.b == b).all()
    client.close()


def test_round_trip_through_the_server(pkg, oracle):
    P = oracle.Params.d2048()
    cell, crs, cache, db, client = session(pkg, oracle, P, 512, 0xC11F)
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(cache.ctx)
    h = store.register_server_side(pkg.ClientPackingKeys(cell.keys(), cell.gamma), cache)
    key, pos = cell.sampler_state()
    rng = np.random.default_rng(9)
    total = cell.num_shards * P.n
    idx = [int(x) for x in rng.integers(0, total, 48)]
    seeds = [rng.bytes(32) for _ in idx]
    qs, _ = client.query_batch(idx, seeds, key, pos)
    batch = pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), qs)
    for ms in (0, pkg.MOD_SWITCH_TARGET_36BIT):
        out = pkg.respond_seeded_batch(crs, db, batch, cache, store, mod_switch_target=ms)
        recs = client.extract_batch(out, 512)
        assert recs == [cell.record(i) for i in idx], ms
    # The 45-bit rung is refused: the secret's product could wrap q.
    out45 = pkg.respond_seeded_batch(crs, db, batch, cache, store, mod_switch_target=pkg.MOD_SWITCH_TARGET_45BIT)
    with pytest.raises(pkg.PirError, match="not served"):
        client.extract_batch(out45, 512)
    client.close()


def test_tree_responses_extract(pkg, oracle):
    P = oracle.Params(n=256)
    cell, crs, cache, db, client = session(pkg, oracle, P, 16, 0xC120, galois=True)
    key, pos = cell.sampler_state()
    idx = [0, 5, 300, 767]
    qs, _ = client.query_batch(idx, [bytes([i % 251] * 32) for i in idx], key, pos)
    out = pkg.respond_one_packing_batch(crs, db, qs)
    assert client.extract_batch(out, 16) == [cell.record(i) for i in idx]
    client.close()
