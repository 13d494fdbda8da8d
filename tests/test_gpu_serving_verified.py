"""Real encrypted queries through the serving loop at saturation, every record checked:
the GPU client (DeviceClient) draws a batch of seeded queries from the session's sampler
stream, the continuous-batching loop answers them under the session's registered key with
the 36-bit switch, and the GPU extraction must return each queried record of a 2^18-record
database (128 MiB of 512-byte records, encoded on the GPU from the records' bytes)."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def test_every_served_record_decodes(oracle):
    pkg = load_package()
    P = oracle.Params.d2048()
    entry, entries = 512, 1 << 18
    cell = oracle.Cell(P, entry, 0x5E7E, entries)
    records = cell.database()
    assert len(records) == entry * entries
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_records(cache, records, entry)
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new(cache.ctx)
    h = store.register_server_side(pkg.ClientPackingKeys(cell.keys(), cell.gamma), cache)
    client = pkg.DeviceClient(cache, cell.secret(), P.sigma)
    key, pos = cell.sampler_state()
    rng = np.random.default_rng(11)
    count = 4096
    idx = rng.integers(0, entries, count)
    seeds = [rng.bytes(32) for _ in range(count)]
    qs = []
    for s in range(0, count, 1024):
        part, pos = client.query_batch(idx[s:s + 1024], seeds[s:s + 1024], key, pos)
        qs += part
    shard_ids = np.array([q.shard_id for q in qs], dtype=np.uint32)
    bs = np.stack([q.b for q in qs])
    seed_arr = np.frombuffer(b"".join(q.seed for q in qs), dtype=np.uint8).reshape(count, 32)
    handles = np.full(count, int(h), dtype=np.uint64)
    ms = pkg.MOD_SWITCH_TARGET_36BIT
    with pkg.ServingLoop(cache.ctx, slots=4, max_batch=64) as loop:
        a, b, lat, el = loop.replay(db, store, shard_ids, handles, seed_arr, bs, ms, window=1024)
    got = client.extract_arrays(a, b, ms, entry)
    want = np.frombuffer(records, dtype=np.uint8).reshape(entries, entry)[idx]
    assert (got == want).all()
    assert (lat > 0).all() and el > 0
    client.close()
