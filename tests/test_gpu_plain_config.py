"""The plain method exactly as the reference's public API runs it (respond.rs:1218-1226,
extract.rs:229-263): InspireParams::d2048, a database of 2048 records of 32 bytes (one shard,
16 columns of 16-bit words) of uniform bytes from seed 0, setup_with_rng and one
ClientSession::with_seeded_secret on the seed-0 sampler and rng, one query_seeded at an
index drawn uniformly from [0, 2048), answered by respond_seeded_inspiring with the packing
key inline. The response must be byte-identical to the oracle's and extract must return the
record exactly, on the CPU (the oracle's decode) and on the GPU (DeviceClient)."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def test_plain_method_d2048_2048_records_of_32_bytes(oracle):
    pkg = load_package()
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 32, 0, entries=2048, plain=True)
    assert (cell.gamma, cell.num_shards) == (16, 1)
    index = cell.draw_index(2048)
    shard_id, seed, b = cell.next_query(index)
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs)
    # encode_database on the GPU from the record bytes (no store: the uncached respond).
    db = pkg.EncodedDatabase.from_records(cache, cell.database(), 32)
    keys = pkg.ClientPackingKeys(cell.keys(), cell.gamma)
    query = pkg.SeededClientQuery(shard_id, seed, b, inspiring_packing_keys=keys)
    resp = pkg.respond_seeded_inspiring(crs, db, query)
    ocache = oracle.Cache(P, cell.gamma, cell.w_seed)
    ao, bo = ocache.respond_per_query(cell.columns(0), oracle.expand_seed(seed, P.n), b, cell.keys())
    assert resp.to_binary() == oracle.response_bytes(ao, bo, cell.gamma, P.q)
    ok, record = cell.decode(index, resp.a, resp.b)
    assert ok and record == cell.record(index)
    client = pkg.DeviceClient(cache, cell.secret())
    try:
        assert client.extract_batch([resp], 32) == [cell.record(index)]
    finally:
        client.close()
