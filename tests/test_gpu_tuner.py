"""The launch-shape tuner: one full wave of queries timed under 1, 2 and 4 CTAs per query
for each width, the table saved and loaded, the shape a launch takes from it, and responses
byte-identical whichever shape the table picks."""
import os

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def test_tune_save_load_choose(oracle, tmp_path):
    pkg = load_package()
    ctx = pkg.Context(0)
    table = ctx.tune_launch_shapes([16, 256], reps=1)
    for g, rows in table.items():
        assert sorted(rows) == list(pkg.TUNE_BATCHES)
        for b, ms in rows.items():
            assert len(ms) == 3 and all(x > 0 for x in ms), (g, b, ms)
    path = tmp_path / "shapes.txt"
    ctx.save_tuning(path)
    other = pkg.Context(0)
    with pytest.raises(pkg.PirError, match="no launch-shape entry"):
        other.tuned(256)
    other.load_tuning(path)
    for b in pkg.TUNE_BATCHES:
        assert other.tuned(256, b) == pytest.approx(table[256][b], rel=1e-5)

    def pick(ms):  # the fastest shape, more CTAs only when at least 2% faster
        best = 0
        for k in (1, 2):
            if ms[k] < ms[best] * 0.98:
                best = k
        return (1, 2, 4)[best]

    # A lone query takes the row of one query in flight; between grid points the next row
    # up; beyond the grid the last row.
    assert other.launch_shape_for(256, 1) == pick(table[256][1])
    assert other.launch_shape_for(256, 3) == pick(table[256][4])
    assert other.launch_shape_for(256, 64, in_flight=4096) == pick(table[256][256])
    # Many queries in flight fill the GPU several times over: one CTA per query.
    assert pick(table[256][256]) == 1
    # A table measured on another SM count is refused.
    text = path.read_text().splitlines()
    text[1] = "sms 7"
    bad = tmp_path / "bad.txt"
    bad.write_text("\n".join(text) + "\n")
    with pytest.raises(pkg.PirError, match="another SM count|measured on 7 SMs"):
        other.load_tuning(bad)
    # Responses under the tuned choice equal the oracle's, batch of 1 and of 7.
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 512, 0x7E57)
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs, ctx=other)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    db.precompute_packing_all()
    keys = pkg.ClientPackingKeys(cell.keys(), cell.gamma)
    ocache = oracle.Cache(P, cell.gamma, cell.w_seed)
    for count in (1, 7):
        idx = [(k * 2999 + count) % (cell.num_shards * P.n) for k in range(count)]
        qs = [pkg.SeededBatchQuery(*cell.next_query(i)) for i in idx]
        out = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Inline(keys), qs), cache)
        for q, r in zip(qs, out):
            ao, bo = ocache.respond_per_query(cell.columns(q.shard_id), oracle.expand_seed(q.seed, P.n), q.b,
                                              cell.keys())
            assert r.to_binary() == oracle.response_bytes(ao, bo, cell.gamma)
    other.close()
    ctx.close()
