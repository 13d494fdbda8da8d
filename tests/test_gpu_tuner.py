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
    for g, ms in table.items():
        assert len(ms) == 3 and all(x > 0 for x in ms), (g, ms)
    path = tmp_path / "shapes.txt"
    ctx.save_tuning(path)
    other = pkg.Context(0)
    with pytest.raises(pkg.PirError, match="no launch-shape entry"):
        other.tuned(256)
    other.load_tuning(path)
    assert other.tuned(256) == pytest.approx(table[256], rel=1e-5)
    # A lone query spreads over the most SMs the table finds worth it; a batch that fills
    # the GPU several times over runs one CTA per query.
    t1, t2, t4 = table[256]
    lone = other.launch_shape_for(256, 1, 152)
    assert lone == min((1, 2, 4), key=lambda s: ({1: t1, 2: t2, 4: t4}[s], s))
    assert other.launch_shape_for(256, 4096, 152) == 1
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
