"""Failure handling without a GPU fault: a device allocation made to fail on the host
(ig_debug_fail_alloc_at) refuses its call with IG_ERR_NOMEM, leaves no half-built object
and the context usable, and a retry serves the reference's bytes; RAVEN_PROFILE_RESPOND
prints the reference's profile line."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT, load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def test_injected_allocation_failures(pkg, oracle):
    ctx = pkg.Context.default()
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 32, 0xFA11)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase(cache, cell.num_shards)
    keys = pkg.ClientPackingKeys(cell.keys(), cell.gamma)
    lib = ctx._lib
    # Shard upload: its first allocation fails (the columns), then its second (the u16 copy).
    for k in (1, 2):
        lib.ig_debug_fail_alloc_at(ctx.h, k)
        with pytest.raises(pkg.PirError, match="injected") as e:
            db.set_shard(0, cell.columns(0))
        assert e.value.code == 8
        lib.ig_debug_fail_alloc_at(ctx.h, 0)
    for s in range(cell.num_shards):
        db.set_shard(s, cell.columns(s))
    # Store build: each of its three allocations in turn.
    for k in (1, 2, 3):
        lib.ig_debug_fail_alloc_at(ctx.h, k)
        with pytest.raises(pkg.PirError, match="injected"):
            db.shards[1].precompute_packing()
        lib.ig_debug_fail_alloc_at(ctx.h, 0)
        assert not db.shards[1].packing_store()
    db.precompute_packing_all()
    # Seat registration and the serving loop.
    store = pkg.ServerSessionStore.new(ctx)
    lib.ig_debug_fail_alloc_at(ctx.h, 1)
    with pytest.raises(pkg.PirError, match="injected"):
        store.register_server_side(keys, cache)
    lib.ig_debug_fail_alloc_at(ctx.h, 0)
    assert len(store) == 0
    h = store.register_server_side(keys, cache)
    lib.ig_debug_fail_alloc_at(ctx.h, 1)  # the loop's one device allocation: its budget ring
    with pytest.raises(pkg.PirError, match="injected"):
        pkg.ServingLoop(ctx, slots=2, max_batch=8)
    lib.ig_debug_fail_alloc_at(ctx.h, 0)
    # Everything still answers the reference's bytes.
    rec = set()
    with open(os.path.join(ROOT, "tests", "golden", "seat_kat_lines.txt")) as f:
        rec = set(x.strip() for x in f)
    qs = [pkg.SeededBatchQuery(*cell.next_query(i)) for i in (3, P.n + 9, 2 * P.n + 100)]
    outs = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), qs), cache,
                                    store)
    with pkg.ServingLoop(ctx, slots=2, max_batch=8) as loop:
        served = [loop.wait(loop.submit(crs, db, q, store, h), 60_000) for q in qs]
    for r, s in zip(outs, served):
        assert r.to_binary() == s.to_binary()
    ocache = oracle.Cache(P, cell.gamma, cell.w_seed)
    for q, r in zip(qs, outs):
        ao, bo = ocache.respond_per_query(cell.columns(q.shard_id), oracle.expand_seed(q.seed, P.n), q.b,
                                          cell.keys())
        assert r.to_binary() == oracle.response_bytes(ao, bo, cell.gamma)


def test_profile_env_prints_reference_line():
    code = (
        "import numpy as np, os, sys\n"
        "sys.path.insert(0, os.getcwd())\n"
        "from __graft_entry__ import _package\n"
        "pkg = _package()\n"
        "d = np.load('tests/golden/d256_respond.npz')\n"
        "g = int(d['gamma'])\n"
        "crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=int(d['n']), p=int(d['p'])), d['w_seed'].tobytes(), g)\n"
        "db = pkg.EncodedDatabase.from_columns(pkg.ServerInspiringCache.new(crs), [d['columns']])\n"
        "q = pkg.ClientQuery(0, d['query_a'], d['query_b'], inspiring_packing_keys=pkg.ClientPackingKeys(d['y_body'], g))\n"
        "pkg.respond_inspiring(crs, db, q)\n"
    )
    env = dict(os.environ, RAVEN_PROFILE_RESPOND="1")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "RAVEN_PROFILE num_cols=16 queries=1 column_check_us=" in r.stderr
