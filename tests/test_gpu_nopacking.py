"""The NoPacking responder on the GPU (respond / respond_seeded, respond.rs:614-643,
1229-1237): one ciphertext per column and their sum. Bytes equal the oracle's restatement;
the column ciphertexts decode, through the reference's unpacked extract, to the requested
record; seeded and unseeded queries agree; batches over several shards agree with single
calls."""
import numpy as np
import pytest

from conftest import load_package
from nopacking_decode import extract

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def setup(pkg, oracle, P, entry, seed):
    cell = oracle.Cell(P, entry, seed)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    return cell, crs, db, oracle.Cache(P, cell.gamma, cell.w_seed)


@pytest.mark.parametrize("entry", [32, 256])
def test_nopacking_bytes_and_decode(pkg, oracle, entry):
    P = oracle.Params.d2048()
    cell, crs, db, ocache = setup(pkg, oracle, P, entry, 0x4E50 + entry)
    secret = cell.secret()
    for idx in [0, P.n + 3, 3 * P.n - 1]:
        sid, seed, b = cell.next_query(idx)
        r = pkg.respond_seeded(crs, db, pkg.SeededBatchQuery(sid, seed, b))
        a = oracle.expand_seed(seed, P.n)
        want = ocache.respond_nopacking(cell.columns(sid), a, b)
        assert r.to_binary() == oracle.response_bytes_full(want)
        assert extract(r.column_ciphertexts, secret, P.q, P.p, entry) == cell.record(idx)
        ru = pkg.respond(crs, db, pkg.ClientQuery(sid, a, b))
        assert ru.to_binary() == r.to_binary()


def test_nopacking_batch_matches_single_calls(pkg, oracle):
    P = oracle.Params.d2048()
    cell, crs, db, _ = setup(pkg, oracle, P, 64, 0x4E51)
    qs = [pkg.SeededBatchQuery(*cell.next_query(i)) for i in (5, 2048 + 9, 4095, 4096 + 77, 1)]
    batch = pkg.respond_nopacking_batch(crs, db, qs)
    for q, r in zip(qs, batch):
        assert r.to_binary() == pkg.respond_seeded(crs, db, q).to_binary()


def test_nopacking_single_column_ring256(pkg, oracle):
    """gamma 1 on the d256 ring: one column, the sum equals it."""
    P = oracle.Params(n=256)
    cell, crs, db, ocache = setup(pkg, oracle, P, 2, 0x534D4102)
    sid, seed, b = cell.next_query(3)
    r = pkg.respond_seeded(crs, db, pkg.SeededBatchQuery(sid, seed, b))
    want = ocache.respond_nopacking(cell.columns(sid), oracle.expand_seed(seed, P.n), b)
    assert r.to_binary() == oracle.response_bytes_full(want)
    assert len(r.column_ciphertexts) == 1
    assert (r.a == r.column_ciphertexts[0][0]).all() and (r.b == r.column_ciphertexts[0][1]).all()


def test_nopacking_concurrent_callers_over_lanes(pkg, oracle):
    """Three caller threads over three lanes (each call holds a lane and copies its
    ciphertexts out after releasing the context lock) give the one-lane answers."""
    import threading
    P = oracle.Params.d2048()
    ctx = pkg.Context.default()
    cell, crs, db, _ = setup(pkg, oracle, P, 64, 0x4E52)
    batches = [[pkg.SeededBatchQuery(*cell.next_query((7 * j + 3 * i) % (2 * P.n))) for i in range(3)]
               for j in range(6)]
    want = [[r.to_binary() for r in pkg.respond_nopacking_batch(crs, db, b)] for b in batches]
    got = [None] * len(batches)
    errors = []
    ctx.set_lanes(3)
    try:
        def caller(t):
            try:
                for j in range(t, len(batches), 3):
                    got[j] = [r.to_binary() for r in pkg.respond_nopacking_batch(crs, db, batches[j])]
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
