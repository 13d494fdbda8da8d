"""The OnePacking responder on the GPU (respond_one_packing / respond_seeded_packed,
respond.rs:696-729, 1241-1249): the column LWEs packed by the Galois-automorphism tree of
inspiring/automorph_pack.rs. Bytes equal the oracle's restatement of the tree under the
same Galois keys; responses decode, through extract_packed (extract.rs:184-226), to the
requested record. The reference draws its Galois keys' `a` from OS entropy, so no byte
golden exists for this variant: the keys here are test keys of the cell's secret."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu
KEY_SEED = bytes(range(32))


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def setup(pkg, oracle, P, entry, seed, with_keys=True):
    cell = oracle.Cell(P, entry, seed)
    keys = cell.galois_keys(KEY_SEED)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma,
                        galois_keys=keys if with_keys else None)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    return cell, keys, crs, db, oracle.Cache(P, cell.gamma, cell.w_seed)


@pytest.mark.parametrize("n,entry", [(256, 16), (256, 256), (2048, 32)])
def test_tree_bytes_and_decode(pkg, oracle, n, entry):
    P = oracle.Params(n=n)
    cell, keys, crs, db, ocache = setup(pkg, oracle, P, entry, 0x7EE0 + entry)
    idxs = [0, n + 3, 3 * n - 1] if n == 256 else [5, 2 * n + 9]
    for idx in idxs:
        sid, seed, b = cell.next_query(idx)
        r = pkg.respond_seeded_packed(crs, db, pkg.SeededBatchQuery(sid, seed, b))
        a = oracle.expand_seed(seed, n)
        ao, bo = ocache.respond_one_packing(cell.columns(sid), a, b, keys)
        assert (r.a == ao).all() and (r.b == bo).all(), idx
        wire = r.to_binary()
        assert wire == oracle.response_bytes_tree(ao, bo, cell.gamma)
        ok, rec = cell.decode_tree(idx, r.a, r.b)
        assert ok and rec == cell.record(idx)
        ru = pkg.respond_one_packing(crs, db, pkg.ClientQuery(sid, a, b))
        assert ru.to_binary() == wire
        assert pkg.ServerResponse.from_rims(r.to_rims()).packing_mode == "Tree"


def test_single_column_skips_the_tree(pkg, oracle):
    """pack_lwes with one LWE returns it without the tree or the d scaling
    (automorph_pack.rs:300-306); the bytes follow the restatement."""
    P = oracle.Params(n=256)
    cell, keys, crs, db, ocache = setup(pkg, oracle, P, 2, 0x7EE2)
    assert cell.gamma == 1
    sid, seed, b = cell.next_query(7)
    r = pkg.respond_seeded_packed(crs, db, pkg.SeededBatchQuery(sid, seed, b))
    ao, bo = ocache.respond_one_packing(cell.columns(sid), oracle.expand_seed(seed, P.n), b, keys)
    assert r.to_binary() == oracle.response_bytes_tree(ao, bo, 1)


def test_batch_over_shards_and_mod_switch(pkg, oracle):
    P = oracle.Params(n=256)
    cell, keys, crs, db, ocache = setup(pkg, oracle, P, 64, 0x7EE3)
    qs = [pkg.SeededBatchQuery(*cell.next_query(i)) for i in (1, 300, 700, 2, 511)]
    batch = pkg.respond_one_packing_batch(crs, db, qs)
    for q, r in zip(qs, batch):
        assert r.to_binary() == pkg.respond_seeded_packed(crs, db, q).to_binary()
    # A switched tree response equals the switch of the unswitched one (mod_switch.rs:148-176).
    ms = pkg.MOD_SWITCH_TARGET_36BIT
    sw = pkg.respond_one_packing_batch(crs, db, qs[:2], mod_switch_target=ms)
    for r, s in zip(batch[:2], sw):
        assert (s.a == oracle.mod_switch(r.a, P.q, ms)).all() and (s.b == oracle.mod_switch(r.b, P.q, ms)).all()


def test_refusals(pkg, oracle):
    P = oracle.Params(n=256)
    cell, keys, crs, db, _ = setup(pkg, oracle, P, 16, 0x7EE4, with_keys=False)
    sid, seed, b = cell.next_query(0)
    with pytest.raises(pkg.PirError, match="0 galois keys, but ring_dim 256 packs through 8 tree levels"):
        pkg.respond_seeded_packed(crs, db, pkg.SeededBatchQuery(sid, seed, b))
    cache = db.cache
    with pytest.raises(pkg.PirError, match="7 galois keys, but ring_dim 256 packs through 8 tree levels"):
        cache.set_galois_keys(keys[:7])
    bad = keys.copy()
    bad[3, 1, 0, 5] = P.q
    with pytest.raises(pkg.PirError, match="not a residue"):
        cache.set_galois_keys(bad)
    cache.set_galois_keys(keys)
    r = pkg.respond_seeded_packed(crs, db, pkg.SeededBatchQuery(sid, seed, b))
    assert cell.decode_tree(0, r.a, r.b)[0]


def test_concurrent_callers_over_lanes(pkg, oracle):
    """Three caller threads over three lanes (each call holds a lane with its node stacks
    and copies its responses out after releasing the context lock) give the one-lane
    answers."""
    import threading
    P = oracle.Params(n=256)
    ctx = pkg.Context.default()
    cell, keys, crs, db, _ = setup(pkg, oracle, P, 64, 0x7EE5)
    batches = [[pkg.SeededBatchQuery(*cell.next_query((11 * j + 5 * i) % (2 * P.n))) for i in range(4)]
               for j in range(6)]
    want = [[r.to_binary() for r in pkg.respond_one_packing_batch(crs, db, b)] for b in batches]
    got = [None] * len(batches)
    errors = []
    ctx.set_lanes(3)
    try:
        def caller(t):
            try:
                for j in range(t, len(batches), 3):
                    got[j] = [r.to_binary() for r in pkg.respond_one_packing_batch(crs, db, batches[j])]
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
