"""GPU parity: the CUDA respond path, called through the C ABI, against the CPU oracle
and the reference's recorded bytes. Bit-exact everywhere (integer arithmetic mod q)."""
import os

import numpy as np
import pytest

from conftest import ROOT, load_package

pytestmark = pytest.mark.gpu

D2048_CELLS = [(32, 0x52455300), (32, 0x52455301), (256, 0x52455300), (256, 0x52455301),
               (512, 0x52455300), (512, 0x52455301), (1024, 0x52455300)]


@pytest.fixture(scope="module")
def pkg():
    return load_package()


@pytest.fixture(scope="module")
def ctx(pkg):
    return pkg.Context.default()


def gpu_cell(pkg, oracle, params_o, entry, seed, entries=None, approx=False):
    cell = oracle.Cell(params_o, entry, seed, entries)
    params = pkg.InspireParams(ring_dim=params_o.n, p=params_o.p, approximate_packing_gadget=approx)
    crs = pkg.ServerCrs(params, cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_columns(cache, [cell.columns(s) for s in range(cell.num_shards)])
    keys = pkg.ClientPackingKeys(cell.keys(), cell.gamma)
    return cell, crs, cache, db, keys


def oracle_bytes(oracle, cell, P, sid, seed, b, ms=0):
    cache = oracle.Cache(P, cell.gamma, cell.w_seed)
    a = oracle.expand_seed(seed, P.n)
    ao, bo = cache.respond_per_query(cell.columns(sid), a, b, cell.keys())
    if ms:
        return oracle.response_bytes(oracle.mod_switch(ao, P.q, ms), oracle.mod_switch(bo, P.q, ms), cell.gamma, ms)
    return oracle.response_bytes(ao, bo, cell.gamma, P.q)


def test_d256_fixture_on_gpu(pkg, oracle, ctx):
    d = np.load(os.path.join(ROOT, "tests", "golden", "d256_respond.npz"))
    gamma = int(d["gamma"])
    params = pkg.InspireParams(ring_dim=int(d["n"]), p=int(d["p"]))
    crs = pkg.ServerCrs(params, d["w_seed"].tobytes(), gamma)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_columns(cache, [d["columns"]])
    keys = pkg.ClientPackingKeys(d["y_body"], gamma)
    q = pkg.ClientQuery(0, d["query_a"], d["query_b"], inspiring_packing_keys=keys)
    r1 = pkg.respond_inspiring(crs, db, q).to_binary()
    assert oracle.fnv1a(r1) == int(d["golden_fnv"])
    db.shards[0].precompute_packing()
    assert db.shards[0].packing_store()
    r2 = pkg.respond_inspiring(crs, db, q).to_binary()
    assert r2 == r1
    # The device store holds the reference's step-1 sums word for word (Montgomery form).
    P = oracle.Params(n=int(d["n"]), p=int(d["p"]))
    ost = oracle.Store(oracle.Cache(P, gamma, d["w_seed"].tobytes()), d["columns"])
    assert (db.store_sums(0) == ost.sums()).all()


@pytest.fixture(params=["pair", "single", "quad"])
def launch_shape(request, ctx):
    """The three respond kernels: two CTAs per query and four (clusters, for small batches),
    and one CTA per query."""
    ctx.set_launch_shape({"single": 1, "pair": 2, "quad": 4}[request.param])
    yield request.param
    ctx.set_launch_shape(0)


@pytest.mark.parametrize("entry,seed", D2048_CELLS)
def test_d2048_seat_kat_cells_on_gpu(pkg, oracle, ctx, recorded_lines, launch_shape, entry, seed):
    P = oracle.Params.d2048()
    n = P.n
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, entry, seed)
    rec = set(recorded_lines)
    kb = cell.key_bytes()
    assert f"SESSIONKEY d2048 entry={entry} seed={seed:#x} len={len(kb)} fnv={oracle.fnv1a(kb):#018x}" in rec
    indices = [0, 1, n - 1, n, 2 * n + 17, 3 * n - 1]
    queries = []
    for idx in indices:
        sid, qseed, b = cell.next_query(idx)
        queries.append(pkg.SeededBatchQuery(sid, qseed, b))
    # Per-query branch (no stores), one call per query with the key inline.
    per_query = []
    for idx, q in zip(indices, queries):
        sq = pkg.SeededClientQuery(q.shard_id, q.seed, q.b, inspiring_packing_keys=keys)
        r = pkg.respond_seeded_inspiring(crs, db, sq)
        ok, _ = cell.decode(idx, r.a, r.b)
        assert ok, f"index {idx} decoded to another record"
        wire = r.to_binary()
        line = f"RESP d2048 entry={entry} seed={seed:#x} index={idx} len={len(wire)} fnv={oracle.fnv1a(wire):#018x}"
        assert line in rec, line
        per_query.append(wire)
    # Store branch: every shard folded, one batch under a registered seat.
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new()
    h = store.register_server_side(keys, cache)
    batch = pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), queries)
    served = [r.to_binary() for r in pkg.respond_seeded_batch(crs, db, batch, cache, store)]
    assert served == per_query
    inline = pkg.SeededQueryBatch(pkg.PackingKeySource.Inline(keys), queries)
    assert [r.to_binary() for r in pkg.respond_seeded_batch(crs, db, inline, cache)] == per_query
    assert store.remove(h) and not store.get(h) and len(store) == 0


def test_mod_switched_batch_matches_oracle(pkg, oracle, ctx, launch_shape):
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 512, 0x4D53)
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new()
    h = store.register_server_side(keys, cache)
    ms = pkg.MOD_SWITCH_TARGET_36BIT
    qs, refs = [], []
    for idx in [3, 2048 + 99, 4095, 6000]:
        sid, seed, b = cell.next_query(idx)
        qs.append(pkg.SeededBatchQuery(sid, seed, b))
        refs.append(oracle_bytes(oracle, cell, P, sid, seed, b, ms))
    out = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), qs), cache,
                                   store, mod_switch_target=ms)
    wires = [r.to_binary() for r in out]
    assert all(len(w) == 10_446 for w in wires)
    assert wires == refs


def test_approximate_gadget_matches_oracle(pkg, oracle, ctx, launch_shape):
    P = oracle.Params.d2048_approximate_gadget()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 64, 0xA9, approx=True)
    assert cache.key_rows == 2
    db.precompute_packing_all()
    for idx in [5, 2048 + 700]:
        sid, seed, b = cell.next_query(idx)
        r = pkg.respond_seeded_inspiring(crs, db, pkg.SeededClientQuery(sid, seed, b, inspiring_packing_keys=keys))
        assert r.to_binary() == oracle_bytes(oracle, cell, P, sid, seed, b)
        assert cell.decode(idx, r.a, r.b)[0]


def test_serial_expansion_path_matches(pkg, oracle, ctx, launch_shape):
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 32, 0x5E1)
    sid, seed, b = cell.next_query(77)
    q = pkg.SeededClientQuery(sid, seed, b, inspiring_packing_keys=keys)
    fast = pkg.respond_seeded_inspiring(crs, db, q).to_binary()
    ctx._lib.ig_debug_force_serial_expand(ctx.h, 1)
    try:
        slow = pkg.respond_seeded_inspiring(crs, db, q).to_binary()
    finally:
        ctx._lib.ig_debug_force_serial_expand(ctx.h, 0)
    assert slow == fast == oracle_bytes(oracle, cell, P, sid, seed, b)


def test_store_refuses_edited_columns_whole_batch(pkg, oracle, ctx):
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 32, 0xED17)
    db.precompute_packing_all()
    q0 = pkg.SeededBatchQuery(*cell.next_query(10))
    q1 = pkg.SeededBatchQuery(*cell.next_query(2048 + 10))
    cols = cell.columns(1)
    cols[5, 100] ^= 1
    db.set_shard(1, cols)
    batch = pkg.SeededQueryBatch(pkg.PackingKeySource.Inline(keys), [q0, q1])
    with pytest.raises(pkg.PirError, match="packing store refused") as e:
        pkg.respond_seeded_batch(crs, db, batch, cache)
    assert e.value.code == 5
    # Rebuilding the store serves the edited shard again.
    db.shards[1].precompute_packing()
    assert len(pkg.respond_seeded_batch(crs, db, batch, cache)) == 2


def test_store_tags_follow_every_column_change(pkg, oracle, ctx):
    """The tag check runs where the columns change (host upload, device upload, encode):
    the same columns again keep the store served with the oracle's bytes, any edit refuses
    the shard until its store is rebuilt."""
    import torch

    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 32, 0x7A65)
    db.precompute_packing_all()
    sid, seed, b = cell.next_query(2048 + 3)
    q = pkg.SeededClientQuery(sid, seed, b, inspiring_packing_keys=keys)
    want = oracle_bytes(oracle, cell, P, sid, seed, b)
    assert pkg.respond_seeded_inspiring(crs, db, q).to_binary() == want
    cols = cell.columns(1)
    db.set_shard(1, cols)  # the same words: the tags still match
    assert pkg.respond_seeded_inspiring(crs, db, q).to_binary() == want
    edited = cols.copy()
    edited[3, 2047] ^= 1 << 7
    d_cols = torch.from_numpy(edited.view(np.int64)).cuda()
    torch.cuda.synchronize()
    db.set_shard_device(1, d_cols.data_ptr())
    with pytest.raises(pkg.PirError, match="packing store refused") as e:
        pkg.respond_seeded_inspiring(crs, db, q)
    assert e.value.code == 5
    d_cols = torch.from_numpy(cols.view(np.int64)).cuda()  # the original words restore the tags
    torch.cuda.synchronize()
    db.set_shard_device(1, d_cols.data_ptr())
    assert pkg.respond_seeded_inspiring(crs, db, q).to_binary() == want
    # Records encoded over the stored shard: other bytes refuse it, a rebuild serves them.
    rec = bytearray(cell.database()[2048 * 32:2 * 2048 * 32])
    rec[5] ^= 0xFF
    db.encode_records(bytes(rec), 32, first_shard=1)
    with pytest.raises(pkg.PirError, match="packing store refused"):
        pkg.respond_seeded_inspiring(crs, db, q)
    db.shards[1].precompute_packing()
    assert len(pkg.respond_seeded_inspiring(crs, db, q).to_binary()) == len(want)


def test_non_canonical_column_words_read_as_residues(pkg, oracle, ctx):
    """Words >= q are served as their residue on both branches (shard_store tests 204-257)."""
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 32, 0xB16)
    cols = cell.columns(0)
    cols[0, :64] += np.uint64(pkg.DEFAULT_Q)
    cols[1, 64:80] = np.uint64(2**64 - 1)
    db.set_shard(0, cols)
    sid, seed, b = cell.next_query(5)
    q = pkg.SeededClientQuery(sid, seed, b, inspiring_packing_keys=keys)
    r1 = pkg.respond_seeded_inspiring(crs, db, q).to_binary()
    db.shards[0].precompute_packing()
    r2 = pkg.respond_seeded_inspiring(crs, db, q).to_binary()
    ocache = oracle.Cache(P, cell.gamma, cell.w_seed)
    ao, bo = ocache.respond_per_query(cols, oracle.expand_seed(seed, P.n), b, cell.keys())
    assert r1 == r2 == oracle.response_bytes(ao, bo, cell.gamma)


def test_refusals(pkg, oracle, ctx):
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 32, 0x12)
    store = pkg.ServerSessionStore.new()
    with pytest.raises(pkg.PirError, match="packing-key material mismatch"):
        store.register_server_side(pkg.ClientPackingKeys(cell.keys()[:2], cell.gamma), cache)
    with pytest.raises(pkg.PirError, match="packing-key width mismatch"):
        store.register_server_side(pkg.ClientPackingKeys(cell.keys(), 32), cache)
    sid, seed, b = cell.next_query(1)
    q = pkg.SeededBatchQuery(sid, seed, b)
    with pytest.raises(pkg.PirError, match="no entry for session_handle"):
        pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(1 << 60), [q]),
                                 cache, store)
    bad = pkg.SeededBatchQuery(7, seed, b)
    with pytest.raises(pkg.PirError, match="shard 7 not found"):
        pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Inline(keys), [q, bad]), cache)
    with pytest.raises(pkg.PirError, match="InspiRING packing width"):
        pkg.ServerInspiringCache.new(pkg.ServerCrs(pkg.InspireParams.d2048(), cell.w_seed, 24))
    h1 = store.register_server_side(keys, cache)
    h2 = store.register_server_side(keys, cache)
    assert h2 > h1 and len(store) == 2


def test_batch_across_many_shards(pkg, oracle, ctx, launch_shape):
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 512, 0x5A5A, entries=2048 * 8)
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new()
    h = store.register_server_side(keys, cache)
    rng = np.random.default_rng(7)
    idx = [int(i) for i in rng.integers(0, 2048 * 8, size=24)]
    qs, raw = [], []
    for i in idx:
        sid, seed, b = cell.next_query(i)
        qs.append(pkg.SeededBatchQuery(sid, seed, b))
        raw.append((sid, seed, b))
    out = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(h), qs), cache, store)
    for k, (i, r) in enumerate(zip(idx, out)):
        assert cell.decode(i, r.a, r.b)[0]
        if k < 6:
            assert r.to_binary() == oracle_bytes(oracle, cell, P, *raw[k])


def test_d256_single_prime_kat_lines_on_gpu(pkg, oracle, ctx, recorded_lines, launch_shape):
    """The reference's d256 single-prime RESP lines (gamma 1, 2, 16, 32 and 128) from the GPU,
    per-query branch and store branch: small and partial scan rows, a one-link and a
    no-link recursion, and the even-log-n transforms."""
    P = oracle.Params(n=256)
    rec = set(recorded_lines)
    for entry in [2, 4, 32, 64, 256]:
        seed = 0x534D4100 + entry
        cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, entry, seed)
        qs = []
        for idx in [0, 255, 256, 511, 700]:
            sid, qseed, b = cell.next_query(idx)
            qs.append((idx, pkg.SeededBatchQuery(sid, qseed, b)))
        for idx, q in qs:
            r = pkg.respond_seeded_inspiring(crs, db, pkg.SeededClientQuery(q.shard_id, q.seed, q.b,
                                                                            inspiring_packing_keys=keys))
            wire = r.to_binary()
            line = f"RESP d256-single-l3 entry={entry} seed={seed:#x} index={idx} len={len(wire)} fnv={oracle.fnv1a(wire):#018x}"
            assert line in rec, line
        db.precompute_packing_all()
        batch = pkg.SeededQueryBatch(pkg.PackingKeySource.Inline(keys), [q for _, q in qs])
        for (idx, _), r in zip(qs, pkg.respond_seeded_batch(crs, db, batch, cache)):
            wire = r.to_binary()
            line = f"RESP d256-single-l3 entry={entry} seed={seed:#x} index={idx} len={len(wire)} fnv={oracle.fnv1a(wire):#018x}"
            assert line in rec, line


def test_one_shard_and_repeated_queries(pkg, oracle, ctx, launch_shape):
    """Collisions: a batch whose queries all name one shard, with the same query repeated,
    answers each query exactly as a batch of one does. An empty batch resolves its key and
    answers nothing, as respond_seeded_batch's map over no queries does (respond.rs:1196-1201):
    an empty list under a registered key, a refusal under an unknown handle."""
    P = oracle.Params.d2048()
    cell, crs, cache, db, keys = gpu_cell(pkg, oracle, P, 256, 0xC011)
    db.precompute_packing_all()
    store = pkg.ServerSessionStore.new()
    h = store.register_server_side(keys, cache)
    src = pkg.PackingKeySource.Registered(h)
    qs = [pkg.SeededBatchQuery(*cell.next_query(P.n + (k * 37) % P.n)) for k in range(12)]
    batch = qs + [qs[3]] * 5 + qs[:3]
    out = pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(src, batch), cache, store)
    alone = {id(q): pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(src, [q]), cache, store)[0].to_binary()
             for q in qs}
    assert [r.to_binary() for r in out] == [alone[id(q)] for q in batch]
    assert pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(src, []), cache, store) == []
    with pytest.raises(pkg.PirError, match="no entry for session_handle"):
        pkg.respond_seeded_batch(crs, db, pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(1 << 60), []), cache,
                                 store)
