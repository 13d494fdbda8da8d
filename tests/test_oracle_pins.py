"""Pins the CPU oracle to the reference's own golden vectors before it is trusted as the
checker for the GPU path: sampler stream hashes (src/math/gaussian.rs:335-351), the d=256
respond fixture (tests/respond_byte_identity_kat.rs:109) and the recorded seat KAT lines
(tests/packing_seat_byte_identity_kat.rs:162-229)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_gaussian_stream_hashes(oracle):
    pins = [line.split() for line in open(os.path.join(GOLDEN, "gaussian_stream_pins.txt"))]
    assert len(pins) == 5
    for sigma, seed, want in pins:
        assert oracle.gaussian_stream_fnv(float(sigma), int(seed), 200_000) == int(want, 16)


def _d256(oracle):
    d = np.load(os.path.join(GOLDEN, "d256_respond.npz"))
    P = oracle.Params(n=int(d["n"]), q=int(d["q"]), p=int(d["p"]), sigma=float(d["sigma"]),
                      gadget_base=int(d["gadget_base"]), gadget_len=int(d["gadget_len"]))
    return d, P


def test_d256_fixture_per_query_and_store(oracle):
    d, P = _d256(oracle)
    cache = oracle.Cache(P, int(d["gamma"]), d["w_seed"].tobytes())
    a, b = cache.respond_per_query(d["columns"], d["query_a"], d["query_b"], d["y_body"])
    resp = oracle.response_bytes(a, b, int(d["gamma"]), P.q)
    assert oracle.fnv1a(resp) == int(d["golden_fnv"]) == 0x796A80CA60D31A52
    store = oracle.Store(cache, d["columns"])
    a2, b2 = store.respond(d["columns"], d["query_a"], d["query_b"], d["y_body"])
    assert (a2 == a).all() and (b2 == b).all()


def test_store_refuses_edited_column(oracle):
    d, P = _d256(oracle)
    cache = oracle.Cache(P, int(d["gamma"]), d["w_seed"].tobytes())
    store = oracle.Store(cache, d["columns"])
    edited = d["columns"].copy()
    edited[3, 17] ^= 1
    with pytest.raises(ValueError):
        store.respond(edited, d["query_a"], d["query_b"], d["y_body"])


def _replay(oracle, tag, P, entry, seed, indices, store_path):
    cell = oracle.Cell(P, entry, seed)
    kb = cell.key_bytes()
    lines = [f"SESSIONKEY {tag} entry={entry} seed={seed:#x} len={len(kb)} fnv={oracle.fnv1a(kb):#018x}"]
    cache = oracle.Cache(P, cell.gamma, cell.w_seed)
    stores = {}
    y = cell.keys()
    for idx in indices:
        sid, qseed, b = cell.next_query(idx)
        a = oracle.expand_seed(qseed, P.n, P.q)
        cols = cell.columns(sid)
        if store_path:
            if sid not in stores:
                stores[sid] = oracle.Store(cache, cols)
            ao, bo = stores[sid].respond(cols, a, b, y)
        else:
            ao, bo = cache.respond_per_query(cols, a, b, y)
        ok, _ = cell.decode(idx, ao, bo)
        assert ok, f"{tag} entry={entry} index {idx} decoded to another record"
        r = oracle.response_bytes(ao, bo, cell.gamma, P.q)
        lines.append(f"RESP {tag} entry={entry} seed={seed:#x} index={idx} len={len(r)} fnv={oracle.fnv1a(r):#018x}")
    return lines


D2048_CELLS = [(32, 0x52455300), (32, 0x52455301), (256, 0x52455300), (256, 0x52455301),
               (512, 0x52455300), (512, 0x52455301), (1024, 0x52455300)]


@pytest.mark.parametrize("store_path", [False, True], ids=["per_query", "store"])
def test_d2048_seat_kat_lines(oracle, recorded_lines, store_path):
    P = oracle.Params.d2048()
    d = P.n
    served = []
    for entry, seed in D2048_CELLS:
        served += _replay(oracle, "d2048", P, entry, seed, [0, 1, d - 1, d, 2 * d + 17, 3 * d - 1], store_path)
    rec = set(recorded_lines)
    missing = [line for line in served if line not in rec]
    assert not missing, missing[:3]
    assert len(served) == sum(1 for line in recorded_lines if line.split(" ")[1] == "d2048")


@pytest.mark.parametrize("store_path", [False, True], ids=["per_query", "store"])
def test_d256_single_prime_seat_kat_lines(oracle, recorded_lines, store_path):
    P = oracle.Params(n=256)
    served = []
    for entry in [2, 4, 32, 64, 256]:
        served += _replay(oracle, "d256-single-l3", P, entry, 0x534D4100 + entry, [0, 255, 256, 511, 700], store_path)
    rec = set(recorded_lines)
    missing = [line for line in served if line not in rec]
    assert not missing, missing[:3]
    assert len(served) == sum(1 for line in recorded_lines if line.split(" ")[1] == "d256-single-l3")


def test_approximate_gadget_paths_agree_and_decode(oracle):
    """No byte golden exists for the approximate gadget (the reference checks cross-path
    equality and decode only, tests/approximate_packing_gadget.rs)."""
    P = oracle.Params.d2048_approximate_gadget()
    cell = oracle.Cell(P, 64, 0xA9)
    assert cell.key_rows == 2 and len(cell.key_bytes()) == 8 + 2 * 15409 + 8 + 1 + 8
    cache = oracle.Cache(P, cell.gamma, cell.w_seed)
    y = cell.keys()
    for idx in [5, 2048 + 700]:
        sid, qseed, b = cell.next_query(idx)
        a = oracle.expand_seed(qseed, P.n)
        cols = cell.columns(sid)
        a1, b1 = cache.respond_per_query(cols, a, b, y)
        a2, b2 = oracle.Store(cache, cols).respond(cols, a, b, y)
        assert (a1 == a2).all() and (b1 == b2).all()
        assert cell.decode(idx, a1, b1)[0]


def test_mod_switched_response_size(oracle):
    """36-bit mod switch: 10,446 bytes at 512-byte records (src/pir/mod_switch.rs:985)."""
    P = oracle.Params.d2048()
    a = np.arange(P.n, dtype=np.uint64) * 7919 % P.q
    b = np.arange(P.n, dtype=np.uint64) * 104729 % P.q
    t = oracle.MOD_SWITCH_TARGET_36BIT
    ms_a, ms_b = oracle.mod_switch(a), oracle.mod_switch(b)
    assert (ms_a < t).all()
    assert len(oracle.response_bytes(ms_a, ms_b, 256, t)) == 10_446
    # c' = floor((c*q' + floor(q/2)) / q) mod q'
    for c in [0, 1, P.q // 2, P.q - 1, 123456789123]:
        want = ((c * t + P.q // 2) // P.q) % t
        assert int(oracle.mod_switch(np.array([c], dtype=np.uint64))[0]) == want


def test_special_modulus_pinned_wire_digests(oracle):
    """tests/special_modulus_kat.rs:349-380: Client::from_seed([42; 32]), 2048 cells from
    seed_from_u64(42), row 1234 — key, query and response bytes pinned by FNV-1a."""
    pins = dict(line.split() for line in open(os.path.join(GOLDEN, "special_modulus_pins.txt")))
    client = oracle.SmClient(bytes([42] * 32))
    server = oracle.SmServer()
    cells = oracle.sm_kat_cells(42, 2048)
    table = server.table(cells)
    seat = server.seat(client.key())
    kb = client.key_bytes()
    seed, body = client.query(1234)
    qb = oracle.sm_query_bytes(seed, body)
    mask, rbody = server.respond(table, seat, seed, body)
    rb = oracle.sm_response_bytes(mask, rbody)
    assert (len(kb), len(qb), len(rb)) == (15_394, 7_456, 9_208)
    assert oracle.fnv1a(kb) == int(pins["key"], 16)
    assert oracle.fnv1a(qb) == int(pins["query"], 16)
    assert oracle.fnv1a(rb) == int(pins["response"], 16)
    assert client.decode(mask, rbody) == cells[1234 * 256:1234 * 256 + 246]


def test_nopacking_restatement_decodes(oracle):
    """The oracle's NoPacking respond (respond.rs:614-643) decodes, through the reference's
    unpacked extract, to the requested record, and its sum ciphertext is the column sum."""
    from nopacking_decode import extract
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 32, 0x52455300)
    cache = oracle.Cache(P, cell.gamma, cell.w_seed)
    secret = cell.secret()
    for idx in [0, 1, P.n + 7]:
        sid, seed, b = cell.next_query(idx)
        out = cache.respond_nopacking(cell.columns(sid), oracle.expand_seed(seed, P.n), b)
        assert (out[1:].astype(object).sum(axis=0) % P.q == out[0].astype(object)).all()
        rec = extract([(out[j, 0], out[j, 1]) for j in range(1, cell.gamma + 1)], secret, P.q, P.p, 32)
        assert rec == cell.record(idx), idx
        wire = oracle.response_bytes_full(out)
        bits = 60
        poly = 8 + (P.n * bits + 7) // 8 + 41
        assert len(wire) == 4 + 2 * poly + 8 + cell.gamma * 2 * poly + 1


def test_tree_restatement_decodes(oracle):
    """The oracle's OnePacking respond (respond.rs:696-729, the automorphism tree of
    automorph_pack.rs) under test Galois keys of the cell's secret decodes, through
    extract_packed's d^-1 scaling (extract.rs:184-226), to the requested record; the tree
    response's wire is the packed one with packing_mode Some(Tree)."""
    P = oracle.Params(n=256)
    cell = oracle.Cell(P, 16, 0x7EE0)
    keys = cell.galois_keys(bytes(range(32)))
    assert keys.shape == (8, 3, 2, P.n)
    cache = oracle.Cache(P, cell.gamma, cell.w_seed)
    for idx in [0, 5, P.n + 3]:
        sid, seed, b = cell.next_query(idx)
        ao, bo = cache.respond_one_packing(cell.columns(sid), oracle.expand_seed(seed, P.n), b, keys)
        ok, rec = cell.decode_tree(idx, ao, bo)
        assert ok and rec == cell.record(idx), idx
        packed = oracle.response_bytes(ao, bo, cell.gamma)
        tree = oracle.response_bytes_tree(ao, bo, cell.gamma)
        assert tree[:-4] == packed[:-4] and packed[-4:] == bytes(4) and tree[-4:] == bytes([1, 0, 0, 0])


def test_plain_method_cell_round_trips(oracle):
    """The plain method's inputs (2048 uniform records of 32 bytes from seed 0, the seeded
    setup and session, a uniform index) through the oracle's uncached respond: extract
    returns the record."""
    P = oracle.Params.d2048()
    cell = oracle.Cell(P, 32, 0, entries=2048, plain=True)
    assert (cell.gamma, cell.num_shards) == (16, 1)
    index = cell.draw_index(2048)
    assert 0 <= index < 2048
    sid, seed, b = cell.next_query(index)
    assert sid == 0
    ao, bo = oracle.Cache(P, cell.gamma, cell.w_seed).respond_per_query(
        cell.columns(0), oracle.expand_seed(seed, P.n), b, cell.keys())
    ok, record = cell.decode(index, ao, bo)
    assert ok and record == cell.record(index)
    assert len(set(cell.database())) > 200  # uniform bytes, not the fixture's formula
