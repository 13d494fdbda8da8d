"""GPU parity of the special_modulus path against the CPU oracle and the reference's
PINNED wire digests (tests/special_modulus_kat.rs:349-380). Bit-exact (32-bit integer
arithmetic mod q and p)."""
import os

import numpy as np
import pytest

from conftest import ROOT, load_package

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def sm():
    return load_package().special_modulus


def test_pinned_wire_digests_on_gpu(sm, oracle):
    pins = dict(line.split() for line in open(os.path.join(GOLDEN, "special_modulus_pins.txt")))
    client = oracle.SmClient(bytes([42] * 32))
    cells = oracle.sm_kat_cells(42, 2048)
    server = sm.Server()
    table = server.table(cells)
    ms, kq, kp = client.key()
    seat = server.seat(sm.PackingKey(ms, kq, kp))
    assert oracle.fnv1a(client.key_bytes()) == int(pins["key"], 16)
    seed, body = client.query(1234)
    assert oracle.fnv1a(oracle.sm_query_bytes(seed, body)) == int(pins["query"], 16)
    resp = server.respond(table, seat, sm.Query(seed, body))
    wire = resp.to_bytes()
    assert len(wire) == 9_208
    assert oracle.fnv1a(wire) == int(pins["response"], 16)
    assert client.decode(resp.mask, resp.body) == cells[1234 * 256:1234 * 256 + 246]
    # The device table holds the reference's step-1 words (Montgomery form) exactly.
    ost = oracle.SmServer().table(cells)
    assert (server.table_step1(table) == ost.step1()).all()


def test_mixed_batch_matches_oracle(sm, oracle):
    """Several shards (one partial), several seated keys, one batch."""
    server = sm.Server()
    oserver = oracle.SmServer()
    rng = np.random.default_rng(3)
    shard_cells = []
    for rows in (2048, 2048, 700):
        c = np.zeros((rows, 256), dtype=np.uint8)
        c[:, :246] = rng.integers(0, 256, (rows, 246), dtype=np.uint8)
        shard_cells.append(c.tobytes())
    tables = [server.table(c) for c in shard_cells]
    otables = [oserver.table(c) for c in shard_cells]
    clients = [oracle.SmClient(bytes([s] * 32)) for s in (1, 2, 3)]
    seats = [server.seat(sm.PackingKey(*cl.key())) for cl in clients]
    oseats = [oserver.seat(cl.key()) for cl in clients]
    qs, meta = [], []
    for k in range(12):
        t, s = k % 3, (k * 7) % 3
        row = int(rng.integers(0, 2048))
        seed, body = clients[s].query(row)
        qs.append(sm.Query(seed, body))
        meta.append((t, s, row, seed, body))
    out = server.respond_batch([tables[m[0]] for m in meta], [seats[m[1]] for m in meta], qs)
    for (t, s, row, seed, body), r in zip(meta, out):
        mask, obody = oserver.respond(otables[t], oseats[s], seed, body)
        assert (r.mask == mask).all() and (r.body == obody).all()
        rec = clients[s].decode(r.mask, r.body)
        want = shard_cells[t][row * 256:row * 256 + 246] if row * 256 < len(shard_cells[t]) else bytes(246)
        assert rec == want


def test_refusals(sm, oracle):
    server = sm.Server()
    bad = bytearray(256)
    bad[250] = 1
    with pytest.raises(load_package().PirError, match="bytes past its 246-byte record"):
        server.table(bytes(bad))
    with pytest.raises(load_package().PirError, match="not at most"):
        server.table(bytes(300))
    ms, kq, kp = oracle.SmClient(bytes([9] * 32)).key()
    kq2 = kq.copy()
    kq2[5] = sm.Params().q
    with pytest.raises(load_package().PirError, match="not a residue"):
        server.seat(sm.PackingKey(ms, kq2, kp))
    seat = server.seat(sm.PackingKey(ms, kq, kp))
    table = server.table(bytes(256))
    body = np.zeros(2048, dtype=np.uint32)
    body[0] = sm.Params().q
    with pytest.raises(load_package().PirError, match="does not fit the set"):
        server.respond(table, seat, sm.Query(bytes(32), body))
    with pytest.raises(load_package().PirError, match="ring dimension"):
        sm.Server(sm.Params(ring_dim=1024, gamma=256, cell_bytes=128, record_bytes=120))


def test_concurrent_callers_over_lanes(oracle):
    """Server::respond from three threads over three lanes equals the one-lane answers."""
    import threading
    pkg = load_package()
    ctx = pkg.Context.default()
    sm = pkg.special_modulus
    server = sm.Server(ctx=ctx)
    rng = np.random.default_rng(31)
    cells = np.zeros((2048, 256), dtype=np.uint8)
    cells[:, :246] = rng.integers(0, 256, (2048, 246), dtype=np.uint8)
    table = server.table(cells.tobytes())
    seat = server.seat(sm.PackingKey(rng.bytes(32), rng.integers(0, 536_813_569, 2048, dtype=np.uint32),
                                     rng.integers(0, 2_147_389_441, 2048, dtype=np.uint32)))
    batches = [[sm.Query(rng.bytes(32), rng.integers(0, 536_813_569, 2048, dtype=np.uint32)) for _ in range(4)]
               for _ in range(6)]
    want = [[r.to_bytes() for r in server.respond_batch([table] * 4, [seat] * 4, b)] for b in batches]
    got = [None] * len(batches)
    errors = []
    ctx.set_lanes(3)
    try:
        def caller(t):
            try:
                for j in range(t, len(batches), 3):
                    got[j] = [r.to_bytes() for r in server.respond_batch([table] * 4, [seat] * 4, batches[j])]
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


@pytest.mark.parametrize("q", [536_903_681, 1_073_750_017])
def test_other_ciphertext_primes_match_oracle(oracle, q):
    """Ciphertext primes at or above 2^29 leave no room for the kernel's unreduced q-limb
    values (below 8q), so they take the fully reduced passes; the answers equal the oracle's
    over the same prime and decode to the record."""
    pkg = load_package()
    sm = pkg.special_modulus
    server = sm.Server(sm.Params(q=q))
    oserver = oracle.SmServer(q=q)
    rng = np.random.default_rng(q % 1000)
    cells = np.zeros((2048, 256), dtype=np.uint8)
    cells[:, :246] = rng.integers(0, 256, (2048, 246), dtype=np.uint8)
    table, otable = server.table(cells.tobytes()), oserver.table(cells.tobytes())
    client = oracle.SmClient(bytes([77] * 32), q=q)
    seat, oseat = server.seat(sm.PackingKey(*client.key())), oserver.seat(client.key())
    rows = [0, 1, 1000, 2047]
    qs = [client.query(r) for r in rows]
    out = server.respond_batch([table] * len(rows), [seat] * len(rows), [sm.Query(s, b) for s, b in qs])
    for row, (seed, body), r in zip(rows, qs, out):
        mask, obody = oserver.respond(otable, oseat, seed, body)
        assert (r.mask == mask).all() and (r.body == obody).all(), row
        assert client.decode(r.mask, r.body) == cells[row, :246].tobytes()
