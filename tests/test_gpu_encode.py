"""encode_database on the GPU (ig_db_encode_records): entries split into shards of ring_dim
rows and 16-bit little-endian columns, written straight into HBM. A database encoded from a
KAT cell's records must answer the reference's recorded bytes; an odd entry size with a
partial last shard must match the same split done on the host."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def host_columns(records: bytes, entry_size: int, n: int, shards: int):
    """encode_db.rs:74-168 restated: column j of row k is bytes 2j, 2j+1 of entry k."""
    gamma = max(1, (entry_size + 1) // 2)
    entries = len(records) // entry_size
    out = np.zeros((shards, gamma, n), dtype=np.uint64)
    raw = np.frombuffer(records[:entries * entry_size], dtype=np.uint8).reshape(entries, entry_size)
    for e in range(entries):
        s, k = divmod(e, n)
        for j in range(gamma):
            lo = raw[e, 2 * j] if 2 * j < entry_size else 0
            hi = raw[e, 2 * j + 1] if 2 * j + 1 < entry_size else 0
            out[s, j, k] = int(lo) | (int(hi) << 8)
    return out


def test_kat_cell_from_records(pkg, oracle, recorded_lines):
    P = oracle.Params.d2048()
    entry, seed = 256, 0x52455300
    cell = oracle.Cell(P, entry, seed)
    records = b"".join(cell.record(i) for i in range(cell.num_shards * P.n))
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), cell.w_seed, cell.gamma)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase.from_records(cache, records, entry)
    assert db.num_shards == cell.num_shards
    db.precompute_packing_all()
    keys = pkg.ClientPackingKeys(cell.keys(), cell.gamma)
    rec = set(recorded_lines)
    n = P.n
    for idx in [0, 1, n - 1, n, 2 * n + 17, 3 * n - 1]:
        sid, qseed, b = cell.next_query(idx)
        r = pkg.respond_seeded_inspiring(crs, db, pkg.SeededClientQuery(sid, qseed, b, inspiring_packing_keys=keys))
        wire = r.to_binary()
        line = f"RESP d2048 entry={entry} seed={seed:#x} index={idx} len={len(wire)} fnv={oracle.fnv1a(wire):#018x}"
        assert line in rec, line


def test_odd_entry_partial_shard_matches_host_split(pkg, oracle):
    torch = pytest.importorskip("torch")
    P = oracle.Params(n=256)
    n, entry = P.n, 7  # four columns, the last holding one byte
    rng = np.random.default_rng(7)
    records = rng.integers(0, 256, size=(5 * n // 2) * entry, dtype=np.uint8).tobytes()  # 2.5 shards
    w_seed = bytes(range(32))
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=n, p=P.p), w_seed, 4)
    cache = pkg.ServerInspiringCache.new(crs)
    host = host_columns(records, entry, n, 3)
    ref_db = pkg.EncodedDatabase.from_columns(cache, list(host))
    gpu_db = pkg.EncodedDatabase.from_records(cache, records, entry)
    dev_db = pkg.EncodedDatabase(cache, 3)
    d_rec = torch.from_numpy(np.frombuffer(records, dtype=np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    dev_db.encode_records(None, entry, device_ptr=d_rec.data_ptr(), nbytes=len(records))
    keys = pkg.ClientPackingKeys(rng.integers(0, pkg.DEFAULT_Q, size=(3, n), dtype=np.uint64), 4)
    for db in (ref_db, gpu_db, dev_db):
        db.precompute_packing_all()
    for sid in range(3):
        seed = bytes(rng.integers(0, 256, 32, dtype=np.uint8))
        b = rng.integers(0, pkg.DEFAULT_Q, n, dtype=np.uint64)
        q = pkg.SeededClientQuery(sid, seed, b, inspiring_packing_keys=keys)
        want = pkg.respond_seeded_inspiring(crs, ref_db, q).to_binary()
        assert pkg.respond_seeded_inspiring(crs, gpu_db, q).to_binary() == want
        assert pkg.respond_seeded_inspiring(crs, dev_db, q).to_binary() == want
    # The store of a GPU-encoded shard equals the one built from the host split.
    assert (gpu_db.store_sums(2) == ref_db.store_sums(2)).all()


def test_encode_refusals(pkg, oracle):
    P = oracle.Params(n=256)
    crs = pkg.ServerCrs(pkg.InspireParams(ring_dim=P.n, p=P.p), bytes(32), 4)
    cache = pkg.ServerInspiringCache.new(crs)
    db = pkg.EncodedDatabase(cache, 1)
    with pytest.raises(pkg.PirError, match="columns") as e:
        db.encode_records(bytes(16 * 256), 16)  # 8 columns against gamma 4
    assert e.value.code == 3
    with pytest.raises(pkg.PirError, match="shards"):
        db.encode_records(bytes(8 * 300), 8)  # 300 entries need 2 shards
