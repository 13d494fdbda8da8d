"""The RIMS codec (encode_response_packed / decode_response_packed, mod_switch.rs:254-521)
on the host: the frame lengths the reference pins (11,543 B at the 36-bit switch and
13,847 B at 45 bits for gamma 256, mod_switch.rs:800-816 and 978-987), its legacy-frame
and malformed-frame refusals (818-879), and byte equality with the oracle's restatement
for packed and unpacked responses."""
import numpy as np
import pytest

from conftest import load_package


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def test_pinned_frame_lengths(pkg):
    n = 2048
    zero = np.zeros(n, dtype=np.uint64)
    r45 = pkg.ServerResponse(zero, zero, 256, pkg.MOD_SWITCH_TARGET_45BIT)
    assert len(r45.to_rims()) == 13_847
    ms = pkg.MOD_SWITCH_TARGET_36BIT
    rng = np.random.default_rng(5)
    a, b = (rng.integers(0, ms, n, dtype=np.uint64) for _ in range(2))
    r36 = pkg.ServerResponse(a, b, 256, ms)
    rims = r36.to_rims()
    assert len(rims) == 11_543 and len(r36.to_binary()) == 10_446 < len(rims)
    back = pkg.ServerResponse.from_rims(rims)
    assert back.modulus == ms and back.packed_coefficients == 256 and back.packing_mode == "Inspiring"
    assert (back.a == a).all() and (back.b[:256] == b[:256]).all() and not back.b[256:].any()


def test_legacy_v1_frame_is_refused(pkg):
    frame = bytearray(b"RIMS") + bytes([1]) + (257).to_bytes(8, "little") + (2).to_bytes(4, "little")
    frame += bytes([2, 0]) + (0).to_bytes(4, "little") + bytes([1, 0, 2, 0, 3, 0, 4, 0])
    with pytest.raises(pkg.PirError, match="unsupported version 1"):
        pkg.ServerResponse.from_rims(bytes(frame))
    frame[4] = 2
    r = pkg.ServerResponse.from_rims(bytes(frame))
    assert r.packing_mode is None and r.column_ciphertexts == []
    assert list(r.a) == [1, 2] and list(r.b) == [3, 4]


def test_malformed_frames_are_refused(pkg):
    valid = bytearray(pkg.ServerResponse(np.zeros(2, np.uint64), np.zeros(2, np.uint64), 1, 257).to_rims())
    assert pkg.ServerResponse.from_rims(bytes(valid)).packed_coefficients == 1
    cases = {}

    def case(name, edit):
        x = bytearray(valid)
        edit(x)
        cases[name] = bytes(x)

    case("version", lambda x: x.__setitem__(4, 1))
    case("modulus", lambda x: x.__setitem__(slice(5, 13), bytes(8)))
    case("ring_dim", lambda x: x.__setitem__(slice(13, 17), bytes(4)))
    case("width", lambda x: x.__setitem__(17, 1))
    case("zero retained", lambda x: x.__setitem__(slice(19, 23), bytes(4)))
    case("excess retained", lambda x: x.__setitem__(slice(19, 23), (3).to_bytes(4, "little")))
    case("truncated", lambda x: x.pop())
    case("trailing", lambda x: x.append(0))
    case("non-canonical", lambda x: x.__setitem__(slice(23, 25), (257).to_bytes(2, "little")))
    case("mode", lambda x: x.__setitem__(18, 3))
    case("magic", lambda x: x.__setitem__(0, ord("X")))
    messages = {
        "version": "unsupported version", "modulus": "must be positive", "ring_dim": "must be positive",
        "width": "does not match modulus width", "zero retained": "outside 1..=2", "excess retained": "outside 1..=2",
        "truncated": "payload length mismatch", "trailing": "payload length mismatch",
        "non-canonical": "not canonical for modulus 257", "mode": "unknown packing_mode byte 3",
        "magic": "bad magic",
    }
    for name, frame in cases.items():
        with pytest.raises(pkg.PirError, match=messages[name]):
            pkg.ServerResponse.from_rims(frame)
    with pytest.raises(pkg.PirError, match="bad magic"):
        pkg.ServerResponse.from_rims(b"RIMS")


def test_frames_equal_the_oracle_restatement(pkg, oracle):
    rng = np.random.default_rng(11)
    q = pkg.DEFAULT_Q
    for n, retained, modulus in [(2048, 16, q), (2048, 256, pkg.MOD_SWITCH_TARGET_36BIT), (256, 256, 257)]:
        a, b = (rng.integers(0, modulus, n, dtype=np.uint64) for _ in range(2))
        got = pkg.ServerResponse(a, b, retained, modulus).to_rims()
        assert got == oracle.rims_bytes(a, b, modulus, retained)
    # Unpacked (NoPacking): b whole and the column ciphertexts.
    n = 256
    cols = [tuple(rng.integers(0, q, n, dtype=np.uint64) for _ in range(2)) for _ in range(3)]
    a, b = (rng.integers(0, q, n, dtype=np.uint64) for _ in range(2))
    r = pkg.ServerResponse(a, b, None, q, cols)
    frame = r.to_rims()
    assert frame == oracle.rims_bytes(a, b, q, columns=cols)
    back = pkg.ServerResponse.from_rims(frame)
    assert back.packing_mode is None and back.packed_coefficients is None and len(back.column_ciphertexts) == 3
    assert all((x == y).all() and (u == v).all() for (x, u), (y, v) in zip(back.column_ciphertexts, cols))
    assert (back.a == a).all() and (back.b == b).all()
    # A tree-mode frame decodes with its mode (the reference's tree responder writes byte 2).
    tree = bytearray(pkg.ServerResponse(a, b, 8, q).to_rims())
    tree[18] = 2
    assert pkg.ServerResponse.from_rims(bytes(tree)).packing_mode == "Tree"


def test_non_canonical_coefficient_is_refused(pkg):
    a = np.zeros(16, dtype=np.uint64)
    b = a.copy()
    b[3] = 257
    with pytest.raises(pkg.PirError):
        pkg.ServerResponse(a, b, 4, 257).to_rims()
