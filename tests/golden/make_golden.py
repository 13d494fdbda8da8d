"""Regenerates the golden files in this directory from the reference's checked-in
fixtures (test infrastructure; run where the reference tree is mounted):

    python tests/golden/make_golden.py /path/to/inspire-rs

Outputs (all small, committed):
  d256_respond.npz        the inputs of tests/fixtures/respond_byte_identity_d256.bin
                          (ServerCrs, EncodedDatabase, ClientQuery at d=256, gamma=16),
                          decoded from bincode into plain arrays, plus the golden
                          FNV-1a of the response bytes pinned by
                          tests/respond_byte_identity_kat.rs:109.
  seat_kat_lines.txt      tests/fixtures/packing_seat_response_kat.txt verbatim: the
                          recorded SESSIONKEY/RESP digests of every InspiRING responder.
  special_modulus_pins.txt  the PINNED digests of tests/special_modulus_kat.rs.
  gaussian_stream_pins.txt  the sampler stream hashes of src/math/gaussian.rs.
"""
import os
import re
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from bincode_reader import Reader, read_gadget, read_poly, read_rlwe  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def decode_d256(path):
    r = Reader(open(path, "rb").read())
    params = dict(ring_dim=r.u64(), q=r.u64(), moduli=r.vec(r.u64), p=r.u64(), sigma=r.f64(),
                  gadget_base=r.u64(), query_gadget_len=r.u64(), packing_gadget_len=r.u64(),
                  label=r.u32())
    for _ in range(r.u64()):  # galois keys: rows then gadget
        r.vec(lambda: read_rlwe(r))
        read_gadget(r)
    read_gadget(r)  # rgsw gadget
    w_seed = r.take(32)
    r.take(32)  # v_seed
    num_columns = r.u64()
    shards = r.vec(lambda: (r.u32(), r.vec(lambda: read_poly(r))))
    config = (r.u64(), r.u64(), r.u64())
    shard_id = r.u32()
    rows = r.vec(lambda: read_rlwe(r))
    read_gadget(r)
    packing_mode = r.u32()
    has_keys = r.u8()
    assert has_keys == 1
    y_body = r.vec(lambda: read_poly(r))
    z_body = r.vec(lambda: read_poly(r))
    r.u8()
    key_width = r.u64()
    has_handle = r.u8()
    assert not has_handle and not z_body and packing_mode == 0
    assert r.done(), "fixture not consumed exactly"
    n = params["ring_dim"]
    cols = np.array([p["coeffs"] for p in shards[shard_id][1]], dtype=np.uint64)
    assert cols.shape == (num_columns, n) and key_width == num_columns
    return dict(
        n=n, q=params["q"], p=params["p"], sigma=params["sigma"],
        gadget_base=params["gadget_base"], gadget_len=params["packing_gadget_len"],
        w_seed=np.frombuffer(w_seed, dtype=np.uint8), gamma=num_columns,
        shard_config=np.array(config, dtype=np.uint64), columns=cols,
        query_a=np.array(rows[0]["a"]["coeffs"], dtype=np.uint64),
        query_b=np.array(rows[0]["b"]["coeffs"], dtype=np.uint64),
        y_body=np.array([p["coeffs"] for p in y_body], dtype=np.uint64),
    )


def main(ref):
    fx = os.path.join(ref, "tests", "fixtures")
    d = decode_d256(os.path.join(fx, "respond_byte_identity_d256.bin"))
    kat_src = open(os.path.join(ref, "tests", "respond_byte_identity_kat.rs")).read()
    golden = int(re.search(r"GOLDEN_FNV1A: u64 = (0x[0-9a-f_]+);", kat_src).group(1).replace("_", ""), 16)
    np.savez_compressed(os.path.join(HERE, "d256_respond.npz"), golden_fnv=np.uint64(golden),
                        **{k: (np.array(v) if not isinstance(v, np.ndarray) else v) for k, v in d.items()})
    with open(os.path.join(fx, "packing_seat_response_kat.txt")) as f, \
            open(os.path.join(HERE, "seat_kat_lines.txt"), "w") as g:
        g.write(f.read())
    sm = open(os.path.join(ref, "tests", "special_modulus_kat.rs")).read()
    m = re.search(r"const PINNED: \[u64; 3\] = \[(.*?)\];", sm, re.S)
    pins = [x.strip().rstrip(",").replace("_", "") for x in m.group(1).split(",") if x.strip()]
    with open(os.path.join(HERE, "special_modulus_pins.txt"), "w") as g:
        g.write("key {}\nquery {}\nresponse {}\n".format(*pins))
    ga = open(os.path.join(ref, "src", "math", "gaussian.rs")).read()
    with open(os.path.join(HERE, "gaussian_stream_pins.txt"), "w") as g:
        for s, seed, want in re.findall(r"\(([0-9.]+), (\d+), (0x[0-9a-f_]+)\)", ga):
            g.write(f"{s} {seed} {want.replace('_', '')}\n")
    print("golden files written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
