"""Minimal reader for the bincode 1.3 (fixint, little-endian) layout the reference's
serde derives produce. Test infrastructure: used only to turn the reference's checked-in
fixtures into the golden files in this directory."""
import struct


class Reader:
    def __init__(self, data: bytes):
        self.b = data
        self.o = 0

    def take(self, n):
        if self.o + n > len(self.b):
            raise ValueError(f"read past end: need {n} at {self.o} of {len(self.b)}")
        v = self.b[self.o:self.o + n]
        self.o += n
        return v

    def u8(self):
        return self.take(1)[0]

    def u32(self):
        return struct.unpack("<I", self.take(4))[0]

    def u64(self):
        return struct.unpack("<Q", self.take(8))[0]

    def f64(self):
        return struct.unpack("<d", self.take(8))[0]

    def vec(self, elem):
        n = self.u64()
        return [elem() for _ in range(n)]

    def done(self):
        return self.o == len(self.b)


def unpack_tight(packed: bytes, moduli, dim):
    """Tight coefficient codec: ceil(log2(max modulus)) bits per value, LSB first
    (src/math/poly.rs:227-284 of the reference)."""
    if not moduli:
        return []
    bits = (max(moduli) - 1).bit_length()
    count = dim * len(moduli)
    whole = int.from_bytes(packed, "little")
    mask = (1 << bits) - 1
    return [(whole >> (i * bits)) & mask for i in range(count)]


def read_poly(r: Reader):
    """`Poly` in its tight (non-human-readable) wire form: TightPolyWire
    {coeffs: bytes, moduli: Vec<u64>, q, dim, crt_q0_inv_mod_q1, is_ntt}."""
    packed = bytes(r.vec(r.u8))
    moduli = r.vec(r.u64)
    q = r.u64()
    dim = r.u64()
    crt_inv = r.u64()
    is_ntt = r.u8()
    coeffs = unpack_tight(packed, moduli, dim)
    return {"coeffs": coeffs, "moduli": moduli, "q": q, "dim": dim,
            "crt_inv": crt_inv, "is_ntt": is_ntt}


def read_rlwe(r):
    return {"a": read_poly(r), "b": read_poly(r)}


def read_gadget(r):
    return {"base": r.u64(), "len": r.u64(), "q": r.u64()}
