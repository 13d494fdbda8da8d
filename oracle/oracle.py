"""ctypes front of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module, as the
checker and the timed CPU baseline. The product package never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

DEFAULT_Q = 1152921504606830593
MOD_SWITCH_TARGET_36BIT = 68_718_428_161

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        V, P, U64, I = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        sig = {
            "orc_last_error": (ctypes.c_char_p, []),
            "orc_set_threads": (None, [I]),
            "orc_max_threads": (I, []),
            "orc_fnv1a": (U64, [P, U64]),
            "orc_gaussian_stream_fnv": (U64, [ctypes.c_double, U64, U64]),
            "orc_expand_seed": (None, [P, U64, U64, P]),
            "orc_chacha_u64s": (None, [P, U64, U64, P]),
            "orc_ntt_forward": (I, [U64, U64, P]),
            "orc_ntt_inverse": (I, [U64, U64, P]),
            "orc_cache_new": (V, [U64, U64, U64, ctypes.c_double, U64, U64, I, U64, P]),
            "orc_cache_free": (None, [V]),
            "orc_cache_tables": (None, [V, P]),
            "orc_cache_w_all_ntt": (None, [V, P]),
            "orc_respond_per_query": (I, [V, P, P, P, P, P, P]),
            "orc_respond_nopacking": (I, [V, P, P, P, P]),
            "orc_response_bytes_full": (U64, [P, U64, U64, U64, P, U64]),
            "orc_store_build": (V, [V, P, U64]),
            "orc_store_free": (None, [V]),
            "orc_store_sums": (None, [V, V, P]),
            "orc_respond_store": (I, [V, V, P, P, P, P, P, P]),
            "orc_store_scan": (I, [V, V, P, P, P]),
            "orc_mod_switch": (None, [P, U64, U64, U64, P]),
            "orc_response_bytes": (U64, [P, P, U64, U64, U64, P, U64]),
            "orc_response_bytes_tree": (U64, [P, P, U64, U64, U64, P, U64]),
            "orc_respond_one_packing": (I, [V, P, P, P, P, U64, P, P]),
            "orc_cell_galois_keys": (None, [V, P, P]),
            "orc_cell_decode_tree": (I, [V, U64, P, P, P]),
            "orc_cell_sampler_state": (None, [V, P, P]),
            "orc_cell_db": (U64, [V, P, U64]),
            "orc_cell_build": (V, [U64, U64, U64, ctypes.c_double, U64, U64, I, U64, U64, U64]),
            "orc_cell_build_seeded": (V, [U64, U64, U64, ctypes.c_double, U64, U64, I, U64, U64, U64]),
            "orc_cell_draw_index": (U64, [V, U64]),
            "orc_cell_free": (None, [V]),
            "orc_cell_info": (None, [V, P, P, P, P]),
            "orc_cell_columns": (None, [V, U64, P]),
            "orc_cell_keys": (None, [V, P]),
            "orc_cell_secret": (None, [V, P]),
            "orc_cell_key_bytes": (U64, [V, P, U64]),
            "orc_cell_next_query": (None, [V, U64, P, P, P]),
            "orc_cell_decode": (I, [V, U64, P, P, P]),
            "orc_cell_record": (None, [V, U64, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fnv1a(b: bytes) -> int:
    arr = np.frombuffer(b, dtype=np.uint8)
    return lib().orc_fnv1a(_p(arr), len(b))


class Params:
    """Single-prime InspireParams (params.rs:137-196 of the reference)."""

    def __init__(self, n=2048, q=DEFAULT_Q, p=65537, sigma=6.4, gadget_base=1 << 20, gadget_len=3,
                 approx=False):
        self.n, self.q, self.p, self.sigma = n, q, p, sigma
        self.gadget_base, self.gadget_len, self.approx = gadget_base, gadget_len, approx

    @property
    def key_rows(self):
        return self.gadget_len - (1 if self.approx else 0)

    def args(self):
        return (self.n, self.q, self.p, self.sigma, self.gadget_base, self.gadget_len, int(self.approx))

    @staticmethod
    def d2048():
        return Params()

    @staticmethod
    def d2048_approximate_gadget():
        return Params(approx=True)


class Cache:
    """PackParams + OfflinePackingKeys for (params, gamma, w_seed)."""

    def __init__(self, params: Params, gamma: int, w_seed: bytes):
        self.params, self.gamma = params, gamma
        seed = np.frombuffer(bytes(w_seed), dtype=np.uint8).copy()
        self.h = lib().orc_cache_new(*params.args(), gamma, _p(seed))
        if not self.h:
            raise RuntimeError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cache_free(self.h)

    def tables(self):
        out = np.zeros((self.gamma, self.params.n), dtype=np.uint32)
        lib().orc_cache_tables(self.h, _p(out))
        return out

    def w_all_ntt(self):
        out = np.zeros((self.gamma - 1, self.params.key_rows, self.params.n), dtype=np.uint64)
        lib().orc_cache_w_all_ntt(self.h, _p(out))
        return out

    def respond_per_query(self, columns, a, b, y_body):
        n = self.params.n
        columns = np.ascontiguousarray(columns, dtype=np.uint64)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        y = np.ascontiguousarray(y_body, dtype=np.uint64)
        ao = np.zeros(n, dtype=np.uint64)
        bo = np.zeros(n, dtype=np.uint64)
        rc = lib().orc_respond_per_query(self.h, _p(columns), _p(a), _p(b), _p(y), _p(ao), _p(bo))
        if rc:
            raise RuntimeError(lib().orc_last_error().decode())
        return ao, bo

    def respond_nopacking(self, columns, a, b):
        """respond (respond.rs:614-643): (gamma + 1) x 2 x n words, the column sum first."""
        n, g = self.params.n, self.gamma
        columns = np.ascontiguousarray(columns, dtype=np.uint64)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        out = np.zeros((g + 1, 2, n), dtype=np.uint64)
        if lib().orc_respond_nopacking(self.h, _p(columns), _p(a), _p(b), _p(out)):
            raise RuntimeError(lib().orc_last_error().decode())
        return out


    def respond_one_packing(self, columns, a, b, galois_keys):
        """respond_one_packing (respond.rs:696-729): the Galois-automorphism tree over the
        column LWEs; galois_keys is (log d, rows, 2, n) in coefficient form."""
        n = self.params.n
        columns = np.ascontiguousarray(columns, dtype=np.uint64)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        keys = np.ascontiguousarray(galois_keys, dtype=np.uint64)
        ao = np.zeros(n, dtype=np.uint64)
        bo = np.zeros(n, dtype=np.uint64)
        if lib().orc_respond_one_packing(self.h, _p(columns), _p(a), _p(b), _p(keys), keys.shape[0], _p(ao), _p(bo)):
            raise RuntimeError(lib().orc_last_error().decode())
        return ao, bo


class Store:
    """ShardPackingStore restated: step-1 sums + tags over one shard's columns."""

    def __init__(self, cache: Cache, columns, key_seed=0x7A6):
        self.cache = cache
        cols = np.ascontiguousarray(columns, dtype=np.uint64)
        self.h = lib().orc_store_build(cache.h, _p(cols), key_seed)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_store_free(self.h)

    def sums(self):
        out = np.zeros((self.cache.gamma, self.cache.params.n), dtype=np.uint64)
        lib().orc_store_sums(self.cache.h, self.h, _p(out))
        return out

    def respond(self, columns, a, b, y_body):
        n = self.cache.params.n
        cols = np.ascontiguousarray(columns, dtype=np.uint64)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        y = np.ascontiguousarray(y_body, dtype=np.uint64)
        ao = np.zeros(n, dtype=np.uint64)
        bo = np.zeros(n, dtype=np.uint64)
        rc = lib().orc_respond_store(self.cache.h, self.h, _p(cols), _p(a), _p(b), _p(y), _p(ao), _p(bo))
        if rc:
            raise ValueError("packing store refused: a column is not the column the store was built from")
        return ao, bo

    def scan(self, columns, b):
        n = self.cache.params.n
        cols = np.ascontiguousarray(columns, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        out = np.zeros(n, dtype=np.uint64)
        rc = lib().orc_store_scan(self.cache.h, self.h, _p(cols), _p(b), _p(out))
        return rc == 0, out


def expand_seed(seed: bytes, n: int, q: int = DEFAULT_Q):
    s = np.frombuffer(bytes(seed), dtype=np.uint8).copy()
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_expand_seed(_p(s), n, q, _p(out))
    return out


def chacha_u64s(seed: bytes, stream: int, count: int):
    s = np.frombuffer(bytes(seed), dtype=np.uint8).copy()
    out = np.zeros(count, dtype=np.uint64)
    lib().orc_chacha_u64s(_p(s), stream, count, _p(out))
    return out


def ntt_forward(c, q=DEFAULT_Q):
    c = np.array(c, dtype=np.uint64)
    if lib().orc_ntt_forward(len(c), q, _p(c)):
        raise RuntimeError(lib().orc_last_error().decode())
    return c


def ntt_inverse(c, q=DEFAULT_Q):
    c = np.array(c, dtype=np.uint64)
    if lib().orc_ntt_inverse(len(c), q, _p(c)):
        raise RuntimeError(lib().orc_last_error().decode())
    return c


def mod_switch(c, q_old=DEFAULT_Q, q_new=MOD_SWITCH_TARGET_36BIT):
    c = np.ascontiguousarray(c, dtype=np.uint64)
    out = np.zeros_like(c)
    lib().orc_mod_switch(_p(c), len(c), q_old, q_new, _p(out))
    return out


def response_bytes(a, b, retained, modulus=DEFAULT_Q) -> bytes:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    L = lib().orc_response_bytes(_p(a), _p(b), len(a), retained, modulus, None, 0)
    out = np.zeros(L, dtype=np.uint8)
    lib().orc_response_bytes(_p(a), _p(b), len(a), retained, modulus, _p(out), L)
    return out.tobytes()


def response_bytes_tree(a, b, retained, modulus=DEFAULT_Q) -> bytes:
    """ServerResponse bytes of a tree-packed response (packing_mode Some(Tree))."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    L = lib().orc_response_bytes_tree(_p(a), _p(b), len(a), retained, modulus, None, 0)
    out = np.zeros(L, dtype=np.uint8)
    lib().orc_response_bytes_tree(_p(a), _p(b), len(a), retained, modulus, _p(out), L)
    return out.tobytes()


def response_bytes_full(cts, modulus=DEFAULT_Q) -> bytes:
    """Unpacked ServerResponse bytes: cts is (count, 2, n), the response ciphertext first."""
    cts = np.ascontiguousarray(cts, dtype=np.uint64)
    count, _, n = cts.shape
    L = lib().orc_response_bytes_full(_p(cts), count, n, modulus, None, 0)
    out = np.zeros(L, dtype=np.uint8)
    lib().orc_response_bytes_full(_p(cts), count, n, modulus, _p(out), L)
    return out.tobytes()


def rims_bytes(a, b, modulus, retained=None, columns=(), mode=None) -> bytes:
    """encode_response_packed (mod_switch.rs:254-345) restated: magic "RIMS", version 2,
    target modulus u64 LE, ring_dim u32 LE, bytes per coefficient ceil(bits(modulus-1)/8)
    (at least one), packing mode byte (0 none, 1 InspiRING, 2 tree), shape u32 LE (columns
    unpacked, retained packed), then a, the retained b and each column's a and b, each
    coefficient in that many little-endian bytes. mode defaults to 1 when retained is given."""
    n = len(a)
    if mode is None:
        mode = 0 if retained is None else 1
    width = (max(1, int(modulus - 1).bit_length()) + 7) // 8
    out = bytearray(b"RIMS") + bytes([2]) + int(modulus).to_bytes(8, "little") + n.to_bytes(4, "little")
    out += bytes([width, mode]) + (len(columns) if mode == 0 else retained).to_bytes(4, "little")

    def poly(c, count):
        for x in list(c)[:count]:
            assert int(x) < modulus
            out.extend(int(x).to_bytes(8, "little")[:width])

    poly(a, n)
    poly(b, n if mode == 0 else retained)
    for ca, cb in columns:
        poly(ca, n)
        poly(cb, n)
    return bytes(out)


class Cell:
    """A KAT cell: database, setup, client session and the reproducible query stream of the
    reference's tests/packing_key_fixture/mod.rs:90-146."""

    def __init__(self, params: Params, entry_size: int, seed: int, entries=None, plain=False):
        """plain=True: the plain method as the reference's public API runs it instead of the
        fixture: records of uniform bytes from ChaCha20Rng::seed_from_u64(seed), setup_with_rng
        and ClientSession::with_seeded_secret on GaussianSampler::with_seed(sigma, seed) and
        ChaCha20Rng::seed_from_u64(seed); draw_index gives a query index from that rng."""
        self.params, self.entry_size, self.seed = params, entry_size, seed
        entries = 3 * params.n if entries is None else entries
        build = lib().orc_cell_build_seeded if plain else lib().orc_cell_build
        self.h = build(*params.args(), entry_size, seed, entries)
        if not self.h:
            raise RuntimeError(lib().orc_last_error().decode())
        g, ns, kr = (ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64())
        w = np.zeros(32, dtype=np.uint8)
        lib().orc_cell_info(self.h, ctypes.byref(g), ctypes.byref(ns), ctypes.byref(kr), _p(w))
        self.gamma, self.num_shards, self.key_rows = g.value, ns.value, kr.value
        self.w_seed = w.tobytes()

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cell_free(self.h)

    def columns(self, shard):
        out = np.zeros((self.gamma, self.params.n), dtype=np.uint64)
        lib().orc_cell_columns(self.h, shard, _p(out))
        return out

    def keys(self):
        out = np.zeros((self.key_rows, self.params.n), dtype=np.uint64)
        lib().orc_cell_keys(self.h, _p(out))
        return out

    def secret(self):
        out = np.zeros(self.params.n, dtype=np.uint64)
        lib().orc_cell_secret(self.h, _p(out))
        return out

    def key_bytes(self) -> bytes:
        L = lib().orc_cell_key_bytes(self.h, None, 0)
        out = np.zeros(L, dtype=np.uint8)
        lib().orc_cell_key_bytes(self.h, _p(out), L)
        return out.tobytes()

    def draw_index(self, bound):
        """rand's gen_range(0..bound) on the cell's rng."""
        return int(lib().orc_cell_draw_index(self.h, bound))

    def next_query(self, index):
        sid = ctypes.c_uint32()
        seed = np.zeros(32, dtype=np.uint8)
        b = np.zeros(self.params.n, dtype=np.uint64)
        lib().orc_cell_next_query(self.h, index, ctypes.byref(sid), _p(seed), _p(b))
        return sid.value, seed.tobytes(), b

    def decode(self, index, a, b):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        rec = np.zeros(self.entry_size, dtype=np.uint8)
        ok = lib().orc_cell_decode(self.h, index, _p(a), _p(b), _p(rec))
        return bool(ok), rec.tobytes()

    def record(self, index):
        out = np.zeros(self.entry_size, dtype=np.uint8)
        lib().orc_cell_record(self.h, index, _p(out))
        return out.tobytes()

    def galois_keys(self, seed: bytes):
        """Test Galois keys of this cell's secret, (log d, rows, 2, n): a from ChaCha20(seed),
        small errors (the reference draws its keys' a from OS entropy)."""
        log_d = self.params.n.bit_length() - 1
        out = np.zeros((log_d, self.params.gadget_len, 2, self.params.n), dtype=np.uint64)
        s = np.frombuffer(seed, dtype=np.uint8).copy()
        lib().orc_cell_galois_keys(self.h, _p(s), _p(out))
        return out

    def database(self) -> bytes:
        """The cell's records, concatenated (the fixture's database formula)."""
        L = lib().orc_cell_db(self.h, None, 0)
        out = np.zeros(L, dtype=np.uint8)
        lib().orc_cell_db(self.h, _p(out), L)
        return out.tobytes()

    def sampler_state(self):
        """(ChaCha20 key bytes, 32-bit words consumed) of the session's Gaussian sampler."""
        key = np.zeros(32, dtype=np.uint8)
        pos = ctypes.c_uint64()
        lib().orc_cell_sampler_state(self.h, _p(key), ctypes.byref(pos))
        return key.tobytes(), pos.value

    def decode_tree(self, index, a, b):
        """extract_packed for a tree response (extract.rs:184-226)."""
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        rec = np.zeros(self.entry_size, dtype=np.uint8)
        ok = lib().orc_cell_decode_tree(self.h, index, _p(a), _p(b), _p(rec))
        return bool(ok), rec.tobytes()


def gaussian_stream_fnv(sigma, seed, count):
    return lib().orc_gaussian_stream_fnv(sigma, seed, count)


# ---------------------------------------------------------------------------------------
# special_modulus (src/special_modulus/ of the reference): ring 2048, q = 536813569,
# p = 2147389441, 256-byte cells, 246-byte records, gamma 512.
SM_D, SM_GAMMA, SM_Q, SM_P, SM_CELL, SM_RECORD = 2048, 512, 536813569, 2147389441, 256, 246
_sm_bound = False


def _sm_lib():
    global _sm_bound
    L = lib()
    if not _sm_bound:
        V, P, U64 = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64
        sig = {
            "orc_sm_server_new": (V, []), "orc_sm_server_free": (None, [V]),
            "orc_sm_server_new_q": (V, [U64]), "orc_sm_client_new_q": (V, [P, U64]),
            "orc_sm_client_new": (V, [P]), "orc_sm_client_free": (None, [V]),
            "orc_sm_client_key": (None, [V, P, P, P]), "orc_sm_client_key_bytes": (U64, [V, P, U64]),
            "orc_sm_client_query": (None, [V, U64, P, P]), "orc_sm_client_decode": (U64, [V, P, P, P]),
            "orc_sm_table_new": (V, [V, P, U64]), "orc_sm_table_free": (None, [V]),
            "orc_sm_table_step1": (None, [V, P]),
            "orc_sm_seat_new": (V, [V, P, P, P]), "orc_sm_seat_free": (None, [V]),
            "orc_sm_respond": (None, [V, V, V, P, P, P, P]),
            "orc_sm_query_bytes": (U64, [P, P, P, U64]), "orc_sm_response_bytes": (U64, [P, P, P, U64]),
            "orc_sm_kat_cells": (None, [U64, U64, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _sm_bound = True
    return L


def _bytes_of(fn, *args):
    n = fn(*args, None, 0)
    out = np.zeros(n, dtype=np.uint8)
    fn(*args, _p(out), n)
    return out.tobytes()


class SmServer:
    def __init__(self, q=None):
        """q: another ciphertext prime for the ring2048_cell256 set (default 536813569)."""
        self.h = _sm_lib().orc_sm_server_new() if q is None else _sm_lib().orc_sm_server_new_q(q)

    def __del__(self):
        if getattr(self, "h", None):
            _sm_lib().orc_sm_server_free(self.h)

    def table(self, cells: bytes):
        return SmTable(self, cells)

    def seat(self, key):
        return SmSeat(self, key)

    def respond(self, table, seat, seed: bytes, body):
        s = np.frombuffer(seed, dtype=np.uint8).copy()
        b = np.ascontiguousarray(body, dtype=np.uint32)
        mask = np.zeros(SM_D, dtype=np.uint32)
        out = np.zeros(2 * SM_RECORD, dtype=np.uint32)
        _sm_lib().orc_sm_respond(self.h, table.h, seat.h, _p(s), _p(b), _p(mask), _p(out))
        return mask, out


class SmTable:
    def __init__(self, server, cells: bytes):
        c = np.frombuffer(cells, dtype=np.uint8).copy()
        self.h = _sm_lib().orc_sm_table_new(server.h, _p(c), len(cells))

    def __del__(self):
        if getattr(self, "h", None):
            _sm_lib().orc_sm_table_free(self.h)

    def step1(self):
        out = np.zeros((SM_GAMMA, SM_D), dtype=np.uint32)
        _sm_lib().orc_sm_table_step1(self.h, _p(out))
        return out


class SmSeat:
    def __init__(self, server, key):
        ms = np.frombuffer(key[0], dtype=np.uint8).copy()
        kq = np.ascontiguousarray(key[1], dtype=np.uint32)
        kp = np.ascontiguousarray(key[2], dtype=np.uint32)
        self.h = _sm_lib().orc_sm_seat_new(server.h, _p(ms), _p(kq), _p(kp))

    def __del__(self):
        if getattr(self, "h", None):
            _sm_lib().orc_sm_seat_free(self.h)


class SmClient:
    """Client::from_seed of the reference (special_modulus/client.rs:137-143)."""

    def __init__(self, seed: bytes, q=None):
        s = np.frombuffer(seed, dtype=np.uint8).copy()
        self.h = _sm_lib().orc_sm_client_new(_p(s)) if q is None else _sm_lib().orc_sm_client_new_q(_p(s), q)

    def __del__(self):
        if getattr(self, "h", None):
            _sm_lib().orc_sm_client_free(self.h)

    def key(self):
        ms = np.zeros(32, dtype=np.uint8)
        kq = np.zeros(SM_D, dtype=np.uint32)
        kp = np.zeros(SM_D, dtype=np.uint32)
        _sm_lib().orc_sm_client_key(self.h, _p(ms), _p(kq), _p(kp))
        return ms.tobytes(), kq, kp

    def key_bytes(self):
        return _bytes_of(_sm_lib().orc_sm_client_key_bytes, self.h)

    def query(self, row):
        seed = np.zeros(32, dtype=np.uint8)
        body = np.zeros(SM_D, dtype=np.uint32)
        _sm_lib().orc_sm_client_query(self.h, row, _p(seed), _p(body))
        return seed.tobytes(), body

    def decode(self, mask, body):
        m = np.ascontiguousarray(mask, dtype=np.uint32)
        b = np.ascontiguousarray(body, dtype=np.uint32)
        out = np.zeros(SM_RECORD, dtype=np.uint8)
        n = _sm_lib().orc_sm_client_decode(self.h, _p(m), _p(b), _p(out))
        return out[:n].tobytes()


def sm_query_bytes(seed, body):
    s = np.frombuffer(seed, dtype=np.uint8).copy()
    b = np.ascontiguousarray(body, dtype=np.uint32)
    return _bytes_of(_sm_lib().orc_sm_query_bytes, _p(s), _p(b))


def sm_response_bytes(mask, body):
    m = np.ascontiguousarray(mask, dtype=np.uint32)
    b = np.ascontiguousarray(body, dtype=np.uint32)
    return _bytes_of(_sm_lib().orc_sm_response_bytes, _p(m), _p(b))


def sm_kat_cells(seed, rows):
    out = np.zeros(rows * SM_CELL, dtype=np.uint8)
    _sm_lib().orc_sm_kat_cells(seed, rows, _p(out))
    return out.tobytes()
