"""inspire_gb300 — the InsPIRe server respond path on one GB300 (sm_103a).

Python front of libinspire_gb300.so (C ABI: include/inspire_gb300.h), mirroring the
reference crate's public API for this path (raven-inspire, src/lib.rs:37-48):

    ServerInspiringCache.new(crs, encoded_db)          respond.rs:926-941
    ShardData.precompute_packing(...)                  setup.rs:335-340
    ServerSessionStore.register_server_side/get/remove/len   session.rs:829-895
    respond_seeded_inspiring(crs, encoded_db, query)   respond.rs:1218-1226
    respond_seeded_batch(crs, encoded_db, batch, cache, session_store)  respond.rs:1189-1202
    mod_switch_response_checked(params, response, target)  fused: mod_switch_target= on the
                                                       respond calls (mod_switch.rs:178-186)
    ServerResponse.to_binary()                         respond.rs:387-390
    ServingLoop.submit/wait/stats                      continuous batching of single queries
                                                       (no single counterpart in the reference)

Every refusal raises PirError with the reference's message. Compute runs only in the
CUDA library: when it cannot be loaded (no build, no GPU) the calls raise, and there is
no CPU fallback.
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build

__all__ = [
    "PirError", "InspireParams", "ServerCrs", "ShardData", "EncodedDatabase", "ServerInspiringCache",
    "ServerSessionStore", "ServerSessionHandle", "ClientPackingKeys", "SeededBatchQuery", "SeededClientQuery",
    "SeededQueryBatch", "PackingKeySource", "ServerResponse", "respond_seeded_inspiring", "respond_seeded_batch", "respond_inspiring",
    "respond", "respond_seeded", "respond_nopacking_batch",
    "check_mod_switch_noise_budget", "ClientQuery", "Context", "DEFAULT_Q",
    "MOD_SWITCH_TARGET_36BIT", "MOD_SWITCH_TARGET_45BIT", "library_path", "special_modulus", "ServingLoop",
    "respond_one_packing", "respond_seeded_packed", "respond_one_packing_batch", "DeviceClient",
    "ServeTicket",
]

DEFAULT_Q = 1152921504606830593
MOD_SWITCH_TARGET_36BIT = 68_718_428_161
TUNE_BATCHES = (1, 4, 16, 32, 64, 128, 256)  # batch sizes the launch-shape tuner measures
MOD_SWITCH_TARGET_45BIT = 35_184_372_060_161

IG_OK = 0
IG_ERR_STORE_REFUSED = 5
IG_ERR_PENDING = 11


class PirError(Exception):
    """PirError(String) of the reference (src/pir/error.rs): every refusal."""

    def __init__(self, message, code=None):
        super().__init__(message)
        self.code = code


_lib = None


def library_path():
    return _build.LIB


class ServeStats(ctypes.Structure):
    _fields_ = [("served", ctypes.c_uint64), ("refused", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("waiting", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64), ("mean_batch", ctypes.c_double),
                ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double), ("max_us", ctypes.c_double),
                ("budget_bytes", ctypes.c_uint64), ("inflight_bytes", ctypes.c_uint64),
                ("peak_inflight_bytes", ctypes.c_uint64), ("queue_p50_us", ctypes.c_double),
                ("queue_p99_us", ctypes.c_double), ("exec_p50_us", ctypes.c_double),
                ("exec_p99_us", ctypes.c_double)]


def _load():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    L = ctypes.CDLL(path)
    P, U64, U32, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
    pu64 = ctypes.POINTER(ctypes.c_uint64)
    sig = {
        "ig_ctx_create": (I, [I, ctypes.POINTER(P)]),
        "ig_ctx_destroy": (None, [P]),
        "ig_last_error": (I, [P, ctypes.c_char_p, ctypes.c_size_t]),
        "ig_ctx_stream": (P, [P]),
        "ig_ctx_device_bytes": (U64, [P]),
        "ig_crs_create": (I, [P, U32, U64, U64, U64, U32, I, U32, P, pu64]),
        "ig_crs_destroy": (I, [P, U64]),
        "ig_crs_key_rows": (I, [P, U64, ctypes.POINTER(U32)]),
        "ig_db_create": (I, [P, U64, U32, pu64]),
        "ig_db_destroy": (I, [P, U64]),
        "ig_db_set_shard": (I, [P, U64, U32, P]),
        "ig_db_set_shard_device": (I, [P, U64, U32, P]),
        "ig_db_encode_records": (I, [P, U64, U32, P, ctypes.c_size_t, U32, I]),
        "ig_db_precompute_packing": (I, [P, U64, U32]),
        "ig_db_precompute_packing_all": (I, [P, U64]),
        "ig_db_drop_packing_store": (I, [P, U64, U32]),
        "ig_db_has_store": (I, [P, U64, U32, ctypes.POINTER(I)]),
        "ig_session_store_create": (I, [P, pu64]),
        "ig_session_store_destroy": (I, [P, U64]),
        "ig_session_register": (I, [P, U64, U64, P, U32, U32, pu64]),
        "ig_session_remove": (I, [P, U64, U64, ctypes.POINTER(I)]),
        "ig_session_len": (I, [P, U64, pu64]),
        "ig_session_contains": (I, [P, U64, U64, ctypes.POINTER(I)]),
        "ig_respond_seeded_batch": (I, [P, U64, U64, U64, P, U32, U32, U32, P, P, P, U64, P, P]),
        "ig_respond_seeded_batch_device": (I, [P, U64, U64, U64, U32, P, P, P, U64, P, P, P]),
        "ig_respond_mixed_batch": (I, [P, U32, P, P, P, P, P, P, P, P, P]),
        "ig_respond_mixed_batch_device": (I, [P, U32, P, P, P, P, P, P, P, P, P, P]),
        "ig_respond_batch": (I, [P, U64, U64, U64, P, U32, U32, U32, P, P, P, U64, P, P]),
        "ig_response_encode": (I, [P, P, U32, U32, U64, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "ig_response_encode_full": (I, [P, U32, U32, U64, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "ig_respond_nopacking_batch": (I, [P, U64, U32, P, P, P, P, P]),
        "ig_response_encode_device": (I, [P, U32, P, P, U32, U32, U64, P, ctypes.POINTER(ctypes.c_size_t), P]),
        "ig_response_encode_tree": (I, [P, P, U32, U32, U64, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "ig_crs_set_galois_keys": (I, [P, U64, U32, U32, P]),
        "ig_client_create": (I, [P, U64, P, ctypes.c_double, pu64]),
        "ig_client_destroy": (I, [P, U64]),
        "ig_client_query_batch": (I, [P, U64, U32, P, P, P, pu64, P, P]),
        "ig_client_extract_batch": (I, [P, U64, U32, P, P, U64, U32, I, P]),
        "ig_respond_one_packing_batch": (I, [P, U64, U32, P, P, P, P, U64, P, P]),
        "ig_response_encode_rims": (I, [P, P, U32, U32, U32, P, U32, U64, P, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t)]),
        "ig_response_decode_rims": (I, [P, ctypes.c_size_t, ctypes.POINTER(U64), ctypes.POINTER(U32),
                                        ctypes.POINTER(U32), ctypes.POINTER(U32), ctypes.POINTER(U32), P, P, P,
                                        ctypes.c_char_p, ctypes.c_size_t]),
        "ig_response_encode_rims_device": (I, [P, U32, P, P, U32, U32, U64, P, ctypes.POINTER(ctypes.c_size_t), P]),
        "ig_debug_force_serial_expand": (I, [P, I]),
        "ig_profile_enable": (I, [P, I]),
        "ig_profile_read": (I, [P, P, P, I, I]),
        "ig_launch_count": (U64, [P]),
        "ig_ctx_set_pair_threshold": (I, [P, U32]),
        "ig_ctx_set_launch_shape": (I, [P, U32]),
        "ig_tune_launch_shapes": (I, [P, U32, P, U32, U32]),
        "ig_tune_get": (I, [P, U32, U32, U32, P]),
        "ig_tune_choose": (I, [P, U32, U32, U32, U32, ctypes.POINTER(U32)]),
        "ig_tune_save": (I, [P, ctypes.c_char_p]),
        "ig_tune_load": (I, [P, ctypes.c_char_p]),
        "ig_sm_server_create": (I, [P, U32, U32, U64, U64, U32, U32, U32, pu64]),
        "ig_sm_server_destroy": (I, [P, U64]),
        "ig_sm_seat": (I, [P, U64, P, P, P, pu64]),
        "ig_sm_seat_destroy": (I, [P, U64]),
        "ig_sm_table": (I, [P, U64, P, ctypes.c_size_t, pu64]),
        "ig_sm_table_destroy": (I, [P, U64]),
        "ig_sm_table_step1": (I, [P, U64, P]),
        "ig_sm_respond_batch": (I, [P, U64, U32, P, P, P, P, P, P]),
        "ig_sm_respond_batch_device": (I, [P, U64, U32, P, P, P, P, P, P, P]),
        "ig_sm_response_encode": (I, [P, U32, P, U32, U64, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "ig_debug_store_sums": (I, [P, U64, U32, P]),
        "ig_debug_fail_alloc_at": (I, [P, U32]),
        "ig_serve_create": (I, [P, U32, U32, U64, ctypes.POINTER(P)]),
        "ig_serve_submit": (I, [P, U64, U64, U64, U32, P, P, U32, U64, P, P, pu64]),
        "ig_serve_submit_wire": (I, [P, U64, U64, U64, U32, P, P, U32, U64, P, ctypes.c_size_t,
                                     ctypes.POINTER(ctypes.c_size_t), pu64]),
        "ig_serve_wait": (I, [P, U64, ctypes.c_int64, pu64, ctypes.c_char_p, ctypes.c_size_t]),
        "ig_serve_stats": (I, [P, ctypes.POINTER(ServeStats), I]),
        "ig_serve_destroy": (I, [P]),
        "ig_serve_replay": (I, [P, U64, U64, U32, P, P, P, P, U32, U64, P, U32, P, P, P,
                                ctypes.POINTER(ctypes.c_double)]),
        "ig_butterfly_peak": (I, [P, I, I, ctypes.POINTER(ctypes.c_double)]),
        "ig_ctx_set_lanes": (I, [P, U32]),
        "ig_ctx_join": (I, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _u64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    if shape is not None and a.shape != shape:
        raise PirError(f"wire shape refused: expected an array of shape {shape}, got {a.shape}")
    return a


class Context:
    """One device and one CUDA stream; every object below lives in one context."""

    _default = {}

    def __init__(self, device=0):
        L = _load()
        h = ctypes.c_void_p()
        rc = L.ig_ctx_create(device, ctypes.byref(h))
        if rc != IG_OK:
            raise PirError(f"cannot open CUDA device {device} (status {rc}); the respond path has no CPU fallback",
                           rc)
        self.h, self.device, self._lib = h, device, L

    @classmethod
    def default(cls, device=0):
        if device not in cls._default:
            cls._default[device] = Context(device)
        return cls._default[device]

    def check(self, rc):
        if rc != IG_OK:
            buf = ctypes.create_string_buffer(2048)
            self._lib.ig_last_error(self.h, buf, 2048)
            raise PirError(buf.value.decode(), rc)

    @property
    def stream(self):
        return self._lib.ig_ctx_stream(self.h)

    @property
    def device_bytes(self):
        return self._lib.ig_ctx_device_bytes(self.h)

    def set_launch_shape(self, ctas):
        """CTAs per query of every later respond launch: 1, 2 or 4; 0 lets each launch choose."""
        self.check(self._lib.ig_ctx_set_launch_shape(self.h, int(ctas)))

    def tune_launch_shapes(self, gammas, ring_dim=2048, reps=3):
        """Measures launches of 1 .. 256 queries under 1, 2 and 4 CTAs per query for each
        width; returns {gamma: {batch: (ms_1, ms_2, ms_4)}} and keeps the table for later
        launches."""
        g = np.ascontiguousarray(gammas, dtype=np.uint32)
        self.check(self._lib.ig_tune_launch_shapes(self.h, int(ring_dim), _ptr(g), len(g), int(reps)))
        return {int(x): {b: self.tuned(int(x), b, ring_dim) for b in TUNE_BATCHES} for x in g}

    def tuned(self, gamma, queries=1, ring_dim=2048):
        """The tuned row (ms under 1, 2, 4 CTAs per query) for `queries` in flight."""
        ms = np.zeros(3, dtype=np.float64)
        self.check(self._lib.ig_tune_get(self.h, int(ring_dim), int(gamma), int(queries), _ptr(ms)))
        return tuple(float(x) for x in ms)

    def launch_shape_for(self, gamma, count, in_flight=None, ring_dim=2048):
        """CTAs per query a launch of `count` queries would take with `in_flight` queries
        expected on the device (default: the launch alone)."""
        out = ctypes.c_uint32()
        self.check(self._lib.ig_tune_choose(self.h, int(ring_dim), int(gamma), int(count),
                                            int(count if in_flight is None else in_flight), ctypes.byref(out)))
        return out.value

    def save_tuning(self, path):
        self.check(self._lib.ig_tune_save(self.h, str(path).encode()))

    def load_tuning(self, path):
        self.check(self._lib.ig_tune_load(self.h, str(path).encode()))

    def set_pair_threshold(self, max_queries):
        """The fixed launch rule (no tuned table): four CTAs per query while twice the
        queries expected in flight fit max_queries, two while they fit it, else one
        (0: one CTA per query always)."""
        self.check(self._lib.ig_ctx_set_pair_threshold(self.h, int(max_queries)))

    def response_wire_len(self, ring_dim, retained, modulus):
        """Bytes of one ServerResponse wire (respond.rs:111-176) at these sizes."""
        n = ctypes.c_size_t()
        self.check(self._lib.ig_response_encode_device(self.h, 0, None, None, ring_dim, retained, modulus, None,
                                                       ctypes.byref(n), None))
        return n.value

    def response_wire_device(self, count, d_a, d_b, ring_dim, retained, modulus, d_out, d_status):
        """Encodes `count` device-resident responses into d_out on the context stream
        (ig_response_encode_device); returns the bytes per response."""
        n = ctypes.c_size_t()
        self.check(self._lib.ig_response_encode_device(self.h, count, ctypes.c_void_p(d_a), ctypes.c_void_p(d_b),
                                                       ring_dim, retained, modulus, ctypes.c_void_p(d_out),
                                                       ctypes.byref(n), ctypes.c_void_p(d_status)))
        return n.value

    def response_rims_device(self, count, d_a, d_b, ring_dim, retained, modulus, d_out, d_status):
        """RIMS frames (mod_switch.rs:254-345) of `count` device-resident InspiRING responses
        into d_out on the context stream (ig_response_encode_rims_device); with d_out 0 it
        only sizes one frame. Returns the bytes per frame."""
        n = ctypes.c_size_t()
        self.check(self._lib.ig_response_encode_rims_device(
            self.h, count, ctypes.c_void_p(d_a), ctypes.c_void_p(d_b), ring_dim, retained, modulus,
            ctypes.c_void_p(d_out) if d_out else None, ctypes.byref(n), ctypes.c_void_p(d_status)))
        return n.value

    def set_lanes(self, lanes):
        """Streams the device-resident batch entry rotates over (1 = the context stream)."""
        self.check(self._lib.ig_ctx_set_lanes(self.h, int(lanes)))

    def join(self):
        """Orders the context stream after all lane work."""
        self.check(self._lib.ig_ctx_join(self.h))

    def butterfly_peak(self, blocks_per_sm=4, iters=4096):
        """Measured rate of lazy mod-q butterflies (one Shoup product each) in registers, per
        second: the integer ceiling of the transform work."""
        v = ctypes.c_double()
        self.check(self._lib.ig_butterfly_peak(self.h, blocks_per_sm, iters, ctypes.byref(v)))
        return v.value

    @property
    def launch_count(self):
        return self._lib.ig_launch_count(self.h)

    def profile(self, on=True):
        self.check(self._lib.ig_profile_enable(self.h, int(on)))

    def profile_read(self, reset=True):
        """Summed device milliseconds and launch counts per region: scan, respond, fold."""
        ms = np.zeros(3, dtype=np.float64)
        cnt = np.zeros(3, dtype=np.uint64)
        self.check(self._lib.ig_profile_read(self.h, _ptr(ms), _ptr(cnt), 3, int(reset)))
        return {name: (float(ms[i]), int(cnt[i])) for i, name in enumerate(["scan", "respond", "fold"])}

    def close(self):
        if self.h:
            self._lib.ig_ctx_destroy(self.h)
            self.h = None


class InspireParams:
    """InspireParams (params.rs:137-196), the single-prime sets the GPU serves."""

    def __init__(self, ring_dim=2048, q=DEFAULT_Q, p=65537, sigma=6.4, gadget_base=1 << 20,
                 packing_gadget_len=3, approximate_packing_gadget=False):
        self.ring_dim, self.q, self.p, self.sigma = ring_dim, q, p, sigma
        self.gadget_base, self.packing_gadget_len = gadget_base, packing_gadget_len
        self.approximate_packing_gadget = approximate_packing_gadget

    @staticmethod
    def d2048():
        return InspireParams()

    @staticmethod
    def d2048_approximate_gadget():
        return InspireParams(approximate_packing_gadget=True)

    def moduli(self):
        return [self.q]

    def delta(self):
        return self.q // self.p

    def packing_key_rows(self):
        return self.packing_gadget_len - (1 if self.approximate_packing_gadget else 0)


class ServerCrs:
    """The public parameters a responder needs (setup.rs:75-96): params, w_seed, width."""

    def __init__(self, params: InspireParams, inspiring_w_seed: bytes, inspiring_num_columns: int,
                 galois_keys=None):
        """galois_keys: the tree responder's keys (setup.rs:435-445), log2(ring_dim) x rows x
        (a, b) x ring_dim coefficient-form words, or None (the published CRS strips them)."""
        if len(inspiring_w_seed) != 32:
            raise PirError("inspiring_w_seed must be 32 bytes")
        self.params, self.inspiring_w_seed = params, bytes(inspiring_w_seed)
        self.inspiring_num_columns = int(inspiring_num_columns)
        self.galois_keys = None if galois_keys is None else np.ascontiguousarray(galois_keys, dtype=np.uint64)

    def ring_dim(self):
        return self.params.ring_dim

    def modulus(self):
        return self.params.q


class ServerInspiringCache:
    """Per-CRS device constants: pack params and offline keys (respond.rs:869-1013)."""

    def __init__(self, crs: ServerCrs, ctx: Context = None):
        self.ctx = ctx or Context.default()
        self.crs = crs
        p = crs.params
        seed = np.frombuffer(crs.inspiring_w_seed, dtype=np.uint8).copy()
        h = ctypes.c_uint64()
        self.ctx.check(self.ctx._lib.ig_crs_create(
            self.ctx.h, p.ring_dim, p.q, p.p, p.gadget_base, p.packing_gadget_len,
            int(p.approximate_packing_gadget), crs.inspiring_num_columns, _ptr(seed), ctypes.byref(h)))
        self.h = h.value
        if crs.galois_keys is not None:
            self.set_galois_keys(crs.galois_keys)

    def set_galois_keys(self, keys):
        """Uploads ServerCrs::galois_keys (ig_crs_set_galois_keys) for the tree responder."""
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        if k.ndim != 4 or k.shape[2] != 2 or k.shape[3] != self.crs.params.ring_dim:
            raise PirError("galois keys must be (keys, rows, 2, ring_dim) coefficient-form words")
        self.ctx.check(self.ctx._lib.ig_crs_set_galois_keys(self.ctx.h, self.h, k.shape[0], k.shape[1], _ptr(k)))

    @staticmethod
    def new(crs: ServerCrs, encoded_db=None, ctx: Context = None):
        if encoded_db is not None and encoded_db.num_columns != crs.inspiring_num_columns:
            raise PirError(f"ServerInspiringCache::new: shard column count {encoded_db.num_columns} != CRS width "
                           f"{crs.inspiring_num_columns}")
        return ServerInspiringCache(crs, ctx)

    @property
    def key_rows(self):
        r = ctypes.c_uint32()
        self.ctx.check(self.ctx._lib.ig_crs_key_rows(self.ctx.h, self.h, ctypes.byref(r)))
        return r.value


class ShardData:
    """One shard of the device-resident database (setup.rs:280-375)."""

    def __init__(self, db, shard_id):
        self.db, self.id = db, shard_id

    def precompute_packing(self):
        self.db.ctx.check(self.db.ctx._lib.ig_db_precompute_packing(self.db.ctx.h, self.db.h, self.id))

    def drop_packing_store(self):
        self.db.ctx.check(self.db.ctx._lib.ig_db_drop_packing_store(self.db.ctx.h, self.db.h, self.id))

    def packing_store(self):
        out = ctypes.c_int()
        self.db.ctx.check(self.db.ctx._lib.ig_db_has_store(self.db.ctx.h, self.db.h, self.id, ctypes.byref(out)))
        return bool(out.value)

    def set_columns(self, columns):
        self.db.set_shard(self.id, columns)


class EncodedDatabase:
    """Shards of gamma column polynomials (setup.rs:272-289) held in HBM."""

    def __init__(self, cache: ServerInspiringCache, num_shards: int):
        self.ctx, self.cache = cache.ctx, cache
        self.num_shards = int(num_shards)
        self.num_columns = cache.crs.inspiring_num_columns
        self.ring_dim = cache.crs.params.ring_dim
        h = ctypes.c_uint64()
        self.ctx.check(self.ctx._lib.ig_db_create(self.ctx.h, cache.h, self.num_shards, ctypes.byref(h)))
        self.h = h.value
        self.shards = [ShardData(self, i) for i in range(self.num_shards)]

    @staticmethod
    def from_columns(cache, shard_columns):
        db = EncodedDatabase(cache, len(shard_columns))
        for i, cols in enumerate(shard_columns):
            db.set_shard(i, cols)
        return db

    @staticmethod
    def from_records(cache, records: bytes, entry_size: int, num_shards: int = None):
        """encode_database (encode_db.rs:74-134) on the GPU: concatenated entries of
        entry_size bytes split into shards of ring_dim entries and 16-bit columns."""
        entries = len(records) // entry_size
        ring = cache.crs.params.ring_dim
        db = EncodedDatabase(cache, num_shards or max(1, (entries + ring - 1) // ring))
        db.encode_records(records, entry_size)
        return db

    def encode_records(self, records, entry_size: int, device_ptr: int = None, nbytes: int = None,
                       first_shard: int = 0):
        """Writes shards first_shard.. from concatenated entries (host bytes, or a device
        pointer with its byte count)."""
        if device_ptr is not None:
            self.ctx.check(self.ctx._lib.ig_db_encode_records(self.ctx.h, self.h, int(first_shard),
                                                              ctypes.c_void_p(device_ptr), int(nbytes),
                                                              int(entry_size), 1))
            return
        buf = np.frombuffer(bytes(records), dtype=np.uint8)
        self.ctx.check(self.ctx._lib.ig_db_encode_records(self.ctx.h, self.h, int(first_shard), _ptr(buf), buf.size,
                                                          int(entry_size), 0))

    def set_shard(self, shard_id, columns):
        cols = _u64(columns, (self.num_columns, self.ring_dim))
        self.ctx.check(self.ctx._lib.ig_db_set_shard(self.ctx.h, self.h, shard_id, _ptr(cols)))

    def set_shard_device(self, shard_id, device_ptr: int):
        self.ctx.check(self.ctx._lib.ig_db_set_shard_device(self.ctx.h, self.h, shard_id, ctypes.c_void_p(device_ptr)))

    def precompute_packing_all(self):
        self.ctx.check(self.ctx._lib.ig_db_precompute_packing_all(self.ctx.h, self.h))

    def store_sums(self, shard_id):
        out = np.zeros((self.num_columns, self.ring_dim), dtype=np.uint64)
        self.ctx.check(self.ctx._lib.ig_debug_store_sums(self.ctx.h, self.h, shard_id, _ptr(out)))
        return out


class ServerSessionHandle(int):
    """ServerSessionHandle(u64) (query.rs:98)."""


class ClientPackingKeys:
    """The uploaded key body (inspiring2.rs:684-698): key_rows x ring_dim coefficients."""

    def __init__(self, y_body, num_to_pack):
        self.y_body = np.ascontiguousarray(y_body, dtype=np.uint64)
        self.num_to_pack = int(num_to_pack)


class ServerSessionStore:
    """Registered packing-key seats by handle (session.rs:700-895)."""

    def __init__(self, ctx: Context = None):
        self.ctx = ctx or Context.default()
        h = ctypes.c_uint64()
        self.ctx.check(self.ctx._lib.ig_session_store_create(self.ctx.h, ctypes.byref(h)))
        self.h = h.value

    @staticmethod
    def new(ctx=None):
        return ServerSessionStore(ctx)

    def register_server_side(self, keys: ClientPackingKeys, cache: ServerInspiringCache):
        y = np.ascontiguousarray(keys.y_body, dtype=np.uint64)
        if y.ndim != 2 or y.shape[1] != cache.crs.params.ring_dim:
            raise PirError(f"packing-key y_body dimension {y.shape[-1] if y.ndim else 0}, expected "
                           f"{cache.crs.params.ring_dim}; rebuild the keys from the current CRS")
        h = ctypes.c_uint64()
        self.ctx.check(self.ctx._lib.ig_session_register(self.ctx.h, self.h, cache.h, _ptr(y), y.shape[0],
                                                         keys.num_to_pack, ctypes.byref(h)))
        return ServerSessionHandle(h.value)

    def get(self, handle):
        out = ctypes.c_int()
        self.ctx.check(self.ctx._lib.ig_session_contains(self.ctx.h, self.h, int(handle), ctypes.byref(out)))
        return bool(out.value)

    def remove(self, handle):
        out = ctypes.c_int()
        self.ctx.check(self.ctx._lib.ig_session_remove(self.ctx.h, self.h, int(handle), ctypes.byref(out)))
        return bool(out.value)

    def __len__(self):
        out = ctypes.c_uint64()
        self.ctx.check(self.ctx._lib.ig_session_len(self.ctx.h, self.h, ctypes.byref(out)))
        return out.value

    def is_empty(self):
        return len(self) == 0


class SeededBatchQuery:
    """One seeded row request (query.rs:141-171): shard_id, the `a` seed and b."""

    def __init__(self, shard_id, seed: bytes, b):
        if len(seed) != 32:
            raise PirError("seeded RGSW row seed must be 32 bytes")
        self.shard_id, self.seed = int(shard_id), bytes(seed)
        self.b = np.ascontiguousarray(b, dtype=np.uint64)


class ClientQuery:
    """An unseeded query row (query.rs:103-120): `a` travels in full."""

    def __init__(self, shard_id, a, b, inspiring_packing_keys=None, session_handle=None):
        self.shard_id = int(shard_id)
        self.a = np.ascontiguousarray(a, dtype=np.uint64)
        self.b = np.ascontiguousarray(b, dtype=np.uint64)
        self.seed = None
        self.inspiring_packing_keys, self.session_handle = inspiring_packing_keys, session_handle


class SeededClientQuery(SeededBatchQuery):
    """A single query with its packing key inline or by handle (query.rs:103-135)."""

    def __init__(self, shard_id, seed, b, inspiring_packing_keys=None, session_handle=None):
        super().__init__(shard_id, seed, b)
        self.inspiring_packing_keys, self.session_handle = inspiring_packing_keys, session_handle


class PackingKeySource:
    """PackingKeySource::{Inline, Registered} (query.rs:176-181)."""

    def __init__(self, inline: ClientPackingKeys = None, registered=None):
        if (inline is None) == (registered is None):
            raise PirError("a packing key source is either inline keys or a registered handle")
        self.inline, self.registered = inline, registered

    @staticmethod
    def Inline(keys):
        return PackingKeySource(inline=keys)

    @staticmethod
    def Registered(handle):
        return PackingKeySource(registered=handle)


class SeededQueryBatch:
    """Queries answered under one packing key (query.rs:186-211)."""

    def __init__(self, packing_key: PackingKeySource, queries):
        self.packing_key, self.queries = packing_key, list(queries)


class ServerResponse:
    """ServerResponse (respond.rs:27-41). Packed (InspiRING): a, b, of which the first
    `packed_coefficients` b words cross the wire, over `modulus`. Unpacked (NoPacking):
    packed_coefficients None, (a, b) the sum of `column_ciphertexts`, a list of (a, b)."""

    def __init__(self, a, b, packed_coefficients, modulus=DEFAULT_Q, column_ciphertexts=None):
        self.a, self.b = a, b
        self.packed_coefficients = None if packed_coefficients is None else int(packed_coefficients)
        self.modulus = int(modulus)
        self.column_ciphertexts = column_ciphertexts or []
        self.packing_mode = None if packed_coefficients is None else "Inspiring"

    def to_binary(self) -> bytes:
        L = _load()
        if self.packed_coefficients is None:
            cts = np.ascontiguousarray(
                np.stack([np.stack([self.a, self.b])] + [np.stack([ca, cb]) for ca, cb in self.column_ciphertexts]),
                dtype=np.uint64)
            n = ctypes.c_size_t()
            count, _, ring = cts.shape
            if L.ig_response_encode_full(_ptr(cts), count, ring, self.modulus, None, 0, ctypes.byref(n)):
                raise PirError("ServerResponse encode refused: coefficients must be canonical")
            out = np.zeros(n.value, dtype=np.uint8)
            L.ig_response_encode_full(_ptr(cts), count, ring, self.modulus, _ptr(out), n.value, ctypes.byref(n))
            return out.tobytes()
        a = np.ascontiguousarray(self.a, dtype=np.uint64)
        b = np.ascontiguousarray(self.b, dtype=np.uint64)
        n = ctypes.c_size_t()
        enc = L.ig_response_encode_tree if self.packing_mode == "Tree" else L.ig_response_encode
        rc = enc(_ptr(a), _ptr(b), len(a), self.packed_coefficients, self.modulus, None, 0, ctypes.byref(n))
        if rc:
            raise PirError(f"ServerResponse encode refused (status {rc}): coefficients must be canonical")
        out = np.zeros(n.value, dtype=np.uint8)
        enc(_ptr(a), _ptr(b), len(a), self.packed_coefficients, self.modulus, _ptr(out), n.value, ctypes.byref(n))
        return out.tobytes()

    _RIMS_MODES = {None: 0, "Inspiring": 1, "Tree": 2}

    def to_rims(self) -> bytes:
        """encode_response_packed (mod_switch.rs:254-345): the self-describing RIMS frame,
        every coefficient in ceil(bits / 8) little-endian bytes."""
        L = _load()
        a = np.ascontiguousarray(self.a, dtype=np.uint64)
        b = np.ascontiguousarray(self.b, dtype=np.uint64)
        mode = self._RIMS_MODES[self.packing_mode]
        retained = 0 if mode == 0 else self.packed_coefficients
        cts = None
        if self.column_ciphertexts:
            cts = np.ascontiguousarray(np.stack([np.stack([ca, cb]) for ca, cb in self.column_ciphertexts]),
                                       dtype=np.uint64)
        ncols = 0 if cts is None else len(cts)
        n = ctypes.c_size_t()
        args = (_ptr(a), _ptr(b), len(a), retained, mode, None if cts is None else _ptr(cts), ncols, self.modulus)
        rc = L.ig_response_encode_rims(*args, None, 0, ctypes.byref(n))
        if rc:
            raise PirError(f"encode_response_packed refused (status {rc}): shape or non-canonical coefficient")
        out = np.zeros(n.value, dtype=np.uint8)
        L.ig_response_encode_rims(*args, _ptr(out), n.value, ctypes.byref(n))
        return out.tobytes()

    @staticmethod
    def from_rims(data: bytes) -> "ServerResponse":
        """decode_response_packed (mod_switch.rs:367-521)."""
        L = _load()
        buf = np.frombuffer(bytes(data), dtype=np.uint8).copy()
        modulus, ring, mode, retained, ncols = (ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32(),
                                                ctypes.c_uint32(), ctypes.c_uint32())
        err = ctypes.create_string_buffer(512)
        hdr = [ctypes.byref(x) for x in (modulus, ring, mode, retained, ncols)]
        if L.ig_response_decode_rims(_ptr(buf) if len(buf) else None, len(buf), *hdr, None, None, None, err,
                                     len(err)):
            raise PirError(err.value.decode())
        n = ring.value
        a = np.zeros(n, dtype=np.uint64)
        b = np.zeros(n, dtype=np.uint64)
        cts = np.zeros((max(ncols.value, 1), 2, n), dtype=np.uint64)
        L.ig_response_decode_rims(_ptr(buf), len(buf), *hdr, _ptr(a), _ptr(b), _ptr(cts), err, len(err))
        packing_mode = {0: None, 1: "Inspiring", 2: "Tree"}[mode.value]
        r = ServerResponse(a, b, None if packing_mode is None else retained.value, modulus.value,
                           [(cts[j, 0], cts[j, 1]) for j in range(ncols.value)])
        r.packing_mode = packing_mode
        return r


def check_mod_switch_noise_budget(params: InspireParams, target_modulus: int):
    """mod_switch.rs:111-146: refuse a target whose rounding noise can break decryption."""
    if target_modulus <= 0 or target_modulus > params.q or target_modulus < params.p:
        raise PirError(f"mod-switch target_modulus {target_modulus} outside [p, q]")
    if target_modulus % (2 * params.ring_dim) != 1:
        raise PirError(f"mod-switch target_modulus {target_modulus} is not NTT-friendly: must satisfy "
                       f"q' == 1 (mod 2*d) where d={params.ring_dim}")
    d, p, q_old, q_new, sigma = float(params.ring_dim), float(params.p), float(params.q), float(target_modulus), params.sigma
    s_max = 7.0 * sigma
    round_noise = 0.5 + d * 0.5 * s_max
    scaled_old = (q_new / q_old) * (q_old / (4.0 * p))
    total = round_noise + scaled_old + float(target_modulus % params.p)
    budget = q_new / (2.0 * p)
    if total >= budget:
        raise PirError(f"mod-switch noise-budget violation: total_noise={total:.0f} >= budget={budget:.0f}")


def _batch(crs, encoded_db, queries, packing_key, session_store, mod_switch_target):
    cache = encoded_db.cache
    ctx = encoded_db.ctx
    if cache.crs is not crs and (cache.crs.inspiring_w_seed != crs.inspiring_w_seed or
                                 cache.crs.inspiring_num_columns != crs.inspiring_num_columns):
        raise PirError("cached pack params do not match CRS params")
    n = crs.params.ring_dim
    count = len(queries)
    shard_ids = np.array([q.shard_id for q in queries], dtype=np.uint32)
    unseeded = count > 0 and queries[0].seed is None
    if any((q.seed is None) != unseeded for q in queries):
        raise PirError("a batch is all seeded or all unseeded queries")
    if unseeded:
        seeds = np.stack([_u64(q.a, (n,)) for q in queries])
    else:
        seeds = np.frombuffer(b"".join(q.seed for q in queries), dtype=np.uint8).copy()
    bs = np.stack([_u64(q.b, (n,)) for q in queries]) if count else np.zeros((0, n), dtype=np.uint64)
    a_out = np.zeros((count, n), dtype=np.uint64)
    b_out = np.zeros((count, n), dtype=np.uint64)
    if packing_key.inline is not None:
        y = _u64(packing_key.inline.y_body)
        if y.ndim != 2 or y.shape[1] != n:
            raise PirError(f"packing-key y_body must be key_rows x {n} coefficients")
        args = (0, 0, _ptr(y), y.shape[0], packing_key.inline.num_to_pack)
    else:
        if session_store is None:
            raise PirError(f"query references session_handle {int(packing_key.registered)} but no "
                           "ServerSessionStore was supplied to respond_*_with_session")
        args = (session_store.h, int(packing_key.registered), None, 0, 0)
    ms = int(mod_switch_target or 0)
    if ms:
        check_mod_switch_noise_budget(crs.params, ms)
    fn = ctx._lib.ig_respond_batch if unseeded else ctx._lib.ig_respond_seeded_batch
    ctx.check(fn(ctx.h, encoded_db.h, *args, count, _ptr(shard_ids), _ptr(seeds), _ptr(bs), ms, _ptr(a_out),
                 _ptr(b_out)))
    modulus = ms or crs.params.q
    return [ServerResponse(a_out[i], b_out[i], crs.inspiring_num_columns, modulus) for i in range(count)]


def respond_seeded_batch(crs: ServerCrs, encoded_db: EncodedDatabase, batch: SeededQueryBatch,
                         cache: ServerInspiringCache = None, session_store: ServerSessionStore = None,
                         mod_switch_target: int = 0):
    """respond_seeded_batch (respond.rs:1189-1202): every query under the batch's one
    packing key, in order; refused whole on the first error."""
    return _batch(crs, encoded_db, batch.queries, batch.packing_key, session_store, mod_switch_target)


def respond_inspiring(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery,
                      session_store: ServerSessionStore = None, mod_switch_target: int = 0):
    """respond_inspiring / respond_inspiring_cached_with_session (respond.rs:736-759,
    1053-1091) for an unseeded query."""
    return respond_seeded_inspiring(crs, encoded_db, query, session_store, mod_switch_target)


def respond_seeded_inspiring(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededClientQuery,
                             session_store: ServerSessionStore = None, mod_switch_target: int = 0):
    """respond_seeded_inspiring (respond.rs:1218-1226) and its _with_session sibling
    (1238-1248): one query, key inline or by handle."""
    keys, handle = query.inspiring_packing_keys, query.session_handle
    if keys is not None and handle is not None:
        raise PirError(f"query has both inlined inspiring_packing_keys AND session_handle {int(handle)}; "
                       "exactly one must be set")
    if keys is None and handle is None:
        raise PirError("InspiRING client packing keys missing from query (neither inlined nor session_handle set)")
    src = PackingKeySource.Inline(keys) if keys is not None else PackingKeySource.Registered(handle)
    return _batch(crs, encoded_db, [query], src, session_store, mod_switch_target)[0]


class MixedQuery:
    """One query of a mixed launch: a seeded query on `encoded_db` under seat `handle` of
    `session_store`, its response switched to mod_switch_target (0: none)."""

    def __init__(self, encoded_db, session_store, handle, query: SeededBatchQuery, mod_switch_target: int = 0):
        self.db, self.store, self.handle = encoded_db, session_store, int(handle)
        self.query, self.mod_switch_target = query, int(mod_switch_target or 0)


def respond_mixed_batch(queries) -> list:
    """Queries of several databases, parameter sets, seats and switch targets in one launch:
    the responses respond_seeded_batch gives each query under its own key and database
    (respond.rs:1189-1202), in order; refused whole on the first error. Every database must
    share one ring and one context."""
    count = len(queries)
    if count == 0:
        return []
    ctx = queries[0].db.ctx
    n = queries[0].db.ring_dim
    # One pass over the queries: the checks, and the per-query fields as lists.
    dbs, stores, handles, sids, ms, seeds = [], [], [], [], [], []
    bs = np.empty((count, n), dtype=np.uint64)
    budget_checked = set()
    for i, q in enumerate(queries):
        db, query = q.db, q.query
        if db.ctx is not ctx:
            raise PirError("a mixed launch runs on one context")
        if query.seed is None or len(query.seed) != 32:
            raise PirError("mixed launches take seeded queries (32-byte seed)")
        target = q.mod_switch_target
        if target:
            params = db.cache.crs.params
            if (id(params), target) not in budget_checked:
                check_mod_switch_noise_budget(params, target)
                budget_checked.add((id(params), target))
        if query.b.shape != (n,):
            raise PirError(f"wire shape refused: expected an array of shape {(n,)}, got {query.b.shape}")
        bs[i] = query.b
        dbs.append(db.h)
        stores.append(q.store.h)
        handles.append(q.handle)
        sids.append(query.shard_id)
        ms.append(target)
        seeds.append(query.seed)
    dbs = np.array(dbs, dtype=np.uint64)
    stores = np.array(stores, dtype=np.uint64)
    handles = np.array(handles, dtype=np.uint64)
    sids = np.array(sids, dtype=np.uint32)
    ms = np.array(ms, dtype=np.uint64)
    seeds = np.frombuffer(b"".join(seeds), dtype=np.uint8).copy()
    a_out = np.empty((count, n), dtype=np.uint64)
    b_out = np.empty((count, n), dtype=np.uint64)
    ctx.check(ctx._lib.ig_respond_mixed_batch(ctx.h, count, _ptr(dbs), _ptr(stores), _ptr(handles), _ptr(sids),
                                              _ptr(seeds), _ptr(bs), _ptr(ms), _ptr(a_out), _ptr(b_out)))
    return [ServerResponse(a_out[i], b_out[i], q.db.num_columns, q.mod_switch_target or q.db.cache.crs.params.q)
            for i, q in enumerate(queries)]


class ServeTicket:
    """One submitted request of a ServingLoop; owns the buffers its result lands in."""

    def __init__(self, loop, ticket, a_out, b_out, modulus, packed, wire=None):
        self.loop, self.ticket = loop, ticket
        self._a, self._b, self._modulus, self._packed = a_out, b_out, modulus, packed
        self._wire = wire  # (buffer, length) for wire requests
        self.latency_us = None
        self.done = False


class ServingLoop:
    """Continuous batching of individually arriving seeded queries (the C ABI's ig_serve_*).

    The reference's server answers one respond_seeded_batch call at a time
    (respond.rs:1189-1202); here requests are submitted one by one, a dispatcher thread
    batches the oldest waiting requests on one ring (parameter sets, record widths, seats and
    mod-switch targets may differ within a batch), and `slots` batches run concurrently on
    their own streams. Admission is by memory: a request joins a batch while the bytes of its
    key and buffers fit in `hbm_budget_bytes` (0: room for every slot full of the largest
    requests) next to the batches in flight. A request's response equals
    respond_seeded_batch's for the same query."""

    def __init__(self, ctx: Context = None, slots=4, max_batch=64, hbm_budget_bytes=0):
        self.ctx = ctx or Context.default()
        self.h = None
        self._live = {}  # tickets whose result buffers the loop may still write
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx._lib.ig_serve_create(self.ctx.h, slots, max_batch, hbm_budget_bytes,
                                                     ctypes.byref(h)))
        self.h = h

    def submit(self, crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededBatchQuery,
               session_store: ServerSessionStore, handle, mod_switch_target: int = 0,
               wire: bool = False) -> ServeTicket:
        """Queues one query; with wire=True the ticket resolves to the ServerResponse bytes,
        built on the GPU, instead of a ServerResponse."""
        if self.h is None:
            raise PirError("serving loop is closed")
        n = crs.params.ring_dim
        if query.seed is None or len(query.seed) != 32:
            raise PirError("the serving loop takes seeded queries (32-byte seed)")
        b = _u64(query.b, (n,))
        seed = np.frombuffer(bytes(query.seed), dtype=np.uint8).copy()
        ms = int(mod_switch_target or 0)
        if ms:
            check_mod_switch_noise_budget(crs.params, ms)
        t = ctypes.c_uint64()
        if wire:
            cap = 78 + 2 * ((n * 64 + 7) // 8)
            buf = np.zeros(cap, dtype=np.uint8)
            length = ctypes.c_size_t()
            self.ctx.check(self.ctx._lib.ig_serve_submit_wire(self.h, encoded_db.h, session_store.h, int(handle),
                                                              int(query.shard_id), _ptr(seed), _ptr(b), n, ms,
                                                              _ptr(buf), cap, ctypes.byref(length), ctypes.byref(t)))
            ticket = ServeTicket(self, t.value, None, None, ms or crs.params.q, crs.inspiring_num_columns,
                                 wire=(buf, length))
            self._live[t.value] = ticket
            return ticket
        a_out = np.zeros(n, dtype=np.uint64)
        b_out = np.zeros(n, dtype=np.uint64)
        self.ctx.check(self.ctx._lib.ig_serve_submit(self.h, encoded_db.h, session_store.h, int(handle),
                                                     int(query.shard_id), _ptr(seed), _ptr(b), n, ms, _ptr(a_out),
                                                     _ptr(b_out), ctypes.byref(t)))
        ticket = ServeTicket(self, t.value, a_out, b_out, ms or crs.params.q, crs.inspiring_num_columns)
        self._live[t.value] = ticket
        return ticket

    def wait(self, ticket: ServeTicket, timeout_ms: int = -1) -> ServerResponse:
        """Blocks until the request finishes; raises PirError with the refusal otherwise."""
        if self.h is None:
            raise PirError("serving loop is closed")
        lat = ctypes.c_uint64()
        err = ctypes.create_string_buffer(1024)
        rc = self.ctx._lib.ig_serve_wait(self.h, ticket.ticket, int(timeout_ms), ctypes.byref(lat), err, len(err))
        if rc != IG_ERR_PENDING:
            ticket.done = True
            self._live.pop(ticket.ticket, None)
        if rc != 0:
            raise PirError(err.value.decode(errors="replace"), rc)
        ticket.latency_us = lat.value / 1e3
        if ticket._wire is not None:
            buf, length = ticket._wire
            return buf[:length.value].tobytes()
        return ServerResponse(ticket._a, ticket._b, ticket._packed, ticket._modulus)

    def replay(self, encoded_db, session_store, shard_ids, handles, seeds, bs, mod_switch_target=0,
               arrival_ns=None, window=0):
        """Native load driver (ig_serve_replay): submits the trace on schedule (arrival_ns,
        open loop) or with `window` requests outstanding (closed loop) and returns
        (a, b, latency_ns, elapsed_s)."""
        shard_ids = np.ascontiguousarray(shard_ids, dtype=np.uint32)
        handles = np.ascontiguousarray(handles, dtype=np.uint64)
        seeds = np.ascontiguousarray(seeds, dtype=np.uint8)
        bs = np.ascontiguousarray(bs, dtype=np.uint64)
        count, n = bs.shape
        arr = None if arrival_ns is None else np.ascontiguousarray(arrival_ns, dtype=np.uint64)
        # Written once here, so the first-touch page faults of the result arrays (hundreds of
        # MB for a long trace) are taken before the trace starts, not by the loop's completer.
        a = np.empty((count, n), dtype=np.uint64)
        b = np.empty((count, n), dtype=np.uint64)
        a.fill(0)
        b.fill(0)
        lat = np.zeros(count, dtype=np.uint64)
        el = ctypes.c_double()
        self.ctx.check(self.ctx._lib.ig_serve_replay(
            self.h, encoded_db.h, session_store.h, count, _ptr(shard_ids), _ptr(handles), _ptr(seeds), _ptr(bs), n,
            int(mod_switch_target or 0), _ptr(arr), int(window), _ptr(a), _ptr(b), _ptr(lat), ctypes.byref(el)))
        return a, b, lat, el.value

    def stats(self, reset=False) -> dict:
        st = ServeStats()
        self.ctx.check(self.ctx._lib.ig_serve_stats(self.h, ctypes.byref(st), 1 if reset else 0))
        return {k: getattr(st, k) for k, _ in ServeStats._fields_}

    def close(self):
        if self.h is not None:
            self.ctx._lib.ig_serve_destroy(self.h)  # finishes every submitted request first
            self.h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _nopacking(crs, encoded_db, queries):
    ctx = encoded_db.ctx
    n, g = crs.params.ring_dim, crs.inspiring_num_columns
    count = len(queries)
    if count == 0:
        raise PirError("empty batch")
    unseeded = queries[0].seed is None
    if any((q.seed is None) != unseeded for q in queries):
        raise PirError("a batch is all seeded or all unseeded queries")
    shard_ids = np.array([q.shard_id for q in queries], dtype=np.uint32)
    if unseeded:
        seeds, a_in = None, np.stack([_u64(q.a, (n,)) for q in queries])
    else:
        seeds, a_in = np.frombuffer(b"".join(q.seed for q in queries), dtype=np.uint8).copy(), None
    bs = np.stack([_u64(q.b, (n,)) for q in queries])
    out = np.zeros((count, g + 1, 2, n), dtype=np.uint64)
    ctx.check(ctx._lib.ig_respond_nopacking_batch(ctx.h, encoded_db.h, count, _ptr(shard_ids), _ptr(seeds),
                                                  _ptr(a_in), _ptr(bs), _ptr(out)))
    return [ServerResponse(out[i, 0, 0], out[i, 0, 1], None, crs.params.q,
                           column_ciphertexts=[(out[i, j, 0], out[i, j, 1]) for j in range(1, g + 1)])
            for i in range(count)]


def respond(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery) -> ServerResponse:
    """respond (respond.rs:614-643): the NoPacking variant, one ciphertext per column and
    their sum, for an unseeded query."""
    return _nopacking(crs, encoded_db, [query])[0]


def respond_seeded(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededBatchQuery) -> ServerResponse:
    """respond_seeded (respond.rs:1229-1237): the query's `a` expanded from its seed, then
    respond."""
    return _nopacking(crs, encoded_db, [query])[0]


def respond_nopacking_batch(crs: ServerCrs, encoded_db: EncodedDatabase, queries) -> list:
    """NoPacking responses of many queries in one launch sequence (seeded or unseeded)."""
    return _nopacking(crs, encoded_db, list(queries))


class DeviceClient:
    """A ClientSession's query batch and record extraction on the GPU (session.rs:377-434,
    extract.rs:184-263), for driving the server with real encrypted queries at saturation
    and checking every answer. `secret` is the session's RLWE secret (ring_dim words mod q)."""

    def __init__(self, cache: "ServerInspiringCache", secret, sigma: float = 6.4):
        self.ctx, self.crs = cache.ctx, cache.crs
        s = _u64(secret, (self.crs.params.ring_dim,))
        h = ctypes.c_uint64()
        self.ctx.check(self.ctx._lib.ig_client_create(self.ctx.h, cache.h, _ptr(s), float(sigma), ctypes.byref(h)))
        self.h = h.value

    def close(self):
        if self.h:
            self.ctx._lib.ig_client_destroy(self.ctx.h, self.h)
            self.h = None

    def query_batch(self, indices, seeds, sampler_key: bytes, sampler_word: int):
        """Seeded queries for global `indices` with `a` seeds (32 bytes each) and errors from the
        sampler (ChaCha20 key, 32-bit words consumed). Returns (SeededBatchQuery list, the
        sampler's new word position)."""
        n = self.crs.params.ring_dim
        idx = np.ascontiguousarray(indices, dtype=np.uint64)
        count = len(idx)
        sd = np.frombuffer(b"".join(bytes(x) for x in seeds), dtype=np.uint8).copy()
        if len(sd) != 32 * count or len(sampler_key) != 32:
            raise PirError("query_batch needs one 32-byte seed per index and a 32-byte sampler key")
        key = np.frombuffer(bytes(sampler_key), dtype=np.uint8).copy()
        pos = ctypes.c_uint64(int(sampler_word))
        sids = np.zeros(count, dtype=np.uint32)
        b = np.zeros((count, n), dtype=np.uint64)
        self.ctx.check(self.ctx._lib.ig_client_query_batch(self.ctx.h, self.h, count, _ptr(idx), _ptr(sd), _ptr(key),
                                                           ctypes.byref(pos), _ptr(sids), _ptr(b)))
        qs = [SeededBatchQuery(int(sids[i]), bytes(seeds[i]), b[i]) for i in range(count)]
        return qs, pos.value

    def extract_arrays(self, a, b, modulus: int, entry_size: int, tree: bool = False) -> np.ndarray:
        """Records (count x entry_size bytes) of packed responses given as (count, n) arrays."""
        n = self.crs.params.ring_dim
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        if a.ndim != 2 or a.shape != b.shape or a.shape[1] != n:
            raise PirError(f"responses must be (count, {n}) arrays")
        out = np.zeros((a.shape[0], entry_size), dtype=np.uint8)
        self.ctx.check(self.ctx._lib.ig_client_extract_batch(self.ctx.h, self.h, a.shape[0], _ptr(a), _ptr(b),
                                                             int(modulus), int(entry_size), int(tree), _ptr(out)))
        return out

    def extract_batch(self, responses, entry_size: int):
        """Records of packed responses (InspiRING or tree, unswitched or switched)."""
        n = self.crs.params.ring_dim
        count = len(responses)
        if count == 0:
            return []
        modulus = responses[0].modulus
        tree = responses[0].packing_mode == "Tree"
        if any(r.modulus != modulus or (r.packing_mode == "Tree") != tree for r in responses):
            raise PirError("extract_batch takes responses of one modulus and one packing mode")
        a = np.stack([_u64(r.a, (n,)) for r in responses])
        b = np.stack([_u64(r.b, (n,)) for r in responses])
        out = np.zeros((count, entry_size), dtype=np.uint8)
        self.ctx.check(self.ctx._lib.ig_client_extract_batch(self.ctx.h, self.h, count, _ptr(a), _ptr(b),
                                                             int(modulus), int(entry_size), int(tree), _ptr(out)))
        return [out[i].tobytes() for i in range(count)]


def _one_packing(crs, encoded_db, queries, mod_switch_target=0):
    ctx = encoded_db.ctx
    n, g = crs.params.ring_dim, crs.inspiring_num_columns
    count = len(queries)
    if count == 0:
        raise PirError("empty batch")
    unseeded = queries[0].seed is None
    if any((q.seed is None) != unseeded for q in queries):
        raise PirError("a batch is all seeded or all unseeded queries")
    if mod_switch_target:
        check_mod_switch_noise_budget(crs.params, mod_switch_target)
    shard_ids = np.array([q.shard_id for q in queries], dtype=np.uint32)
    if unseeded:
        seeds, a_in = None, np.stack([_u64(q.a, (n,)) for q in queries])
    else:
        seeds, a_in = np.frombuffer(b"".join(q.seed for q in queries), dtype=np.uint8).copy(), None
    bs = np.stack([_u64(q.b, (n,)) for q in queries])
    a = np.zeros((count, n), dtype=np.uint64)
    b = np.zeros((count, n), dtype=np.uint64)
    ctx.check(ctx._lib.ig_respond_one_packing_batch(ctx.h, encoded_db.h, count, _ptr(shard_ids), _ptr(seeds),
                                                    _ptr(a_in), _ptr(bs), int(mod_switch_target), _ptr(a), _ptr(b)))
    out = []
    for i in range(count):
        r = ServerResponse(a[i], b[i], g, mod_switch_target or crs.params.q)
        r.packing_mode = "Tree"
        out.append(r)
    return out


def respond_one_packing(crs: ServerCrs, encoded_db: EncodedDatabase, query: ClientQuery,
                        mod_switch_target: int = 0) -> ServerResponse:
    """respond_one_packing (respond.rs:696-729): the column LWEs packed by the Galois-
    automorphism tree into one ciphertext holding column k at coefficient k, scaled by d.
    Needs the CRS's Galois keys."""
    return _one_packing(crs, encoded_db, [query], mod_switch_target)[0]


def respond_seeded_packed(crs: ServerCrs, encoded_db: EncodedDatabase, query: SeededBatchQuery,
                          mod_switch_target: int = 0) -> ServerResponse:
    """respond_seeded_packed (respond.rs:1241-1249): the seed expanded, then
    respond_one_packing."""
    return _one_packing(crs, encoded_db, [query], mod_switch_target)[0]


def respond_one_packing_batch(crs: ServerCrs, encoded_db: EncodedDatabase, queries, mod_switch_target: int = 0):
    """OnePacking responses of many queries in one launch (seeded or unseeded)."""
    return _one_packing(crs, encoded_db, list(queries), mod_switch_target)


class _SpecialModulus:
    """The special_modulus variant (reference src/special_modulus/): Params, Server,
    ShardTable, KeySeat, Query and Response over 32-bit words, run on the GPU."""

    class Params:
        """Params::ring2048_cell256 (special_modulus/mod.rs:84-95)."""

        def __init__(self, ring_dim=2048, gamma=512, q=536_813_569, special_prime=2_147_389_441, cell_bytes=256,
                     record_bytes=246, sigma=6.4, key_mask_version=2):
            self.ring_dim, self.gamma, self.q, self.special_prime = ring_dim, gamma, q, special_prime
            self.cell_bytes, self.record_bytes, self.sigma = cell_bytes, record_bytes, sigma
            self.key_mask_version = key_mask_version

        @staticmethod
        def ring2048_cell256():
            return _SpecialModulus.Params()

        def body_coefficients(self):
            return 2 * self.record_bytes

    class PackingKey:
        """A decoded packing key (wire.rs:37-43): mask seed and the two limbs."""

        def __init__(self, mask_seed: bytes, q, p):
            self.mask_seed = bytes(mask_seed)
            self.q = np.ascontiguousarray(q, dtype=np.uint32)
            self.p = np.ascontiguousarray(p, dtype=np.uint32)

    class Query:
        def __init__(self, seed: bytes, body):
            self.seed = bytes(seed)
            self.body = np.ascontiguousarray(body, dtype=np.uint32)

    class Response:
        def __init__(self, mask, body, q):
            self.mask, self.body, self.q = mask, body, q

        def to_bytes(self) -> bytes:
            L = _load()
            m = np.ascontiguousarray(self.mask, dtype=np.uint32)
            b = np.ascontiguousarray(self.body, dtype=np.uint32)
            n = ctypes.c_size_t()
            if L.ig_sm_response_encode(_ptr(m), len(m), _ptr(b), len(b), self.q, None, 0, ctypes.byref(n)):
                raise PirError("response coefficient is not a residue")
            out = np.zeros(n.value, dtype=np.uint8)
            L.ig_sm_response_encode(_ptr(m), len(m), _ptr(b), len(b), self.q, _ptr(out), n.value, ctypes.byref(n))
            return out.tobytes()

    class Server:
        """Server::new (server.rs:145-164): seat, table and respond on one device."""

        def __init__(self, params=None, ctx: Context = None):
            self.ctx = ctx or Context.default()
            self.params = params or _SpecialModulus.Params()
            p = self.params
            h = ctypes.c_uint64()
            self.ctx.check(self.ctx._lib.ig_sm_server_create(
                self.ctx.h, p.ring_dim, p.gamma, p.q, p.special_prime, p.cell_bytes, p.record_bytes,
                p.key_mask_version, ctypes.byref(h)))
            self.h = h.value

        def seat(self, key):
            h = ctypes.c_uint64()
            ms = np.frombuffer(key.mask_seed, dtype=np.uint8).copy()
            if len(key.q) != self.params.ring_dim or len(key.p) != self.params.ring_dim:
                raise PirError(f"packing key needs {self.params.ring_dim} coefficients per limb")
            self.ctx.check(self.ctx._lib.ig_sm_seat(self.ctx.h, self.h, _ptr(ms), _ptr(key.q), _ptr(key.p),
                                                    ctypes.byref(h)))
            return h.value

        def table(self, cells: bytes):
            h = ctypes.c_uint64()
            c = np.frombuffer(bytes(cells), dtype=np.uint8).copy()
            self.ctx.check(self.ctx._lib.ig_sm_table(self.ctx.h, self.h, _ptr(c) if len(c) else None, len(c),
                                                     ctypes.byref(h)))
            return h.value

        def table_step1(self, table):
            out = np.zeros((self.params.gamma, self.params.ring_dim), dtype=np.uint32)
            self.ctx.check(self.ctx._lib.ig_sm_table_step1(self.ctx.h, table, _ptr(out)))
            return out

        def respond(self, table, seat, query):
            return self.respond_batch([table], [seat], [query])[0]

        def respond_batch(self, tables, seats, queries):
            n, nb = self.params.ring_dim, self.params.body_coefficients()
            count = len(queries)
            if count == 0 or len(tables) != count or len(seats) != count:
                raise PirError("a batch needs one table and one seat per query")
            th = np.array(tables, dtype=np.uint64)
            sh = np.array(seats, dtype=np.uint64)
            seeds = np.frombuffer(b"".join(q.seed for q in queries), dtype=np.uint8).copy()
            bodies = np.stack([q.body for q in queries]).astype(np.uint32)
            if bodies.shape != (count, n):
                raise PirError("query does not fit the set")
            mask = np.zeros((count, n), dtype=np.uint32)
            body = np.zeros((count, nb), dtype=np.uint32)
            self.ctx.check(self.ctx._lib.ig_sm_respond_batch(self.ctx.h, self.h, count, _ptr(th), _ptr(sh),
                                                             _ptr(seeds), _ptr(bodies), _ptr(mask), _ptr(body)))
            return [_SpecialModulus.Response(mask[i], body[i], self.params.q) for i in range(count)]


special_modulus = _SpecialModulus
