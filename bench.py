"""Benchmark of the InsPIRe respond path on GB300.

Workload (the reference's headline serving configuration): InspireParams::d2048, 512-byte
records (gamma = 256 columns per shard), 2^20 records = 512 shards, a packing store folded
on every shard, one session key registered by handle, batches of 64 queries with uniform
indices answered through respond_seeded_batch, responses mod-switched to 36 bits; a step is
16 such batches. Inputs are seeded synthetic data of those shapes: uniform 16-bit column
words (the encoding of uniform random record bytes), uniform key and query words mod q.
After the timed region, sampled responses of it are recomputed by the CPU oracle and must
match byte for byte (`parity_checked`).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload served-batch|special-modulus|mixed|serving-sweep|one-packing|no-packing]
                    [--headline-only]

--workload special-modulus times the special_modulus batch of 256, mixed six parameter sets
(32/512/2048 B records under both gadgets, batch sizes 1-512), serving-sweep the serving
loop over 2^25 records and 1000 seats, one-packing the tree responder, no-packing the
NoPacking responder. On one GPU at the default database size, the served-batch run also
runs those five after the headline, each at its own defaults, and reports them under
`workloads` (--headline-only skips them).

Prints one JSON line. `value` = queries/s over K device-resident steps (CUDA events on
the library's stream); `e2e` = the same through the public API with host buffers;
`cpu_baseline` = the CPU oracle (a port of the reference's respond path) on a bounded
sample on this host's cores. `--impl reference` times that CPU port alone on the whole
configuration (every shard stored, one batch of 64 per step).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

# The oracle's OpenMP workers (byte checks between GPU legs, the CPU samples) sleep as soon
# as a parallel region ends instead of spinning on the host cores the GPU legs' threads use.
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_RING = 2048
GAMMA = 256
ENTRY_BYTES = 512
NUM_SHARDS = 512  # 2^20 records / 2048 per shard
BATCH = 64
BATCHES_PER_STEP = 16  # a step answers 16 batches of 64 (1024 queries), about 17 ms on one GB300
SERVE_REQUESTS = 16384  # requests of each serving-loop leg past its warm-up, whatever --steps is
Q = 1152921504606830593
MS_TARGET = 68_718_428_161
SHARD_DB_BYTES = N_RING * ENTRY_BYTES  # the queried shard's records: 1 MiB
METRIC = "respond queries/s (served batch of 64, d2048, 512 B records, 2^20 records, 36-bit mod switch)"
CONFIG = {"workload": "d2048 TwoPacking, 512-byte records x 2^20 (512 shards, gamma 256), packing store on "
                      "every shard, batches of 64 under one registered key, uniform indices, 36-bit mod switch",
          "ring_dim": N_RING, "gamma": GAMMA, "records": 1 << 20, "shards": NUM_SHARDS, "batch": BATCH,
          "mod_switch_bits": 36, "l2": "inputs larger than L2: each batch reads 64 random shards' columns and "
                                       "stores (8 MiB per query, 512 MiB per batch)"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM bytes (read + write) of one k_scan launch of this workload, from an ncu capture of a
# batch of 64 queries of gamma 256 on a 512-shard database with L2 flushed before the launch
# (dram__bytes_read.sum + dram__bytes_write.sum: 66,102,528 + 508,416; the command is in
# profiles/k_scan_batch64_d2048_g256.md). It sits just under the algorithmic bytes: each
# byte is read once.
SCAN_TRAFFIC_BYTES = 66_610_944
# Heavy integer pipe (IMAD, IMAD.WIDE, IMAD.HI) busy cycles of k_respond per query, summed
# over the four sub-partitions of each SM: sm__pipe_fmaheavy_cycles_active.sum of one
# 64-query launch of this workload's timed region (1,043,445,848) / 64, from the ncu
# capture in profiles/k_respond_single_batch64_d2048_g256.md. The pipe offers four such
# cycles per SM per clock.
RESPOND_HEAVY_CYCLES_PER_QUERY = 16_303_841


def shard_seed(rank, s):
    """Seed of shard s's synthetic columns, so a shard can be regenerated for the oracle."""
    return (1 + rank) * 1_000_003 + s


def shard_columns_device(torch, rank, s):
    g = torch.Generator(device="cuda")
    g.manual_seed(shard_seed(rank, s))
    return torch.randint(0, 1 << 16, (GAMMA, N_RING), generator=g, device="cuda", dtype=torch.int64)


def rand_words(rng, shape):
    return rng.integers(0, Q, size=shape, dtype=np.uint64)


# ------------------------------------------------------------------------------------
# CPU oracle leg (the reference's algorithm restated; test infrastructure only here as
# the timed CPU baseline).
def cpu_sample(batches, warmup_batches=0, build_all=False, shards=NUM_SHARDS, seed=11):
    """The workload on the host's cores through the oracle's store path (the reference's
    respond_seeded_batch restated: seed expansion, column check and b fold, store gather,
    recursion, online gather, 36-bit switch; OpenMP at the reference's rayon sites): batches
    of 64 queries with uniform indices over a database of `shards` shards of gamma 256,
    answered one query after another as respond_seeded_batch answers them. The shards'
    stores are built offline (untimed): all of them with build_all, else the shards the
    sample touches. Timing follows the reference's bench method
    (benches/shard_packing_store_bench.rs:1-60): every sample listed, median/p90/p99."""
    from oracle import oracle as O

    O.build()
    cores = O.lib().orc_max_threads()
    rng = np.random.default_rng(seed)
    P = O.Params.d2048()
    cache = O.Cache(P, GAMMA, rng.bytes(32))
    y = rand_words(rng, (3, N_RING))
    cols, stores = {}, {}

    def shard(s):
        if s not in stores:
            c = np.random.default_rng((seed, s)).integers(0, 1 << 16, (GAMMA, N_RING), dtype=np.uint64)
            cols[s], stores[s] = c, O.Store(cache, c)
        return cols[s], stores[s]

    t0 = time.perf_counter()
    if build_all:
        for s in range(shards):
            shard(s)
    setup_s = time.perf_counter() - t0
    lat, batch_s = [], []
    for bi in range(warmup_batches + batches):
        sids = rng.integers(0, shards * N_RING, BATCH) // N_RING
        queries = [(int(sid), rng.bytes(32), rand_words(rng, N_RING)) for sid in sids]
        for sid, _, _ in queries:
            shard(sid)  # offline precompute_packing, outside the timing
        t_batch = time.perf_counter()
        for sid, seed_b, b in queries:
            tq = time.perf_counter()
            c, st = shard(sid)
            ao, bo = st.respond(c, O.expand_seed(seed_b, N_RING), b, y)
            O.mod_switch(ao, Q, MS_TARGET)
            O.mod_switch(bo, Q, MS_TARGET)
            if bi >= warmup_batches:
                lat.append(time.perf_counter() - tq)
        if bi >= warmup_batches:
            batch_s.append(time.perf_counter() - t_batch)
    qps = BATCH * len(batch_s) / sum(batch_s)
    lat_ms = np.sort(np.array(lat)) * 1e3

    def pct(p):
        return float(lat_ms[min(len(lat_ms) - 1, int(p * len(lat_ms)))])

    return {"value": qps, "unit": "queries/s", "cores": int(cores), "kind": "port",
            "sample": f"{batches} batch(es) of 64 queries with uniform indices over {shards} shards of gamma 256 "
                      f"(512-byte records), {len(stores)} stores built ({'every shard' if build_all else 'the shards the sample touches'}); "
                      "oracle store path + 36-bit switch, one query after another, OpenMP over the reference's "
                      "rayon sites",
            "queries": len(lat), "setup_s": setup_s,
            "batch_s": [round(x, 4) for x in batch_s],
            "query_ms": {"median": pct(0.5), "p90": pct(0.9), "p99": pct(0.99)}}


# ------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.proc, self.lines = device, None, []
        self.first = threading.Event()
        self.t_begin = self.t_end = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5.0)  # the sampler is live before the timed work starts
        except Exception:
            self.proc = None
        self.t_begin = time.perf_counter()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))
            self.first.set()

    def __exit__(self, *a):
        self.t_end = time.perf_counter()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # Samples taken inside the sampled region; a line arrives just after its sample.
        inside = [ln for t, ln in self.lines if self.t_begin is not None and self.t_begin <= t <= self.t_end + 0.05]
        for ln in inside:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "interval_ms": 50,
                "region_s": None if self.t_end is None else round(self.t_end - self.t_begin, 3)}


# Contexts the workloads open; closed between workloads so each starts on a free device.
_OPEN_CONTEXTS = []


def open_context(pkg, device):
    ctx = pkg.Context(device)
    _OPEN_CONTEXTS.append(ctx)
    return ctx


def close_contexts():
    import torch

    while _OPEN_CONTEXTS:
        _OPEN_CONTEXTS.pop().close()
    if torch.cuda.is_available():
        torch.cuda.synchronize()
        torch.cuda.empty_cache()


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("IG_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return rank, world


def max_over_ranks(x, world):
    """Largest value of x over all ranks (the slowest rank sets whole-job throughput)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------------------------
def oracle_check(O, cache_o, y, cols_of, cases):
    """Each case (shard, seed, b, gpu_a, gpu_b) recomputed by the oracle's store path with the
    36-bit switch; raises on the first response whose wire bytes differ. Returns the count."""
    stores = {}
    for sid, seed_b, b, ga, gb in cases:
        if sid not in stores:
            c = cols_of(sid)
            stores[sid] = (c, O.Store(cache_o, c))
        c, st = stores[sid]
        ao, bo = st.respond(c, O.expand_seed(seed_b, N_RING), b, y)
        want = O.response_bytes(O.mod_switch(ao, Q, MS_TARGET), O.mod_switch(bo, Q, MS_TARGET), GAMMA, MS_TARGET)
        got = O.response_bytes(np.asarray(ga, dtype=np.uint64), np.asarray(gb, dtype=np.uint64), GAMMA, MS_TARGET)
        if got != want:
            raise RuntimeError(f"GPU response differs from the oracle's (shard {sid})")
    return len(cases)


def serve_leg(pkg, ctx, db, store, handle, shards, rng, ms, slots, max_batch=BATCH, requests=SERVE_REQUESTS):
    """The continuous-batching loop (ig_serve_*) with host buffers, driven by the native load
    driver (ig_serve_replay) so the client side is not the bottleneck: a closed loop keeping
    4 x slots x max_batch requests outstanding (saturation), then Poisson arrivals at half
    that rate (latency under load). Each leg runs `requests` requests past a warm-up of its
    own; latency runs from submit to the result in the caller's buffer. Returns the stats and
    a few (shard, seed, b, a, b) responses for the oracle check."""
    warm = 4 * slots * max_batch
    total = warm + requests
    sids = (rng.integers(0, shards * N_RING, total) // N_RING).astype(np.uint32)
    handles = np.full(total, int(handle), dtype=np.uint64)
    seeds = rng.integers(0, 256, (total, 32), dtype=np.uint8)
    bs = rand_words(rng, (total, N_RING))
    out = {"slots": slots, "max_batch": max_batch, "requests": requests, "driver": "ig_serve_replay (native)"}
    window = 4 * slots * max_batch
    with pkg.ServingLoop(ctx, slots=slots, max_batch=max_batch) as loop:
        loop.replay(db, store, sids[:warm], handles[:warm], seeds[:warm], bs[:warm], ms, window=window)
        loop.stats(reset=True)
        a, b, lat, el = loop.replay(db, store, sids[warm:], handles[warm:], seeds[warm:], bs[warm:], ms,
                                    window=window)
        st = loop.stats(reset=True)
        sat = requests / el
        lat_ms = np.sort(lat) / 1e6
        out["saturation"] = {"queries_per_s": sat, "p50_ms": float(lat_ms[len(lat_ms) // 2]),
                             "p99_ms": float(lat_ms[int(0.99 * (len(lat_ms) - 1))]), "mean_batch": st["mean_batch"],
                             "window": window}
        picks = [warm + int(i) for i in rng.choice(requests, 2, replace=False)]
        cases = [(int(sids[i]), seeds[i].tobytes(), bs[i], a[i - warm], b[i - warm]) for i in picks]
        rate = 0.5 * sat
        arr = np.cumsum(rng.exponential(1e9 / rate, requests)).astype(np.uint64)
        a, b, lat, el = loop.replay(db, store, sids[warm:], handles[warm:], seeds[warm:], bs[warm:], ms,
                                    arrival_ns=arr)
        st = loop.stats(reset=True)
        lat_ms = np.sort(lat) / 1e6
        out["poisson_half_load"] = {"offered_per_s": rate, "queries_per_s": requests / el,
                                    "p50_ms": float(lat_ms[len(lat_ms) // 2]),
                                    "p99_ms": float(lat_ms[int(0.99 * (len(lat_ms) - 1))]),
                                    "mean_batch": st["mean_batch"]}
        # Light load (5% of saturation), where requests arrive about alone: 2,048 of them.
        low = min(requests, 2048)
        rate = 0.05 * sat
        arr = np.cumsum(rng.exponential(1e9 / rate, low)).astype(np.uint64)
        _, _, lat, el = loop.replay(db, store, sids[warm:warm + low], handles[warm:warm + low], seeds[warm:warm + low],
                                    bs[warm:warm + low], ms, arrival_ns=arr)
        st = loop.stats(reset=True)
        lat_ms = np.sort(lat) / 1e6
        out["poisson_light_load"] = {"offered_per_s": rate, "queries_per_s": low / el, "requests": low,
                                     "p50_ms": float(lat_ms[len(lat_ms) // 2]),
                                     "p99_ms": float(lat_ms[int(0.99 * (len(lat_ms) - 1))]),
                                     "mean_batch": st["mean_batch"]}
    return out, cases


def plain_leg(pkg, crs, db, keys, queries, ms):
    """One query per call through respond_seeded_inspiring with the packing key inline
    (respond.rs:1218-1226): per call the key's seat is built, the shard scanned and the
    query answered alone. Host buffers; latency per call."""
    lat = []
    calls = [pkg.SeededClientQuery(q.shard_id, q.seed, q.b, inspiring_packing_keys=keys) for q in queries]
    for q in calls[:3]:
        pkg.respond_seeded_inspiring(crs, db, q, mod_switch_target=ms)
    t0 = time.perf_counter()
    for q in calls:
        t = time.perf_counter()
        pkg.respond_seeded_inspiring(crs, db, q, mod_switch_target=ms)
        lat.append(time.perf_counter() - t)
    total = time.perf_counter() - t0
    lat.sort()
    return {"calls": len(calls), "queries_per_s": len(calls) / total, "p50_ms": 1e3 * lat[len(lat) // 2],
            "p99_ms": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))]}


def small_batch_leg(pkg, ctx, crs, db, cache, store, handle, shards, rng, ms, calls=20):
    """Latency of small batches under each launch shape: batches of 7 and 1 through
    respond_seeded_batch (host buffers, one synchronous call at a time), at one, two and four
    CTAs per query, and the shape the context picks for that batch alone. Inside a profiler
    range, so an ncu --profile-from-start off capture with -k regex:k_respond_quad -c 1 takes
    the first four-CTA launch of 7 queries."""
    out = {}
    for count in (7, 1):
        qs = [pkg.SeededBatchQuery(int(rng.integers(0, shards)), rng.bytes(32), rand_words(rng, N_RING))
              for _ in range(count)]
        batch = pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(handle), qs)
        row = {"auto_shape": ctx.launch_shape_for(GAMMA, count)}
        for shape in (4, 2, 1):
            ctx.set_launch_shape(shape)
            lat = []
            for r in range(3 + calls):
                t = time.perf_counter()
                pkg.respond_seeded_batch(crs, db, batch, cache, store, mod_switch_target=ms)
                if r >= 3:
                    lat.append(time.perf_counter() - t)
            lat.sort()
            row[f"ctas{shape}"] = {"p50_ms": 1e3 * lat[len(lat) // 2], "max_ms": 1e3 * lat[-1]}
        ctx.set_launch_shape(0)
        out[f"batch{count}"] = row
    out["call"] = f"respond_seeded_batch, host buffers, {calls} timed calls after 3 untimed"
    return out


def run_gb300(args, rank, world):
    import torch

    from __graft_entry__ import _package
    pkg = _package()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = open_context(pkg, local)
    rng = np.random.default_rng(1000 + rank)

    params = pkg.InspireParams.d2048()
    w_seed = rng.integers(0, 256, 32, dtype=np.uint8).tobytes()
    crs = pkg.ServerCrs(params, w_seed, GAMMA)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase(cache, args.shards)
    t_setup = time.perf_counter()
    for s in range(args.shards):
        cols = shard_columns_device(torch, rank, s)
        torch.cuda.current_stream().synchronize()
        db.set_shard_device(s, cols.data_ptr())
    db.precompute_packing_all()
    setup_s = time.perf_counter() - t_setup
    store = pkg.ServerSessionStore.new(ctx)
    y_body = rand_words(rng, (3, N_RING))
    keys = pkg.ClientPackingKeys(y_body, GAMMA)
    handle = store.register_server_side(keys, cache)

    bps = args.batches_per_step
    total = (args.warmup + args.steps) * bps  # batches
    first_timed = args.warmup * bps
    shard_ids = [np.ascontiguousarray(rng.integers(0, args.shards * N_RING, size=BATCH) // N_RING, dtype=np.uint32)
                 for _ in range(total)]
    seeds_h = rng.integers(0, 256, size=(total, BATCH, 32), dtype=np.uint8)
    bs_h = rand_words(rng, (total, BATCH, N_RING))
    d_seeds = torch.from_numpy(seeds_h).cuda()
    d_bs = torch.from_numpy(bs_h.view(np.int64)).cuda()
    lanes = args.lanes
    d_a = torch.empty((lanes, BATCH, N_RING), dtype=torch.int64, device="cuda")
    d_b = torch.empty((lanes, BATCH, N_RING), dtype=torch.int64, device="cuda")
    d_status = torch.zeros((lanes, BATCH), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    lib = ctx._lib
    stream = torch.cuda.ExternalStream(ctx.stream)
    # Consecutive batches of 64 rotate over `lanes` streams, so each batch's scan and
    # recursion overlap the ones before it; with more than one lane the batches run one CTA
    # per query (64 x lanes CTAs in flight), with one lane two CTAs per query.
    pair_default = 76
    q_in_flight = BATCH * lanes
    shape = ("quad (4 CTAs per query)" if 2 * q_in_flight <= pair_default else
             "pair (2 CTAs per query)" if q_in_flight <= pair_default else "single (1 CTA per query)")

    def batch(i):
        k = i % lanes
        ctx.check(lib.ig_respond_seeded_batch_device(
            ctx.h, db.h, store.h, int(handle), BATCH, shard_ids[i].ctypes.data, d_seeds[i].data_ptr(),
            d_bs[i].data_ptr(), MS_TARGET, d_a[k].data_ptr(), d_b[k].data_ptr(), d_status[k].data_ptr()))

    ctx.set_lanes(lanes)
    for i in range(first_timed):
        batch(i)
    ctx.join()
    torch.cuda.synchronize()
    stream.synchronize()
    ctx.set_lanes(lanes)  # restart the rotation at lane 0
    launches0 = ctx.launch_count
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    stream.synchronize()
    with ClockSampler(local) as clk:
        torch.cuda.profiler.start()  # bounds an ncu --profile-from-start off capture
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for i in range(first_timed, total):
                batch(i)
            ctx.join()
            ev1.record(stream)
        torch.cuda.synchronize()
        stream.synchronize()
        torch.cuda.profiler.stop()
    barrier(world)
    ms_total = ev0.elapsed_time(ev1)
    launches = ctx.launch_count - launches0
    if int(d_status.abs().sum().item()) != 0:
        raise RuntimeError("a batch was refused during the timed region")
    ms_max = max_over_ranks(ms_total, world)
    timed_queries = BATCH * (total - first_timed)
    value = world * timed_queries / (ms_max / 1e3)

    # Byte check of what was timed, outside the timing: the last two batches' outputs are
    # still in their lanes; two queries of each (first and last of the batch) against the
    # oracle's store path on the same shards, key and queries.
    from oracle import oracle as O
    O.build()
    cache_o = O.Cache(O.Params.d2048(), GAMMA, w_seed)
    a_h = d_a.cpu().numpy().view(np.uint64)
    b_h = d_b.cpu().numpy().view(np.uint64)
    cases = []
    # The last batch of each lane still holds its outputs: the last two batches with two or
    # more lanes, the last one with one lane (four queries of it then).
    last = [total - 1, total - 2] if lanes > 1 else [total - 1]
    picks = (0, BATCH - 1) if lanes > 1 else (0, 1, BATCH - 2, BATCH - 1)
    for i in last:
        for k in picks:
            cases.append((int(shard_ids[i][k]), seeds_h[i, k].tobytes(), bs_h[i, k], a_h[i % lanes, k],
                          b_h[i % lanes, k]))

    def cols_of(sid):
        return shard_columns_device(torch, rank, sid).cpu().numpy().view(np.uint64)

    checked = oracle_check(O, cache_o, y_body, cols_of, cases)

    # Kernel rooflines: the same batches one at a time (one lane, the launch shape of the
    # timed region), each kernel bracketed by CUDA events on the stream it runs on.
    ctx.set_lanes(1)
    if lanes > 1:
        ctx.set_pair_threshold(0)
    ctx.profile(True)
    prof_batches = min(total - first_timed, 20)
    for i in range(3):
        batch(i)
    ctx.profile_read(reset=True)
    for i in range(first_timed, first_timed + prof_batches):
        batch(i)
    prof = ctx.profile_read(reset=True)
    ctx.profile(False)
    ctx.set_pair_threshold(pair_default)

    # e2e: the public API with host buffers (H2D of seeds and b, D2H of a and b), one
    # synchronous respond_seeded_batch call per batch of 64 from `lanes` caller threads, as a
    # server's worker pool would issue them; with lanes > 1 the calls overlap on the device.
    import threading

    e2e_queries = [[pkg.SeededBatchQuery(int(shard_ids[i][k]), seeds_h[i, k].tobytes(), bs_h[i, k])
                    for k in range(BATCH)] for i in range(total)]
    batches = [pkg.SeededQueryBatch(pkg.PackingKeySource.Registered(handle), qs) for qs in e2e_queries]
    ctx.set_lanes(lanes)
    served = [0] * lanes
    errors = []
    last_out = {}

    def caller(t, idx):
        try:
            for i in idx:
                out = pkg.respond_seeded_batch(crs, db, batches[i], cache, store, mod_switch_target=MS_TARGET)
                served[t] += len(out)
                if i == total - 1:
                    last_out[i] = out
        except Exception as e:  # reported below
            errors.append(e)

    def run_callers(indices):
        threads = [threading.Thread(target=caller, args=(t, indices[t::lanes])) for t in range(lanes)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()

    run_callers(list(range(first_timed)))
    served = [0] * lanes
    barrier(world)
    t0 = time.perf_counter()
    run_callers(list(range(first_timed, total)))
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    ctx.set_lanes(1)
    if errors:
        raise errors[0]
    assert sum(served) == timed_queries
    e2e_value = world * timed_queries / e2e_s
    # The host-buffer path's last batch: the same bytes as the device path's.
    for k in (0, BATCH - 1):
        r = last_out[total - 1][k]
        if not (np.array_equal(np.asarray(r.a, dtype=np.uint64), a_h[(total - 1) % lanes, k]) and
                np.array_equal(np.asarray(r.b, dtype=np.uint64)[:GAMMA], b_h[(total - 1) % lanes, k][:GAMMA])):
            raise RuntimeError("respond_seeded_batch differs from the device path on the same batch")

    serving, serve_cases = serve_leg(pkg, ctx, db, store, handle, args.shards, rng, MS_TARGET, slots=lanes)
    checked += oracle_check(O, cache_o, y_body, cols_of, serve_cases)
    plain = plain_leg(pkg, crs, db, keys, [q for qs in e2e_queries[:1] for q in qs], MS_TARGET)
    torch.cuda.profiler.start()
    small = small_batch_leg(pkg, ctx, crs, db, cache, store, handle, args.shards, rng, MS_TARGET)
    torch.cuda.profiler.stop()

    scan_ms, scan_n = prof["scan"]
    resp_ms, resp_n = prof["respond"]
    scan_avg = scan_ms / max(scan_n, 1)
    resp_avg = resp_ms / max(resp_n, 1)
    # Algorithmic bytes of one scan launch. The shards hold 16-bit record words, which the
    # library keeps as a u16 copy for the scan: per query the gamma columns at 2 bytes a
    # word, the query's b (n words) and gamma folded words out.
    scan_bytes = BATCH * (GAMMA * N_RING * 2 + N_RING * 8 + GAMMA * 8)
    hbm_peak, peak_kind = peaks()
    achieved = scan_bytes / (scan_avg / 1e3) / 1e9
    # The respond kernel is bound by the heavy integer pipe: its roofline counts that pipe's
    # busy cycles (ncu's per-query count, RESPOND_HEAVY_CYCLES_PER_QUERY) against the cycles
    # the pipe offers, four per SM per clock at the SM clock sampled during the timed region.
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    clk_sum = clk.summary()
    mhz = clk_sum["sm_mhz"] or 2070.0
    heavy_achieved = value / world * RESPOND_HEAVY_CYCLES_PER_QUERY / 1e9  # G pipe-cycles/s per GPU
    heavy_peak = sms * 4 * mhz * 1e6 / 1e9
    # Cross-check: modular products per second against a register-only butterfly loop (3
    # transforms of n/2 log n butterflies per link; per slot 7 pointwise products and 2
    # Montgomery reductions of 2 products each).
    links = GAMMA - 1
    modmul_per_query = links * (3 * (N_RING // 2) * 11 + 11 * N_RING) + 3 * (N_RING // 2) * 11
    timed_gmodmul = value / world * modmul_per_query / 1e9
    peak_gmodmul = ctx.butterfly_peak() / 1e9
    return {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 (exact mod q = 2^60-2^14+1)",
        "data": "synthetic: uniform 16-bit column words (uniform record bytes), uniform key/query words mod q",
        "config": dict(CONFIG, **({"shards": args.shards, "records": args.shards * N_RING}
                                  if args.shards != NUM_SHARDS else {})),
        "step": f"{bps} batches of {BATCH} queries, each one respond_seeded_batch_device call "
                f"({bps * BATCH} queries a step)",
        "execution": {"parallelism": f"replicas x{world}" if world > 1 else "single GPU", "lanes": lanes,
                      "launch_shape": shape},
        "parity_checked": checked,
        "parity_note": "outside the timing: 4 responses of the timed region's last batches (first and last "
                       "query of the last two, or four queries of the last with one lane) and 2 served by the "
                       "serving loop, recomputed by the oracle's store path on the same 2^20-record database, "
                       "key and queries, 36-bit switch: wire bytes equal",
        "db_gbs": value * SHARD_DB_BYTES / 1e9,
        "e2e": {"value": e2e_value, "unit": "queries/s",
                "h2d_bytes_per_step": bps * BATCH * (32 + N_RING * 8 + 4),
                "d2h_bytes_per_step": bps * BATCH * 2 * N_RING * 8,
                "callers": lanes, "call": "respond_seeded_batch (one batch of 64 per call)"},
        "roofline": {"kernel": "shard_scan", "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak,
                     "traffic": SCAN_TRAFFIC_BYTES if args.shards == NUM_SHARDS else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, same workload",
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "avg_launch_ms": scan_avg, "algorithmic_bytes_per_launch": scan_bytes,
                     "timing": "one batch of 64 at a time on one lane, CUDA events around each scan launch",
                     "note": "the HBM-facing kernel; the dominant kernel is in roofline_dominant"},
        "roofline_dominant": {"kernel": "respond (fused recursion + online gather, one CTA per query)",
                              "bound": "heavy integer multiply pipe (IMAD/IMAD.WIDE/IMAD.HI)",
                              "achieved": heavy_achieved, "peak": heavy_peak,
                              "unit": "G heavy-pipe sub-partition cycles/s",
                              "frac": heavy_achieved / heavy_peak,
                              "achieved_note": "queries/s over the timed region x the pipe's busy cycles per query "
                                               "(ncu, RESPOND_HEAVY_CYCLES_PER_QUERY)",
                              "peak_source": f"{sms} SMs x 4 sub-partitions x the sampled SM clock ({mhz:.0f} MHz)",
                              "avg_launch_ms": resp_avg, "heavy_cycles_per_query": RESPOND_HEAVY_CYCLES_PER_QUERY,
                              "cross_check": {"unit": "G modmul/s", "achieved": timed_gmodmul,
                                              "butterfly_probe": peak_gmodmul,
                                              "frac_of_probe": timed_gmodmul / peak_gmodmul,
                                              "modmul_per_query": modmul_per_query},
                              "launch_shape": shape, "queries_per_launch": BATCH},
        "gpu_launches": int(launches),
        "setup_s": setup_s,
        "clocks": clk_sum,
        "serving": serving,
        "plain": plain,
        "small_batches": small,
    }


# ------------------------------------------------------------------------------------
# special_modulus workload: ring2048_cell256, 2^22 cells of 256 bytes
# (2048 shards, 1 GiB), a ShardTable per shard, 8 seated keys, batches of 256 uniform rows.
SM_METRIC = "special_modulus respond queries/s (batch 256, 2^22 x 256 B cells, 8 seated keys)"
SM_CONFIG = {"workload": "special_modulus ring2048_cell256: 2^22 cells x 256 B (2048 shards), ShardTable per "
                         "shard, 8 seated keys, batch 256 uniform rows",
             "ring_dim": 2048, "gamma": 512, "cells": 1 << 22, "shards": 2048, "batch": 256, "keys": 8,
             "l2": "inputs larger than L2: each step reads 256 random shards' tables (5 MiB each)"}


def sm_cpu_sample(steps, warmup, queries_per_step=4, seed=12):
    from oracle import oracle as O

    O.build()
    rng = np.random.default_rng(seed)
    server = O.SmServer()
    cells = np.zeros((2048, 256), dtype=np.uint8)
    cells[:, :246] = rng.integers(0, 256, (2048, 246), dtype=np.uint8)
    table = server.table(cells.tobytes())
    client = O.SmClient(rng.bytes(32))
    seat = server.seat(client.key())
    times = []
    for step in range(warmup + steps):
        qs = [client.query(int(rng.integers(0, 2048))) for _ in range(queries_per_step)]
        t0 = time.perf_counter()
        for seed_b, body in qs:
            server.respond(table, seat, seed_b, body)
        if step >= warmup:
            times.append(time.perf_counter() - t0)
    return {"value": queries_per_step * len(times) / sum(times), "unit": "queries/s", "cores": 1, "kind": "port",
            "sample": f"{queries_per_step} queries per step, {steps} steps, one shard table (oracle, one thread as "
                      "the reference's respond_impl)"}


def run_sm(args, rank, world):
    import torch

    from __graft_entry__ import _package
    pkg = _package()
    sm = pkg.special_modulus
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = open_context(pkg, local)
    rng = np.random.default_rng(2 + rank)
    server = sm.Server(ctx=ctx)
    shards = args.shards if args.shards != NUM_SHARDS else 2048
    t_setup = time.perf_counter()

    def shard_cells(s):  # regenerable per shard, for the oracle check
        cells = np.zeros((2048, 256), dtype=np.uint8)
        cells[:, :246] = np.random.default_rng((2 + rank, s)).integers(0, 256, (2048, 246), dtype=np.uint8)
        return cells.tobytes()

    tables = [server.table(shard_cells(s)) for s in range(shards)]
    seats, keys = [], []
    for k in range(8):
        key = (rng.bytes(32), rng.integers(0, 536_813_569, 2048, dtype=np.uint32),
               rng.integers(0, 2_147_389_441, 2048, dtype=np.uint32))
        keys.append(key)
        seats.append(server.seat(sm.PackingKey(*key)))
    setup_s = time.perf_counter() - t_setup
    B = 256
    total = args.warmup + args.steps
    tidx = [rng.integers(0, shards, B) for _ in range(total)]
    sidx = [rng.integers(0, 8, B) for _ in range(total)]
    tsel = [np.array([tables[i] for i in t], dtype=np.uint64) for t in tidx]
    ssel = [np.array([seats[i] for i in t], dtype=np.uint64) for t in sidx]
    seeds_h = rng.integers(0, 256, (total, B, 32), dtype=np.uint8)
    bodies_h = rng.integers(0, 536_813_569, (total, B, 2048), dtype=np.uint32)
    d_seeds = torch.from_numpy(seeds_h).cuda()
    d_bodies = torch.from_numpy(bodies_h.view(np.int32)).cuda()
    lanes = args.lanes
    d_mask = torch.empty((lanes, B, 2048), dtype=torch.int32, device="cuda")
    d_body = torch.empty((lanes, B, 492), dtype=torch.int32, device="cuda")
    d_status = torch.zeros((lanes, B), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    lib = ctx._lib

    def step(i):
        k = i % lanes
        ctx.check(lib.ig_sm_respond_batch_device(ctx.h, server.h, B, tsel[i].ctypes.data, ssel[i].ctypes.data,
                                                  d_seeds[i].data_ptr(), d_bodies[i].data_ptr(), d_mask[k].data_ptr(),
                                                  d_body[k].data_ptr(), d_status[k].data_ptr()))

    stream = torch.cuda.ExternalStream(ctx.stream)
    ctx.set_lanes(lanes)
    for i in range(args.warmup):
        step(i)
    ctx.join()
    torch.cuda.synchronize()
    stream.synchronize()
    ctx.set_lanes(lanes)
    launches0 = ctx.launch_count
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    with ClockSampler(local) as clk:
        torch.cuda.profiler.start()  # bounds an ncu --profile-from-start off capture
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for i in range(args.warmup, total):
                step(i)
            ctx.join()
            ev1.record(stream)
        torch.cuda.synchronize()
        stream.synchronize()
        torch.cuda.profiler.stop()
    launches = ctx.launch_count - launches0
    ctx.set_lanes(1)
    barrier(world)
    if int(d_status.abs().sum().item()) != 0:
        raise RuntimeError("a special-modulus batch reported a device status")
    # Byte check outside the timing: the last batch's first and last queries (its outputs
    # are still in their lane) against the oracle's Server::respond on the same table, key
    # and query.
    from oracle import oracle as O
    O.build()
    oserver = O.SmServer()
    last = total - 1
    mask_h = d_mask[last % lanes].cpu().numpy().view(np.uint32)
    body_h = d_body[last % lanes].cpu().numpy().view(np.uint32)
    checked = 0
    for k in (0, B - 1):
        otable = oserver.table(shard_cells(int(tidx[last][k])))
        oseat = oserver.seat(keys[int(sidx[last][k])])
        m_o, b_o = oserver.respond(otable, oseat, seeds_h[last, k].tobytes(), bodies_h[last, k])
        if not (np.array_equal(m_o, mask_h[k]) and np.array_equal(b_o, body_h[k])):
            raise RuntimeError(f"special_modulus response differs from the oracle (query {k} of the last batch)")
        checked += 1
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    value = world * B * args.steps / (ms / 1e3)
    # e2e: Server::respond for each batch with host buffers, from `lanes` caller threads
    # whose calls overlap on the device (each holds a lane while its batch runs).
    import threading

    qobjs = [[sm.Query(seeds_h[i, k].tobytes(), bodies_h[i, k]) for k in range(B)] for i in range(total)]
    ctx.set_lanes(lanes)
    errors = []

    def caller(idx):
        try:
            for i in idx:
                server.respond_batch(list(tsel[i]), list(ssel[i]), qobjs[i])
        except Exception as e:  # reported below
            errors.append(e)

    def run_callers(indices):
        threads = [threading.Thread(target=caller, args=(indices[t::lanes],)) for t in range(lanes)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()

    run_callers(list(range(args.warmup)))
    t0 = time.perf_counter()
    run_callers(list(range(args.warmup, total)))
    e2e = world * B * args.steps / max_over_ranks(time.perf_counter() - t0, world)
    ctx.set_lanes(1)
    if errors:
        raise errors[0]
    return {
        "metric": SM_METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 (exact mod q and p)",
        "data": "synthetic: uniform record bytes, uniform key and query words",
        "config": dict(SM_CONFIG, shards=shards, lanes=lanes),
        "parity_checked": checked,
        "db_gbs": value * 2048 * 256 / 1e9,
        "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": B * (32 + 2048 * 4),
                "d2h_bytes_per_step": B * (2048 + 492) * 4, "callers": lanes},
        "gpu_launches": int(launches), "setup_s": setup_s, "clocks": clk.summary(),
    }


# ------------------------------------------------------------------------------------
# Serving sweep: 2^25 records of 512 B (16,384 shards, 16 GiB of
# records) encoded on the GPU, a store on every shard, 1000 registered seats, requests with
# uniform index and seat through the continuous-batching loop, driven natively: a closed
# loop to saturation, then Poisson arrivals at fractions of the saturation rate.
# ------------------------------------------------------------------------------------
# OnePacking (the Galois-automorphism tree responder) over the served-batch database:
# 2^20 records of 512 B (512 shards, gamma 256), batches of 152 seeded queries (one per SM)
# through respond_one_packing_batch with host buffers. The Galois keys are uniform words:
# the tree's work does not depend on their values.
TREE_METRIC = "OnePacking respond queries/s (batch 152, d2048, 512 B records, 2^20 records)"


def run_tree(args, rank, world):
    import threading

    import torch

    from __graft_entry__ import _package
    pkg = _package()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = open_context(pkg, local)
    g = torch.Generator(device="cuda")
    g.manual_seed(1 + rank)
    rng = np.random.default_rng(2000 + rank)
    log_n = N_RING.bit_length() - 1
    keys = rand_words(rng, (log_n, 3, 2, N_RING))
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), rng.integers(0, 256, 32, dtype=np.uint8).tobytes(), GAMMA,
                        galois_keys=keys)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase(cache, args.shards)
    for s in range(args.shards):
        cols = torch.randint(0, 1 << 16, (GAMMA, N_RING), generator=g, device="cuda", dtype=torch.int64)
        torch.cuda.current_stream().synchronize()
        db.set_shard_device(s, cols.data_ptr())
    B = 152
    total = args.warmup + args.steps
    batches = [[pkg.SeededBatchQuery(int(rng.integers(0, args.shards)), rng.bytes(32), rand_words(rng, N_RING))
                for _ in range(B)] for _ in range(total)]
    # Caller threads over as many lanes, as a server's worker pool would issue the calls.
    T = max(1, args.lanes)
    ctx.set_lanes(T)

    def run(lo, hi):
        errors = []

        def caller(t):
            try:
                for i in range(lo + t, hi, T):
                    pkg.respond_one_packing_batch(crs, db, batches[i])
            except Exception as e:
                errors.append(e)
        threads = [threading.Thread(target=caller, args=(t,)) for t in range(T)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]

    run(0, args.warmup)
    launches0 = ctx.launch_count
    barrier(world)
    with ClockSampler(local) as clk:
        torch.cuda.profiler.start()
        t0 = time.perf_counter()
        run(args.warmup, total)
        el = max_over_ranks(time.perf_counter() - t0, world)
        torch.cuda.profiler.stop()
    ctx.set_lanes(1)
    value = world * B * args.steps / el
    return {
        "metric": TREE_METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 (exact mod q = 2^60-2^14+1)",
        "data": "synthetic: uniform 16-bit column words, uniform query words and Galois-key words",
        "config": {"workload": "d2048 OnePacking, 512-byte records x 2^20 (512 shards, gamma 256), batch 152, "
                               "unswitched", "shards": args.shards, "batch": B, "callers": T, "lanes": T},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": B * (32 + N_RING * 8 + 4),
                "d2h_bytes_per_step": B * 2 * N_RING * 8,
                "note": "host buffers in and out: one respond_one_packing_batch call per step, from the caller "
                        "threads"},
        "gpu_launches": int(ctx.launch_count - launches0), "clocks": clk.summary(),
    }


# ------------------------------------------------------------------------------------
# NoPacking (respond / respond_seeded, respond.rs:614-643, 1229-1237): the served-batch
# database, batches of 16 seeded queries through the C ABI with host buffers. A response
# is gamma + 1 ciphertexts (8.4 MB at gamma 256), so the batch is small.
NOPACK_METRIC = "NoPacking respond queries/s (batch 16, d2048, 512 B records, 2^20 records)"


def run_nopack(args, rank, world):
    import threading

    import torch

    from __graft_entry__ import _package
    pkg = _package()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = open_context(pkg, local)
    g = torch.Generator(device="cuda")
    g.manual_seed(1 + rank)
    rng = np.random.default_rng(3000 + rank)
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), rng.integers(0, 256, 32, dtype=np.uint8).tobytes(), GAMMA)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    db = pkg.EncodedDatabase(cache, args.shards)
    for s in range(args.shards):
        cols = torch.randint(0, 1 << 16, (GAMMA, N_RING), generator=g, device="cuda", dtype=torch.int64)
        torch.cuda.current_stream().synchronize()
        db.set_shard_device(s, cols.data_ptr())
    B = 16
    total = args.warmup + args.steps
    sids = [np.ascontiguousarray(rng.integers(0, args.shards, B), dtype=np.uint32) for _ in range(total)]
    seeds = [np.frombuffer(rng.bytes(32 * B), dtype=np.uint8).copy() for _ in range(total)]
    bs = [rand_words(rng, (B, N_RING)) for _ in range(total)]
    # Caller threads over as many lanes, as a server's worker pool would issue the calls;
    # each lands its responses in its own pinned host buffer.
    T = max(1, args.lanes)
    ctx.set_lanes(T)
    outs = [torch.empty((B, GAMMA + 1, 2, N_RING), dtype=torch.int64, pin_memory=True) for _ in range(T)]
    lib = ctx._lib

    def step(i, t):
        ctx.check(lib.ig_respond_nopacking_batch(ctx.h, db.h, B, sids[i].ctypes.data, seeds[i].ctypes.data, None,
                                                 bs[i].ctypes.data, outs[t].data_ptr()))

    def run(lo, hi):
        errors = []

        def caller(t):
            try:
                for i in range(lo + t, hi, T):
                    step(i, t)
            except Exception as e:
                errors.append(e)
        threads = [threading.Thread(target=caller, args=(t,)) for t in range(T)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]

    run(0, args.warmup)
    launches0 = ctx.launch_count
    barrier(world)
    with ClockSampler(local) as clk:
        torch.cuda.profiler.start()
        t0 = time.perf_counter()
        run(args.warmup, total)
        el = max_over_ranks(time.perf_counter() - t0, world)
        torch.cuda.profiler.stop()
    ctx.set_lanes(1)
    value = world * B * args.steps / el
    return {
        "metric": NOPACK_METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 (exact mod q = 2^60-2^14+1)",
        "data": "synthetic: uniform 16-bit column words, uniform query words",
        "config": {"workload": "d2048 NoPacking, 512-byte records x 2^20 (512 shards, gamma 256), batch 16, "
                               "seeded queries", "shards": args.shards, "batch": B, "callers": T, "lanes": T},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": B * (32 + N_RING * 8 + 4),
                "d2h_bytes_per_step": B * (GAMMA + 1) * 2 * N_RING * 8,
                "note": "host buffers in and out (responses into pinned memory): one ig_respond_nopacking_batch "
                        "call per step, from the caller threads"},
        "gpu_launches": int(ctx.launch_count - launches0), "clocks": clk.summary(),
    }


# ------------------------------------------------------------------------------------
# Uneven batching over three resident databases: 32 B x 2^22 (gamma 16, 2048 shards), 512 B
# x 2^20 (gamma 256, 512 shards), 2048 B x 2^18 (gamma 1024, 128 shards), records of uniform
# bytes from seeds 3, 4 and 5 encoded on the GPU. 128 keys, half under d2048 and half under
# d2048_approximate_gadget, each registered under one (database width, gadget) set; a
# database serves both gadgets' seats from one store. Every launch carries a batch of a size
# drawn from {1, 7, 33, 128, 512} whose members each draw a key (so they span all three
# databases and both gadgets) and a uniform shard; responses unswitched.
C4_DBS = [(32, 2048, 3), (512, 512, 4), (2048, 128, 5)]  # entry bytes, shards, seed
C4_KEYS = 128
C4_BATCHES = (1, 7, 33, 128, 512)
C4_METRIC = ("uneven-batch respond queries/s (members across 32/512/2048 B record databases and both gadgets, "
             "128 keys, batch sizes 1-512)")


def c4_records(torch, entry, shards, seed, rank):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed + 1000 * rank)
    return torch.randint(0, 256, (shards * N_RING * entry,), dtype=torch.uint8, device="cuda", generator=g)


def run_cfg4(args, rank, world):
    import threading

    import torch

    from __graft_entry__ import _package
    pkg = _package()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = open_context(pkg, local)
    rng = np.random.default_rng(4 + rank)
    store = pkg.ServerSessionStore.new(ctx)
    dbs = []
    t0 = time.perf_counter()
    for entry, shards, seed in C4_DBS:
        if args.shards != NUM_SHARDS:
            shards = max(1, min(shards, args.shards))
        gamma = (entry + 1) // 2
        rec = c4_records(torch, entry, shards, seed, rank)
        torch.cuda.current_stream().synchronize()
        crs = pkg.ServerCrs(pkg.InspireParams.d2048(), rng.integers(0, 256, 32, dtype=np.uint8).tobytes(), gamma)
        cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
        db = pkg.EncodedDatabase(cache, shards)
        db.encode_records(None, entry, device_ptr=rec.data_ptr(), nbytes=rec.numel())
        db.precompute_packing_all()
        del rec
        torch.cuda.empty_cache()
        # The approximate gadget's set of the same width: its seats run on this database.
        crs_a = pkg.ServerCrs(pkg.InspireParams.d2048_approximate_gadget(),
                              rng.integers(0, 256, 32, dtype=np.uint8).tobytes(), gamma)
        cache_a = pkg.ServerInspiringCache.new(crs_a, ctx=ctx)
        dbs.append({"entry": entry, "gamma": gamma, "shards": shards, "seed": seed, "db": db,
                    "sets": [(crs, cache), (crs_a, cache_a)]})
    keys = []  # (database index, gadget index, y_body, handle)
    for k in range(C4_KEYS):
        di, gi = k % len(dbs), (k // len(dbs)) % 2
        d = dbs[di]
        rows = 2 if gi else 3
        y = rand_words(rng, (rows, N_RING))
        h = store.register_server_side(pkg.ClientPackingKeys(y, d["gamma"]), d["sets"][gi][1])
        keys.append((di, gi, y, int(h)))
    setup_s = time.perf_counter() - t0

    total = args.warmup + args.steps
    plan = []  # per launch: key indices, shard ids
    for i in range(total):
        count = int(rng.choice(C4_BATCHES))
        kidx = rng.integers(0, C4_KEYS, count)
        sids = np.array([int(rng.integers(0, dbs[keys[k][0]]["shards"])) for k in kidx], dtype=np.uint32)
        plan.append((count, kidx, sids))
    offs = np.cumsum([0] + [p[0] for p in plan])
    nq = int(offs[-1])
    seeds_h = rng.integers(0, 256, (nq, 32), dtype=np.uint8)
    bs_h = rand_words(rng, (nq, N_RING))
    d_seeds = torch.from_numpy(seeds_h).cuda()
    d_bs = torch.from_numpy(bs_h.view(np.int64)).cuda()
    d_a = torch.empty((nq, N_RING), dtype=torch.int64, device="cuda")
    d_b = torch.empty_like(d_a)
    d_status = torch.zeros(nq, dtype=torch.int32, device="cuda")
    arrays = []
    for count, kidx, sids in plan:
        arrays.append((np.array([dbs[keys[k][0]]["db"].h for k in kidx], dtype=np.uint64),
                       np.full(count, store.h, dtype=np.uint64),
                       np.array([keys[k][3] for k in kidx], dtype=np.uint64), sids,
                       np.zeros(count, dtype=np.uint64)))
    torch.cuda.synchronize()
    lib = ctx._lib
    stream = torch.cuda.ExternalStream(ctx.stream)
    lanes = args.lanes

    def launch(i):
        count = plan[i][0]
        dbh, sth, hh, sids, ms = arrays[i]
        o = int(offs[i])
        ctx.check(lib.ig_respond_mixed_batch_device(
            ctx.h, count, dbh.ctypes.data, sth.ctypes.data, hh.ctypes.data, sids.ctypes.data, d_seeds[o].data_ptr(),
            d_bs[o].data_ptr(), ms.ctypes.data, d_a[o].data_ptr(), d_b[o].data_ptr(), d_status[o:].data_ptr()))

    def timed_region():
        ctx.set_lanes(lanes)
        for i in range(args.warmup):
            launch(i)
        ctx.join()
        stream.synchronize()
        torch.cuda.synchronize()
        ctx.set_lanes(lanes)
        launches0 = ctx.launch_count
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(world)
        with ClockSampler(local) as clk:
            with torch.cuda.stream(stream):
                ev0.record(stream)
                for i in range(args.warmup, total):
                    launch(i)
                ctx.join()
                ev1.record(stream)
            stream.synchronize()
            torch.cuda.synchronize()
        ctx.set_lanes(1)
        if int(d_status.abs().sum().item()) != 0:
            raise RuntimeError("a launch was refused during the timed region")
        return max_over_ranks(ev0.elapsed_time(ev1), world), ctx.launch_count - launches0, clk

    timed_queries = int(offs[-1] - offs[args.warmup])
    # The fixed rule first (no table: four CTAs per query while 2 x count x lanes <= SMs / 2, two
    # while count x lanes <= SMs / 2, else one), then
    # the launch-shape tuner's table for the three widths, then the same launches tuned.
    ms_fixed, _, _ = timed_region()
    t0 = time.perf_counter()
    tuned = ctx.tune_launch_shapes([d["gamma"] for d in dbs], reps=2)
    tune_s = time.perf_counter() - t0
    ms_t, launches, clk = timed_region()
    value = world * timed_queries / (ms_t / 1e3)
    fixed_value = world * timed_queries / (ms_fixed / 1e3)

    # Byte check outside the timing: the last launch's members from each database against
    # the oracle's store path under the member's own key and set.
    from oracle import oracle as O
    O.build()
    a_h = d_a.cpu().numpy().view(np.uint64)
    b_h = d_b.cpu().numpy().view(np.uint64)
    checked, seen = 0, set()
    i_last = total - 1
    while len(seen) < len(dbs) and i_last >= args.warmup:
        count, kidx, sids = plan[i_last]
        for j in range(count):
            di, gi, y, _ = keys[kidx[j]]
            if di in seen:
                continue
            seen.add(di)
            d = dbs[di]
            crs_j = d["sets"][gi][0]
            P = O.Params.d2048_approximate_gadget() if gi else O.Params.d2048()
            rec = c4_records(torch, d["entry"], d["shards"], d["seed"], rank)
            s0 = int(sids[j]) * N_RING * d["entry"]
            shard_bytes = rec[s0:s0 + N_RING * d["entry"]].cpu().numpy()
            cols = np.ascontiguousarray(shard_bytes.view("<u2").reshape(N_RING, d["gamma"]).T, dtype=np.uint64)
            st = O.Store(O.Cache(P, d["gamma"], crs_j.inspiring_w_seed), cols)
            row = int(offs[i_last]) + j
            ao, bo = st.respond(cols, O.expand_seed(seeds_h[row].tobytes(), N_RING), bs_h[row], y)
            if O.response_bytes(ao, bo, d["gamma"]) != O.response_bytes(a_h[row], b_h[row], d["gamma"]):
                raise RuntimeError(f"mixed launch differs from the oracle (database {di}, row {row})")
            checked += 1
            del rec
        i_last -= 1
    torch.cuda.empty_cache()

    # Latency of small batches under each shape: batches of 1 and 7 on the 512-byte and the
    # 2048-byte database (gamma 256 and 1024), one synchronous host-buffer call at a time.
    latency = {}
    for di in (1, 2):
        d = dbs[di]
        hk = next(k for k in keys if k[0] == di and k[1] == 0)[3]
        cell = {}
        for count in (1, 7):
            qs_all = [pkg.MixedQuery(d["db"], store, hk,
                                     pkg.SeededBatchQuery(int(rng.integers(0, d["shards"])), rng.bytes(32),
                                                          rand_words(rng, N_RING)))
                      for _ in range(count)]
            row = {"tuned_choice": ctx.launch_shape_for(d["gamma"], count)}
            for shape in (1, 2, 4):
                ctx.set_launch_shape(shape)
                lat = []
                for r in range(43):
                    t = time.perf_counter()
                    pkg.respond_mixed_batch(qs_all)
                    if r >= 3:
                        lat.append(time.perf_counter() - t)
                lat_ms = np.sort(np.array(lat)) * 1e3
                row[str(shape)] = {"p50_ms": float(lat_ms[len(lat_ms) // 2]),
                                   "p99_ms": float(lat_ms[int(0.99 * (len(lat_ms) - 1))])}
            ctx.set_launch_shape(0)
            cell[f"batch{count}"] = row
        latency[f"gamma{d['gamma']}"] = cell

    # e2e: respond_mixed_batch with host buffers, one call per launch, from `lanes` threads.
    calls = []
    for i, (count, kidx, sids) in enumerate(plan):
        o = int(offs[i])
        calls.append([pkg.MixedQuery(dbs[keys[k][0]]["db"], store, keys[k][3],
                                     pkg.SeededBatchQuery(int(sids[j]), seeds_h[o + j].tobytes(), bs_h[o + j]))
                      for j, k in enumerate(kidx)])
    errors = []

    # The calls differ in size (1 to 512 queries), so the callers take the next call as they
    # free up, as a server's worker pool takes the next request, not a fixed share each.
    def caller(pending, lock):
        try:
            while True:
                with lock:
                    if not pending:
                        return
                    i = pending.pop()
                pkg.respond_mixed_batch(calls[i])
        except Exception as e:  # reported below
            errors.append(e)

    def run_callers(indices):
        pending, lock = list(reversed(indices)), threading.Lock()
        threads = [threading.Thread(target=caller, args=(pending, lock)) for t in range(lanes)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()

    ctx.set_lanes(lanes)
    run_callers(list(range(args.warmup)))
    t0 = time.perf_counter()
    run_callers(list(range(args.warmup, total)))
    e2e = world * timed_queries / max_over_ranks(time.perf_counter() - t0, world)
    ctx.set_lanes(1)
    if errors:
        raise errors[0]

    # The plain per-query GPU path on the same members: one call per query under its own
    # key, database and set (host buffers), over the first 512 timed members.
    flat = [q for c in calls[args.warmup:] for q in c][:512]
    t0 = time.perf_counter()
    for q in flat:
        pkg.respond_mixed_batch([q])
    plain_qps = len(flat) / (time.perf_counter() - t0)
    mix = {str(b): sum(1 for p in plan[args.warmup:] if p[0] == b) for b in C4_BATCHES}
    return {
        "metric": C4_METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 (exact mod q = 2^60-2^14+1)",
        "data": "synthetic: uniform record bytes encoded on the GPU, uniform key and query words",
        "config": {"workload": "three resident databases (32 B x 2^22 gamma 16, 512 B x 2^20 gamma 256, 2048 B x "
                               "2^18 gamma 1024; seeds 3/4/5), 128 keys half exact and half approximate gadget, "
                               "each launch a batch of a size drawn from {1, 7, 33, 128, 512} whose members draw "
                               "a key and a uniform shard, so they span all three databases and both gadgets",
                   "shards": [d["shards"] for d in dbs], "keys": C4_KEYS, "lanes": lanes,
                   "queries": timed_queries, "batch_mix": mix, "mod_switch": None,
                   "l2": "inputs larger than L2: the three databases hold about 10 GiB of columns and stores"},
        "step": "one mixed launch (ig_respond_mixed_batch_device: one scan and one respond launch)",
        "parity_checked": checked,
        "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": int(timed_queries * (32 + N_RING * 8 + 4)
                                                                            / args.steps),
                "d2h_bytes_per_step": int(timed_queries * 2 * N_RING * 8 / args.steps), "callers": lanes,
                "call": "respond_mixed_batch (one launch per call)"},
        "fixed_rule": {"value": fixed_value, "unit": "queries/s",
                       "rule": "four CTAs per query while 2 x count x lanes <= SMs / 2, two while "
                               "count x lanes <= SMs / 2, else one"},
        "launch_shapes": {"tuned_ms_per_launch": {str(g): {str(b): {"1": t[0], "2": t[1], "4": t[2]}
                                                           for b, t in rows.items()} for g, rows in tuned.items()},
                          "tune_s": tune_s,
                          "rule": "per launch the shape the table times fastest at count x lanes queries in flight"},
        "latency": latency,
        "plain_per_query": {"queries_per_s": plain_qps, "queries": len(flat),
                            "call": "one respond_mixed_batch call per query (host buffers)"},
        "gpu_launches": int(launches), "setup_s": setup_s, "clocks": clk.summary(),
        "device_bytes": ctx.device_bytes,
    }


C5_SHARDS = 16384
C5_SEATS = 1000
C5_METRIC = ("served queries/s at saturation (continuous batching, 2^25 x 512 B records, 16,384 shards, "
             "1000 seats of 3- and 2-row gadgets, 36-bit mod switch)")
C5_CHUNK = 512  # shards per piece of records generated on the device (512 MiB), seeded per piece


def c5_records(torch, s0, k, rank):
    g = torch.Generator(device="cuda")
    g.manual_seed(6 + 1000 * rank + s0 // C5_CHUNK)
    return torch.randint(0, 256, (k * N_RING * ENTRY_BYTES,), dtype=torch.uint8, device="cuda", generator=g)


def run_cfg5(args, rank, world):
    import torch

    from __graft_entry__ import _package
    pkg = _package()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = open_context(pkg, local)
    shards = args.shards if args.shards != NUM_SHARDS else C5_SHARDS
    rng = np.random.default_rng(6 + rank)
    crs = pkg.ServerCrs(pkg.InspireParams.d2048(), rng.integers(0, 256, 32, dtype=np.uint8).tobytes(), GAMMA)
    cache = pkg.ServerInspiringCache.new(crs, ctx=ctx)
    # The approximate gadget's set of the same width: its 2-row seats run on the same store.
    crs_a = pkg.ServerCrs(pkg.InspireParams.d2048_approximate_gadget(),
                          rng.integers(0, 256, 32, dtype=np.uint8).tobytes(), GAMMA)
    cache_a = pkg.ServerInspiringCache.new(crs_a, ctx=ctx)
    db = pkg.EncodedDatabase(cache, shards)
    t0 = time.perf_counter()
    for s0 in range(0, shards, C5_CHUNK):
        k = min(C5_CHUNK, shards - s0)
        rec = c5_records(torch, s0, k, rank)
        torch.cuda.current_stream().synchronize()
        db.encode_records(None, ENTRY_BYTES, device_ptr=rec.data_ptr(), nbytes=rec.numel(), first_shard=s0)
        del rec
    encode_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    db.precompute_packing_all()
    store_s = time.perf_counter() - t0
    torch.cuda.empty_cache()
    store = pkg.ServerSessionStore.new(ctx)
    seat_keys = []  # (handle, gadget, y_body): even seats 3-row exact, odd seats 2-row approximate
    for i in range(C5_SEATS):
        gi = i % 2
        y = rand_words(rng, (2 if gi else 3, N_RING))
        seat_keys.append((int(store.register_server_side(pkg.ClientPackingKeys(y, GAMMA), cache_a if gi else cache)),
                          gi, y))
    seats = [h for h, _, _ in seat_keys]
    count = args.requests
    shard_ids = rng.integers(0, shards, count).astype(np.uint32)
    handles = np.array([int(seats[i]) for i in rng.integers(0, C5_SEATS, count)], dtype=np.uint64)
    seeds = rng.integers(0, 256, (count, 32), dtype=np.uint8)
    bs = rand_words(rng, (count, N_RING))
    out = {"metric": C5_METRIC, "unit": "queries/s", "n_gpus": world, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "u64 (exact mod q = 2^60-2^14+1)",
           "data": "synthetic: uniform record bytes encoded on the GPU, uniform key and query words",
           "config": {"workload": "d2048 TwoPacking, 512-byte records x 2^25 (16,384 shards), store on every "
                                  "shard, 1000 seats (500 of 3 rows under d2048, 500 of 2 rows under "
                                  "d2048_approximate_gadget, one store serving both), uniform index and seat per "
                                  "request, 36-bit mod switch",
                      "shards": shards, "records": shards * N_RING, "seats": C5_SEATS, "requests": count,
                      "slots": args.lanes, "max_batch": BATCH},
           "setup_s": {"encode_records": encode_s, "precompute_packing": store_s},
           "device_bytes": ctx.device_bytes}
    slots = args.lanes
    with pkg.ServingLoop(ctx, slots=slots, max_batch=BATCH) as loop:
        w = min(count, 512)
        loop.replay(db, store, shard_ids[:w], handles[:w], seeds[:w], bs[:w], MS_TARGET, window=256)  # warm-up
        with ClockSampler(local) as clk:
            a_out, b_out, lat, el = loop.replay(db, store, shard_ids, handles, seeds, bs, MS_TARGET,
                                                window=4 * slots * BATCH)
        sat = count / el
        # Byte check outside the timing: one response under each gadget against the oracle.
        from oracle import oracle as O
        O.build()
        gadget_of = {h: (gi, y) for h, gi, y in seat_keys}
        checked = 0
        for want_gi in (0, 1):
            i = next(j for j in range(count) if gadget_of[int(handles[j])][0] == want_gi)
            gi, y = gadget_of[int(handles[i])]
            sid = int(shard_ids[i])
            s0 = sid - sid % C5_CHUNK
            rec = c5_records(torch, s0, min(C5_CHUNK, shards - s0), rank)
            off = (sid - s0) * N_RING * ENTRY_BYTES
            shard_bytes = rec[off:off + N_RING * ENTRY_BYTES].cpu().numpy()
            del rec
            cols = np.ascontiguousarray(shard_bytes.view("<u2").reshape(N_RING, GAMMA).T, dtype=np.uint64)
            P = O.Params.d2048_approximate_gadget() if gi else O.Params.d2048()
            w = (crs_a if gi else crs).inspiring_w_seed
            ao, bo = O.Store(O.Cache(P, GAMMA, w), cols).respond(cols, O.expand_seed(seeds[i].tobytes(), N_RING),
                                                                 bs[i], y)
            want = O.response_bytes(O.mod_switch(ao, Q, MS_TARGET), O.mod_switch(bo, Q, MS_TARGET), GAMMA, MS_TARGET)
            if O.response_bytes(a_out[i], b_out[i], GAMMA, MS_TARGET) != want:
                raise RuntimeError(f"served response differs from the oracle (request {i})")
            checked += 1
        torch.cuda.empty_cache()
        out["parity_checked"] = checked
        lat_ms = np.sort(lat) / 1e6
        out["value"] = sat
        out["saturation"] = {"queries_per_s": sat, "p50_ms": float(lat_ms[len(lat_ms) // 2]),
                             "p99_ms": float(lat_ms[int(0.99 * (len(lat_ms) - 1))]),
                             "window": 4 * slots * BATCH}
        out["clocks"] = clk.summary()
        sweep = []
        for frac in (0.05, 0.25, 0.5, 0.75, 0.9):
            rate = frac * sat
            n = min(count, max(256, int(rate * 0.6)))
            arr = np.cumsum(rng.exponential(1e9 / rate, n)).astype(np.uint64)
            _, _, lat, el = loop.replay(db, store, shard_ids[:n], handles[:n], seeds[:n], bs[:n], MS_TARGET,
                                        arrival_ns=arr)
            lat_ms = np.sort(lat) / 1e6
            sweep.append({"offered_per_s": rate, "queries_per_s": n / el, "requests": n,
                          "p50_ms": float(lat_ms[len(lat_ms) // 2]),
                          "p99_ms": float(lat_ms[int(0.99 * (len(lat_ms) - 1))])})
        out["poisson_sweep"] = sweep
        st = loop.stats()
        out["mean_batch"] = st["mean_batch"]
    out["e2e"] = {"value": out["value"], "unit": "queries/s", "h2d_bytes_per_step": BATCH * (32 + N_RING * 8 + 8),
                  "d2h_bytes_per_step": BATCH * 2 * N_RING * 8,
                  "note": "the loop's closed-loop rate: host buffers in, host buffers out"}
    out["steps"] = count // BATCH
    out["warmup"] = 1
    out["ms_per_step"] = 1e3 * BATCH / out["value"]
    return out


# The other workloads the library serves, each at its own default size and step count, run
# after the headline on one GPU so that the one JSON line carries their numbers too.
OTHER_WORKLOADS = ("special-modulus", "mixed", "serving-sweep", "one-packing", "no-packing")
# Default timed steps and lanes of each workload (the measured optimum of lanes).
DEFAULT_STEPS = {"served-batch": 20, "special-modulus": 100, "mixed": 60, "serving-sweep": 0, "one-packing": 20,
                 "no-packing": 300}
DEFAULT_LANES = {"served-batch": 4, "serving-sweep": 4, "mixed": 8}  # 3 otherwise


def compact(line, wall_s):
    out = {k: line[k] for k in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "parity_checked",
                                "gpu_launches") if k in line}
    out["config"] = (line.get("config") or {}).get("workload")
    if "e2e" in line:
        out["e2e"] = {"value": line["e2e"]["value"], "unit": line["e2e"]["unit"]}
    c = line.get("clocks") or {}
    out["clocks"] = {k: c.get(k) for k in ("sm_mhz", "sm_max_mhz", "reasons", "samples")}
    for k in ("fixed_rule", "latency", "saturation", "poisson_sweep"):
        if k in line:
            out[k] = line[k]
    out["wall_s"] = round(wall_s, 1)
    return out


def other_workloads(args, rank, world):
    runs = {"special-modulus": run_sm, "mixed": run_cfg4, "serving-sweep": run_cfg5, "one-packing": run_tree,
            "no-packing": run_nopack}
    out = {}
    for name in OTHER_WORKLOADS:
        sub = argparse.Namespace(**vars(args))
        sub.workload, sub.steps, sub.warmup = name, DEFAULT_STEPS[name], max(args.warmup, 3)
        sub.lanes = DEFAULT_LANES.get(name, 3)
        sub.shards, sub.requests = NUM_SHARDS, 16384
        t0 = time.perf_counter()
        try:
            line = runs[name](sub, rank, world)
        except Exception as e:  # reported in its slot; the headline line still prints
            out[name] = {"error": f"{type(e).__name__}: {e}"[:500], "wall_s": round(time.perf_counter() - t0, 1)}
            try:
                close_contexts()
            except Exception:
                pass
            continue
        close_contexts()
        out[name] = compact(line, time.perf_counter() - t0)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 20 for the served batch, a step being 16 batches of 64, and 100 for "
                         "the special_modulus batch: a timed region of about a third of a second that the 50 ms "
                         "clock sampler sees; 20 for the reference arm, a step being one batch of 64)")
    ap.add_argument("--batches-per-step", type=int, default=BATCHES_PER_STEP,
                    help="batches of 64 in one step of the served-batch workload")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lanes", type=int, default=None,
                    help="streams consecutive batches rotate over in the device-resident timed region, and the "
                         "caller threads and serving slots of the host-buffer legs (default: 4 for the served "
                         "batch of 64 and the serving sweep, 8 for the mixed launches, 3 otherwise; the measured "
                         "optimum of each)")
    ap.add_argument("--workload", default="served-batch",
                    choices=["served-batch", "special-modulus", "mixed", "serving-sweep", "one-packing", "no-packing"],
                    help="served-batch: the InspiRING batch of 64 over 2^20 records (the headline); special-modulus: "
                         "the special_modulus batch of 256; mixed: six parameter sets and batch sizes 1-512; "
                         "serving-sweep: the serving loop over 16,384 shards and 1000 seats; one-packing: the "
                         "tree responder, batches of 152; no-packing: the NoPacking responder, batches of 16")
    ap.add_argument("--requests", type=int, default=16384, help="trace length of the serving sweep")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the other workloads that the default served-batch run measures after the headline "
                         "(one GPU, default database size) and reports under `workloads`")
    ap.add_argument("--shards", type=int, default=NUM_SHARDS,
                    help="shards in the database (smaller values only for profiling captures)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.lanes is None:
        args.lanes = DEFAULT_LANES.get(args.workload, 3)
    if args.steps is None:
        args.steps = 20 if args.impl == "reference" else DEFAULT_STEPS[args.workload]
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        if rank != 0:
            return
        # The whole configuration on the host's cores: all 512 shards with their stores, each
        # step one batch of 64 queries with uniform indices, answered one after another.
        cb = cpu_sample(batches=args.steps, warmup_batches=args.warmup, build_all=True)
        line = {"metric": METRIC, "value": cb["value"], "unit": "queries/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(cb["batch_s"])),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u64 (exact mod q)", "data": "synthetic, same shapes", "config": CONFIG,
                "step": f"one batch of {BATCH} queries (a bounded sample of the workload per step)",
                "execution": {"parallelism": f"CPU, {cb['cores']} threads"},
                "impl": "reference", "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    if args.workload == "one-packing":
        line = run_tree(args, rank, world)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.workload == "no-packing":
        line = run_nopack(args, rank, world)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.workload == "mixed":
        line = run_cfg4(args, rank, world)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.workload == "serving-sweep":
        line = run_cfg5(args, rank, world)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.workload == "special-modulus":
        line = run_sm(args, rank, world)
        if rank == 0:
            if not args.no_cpu_baseline:
                line["cpu_baseline"] = sm_cpu_sample(steps=3, warmup=1)
            print(json.dumps(line))
        return
    line = run_gb300(args, rank, world)
    if world == 1 and args.shards == NUM_SHARDS and not args.headline_only:
        close_contexts()
        line["workloads"] = other_workloads(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            # Two batches of 64 over the same 512-shard shape (about 10 s of CPU work); the
            # stores of the touched shards, over 100 of them, exceed the host's last-level cache.
            # The CPU samples run after all the GPU work, so no GPU leg shares the host with them.
            line["cpu_baseline"] = cpu_sample(batches=2)
            sm = line.get("workloads", {}).get("special-modulus")
            if sm and "value" in sm:
                sm["cpu_baseline"] = sm_cpu_sample(steps=3, warmup=1)
        print(json.dumps(line))


if __name__ == "__main__":
    main()
