// The serving loop: continuous batching of individually submitted respond requests.
//
// Requests (one seeded query each, under a registered seat) enter a queue. A dispatcher
// thread forms a batch from the oldest waiting requests on one ring: databases, parameter
// sets (record widths, exact or approximate gadget), shards, seats and mod-switch targets
// may all differ within a batch, because every query of a launch carries its own set,
// shard entry and target. Admission is by memory. The loop holds a budget of device bytes;
// a request joins a batch only while the bytes its key and its buffers need fit in what the
// batches in flight leave free. Its buffers (query descriptor, shard entry, scan work items,
// seed, b, b fold, a and b out, status, wire bytes) are carved per batch from a device ring
// of the budget's size and returned in launch order; its key (the seat, 49,152 B or
// 32,768 B at ring 2048) counts once while any request on it is in flight. Each batch runs
// on one of `slots` streams, so batches overlap on the device, and requests that arrive
// while others run are admitted as slots and memory free up. A completion thread finishes
// batches in launch order, copies each request's result to its caller's buffers and records
// its latency from submission. A request's result is the one ig_respond_seeded_batch gives
// for the same query, whatever batch it lands in.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/inspire_gb300.h"
#include "ig_internal.hpp"
#include "ig_kernels.cuh"

using namespace ig;

namespace {

typedef std::chrono::steady_clock clk;

constexpr size_t kMaxN = 2048;      // largest ring the respond kernels serve
constexpr size_t kMaxGamma = 1024;  // largest packing width at that ring (gamma <= n/2)
// Largest ServerResponse wire: header and trailer (78 bytes) and two 60-bit tight blocks.
constexpr size_t kMaxWire = 78 + 2 * ((kMaxN * 60 + 7) / 8);
constexpr size_t kAlign = 256;
constexpr size_t kParts = 12;  // sub-buffers of a batch's region, each kAlign-aligned

size_t up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct Req {
  u64 ticket = 0;
  u64 db = 0, store = 0, handle = 0, ms = 0;
  u32 shard = 0, n = 0;
  uint8_t seed[32];
  std::vector<u64> b;
  u64* a_out = nullptr;
  u64* b_out = nullptr;
  uint8_t* wire_out = nullptr;  // wire requests: the ServerResponse bytes instead of a, b
  size_t wire_cap = 0;
  size_t* wire_len = nullptr;
  clk::time_point t_submit, t_launch;  // submission, and its batch's launch
  int status = -1;  // -1 while waiting or in flight
  u64 latency_ns = 0;
  std::string err;
  // Resolved when the request joins a batch.
  igint::RequestView v{};
  size_t wire_bytes = 0;  // its ServerResponse length (wire requests)
};

// Offsets of a batch's buffers within its region of the ring (device and pinned host
// mirror alike). [q, fold) is staged to the device as one copy.
struct Layout {
  size_t q = 0, table = 0, work = 0, seeds = 0, bs = 0, fold = 0, a = 0, b = 0, status = 0, wire = 0, wstatus = 0,
         tmpl = 0, total = 0;
};

Layout layout(size_t count, size_t n, size_t work, size_t fold, size_t wire, size_t tmpl) {
  Layout L;
  size_t o = 0;
  auto put = [&](size_t bytes) {
    const size_t at = o;
    o += up(bytes);
    return at;
  };
  L.q = put(count * sizeof(QueryDev));
  L.table = put(count * sizeof(ShardDev));
  L.work = put(work * 4);
  L.seeds = put(count * 32);
  L.bs = put(count * n * 8);
  L.fold = put(fold * 8);
  L.a = put(count * n * 8);
  L.b = put(count * n * 8);
  L.status = put(count * 4);
  L.wire = put(wire);
  L.wstatus = put(count * 4);
  L.tmpl = put(tmpl);
  L.total = o;
  return L;
}

// Bytes one request adds to a batch's region (its share of every sub-buffer; the batch adds
// kParts x kAlign of rounding once, and a template per (gamma, modulus) group of wire
// requests).
size_t request_bytes(size_t n, u32 gamma, size_t wire) {
  return sizeof(QueryDev) + sizeof(ShardDev) + 4 * (size_t)igk::scan_chunks(gamma) + 32 + n * 8 + (size_t)gamma * 8 +
         2 * n * 8 + 4 + wire + 4;
}

// One (gamma, modulus) group of wire requests in a batch: consecutive rows, one template.
struct WireGroup {
  u32 first = 0, count = 0, gamma = 0;
  u64 modulus = 0;
  size_t len = 0, tmpl_off = 0, out_off = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ready = nullptr;  // context work the batch depends on
  cudaEvent_t done = nullptr;
  std::vector<Req*> reqs;  // rows, in launch order
  std::vector<WireGroup> groups;
  size_t off = 0;  // the batch's region in the ring
  Layout L;
  u32 work_items = 0;
  bool want_ab = false;
  int launch_err = 0;
  u32 ctas = 0;  // CTAs of the batch in flight
  bool busy = false;
};

// A ring over [0, cap) whose regions are returned in the order they were carved.
struct Ring {
  size_t cap = 0, head = 0, tail = 0, used = 0;
  std::deque<std::pair<size_t, size_t>> live;  // (offset, bytes), oldest first

  bool wrapped() const { return head < tail || (head == tail && !live.empty()); }
  bool fits(size_t bytes) const {
    if (live.empty()) return bytes <= cap;
    if (wrapped()) return tail - head >= bytes;
    return cap - head >= bytes || tail >= bytes;
  }
  size_t take(size_t bytes) {  // the caller checked fits()
    if (live.empty()) head = tail = 0;
    const size_t off = (!wrapped() && cap - head < bytes) ? 0 : head;  // wrap: [head, cap) idles
    head = off + bytes;
    live.emplace_back(off, bytes);
    used += bytes;
    return off;
  }
  void give_oldest() {
    used -= live.front().second;
    live.pop_front();
    if (live.empty())
      head = tail = 0;
    else
      tail = live.front().first;
  }
};

}  // namespace

struct ig_serve {
  ig_ctx* ctx = nullptr;
  u32 max_batch = 0, nslots = 0;
  u64 max_waiting = 0;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_slot, cv_done, cv_launched;
  std::deque<Req*> waiting;
  std::unordered_map<u64, Req*> tickets;
  std::deque<u32> launched;  // slot indices in launch order
  bool stop = false;
  std::thread dispatcher, completer;
  u64 next_ticket = 1;
  u64 served = 0, refused = 0, batches = 0, batched_queries = 0;
  u32 inflight_ctas = 0;  // CTAs of all batches in flight
  std::vector<u64> latencies;
  std::vector<u64> queue_ns, exec_ns;  // per served request: submit -> launch, launch -> result
  // Memory admission: the ring of request buffers (device, and its pinned host mirror) and
  // the keys pinned by requests in flight, both counted against `budget`.
  size_t budget = 0;
  Ring ring;
  uint8_t* d_arena = nullptr;
  uint8_t* h_arena = nullptr;
  std::unordered_map<const u64*, u32> seat_refs;  // seat -> requests in flight on it
  size_t seat_bytes = 0;                          // bytes of the seats in seat_refs
  size_t peak_bytes = 0;
  // ServerResponse templates (zero coefficients) by (ring, gamma, modulus).
  std::map<std::tuple<u32, u32, u64>, std::vector<uint8_t>> templates;
  size_t device_bytes = 0;
};

namespace {

// Caller holds s->mu.
void finish(ig_serve* s, Req* r, int status) {
  r->status = status;
  const clk::time_point now = clk::now();
  r->latency_ns = (u64)std::chrono::duration_cast<std::chrono::nanoseconds>(now - r->t_submit).count();
  if (status == IG_OK) {
    s->served++;
    s->latencies.push_back(r->latency_ns);
    s->queue_ns.push_back((u64)std::chrono::duration_cast<std::chrono::nanoseconds>(r->t_launch - r->t_submit).count());
    s->exec_ns.push_back((u64)std::chrono::duration_cast<std::chrono::nanoseconds>(now - r->t_launch).count());
  } else {
    s->refused++;
  }
}

void refuse(ig_serve* s, Req* r, int code, const char* fmt, ...) __attribute__((format(printf, 4, 5)));
void refuse(ig_serve* s, Req* r, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  r->err = buf;
  finish(s, r, code);
}

// The zero-coefficient ServerResponse of (n, gamma, modulus), whose length is the wire's.
// Caller holds s->mu.
const std::vector<uint8_t>* wire_template(ig_serve* s, u32 n, u32 gamma, u64 modulus) {
  auto key = std::make_tuple(n, gamma, modulus);
  auto it = s->templates.find(key);
  if (it != s->templates.end()) return &it->second;
  std::vector<u64> zeros(n, 0);
  std::vector<uint8_t> t(kMaxWire);
  size_t len = 0;
  if (ig_response_encode(zeros.data(), zeros.data(), n, gamma, modulus, t.data(), t.size(), &len) != IG_OK ||
      len > kMaxWire)
    return nullptr;
  t.resize(len);
  return &s->templates.emplace(key, std::move(t)).first->second;
}

// Forms one batch on a free slot from the oldest waiting requests on the head's ring, while
// max_batch and memory allow: a request joins while the batch's region still fits the ring
// and the ring's bytes, the pinned keys' bytes and the batch's stay within the budget
// together. A request that could not fit even alone is refused (IG_ERR_NOMEM); requests the
// context refuses finish here with the refusal. Returns the slot index, or -1 when nothing
// was batched. Caller holds s->mu and has seen a free slot (the context lock is taken
// inside, after s->mu).
int form_batch(ig_serve* s, CrsDev* ring_out) {
  int slot = -1;
  for (u32 k = 0; k < s->nslots; k++)
    if (!s->slots[k].busy) {
      slot = (int)k;
      break;
    }
  if (slot < 0) return -1;
  Slot& sl = s->slots[slot];
  sl.reqs.clear();
  sl.groups.clear();
  u32 n = 0;
  size_t req_sum = 0, work = 0, fold = 0, wire = 0, tmpl = 0, new_seats = 0;
  std::vector<const u64*> batch_seats;
  std::vector<std::pair<u32, u64>> batch_groups;  // (gamma, modulus) of the batch's templates
  for (auto it = s->waiting.begin(); it != s->waiting.end() && sl.reqs.size() < s->max_batch;) {
    Req* r = *it;
    igint::RequestView& v = r->v;
    const int rc = igint::resolve_request(s->ctx, r->db, r->store, r->handle, r->shard, &v);
    if (rc != IG_OK) {
      r->err = v.err;
      finish(s, r, rc);
      it = s->waiting.erase(it);
      continue;
    }
    if (r->n != v.crs.n) {
      refuse(s, r, IG_ERR_SHAPE, "query ring_dim %u does not match the database's ring_dim %u", r->n, v.crs.n);
      it = s->waiting.erase(it);
      continue;
    }
    if (!v.has_store) {
      refuse(s, r, IG_ERR_ARG,
             "shard %u has no packing store; the serving loop serves shards whose store was built "
             "(precompute_packing)",
             r->shard);
      it = s->waiting.erase(it);
      continue;
    }
    if (r->ms && (r->ms >= Q || r->ms < v.p || r->ms % (2ULL * v.crs.n) != 1)) {
      refuse(s, r, IG_ERR_ARG, "mod-switch target_modulus %llu must be in [p, q) and 1 mod 2d",
             (unsigned long long)r->ms);
      it = s->waiting.erase(it);
      continue;
    }
    if (sl.reqs.empty()) n = r->n;
    if (r->n != n) {  // another ring waits for a later batch
      ++it;
      continue;
    }
    const u32 gamma = v.crs.gamma;
    const u64 modulus = r->ms ? r->ms : Q;
    size_t add_tmpl = 0;
    r->wire_bytes = 0;
    if (r->wire_out) {
      const std::vector<uint8_t>* t = wire_template(s, n, gamma, modulus);
      if (!t) {
        refuse(s, r, IG_ERR_SHAPE, "ServerResponse encode refused for gamma %u over modulus %llu", gamma,
               (unsigned long long)modulus);
        it = s->waiting.erase(it);
        continue;
      }
      r->wire_bytes = t->size();
      if (std::find(batch_groups.begin(), batch_groups.end(), std::make_pair(gamma, modulus)) == batch_groups.end())
        add_tmpl = t->size();
    }
    const bool seat_new = s->seat_refs.find(v.seat) == s->seat_refs.end() &&
                          std::find(batch_seats.begin(), batch_seats.end(), v.seat) == batch_seats.end();
    const size_t key_bytes = seat_new ? (size_t)v.seat_rows * n * 8 : 0;
    const size_t mine = request_bytes(n, gamma, r->wire_bytes);
    const size_t region = req_sum + mine + tmpl + add_tmpl + kParts * kAlign;
    const size_t charged = s->ring.used + s->seat_bytes + new_seats + key_bytes + region;
    if (!s->ring.fits(region) || charged > s->budget) {
      const size_t alone = mine + r->wire_bytes + kParts * kAlign + (size_t)v.seat_rows * n * 8;
      if (alone > s->budget) {
        refuse(s, r, IG_ERR_NOMEM,
               "admission refused: the request needs %zu device bytes (its key and buffers), the serving loop's "
               "budget is %zu",
               alone, s->budget);
        it = s->waiting.erase(it);
        continue;
      }
      break;  // waits, in arrival order, for batches in flight to return their memory
    }
    req_sum += mine;
    work += igk::scan_chunks(gamma);
    fold += gamma;
    wire += r->wire_bytes;
    if (add_tmpl) {
      batch_groups.emplace_back(gamma, modulus);
      tmpl += add_tmpl;
    }
    if (key_bytes) {
      batch_seats.push_back(v.seat);
      new_seats += key_bytes;
    }
    sl.reqs.push_back(r);
    it = s->waiting.erase(it);
  }
  if (sl.reqs.empty()) return -1;
  // Rows: longest recursion first (the launch's tail is its shortest queries), then by
  // switch target and wire, so each (gamma, modulus) group of wire requests is consecutive.
  std::stable_sort(sl.reqs.begin(), sl.reqs.end(), [](const Req* x, const Req* y) {
    if (x->v.crs.gamma != y->v.crs.gamma) return x->v.crs.gamma > y->v.crs.gamma;
    if (x->ms != y->ms) return x->ms < y->ms;
    return (x->wire_out != nullptr) < (y->wire_out != nullptr);
  });
  const u32 count = (u32)sl.reqs.size();
  sl.L = layout(count, n, work, fold, wire, tmpl);
  sl.off = s->ring.take(sl.L.total);
  for (Req* r : sl.reqs) s->seat_refs[r->v.seat]++;
  s->seat_bytes += new_seats;
  s->peak_bytes = std::max(s->peak_bytes, s->ring.used + s->seat_bytes);
  // Host side of the region: descriptors, shard entries, work items and templates (the
  // seeds and b are copied in by the dispatcher after it releases the loop's lock).
  uint8_t* h = s->h_arena + sl.off;
  uint8_t* d = s->d_arena + sl.off;
  QueryDev* hq = (QueryDev*)(h + sl.L.q);
  ShardDev* ht = (ShardDev*)(h + sl.L.table);
  u32* hw = (u32*)(h + sl.L.work);
  size_t fold_off = 0, wire_off = 0, tmpl_off = 0;
  u32 work_n = 0;
  sl.want_ab = false;
  for (u32 i = 0; i < count; i++) {
    Req* r = sl.reqs[i];
    const u32 gamma = r->v.crs.gamma;
    ht[i] = r->v.shard;
    QueryDev& q = hq[i];
    q = QueryDev{};
    q.shard = i;
    q.fold_off = (u32)fold_off;
    q.seed = (const u32*)(d + sl.L.seeds + (size_t)i * 32);
    q.b = (const u64*)(d + sl.L.bs) + (size_t)i * n;
    q.seat_R = r->v.seat;
    q.crs = r->v.crs_dev;
    q.ms = r->ms;
    q.row = i;
    for (u32 ch = 0; ch < igk::scan_chunks(gamma); ch++) hw[work_n++] = (i << 12) | ch;
    fold_off += gamma;
    if (!r->wire_out) {
      sl.want_ab = true;
      continue;
    }
    const u64 modulus = r->ms ? r->ms : Q;
    if (sl.groups.empty() || sl.groups.back().gamma != gamma || sl.groups.back().modulus != modulus) {
      // Rows are sorted by (gamma, modulus), so each pair forms one group with one template.
      WireGroup g;
      g.first = i;
      g.gamma = gamma;
      g.modulus = modulus;
      g.len = r->wire_bytes;
      g.out_off = wire_off;
      g.tmpl_off = tmpl_off;
      const std::vector<uint8_t>* t = wire_template(s, n, gamma, modulus);
      memcpy(h + sl.L.tmpl + tmpl_off, t->data(), t->size());
      tmpl_off += t->size();
      sl.groups.push_back(g);
    }
    sl.groups.back().count++;
    wire_off += r->wire_bytes;
  }
  sl.work_items = work_n;
  *ring_out = sl.reqs[0]->v.crs;
  sl.busy = true;
  return slot;
}

void dispatch_loop(ig_serve* s) {
  cudaSetDevice(igint::device(s->ctx));
  for (;;) {
    CrsDev ring{};
    int k;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      for (;;) {
        s->cv_work.wait(lk, [&] { return s->stop || !s->waiting.empty(); });
        if (s->waiting.empty()) return;  // stopped and drained
        s->cv_slot.wait(lk, [&] {
          for (const Slot& x : s->slots)
            if (!x.busy) return true;
          return false;
        });
        // A batch launched into SMs the batches in flight still hold would wait on the device
        // behind them, half-started; held here until it fits the free SMs (one CTA a query),
        // it waits as long and more arrivals join it. A full batch's worth of waiting requests
        // launches at once, so the device stays fed at saturation.
        const u32 sms = (u32)igint::sm_count(s->ctx);
        s->cv_slot.wait(lk, [&] {
          const size_t next = std::min<size_t>(s->waiting.size(), s->max_batch);
          return s->stop || s->launched.empty() || s->waiting.size() >= s->max_batch ||
                 s->inflight_ctas + next <= sms;
        });
        k = form_batch(s, &ring);
        if (k >= 0) break;
        s->cv_done.notify_all();  // requests refused while forming
        // Nothing fit: wait until a batch in flight returns its memory.
        const u64 done_before = s->batches - s->launched.size();
        if (!s->waiting.empty() && !s->launched.empty())
          s->cv_slot.wait(lk, [&] { return s->stop || s->batches - s->launched.size() != done_before; });
      }
    }
    s->cv_done.notify_all();
    Slot& sl = s->slots[k];
    const u32 count = (u32)sl.reqs.size();
    const size_t n = ring.n;
    // Several CTAs per query (a cluster) only while the batches in flight and this one leave
    // at least half the SMs free: a cluster needs its SMs free together within one GPC, and
    // batches of single CTAs scattered over most of the GPCs leave it waiting on the device
    // behind them although enough SMs are free in all. Otherwise one CTA per query does the
    // same work on fewer SMs.
    int ctas;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      const u32 sms = (u32)igint::sm_count(s->ctx);
      ctas = igint::launch_ctas(s->ctx, (u32)n, sl.reqs[0]->v.crs.gamma, count, count + s->inflight_ctas);
      if (s->inflight_ctas != 0 && ctas > 1 && !igint::forced_ctas(s->ctx) &&
          2 * (s->inflight_ctas + (u32)ctas * count) > sms)
        ctas = 1;
      sl.ctas = (u32)ctas * count;
      s->inflight_ctas += sl.ctas;
    }
    uint8_t* h = s->h_arena + sl.off;
    uint8_t* d = s->d_arena + sl.off;
    const Layout& L = sl.L;
    // The batch's requests belong to this slot until it completes: their inputs are copied
    // into the pinned region without the loop's lock.
    for (u32 i = 0; i < count; i++) {
      memcpy(h + L.seeds + (size_t)i * 32, sl.reqs[i]->seed, 32);
      memcpy(h + L.bs + (size_t)i * n * 8, sl.reqs[i]->b.data(), n * 8);
    }
    cudaStream_t st = sl.stream;
    // Ordered after every context call made before this batch formed (shard uploads, stores).
    cudaError_t e = cudaEventRecord(sl.ready, igint::stream(s->ctx));
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, sl.ready, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + L.q, h + L.q, L.fold - L.q, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d + L.status, 0, count * 4, st);
    if (e == cudaSuccess)
      e = igk::shard_scan(ring, (const QueryDev*)(d + L.q), (const ShardDev*)(d + L.table), count,
                          (const u32*)(d + L.work), sl.work_items, (u64*)(d + L.fold), (u32*)(d + L.status), st);
    if (e == cudaSuccess)
      e = igk::respond(ring, (const QueryDev*)(d + L.q), (const ShardDev*)(d + L.table), count,
                       (const u64*)(d + L.fold), (u64*)(d + L.a), (u64*)(d + L.b), (u32*)(d + L.status), 0, ctas, st);
    if (e == cudaSuccess) {
      igint::add_launches(s->ctx, 2);
      e = cudaMemcpyAsync(h + L.status, d + L.status, count * 4, cudaMemcpyDeviceToHost, st);
    }
    // Wire requests: the ServerResponse bytes (tight codec) built next to the words, one
    // wire launch per (gamma, modulus) group of consecutive rows.
    if (e == cudaSuccess && !sl.groups.empty()) {
      e = cudaMemcpyAsync(d + L.tmpl, h + L.tmpl, L.total - L.tmpl, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(d + L.wstatus, 0, count * 4, st);
      for (const WireGroup& g : sl.groups) {
        if (e != cudaSuccess) break;
        const unsigned bits = 64 - __builtin_clzll(g.modulus - 1);
        const u32 a_bytes = (u32)(((u64)n * bits + 7) / 8), b_bytes = (u32)(((u64)g.gamma * bits + 7) / 8);
        e = igk::wire((const u64*)(d + L.a) + (size_t)g.first * n, (const u64*)(d + L.b) + (size_t)g.first * n,
                      g.count, (u32)n, g.gamma, bits, g.modulus, d + L.tmpl + g.tmpl_off, (u32)g.len, 12, a_bytes,
                      12 + a_bytes + 41 + 8, b_bytes, d + L.wire + g.out_off, (u32*)(d + L.wstatus) + g.first, st);
        if (e == cudaSuccess) igint::add_launches(s->ctx, 1);
      }
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(h + L.wire, d + L.wire, L.wstatus + count * 4 - L.wire, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess && sl.want_ab)
      e = cudaMemcpyAsync(h + L.a, d + L.a, L.status - L.a, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(sl.done, st);
    const clk::time_point t_launch = clk::now();
    for (Req* r : sl.reqs) r->t_launch = t_launch;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      sl.launch_err = (int)e;
      s->batches++;
      s->batched_queries += count;
      s->launched.push_back((u32)k);
    }
    s->cv_launched.notify_all();
  }
}

void complete_loop(ig_serve* s) {
  cudaSetDevice(igint::device(s->ctx));
  for (;;) {
    u32 k;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_launched.wait(lk, [&] {
        if (!s->launched.empty()) return true;
        if (!s->stop || !s->waiting.empty()) return false;
        for (const Slot& x : s->slots)
          if (x.busy) return false;
        return true;
      });
      if (s->launched.empty()) return;
      k = s->launched.front();
    }
    Slot& sl = s->slots[k];
    const cudaError_t e = cudaEventSynchronize(sl.done);
    // Outcomes and result copies without the loop's lock (the batch's requests belong to
    // this slot until they finish); then, under it, the requests finish and the memory returns.
    const uint8_t* h = s->h_arena + sl.off;
    const Layout& L = sl.L;
    const u32* h_status = (const u32*)(h + L.status);
    const u32* h_wstatus = (const u32*)(h + L.wstatus);
    enum Outcome { SERVED, LAUNCH, TAG, DEVICE, WIRE_SHAPE, WIRE_CAP };
    std::vector<Outcome> outcome(sl.reqs.size());
    size_t wire_off = 0;
    for (size_t i = 0; i < sl.reqs.size(); i++) {
      Req* r = sl.reqs[i];
      const size_t n = r->n;
      Outcome o = SERVED;
      if (sl.launch_err || e != cudaSuccess) {
        o = LAUNCH;
      } else if (h_status[i] & DEV_TAG_MISMATCH) {
        o = TAG;
      } else if (h_status[i]) {
        o = DEVICE;
      } else if (r->wire_out) {
        if (h_wstatus[i]) {
          o = WIRE_SHAPE;
        } else if (r->wire_bytes > r->wire_cap) {
          o = WIRE_CAP;
        } else {
          memcpy(r->wire_out, h + L.wire + wire_off, r->wire_bytes);
          *r->wire_len = r->wire_bytes;
        }
      } else {
        memcpy(r->a_out, h + L.a + i * n * 8, n * 8);
        memcpy(r->b_out, h + L.b + i * n * 8, n * 8);
      }
      outcome[i] = o;
      wire_off += r->wire_bytes;
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->launched.pop_front();
      for (size_t i = 0; i < sl.reqs.size(); i++) {
        Req* r = sl.reqs[i];
        switch (outcome[i]) {
          case SERVED:
            finish(s, r, IG_OK);
            break;
          case LAUNCH:
            refuse(s, r, IG_ERR_CUDA, "serving launch failed: %s",
                   cudaGetErrorString(sl.launch_err ? (cudaError_t)sl.launch_err : e));
            break;
          case TAG:
            refuse(s, r, IG_ERR_STORE_REFUSED,
                   "shard %u: packing store refused: a column is not the column the store was built from. The "
                   "shard changed after the build; rebuild the store before serving it",
                   r->shard);
            break;
          case DEVICE:
            refuse(s, r, IG_ERR_DEVICE, "respond kernel status %u", h_status[i]);
            break;
          case WIRE_SHAPE:
            refuse(s, r, IG_ERR_SHAPE, "ServerResponse encode refused: coefficients must be canonical");
            break;
          case WIRE_CAP:
            refuse(s, r, IG_ERR_ARG, "wire buffer of %zu bytes is smaller than the %zu-byte response", r->wire_cap,
                   r->wire_bytes);
            break;
        }
      }
      // The batch's memory returns: its region (the oldest in the ring) and its keys.
      for (Req* r : sl.reqs) {
        auto it = s->seat_refs.find(r->v.seat);
        if (it != s->seat_refs.end() && --it->second == 0) {
          s->seat_bytes -= (size_t)r->v.seat_rows * r->n * 8;
          s->seat_refs.erase(it);
        }
      }
      s->ring.give_oldest();
      sl.reqs.clear();
      sl.busy = false;
      s->inflight_ctas -= sl.ctas;
      sl.ctas = 0;
    }
    s->cv_slot.notify_all();
    s->cv_done.notify_all();
  }
}

void free_loop(ig_serve* s) {
  for (auto& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.ready) cudaEventDestroy(sl.ready);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  if (s->d_arena) igint::dfree(s->ctx, s->d_arena, s->budget);
  if (s->h_arena) cudaFreeHost(s->h_arena);
}

}  // namespace

extern "C" {

int ig_serve_create(ig_ctx* ctx, uint32_t slots, uint32_t max_batch, uint64_t hbm_budget_bytes, ig_serve** out) {
  if (!ctx) return IG_ERR_ARG;
  if (!out || slots == 0 || max_batch == 0 || slots > 64 || max_batch > 4096)
    return igint::fail(ctx, IG_ERR_ARG, "ig_serve_create: need 1..64 slots of 1..4096 queries and an out pointer");
  // Default budget: every slot full of the largest requests (gamma 1024 at ring 2048, wire
  // bytes, a key of three rows each).
  const size_t largest = request_bytes(kMaxN, (u32)kMaxGamma, kMaxWire) + kMaxWire + 3 * kMaxN * 8;
  const size_t budget =
      hbm_budget_bytes ? (size_t)hbm_budget_bytes : (size_t)slots * ((size_t)max_batch * largest + kParts * kAlign);
  cudaSetDevice(igint::device(ctx));
  auto* s = new ig_serve();
  s->ctx = ctx;
  s->max_batch = max_batch;
  s->nslots = slots;
  s->max_waiting = (u64)slots * max_batch * 8;
  s->slots.resize(slots);
  s->budget = budget;
  s->ring.cap = budget;
  {
    std::lock_guard<std::mutex> lk(igint::mutex(ctx));
    if (igint::dalloc(ctx, (void**)&s->d_arena, budget) != IG_OK) {
      char why[256];
      ig_last_error(ctx, why, sizeof why);
      s->d_arena = nullptr;
      delete s;
      return igint::fail(ctx, IG_ERR_NOMEM, "serving loop refused: its %zu-byte device budget cannot be allocated (%s)",
                         budget, why);
    }
    s->device_bytes = budget;
    if (cudaHostAlloc((void**)&s->h_arena, budget, 0) != cudaSuccess) {
      s->h_arena = nullptr;
      free_loop(s);
      delete s;
      return igint::fail(ctx, IG_ERR_NOMEM, "serving loop: pinned host allocation of %zu bytes failed", budget);
    }
    for (auto& sl : s->slots)
      if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) ||
          cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming) ||
          cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) {
        free_loop(s);
        delete s;
        return igint::fail(ctx, IG_ERR_CUDA, "serving loop: stream or event creation failed");
      }
  }
  s->dispatcher = std::thread(dispatch_loop, s);
  s->completer = std::thread(complete_loop, s);
  *out = s;
  return IG_OK;
}

int ig_serve_destroy(ig_serve* s) {
  if (!s) return IG_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_slot.notify_all();
  s->dispatcher.join();
  s->cv_launched.notify_all();
  s->completer.join();
  {
    std::lock_guard<std::mutex> lk(igint::mutex(s->ctx));
    free_loop(s);
  }
  for (auto& kv : s->tickets) delete kv.second;
  delete s;
  return IG_OK;
}

static int submit(ig_serve* s, uint64_t db, uint64_t store, uint64_t handle, uint32_t shard_id, const uint8_t* seed,
                  const uint64_t* b, uint32_t ring_dim, uint64_t mod_switch_target, uint64_t* a_out, uint64_t* b_out,
                  uint8_t* wire_out, size_t wire_cap, size_t* wire_len, uint64_t* ticket_out) {
  auto* r = new Req();
  r->wire_out = wire_out;
  r->wire_cap = wire_cap;
  r->wire_len = wire_len;
  r->db = db;
  r->store = store;
  r->handle = handle;
  r->shard = shard_id;
  r->ms = mod_switch_target;
  r->n = ring_dim;
  memcpy(r->seed, seed, 32);
  r->b.assign(b, b + ring_dim);
  r->a_out = a_out;
  r->b_out = b_out;
  r->t_submit = clk::now();
  bool full = false;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop || s->waiting.size() >= s->max_waiting) {
      const size_t w = s->waiting.size();
      delete r;
      return igint::fail(s->ctx, IG_ERR_NOMEM, "admission refused: %zu requests are already waiting (limit %llu)", w,
                         (unsigned long long)s->max_waiting);
    }
    r->ticket = s->next_ticket++;
    s->tickets[r->ticket] = r;
    s->waiting.push_back(r);
    *ticket_out = r->ticket;
    full = s->waiting.size() >= s->max_batch;
  }
  s->cv_work.notify_one();
  if (full) s->cv_slot.notify_all();  // a held dispatcher launches a full batch at once
  return IG_OK;
}

int ig_serve_submit(ig_serve* s, uint64_t db, uint64_t store, uint64_t handle, uint32_t shard_id,
                    const uint8_t* seed, const uint64_t* b, uint32_t ring_dim, uint64_t mod_switch_target,
                    uint64_t* a_out, uint64_t* b_out, uint64_t* ticket_out) {
  if (!s) return IG_ERR_ARG;
  if (!seed || !b || !a_out || !b_out || !ticket_out || ring_dim == 0 || ring_dim > kMaxN)
    return igint::fail(s->ctx, IG_ERR_ARG, "ig_serve_submit: null buffer or ring_dim outside 1..2048");
  return submit(s, db, store, handle, shard_id, seed, b, ring_dim, mod_switch_target, a_out, b_out, nullptr, 0,
                nullptr, ticket_out);
}

int ig_serve_submit_wire(ig_serve* s, uint64_t db, uint64_t store, uint64_t handle, uint32_t shard_id,
                         const uint8_t* seed, const uint64_t* b, uint32_t ring_dim, uint64_t mod_switch_target,
                         uint8_t* wire_out, size_t wire_cap, size_t* wire_len, uint64_t* ticket_out) {
  if (!s) return IG_ERR_ARG;
  if (!seed || !b || !wire_out || !wire_len || !ticket_out || ring_dim == 0 || ring_dim > kMaxN)
    return igint::fail(s->ctx, IG_ERR_ARG, "ig_serve_submit_wire: null buffer or ring_dim outside 1..2048");
  return submit(s, db, store, handle, shard_id, seed, b, ring_dim, mod_switch_target, nullptr, nullptr, wire_out,
                wire_cap, wire_len, ticket_out);
}

int ig_serve_wait(ig_serve* s, uint64_t ticket, int64_t timeout_ms, uint64_t* latency_ns, char* err, size_t err_len) {
  if (!s) return IG_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) {
    if (err && err_len) snprintf(err, err_len, "unknown serving ticket %llu", (unsigned long long)ticket);
    return IG_ERR_HANDLE;
  }
  Req* r = it->second;
  auto done = [&] { return r->status >= 0; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
    if (err && err_len)
      snprintf(err, err_len, "serving ticket %llu not finished within %lld ms", (unsigned long long)ticket,
               (long long)timeout_ms);
    return IG_ERR_PENDING;
  }
  const int st = r->status;
  if (latency_ns) *latency_ns = r->latency_ns;
  if (err && err_len) snprintf(err, err_len, "%s", r->err.c_str());
  s->tickets.erase(it);
  delete r;
  return st;
}

int ig_serve_replay(ig_serve* s, uint64_t db, uint64_t store, uint32_t count, const uint32_t* shard_ids,
                    const uint64_t* handles, const uint8_t* seeds, const uint64_t* bs, uint32_t ring_dim,
                    uint64_t mod_switch_target, const uint64_t* arrival_ns, uint32_t window, uint64_t* a_out,
                    uint64_t* b_out, uint64_t* latency_ns, double* elapsed_s) {
  if (!s) return IG_ERR_ARG;
  if (!shard_ids || !handles || !seeds || !bs || !a_out || !b_out || count == 0 || ring_dim == 0 ||
      (!arrival_ns && window == 0))
    return igint::fail(s->ctx, IG_ERR_ARG, "ig_serve_replay: null buffer, empty trace, or neither arrivals nor window");
  std::vector<u64> tickets(count);
  const auto t0 = clk::now();
  int first_err = IG_OK;
  u32 waited = 0;  // requests [0, waited) already collected
  auto collect = [&](u32 i) {
    u64 lat = 0;
    const int rc = ig_serve_wait(s, tickets[i], -1, &lat, nullptr, 0);
    if (latency_ns) latency_ns[i] = lat;
    if (rc != IG_OK && first_err == IG_OK) first_err = rc;
  };
  for (u32 i = 0; i < count; i++) {
    if (arrival_ns) {
      const auto due = t0 + std::chrono::nanoseconds(arrival_ns[i]);
      while (clk::now() < due) {
        const auto left = due - clk::now();
        if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
      }
    }
    if (window)
      while (i - waited >= window) collect(waited++);
    int rc;
    for (;;) {  // an admission refusal under load waits for the oldest request, then retries
      rc = ig_serve_submit(s, db, store, handles[i], shard_ids[i], seeds + (size_t)i * 32, bs + (size_t)i * ring_dim,
                           ring_dim, mod_switch_target, a_out + (size_t)i * ring_dim, b_out + (size_t)i * ring_dim,
                           &tickets[i]);
      if (rc != IG_ERR_NOMEM || waited == i) break;
      collect(waited++);
    }
    if (rc != IG_OK) {
      for (; waited < i; waited++) collect(waited);
      return rc;
    }
  }
  for (; waited < count; waited++) collect(waited);
  if (elapsed_s) *elapsed_s = std::chrono::duration<double>(clk::now() - t0).count();
  return first_err;
}

int ig_serve_stats(ig_serve* s, ig_serve_stats_t* out, int reset) {
  if (!s || !out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<u64> v = s->latencies, vq = s->queue_ns, ve = s->exec_ns;
  std::sort(v.begin(), v.end());
  std::sort(vq.begin(), vq.end());
  std::sort(ve.begin(), ve.end());
  auto pct_of = [](const std::vector<u64>& x, double p) -> double {
    if (x.empty()) return 0.0;
    size_t i = (size_t)(p * (double)x.size());
    if (i >= x.size()) i = x.size() - 1;
    return (double)x[i] / 1e3;
  };
  auto pct = [&](double p) { return pct_of(v, p); };
  out->served = s->served;
  out->refused = s->refused;
  out->batches = s->batches;
  out->waiting = s->waiting.size();
  out->device_bytes = s->device_bytes;
  out->mean_batch = s->batches ? (double)s->batched_queries / (double)s->batches : 0.0;
  out->p50_us = pct(0.50);
  out->p99_us = pct(0.99);
  out->max_us = v.empty() ? 0.0 : (double)v.back() / 1e3;
  out->budget_bytes = s->budget;
  out->inflight_bytes = s->ring.used + s->seat_bytes;
  out->peak_inflight_bytes = s->peak_bytes;
  out->queue_p50_us = pct_of(vq, 0.50);
  out->queue_p99_us = pct_of(vq, 0.99);
  out->exec_p50_us = pct_of(ve, 0.50);
  out->exec_p99_us = pct_of(ve, 0.99);
  if (reset) {
    s->latencies.clear();
    s->queue_ns.clear();
    s->exec_ns.clear();
    s->served = s->refused = s->batches = s->batched_queries = 0;
    s->peak_bytes = s->ring.used + s->seat_bytes;
  }
  return IG_OK;
}

}  // extern "C"
