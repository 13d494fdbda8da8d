// The serving loop: continuous batching of individually submitted respond requests.
//
// Requests (one seeded query each, under a registered seat) enter a queue. A dispatcher
// thread takes the oldest request and every other waiting request that can share its
// launch: the same parameter set and mod-switch target. Databases, shards and seats may
// differ per query, because each launch carries its own shard table. The batch goes to a
// free slot. Each slot owns a CUDA stream and device and pinned buffers sized when the loop
// is created, so admission is bounded by memory fixed up front and a batch never allocates.
// Batches on different slots overlap on the device, and requests that arrive while others
// run are admitted as soon as a slot frees. A completion thread finishes slots in launch
// order, copies each request's result to its caller's buffers and records its latency from
// submission. A request's result is the one ig_respond_seeded_batch gives for the same
// query, whatever batch it lands in.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/inspire_gb300.h"
#include "ig_internal.hpp"
#include "ig_kernels.cuh"

using namespace ig;

namespace {

typedef std::chrono::steady_clock clk;

constexpr size_t kMaxN = 2048;      // largest ring the respond kernels serve
constexpr size_t kMaxGamma = 2048;  // largest packing width (gamma <= n)
// Largest ServerResponse wire: header and trailer (78 bytes) and two 60-bit tight blocks.
constexpr size_t kMaxWire = 78 + 2 * ((kMaxN * 60 + 7) / 8);

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
  clk::time_point t_submit;
  int status = -1;  // -1 while waiting or in flight
  u64 latency_ns = 0;
  std::string err;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ready = nullptr;  // context work the batch depends on
  cudaEvent_t done = nullptr;
  QueryDev* d_q = nullptr;
  ShardDev* d_table = nullptr;
  uint8_t* d_seeds = nullptr;
  u64* d_bs = nullptr;
  u64* d_fold = nullptr;
  u64* d_a = nullptr;
  u64* d_b = nullptr;
  u32* d_status = nullptr;
  uint8_t* d_wire = nullptr;
  uint8_t* d_tmpl = nullptr;
  u32* d_wstatus = nullptr;
  QueryDev* h_q = nullptr;
  ShardDev* h_table = nullptr;
  uint8_t* h_seeds = nullptr;
  u64* h_bs = nullptr;
  u64* h_a = nullptr;
  u64* h_b = nullptr;
  u32* h_status = nullptr;
  uint8_t* h_wire = nullptr;
  uint8_t* h_tmpl = nullptr;
  u32* h_wstatus = nullptr;
  size_t wire_len = 0;  // bytes per response of the batch in flight (0: no wire requests)
  bool want_ab = false;
  std::vector<Req*> reqs;
  int launch_err = 0;
  u32 ctas = 0;  // CTAs of the batch in flight
  bool busy = false;
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
  size_t device_bytes = 0;
};

namespace {

size_t slot_device_bytes(u32 B) {
  return (size_t)B * (sizeof(QueryDev) + sizeof(ShardDev) + 32 + kMaxN * 8 * 3 + kMaxGamma * 8 + 8 + kMaxWire) +
         kMaxWire;
}

int alloc_slot(ig_serve* s, Slot& sl) {
  const size_t B = s->max_batch;
  auto dev = [&](void** p, size_t bytes) -> int {
    const int rc = igint::dalloc(s->ctx, p, bytes);
    if (!rc) s->device_bytes += bytes;
    return rc;
  };
  int rc;
  if ((rc = dev((void**)&sl.d_q, B * sizeof(QueryDev))) || (rc = dev((void**)&sl.d_table, B * sizeof(ShardDev))) ||
      (rc = dev((void**)&sl.d_seeds, B * 32)) || (rc = dev((void**)&sl.d_bs, B * kMaxN * 8)) ||
      (rc = dev((void**)&sl.d_fold, B * kMaxGamma * 8)) || (rc = dev((void**)&sl.d_a, B * kMaxN * 8)) ||
      (rc = dev((void**)&sl.d_b, B * kMaxN * 8)) || (rc = dev((void**)&sl.d_status, B * 4)) ||
      (rc = dev((void**)&sl.d_wire, B * kMaxWire)) || (rc = dev((void**)&sl.d_tmpl, kMaxWire)) ||
      (rc = dev((void**)&sl.d_wstatus, B * 4)))
    return rc;
  if (cudaHostAlloc((void**)&sl.h_q, B * sizeof(QueryDev), 0) ||
      cudaHostAlloc((void**)&sl.h_table, B * sizeof(ShardDev), 0) || cudaHostAlloc((void**)&sl.h_seeds, B * 32, 0) ||
      cudaHostAlloc((void**)&sl.h_bs, B * kMaxN * 8, 0) || cudaHostAlloc((void**)&sl.h_a, B * kMaxN * 8, 0) ||
      cudaHostAlloc((void**)&sl.h_b, B * kMaxN * 8, 0) || cudaHostAlloc((void**)&sl.h_status, B * 4, 0) ||
      cudaHostAlloc((void**)&sl.h_wire, B * kMaxWire, 0) || cudaHostAlloc((void**)&sl.h_tmpl, kMaxWire, 0) ||
      cudaHostAlloc((void**)&sl.h_wstatus, B * 4, 0))
    return igint::fail(s->ctx, IG_ERR_NOMEM, "serving loop: pinned host allocation of a slot failed");
  if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) ||
      cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming) ||
      cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming))
    return igint::fail(s->ctx, IG_ERR_CUDA, "serving loop: stream or event creation failed");
  return IG_OK;
}

void free_slot(ig_serve* s, Slot& sl) {
  if (sl.stream) cudaStreamSynchronize(sl.stream);
  const size_t B = s->max_batch;
  igint::dfree(s->ctx, sl.d_q, B * sizeof(QueryDev));
  igint::dfree(s->ctx, sl.d_table, B * sizeof(ShardDev));
  igint::dfree(s->ctx, sl.d_seeds, B * 32);
  igint::dfree(s->ctx, sl.d_bs, B * kMaxN * 8);
  igint::dfree(s->ctx, sl.d_fold, B * kMaxGamma * 8);
  igint::dfree(s->ctx, sl.d_a, B * kMaxN * 8);
  igint::dfree(s->ctx, sl.d_b, B * kMaxN * 8);
  igint::dfree(s->ctx, sl.d_status, B * 4);
  igint::dfree(s->ctx, sl.d_wire, B * kMaxWire);
  igint::dfree(s->ctx, sl.d_tmpl, kMaxWire);
  igint::dfree(s->ctx, sl.d_wstatus, B * 4);
  for (void* h : {(void*)sl.h_q, (void*)sl.h_table, (void*)sl.h_seeds, (void*)sl.h_bs, (void*)sl.h_a, (void*)sl.h_b,
                  (void*)sl.h_status, (void*)sl.h_wire, (void*)sl.h_tmpl, (void*)sl.h_wstatus})
    if (h) cudaFreeHost(h);
  if (sl.ready) cudaEventDestroy(sl.ready);
  if (sl.done) cudaEventDestroy(sl.done);
  if (sl.stream) cudaStreamDestroy(sl.stream);
}

// Caller holds s->mu.
void finish(ig_serve* s, Req* r, int status) {
  r->status = status;
  r->latency_ns = (u64)std::chrono::duration_cast<std::chrono::nanoseconds>(clk::now() - r->t_submit).count();
  if (status == IG_OK) {
    s->served++;
    s->latencies.push_back(r->latency_ns);
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

// Forms one batch on a free slot: the oldest waiting request and every later one with the
// same parameter set and mod-switch target, up to max_batch, in arrival order. Requests the
// context refuses finish here with the refusal. Returns the slot index, or -1 when nothing
// was batched. Caller holds s->mu and has seen a free slot (the context lock is taken
// inside, after s->mu).
int form_batch(ig_serve* s, CrsDev* crs_out, u64* ms_out) {
  int slot = -1;
  for (u32 k = 0; k < s->nslots; k++)
    if (!s->slots[k].busy) {
      slot = (int)k;
      break;
    }
  if (slot < 0) return -1;
  Slot& sl = s->slots[slot];
  sl.reqs.clear();
  bool have_head = false;
  u64 crs = 0, ms = 0;
  for (auto it = s->waiting.begin(); it != s->waiting.end() && sl.reqs.size() < s->max_batch;) {
    Req* r = *it;
    igint::RequestView v;
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
    if (!have_head) {
      have_head = true;
      crs = v.crs_handle;
      ms = r->ms;
      *crs_out = v.crs;
      *ms_out = ms;
    }
    if (v.crs_handle != crs || r->ms != ms) {
      ++it;
      continue;
    }
    const u32 i = (u32)sl.reqs.size();
    sl.h_table[i] = v.shard;
    QueryDev& q = sl.h_q[i];
    q.shard = i;
    q.reserved = 0;
    q.seed = (const u32*)(sl.d_seeds + (size_t)i * 32);
    q.b = sl.d_bs + (size_t)i * r->n;
    q.seat_R = v.seat;
    q.a = nullptr;
    sl.reqs.push_back(r);
    it = s->waiting.erase(it);
  }
  if (sl.reqs.empty()) return -1;
  sl.busy = true;
  return slot;
}

void dispatch_loop(ig_serve* s) {
  cudaSetDevice(igint::device(s->ctx));
  for (;;) {
    CrsDev crs{};
    u64 ms = 0;
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
        k = form_batch(s, &crs, &ms);
        if (k >= 0) break;
        s->cv_done.notify_all();  // requests refused while forming
      }
    }
    s->cv_done.notify_all();
    Slot& sl = s->slots[k];
    const u32 count = (u32)sl.reqs.size();
    const size_t n = crs.n;
    // Two CTAs per query only while the SMs left by the batches in flight hold them; with
    // other batches running, one CTA per query does the same work on fewer SMs.
    bool pair;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      pair = (int)count <= igint::pair_threshold(s->ctx) &&
             s->inflight_ctas + 2 * count <= (u32)igint::sm_count(s->ctx);
      sl.ctas = pair ? 2 * count : count;
      s->inflight_ctas += sl.ctas;
    }
    for (u32 i = 0; i < count; i++) {
      memcpy(sl.h_seeds + (size_t)i * 32, sl.reqs[i]->seed, 32);
      memcpy(sl.h_bs + i * n, sl.reqs[i]->b.data(), n * 8);
    }
    cudaStream_t st = sl.stream;
    // Ordered after every context call made before this batch formed (shard uploads, stores).
    cudaError_t e = cudaEventRecord(sl.ready, igint::stream(s->ctx));
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, sl.ready, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.d_q, sl.h_q, count * sizeof(QueryDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(sl.d_table, sl.h_table, count * sizeof(ShardDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.d_seeds, sl.h_seeds, (size_t)count * 32, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.d_bs, sl.h_bs, (size_t)count * n * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_status, 0, count * 4, st);
    if (e == cudaSuccess) e = igk::shard_scan(crs, sl.d_q, sl.d_table, count, sl.d_fold, sl.d_status, 0, nullptr, st);
    if (e == cudaSuccess)
      e = igk::respond(crs, sl.d_q, sl.d_table, count, sl.d_fold, ms, sl.d_a, sl.d_b, sl.d_status, 0, pair, st);
    if (e == cudaSuccess) {
      igint::add_launches(s->ctx, 2);
      e = cudaMemcpyAsync(sl.h_status, sl.d_status, count * 4, cudaMemcpyDeviceToHost, st);
    }
    // Outputs: the coefficient words for requests that want them, the wire bytes (built
    // here from the words, tight codec) for requests that want those.
    sl.want_ab = false;
    sl.wire_len = 0;
    bool want_wire = false;
    for (const Req* r : sl.reqs) (r->wire_out ? want_wire : sl.want_ab) = true;
    if (e == cudaSuccess && want_wire) {
      const u64 modulus = ms ? ms : Q;
      const unsigned bits = 64 - __builtin_clzll(modulus - 1);
      const u32 a_bytes = (u32)(((u64)n * bits + 7) / 8), b_bytes = (u32)(((u64)crs.gamma * bits + 7) / 8);
      std::vector<u64> zeros(n, 0);
      size_t len = 0;
      if (ig_response_encode(zeros.data(), zeros.data(), (u32)n, crs.gamma, modulus, sl.h_tmpl, kMaxWire, &len) ==
              IG_OK &&
          len <= kMaxWire) {
        sl.wire_len = len;
        e = cudaMemcpyAsync(sl.d_tmpl, sl.h_tmpl, len, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_wstatus, 0, count * 4, st);
        if (e == cudaSuccess)
          e = igk::wire(sl.d_a, sl.d_b, count, (u32)n, crs.gamma, bits, modulus, sl.d_tmpl, (u32)len, 12, a_bytes,
                        12 + a_bytes + 41 + 8, b_bytes, sl.d_wire, sl.d_wstatus, st);
        if (e == cudaSuccess) {
          igint::add_launches(s->ctx, 1);
          e = cudaMemcpyAsync(sl.h_wire, sl.d_wire, (size_t)count * len, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(sl.h_wstatus, sl.d_wstatus, count * 4, cudaMemcpyDeviceToHost, st);
      }
    }
    if (e == cudaSuccess && sl.want_ab)
      e = cudaMemcpyAsync(sl.h_a, sl.d_a, (size_t)count * n * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && sl.want_ab)
      e = cudaMemcpyAsync(sl.h_b, sl.d_b, (size_t)count * n * 8, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(sl.done, st);
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
      s->launched.pop_front();
    }
    Slot& sl = s->slots[k];
    const cudaError_t e = cudaEventSynchronize(sl.done);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (size_t i = 0; i < sl.reqs.size(); i++) {
        Req* r = sl.reqs[i];
        if (sl.launch_err || e != cudaSuccess) {
          refuse(s, r, IG_ERR_CUDA, "serving launch failed: %s",
                 cudaGetErrorString(sl.launch_err ? (cudaError_t)sl.launch_err : e));
        } else if (sl.h_status[i] & DEV_TAG_MISMATCH) {
          refuse(s, r, IG_ERR_STORE_REFUSED,
                 "shard %u: packing store refused: a column is not the column the store was built from. The shard "
                 "changed after the build; rebuild the store before serving it",
                 r->shard);
        } else if (sl.h_status[i]) {
          refuse(s, r, IG_ERR_DEVICE, "respond kernel status %u", sl.h_status[i]);
        } else if (r->wire_out) {
          if (sl.wire_len == 0 || sl.h_wstatus[i]) {
            refuse(s, r, IG_ERR_SHAPE, "ServerResponse encode refused: coefficients must be canonical");
          } else if (sl.wire_len > r->wire_cap) {
            refuse(s, r, IG_ERR_ARG, "wire buffer of %zu bytes is smaller than the %zu-byte response", r->wire_cap,
                   sl.wire_len);
          } else {
            memcpy(r->wire_out, sl.h_wire + i * sl.wire_len, sl.wire_len);
            *r->wire_len = sl.wire_len;
            finish(s, r, IG_OK);
          }
        } else {
          memcpy(r->a_out, sl.h_a + i * r->n, (size_t)r->n * 8);
          memcpy(r->b_out, sl.h_b + i * r->n, (size_t)r->n * 8);
          finish(s, r, IG_OK);
        }
      }
      sl.reqs.clear();
      sl.busy = false;
      s->inflight_ctas -= sl.ctas;
      sl.ctas = 0;
    }
    s->cv_slot.notify_all();
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

int ig_serve_create(ig_ctx* ctx, uint32_t slots, uint32_t max_batch, uint64_t hbm_budget_bytes, ig_serve** out) {
  if (!ctx) return IG_ERR_ARG;
  if (!out || slots == 0 || max_batch == 0 || slots > 64 || max_batch > 4096)
    return igint::fail(ctx, IG_ERR_ARG, "ig_serve_create: need 1..64 slots of 1..4096 queries and an out pointer");
  const u64 need = (u64)slot_device_bytes(max_batch) * slots;
  if (hbm_budget_bytes && need > hbm_budget_bytes)
    return igint::fail(ctx, IG_ERR_NOMEM,
                       "serving loop refused: %u slots of %u queries need %llu device bytes, the budget is %llu",
                       slots, max_batch, (unsigned long long)need, (unsigned long long)hbm_budget_bytes);
  cudaSetDevice(igint::device(ctx));
  auto* s = new ig_serve();
  s->ctx = ctx;
  s->max_batch = max_batch;
  s->nslots = slots;
  s->max_waiting = (u64)slots * max_batch * 8;
  s->slots.resize(slots);
  {
    std::lock_guard<std::mutex> lk(igint::mutex(ctx));
    for (auto& sl : s->slots) {
      const int rc = alloc_slot(s, sl);
      if (rc) {
        for (auto& x : s->slots) free_slot(s, x);
        delete s;
        return rc;
      }
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
  s->dispatcher.join();
  s->cv_launched.notify_all();
  s->completer.join();
  {
    std::lock_guard<std::mutex> lk(igint::mutex(s->ctx));
    for (auto& sl : s->slots) free_slot(s, sl);
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
  }
  s->cv_work.notify_one();
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
  std::vector<u64> v = s->latencies;
  std::sort(v.begin(), v.end());
  auto pct = [&](double p) -> double {
    if (v.empty()) return 0.0;
    size_t i = (size_t)(p * (double)v.size());
    if (i >= v.size()) i = v.size() - 1;
    return (double)v[i] / 1e3;
  };
  out->served = s->served;
  out->refused = s->refused;
  out->batches = s->batches;
  out->waiting = s->waiting.size();
  out->device_bytes = s->device_bytes;
  out->mean_batch = s->batches ? (double)s->batched_queries / (double)s->batches : 0.0;
  out->p50_us = pct(0.50);
  out->p99_us = pct(0.99);
  out->max_us = v.empty() ? 0.0 : (double)v.back() / 1e3;
  if (reset) {
    s->latencies.clear();
    s->served = s->refused = s->batches = s->batched_queries = 0;
  }
  return IG_OK;
}

}  // extern "C"
