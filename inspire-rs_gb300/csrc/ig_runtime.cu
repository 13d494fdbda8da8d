// Host runtime behind the C ABI of include/inspire_gb300.h: device residency of the
// per-parameter-set constants, shards, packing stores and seats, request validation with
// the reference's refusal rules, and the launch sequence of a respond batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/inspire_gb300.h"
#include "ig_internal.hpp"
#include "ig_kernels.cuh"

using namespace ig;

namespace {

// ---------------------------------------------------------------------------------------
// Host modular helpers over q.
u64 mulmod(u64 a, u64 b) { return (u64)((u128)a * b % Q); }
u64 powmod(u64 b, u64 e) {
  u64 r = 1;
  b %= Q;
  while (e) {
    if (e & 1) r = mulmod(r, b);
    b = mulmod(b, b);
    e >>= 1;
  }
  return r;
}
u64 invmod(u64 a) { return powmod(a, Q - 2); }
const u64 R_MOD_Q = (u64)((((u128)1) << 64) % Q);

// Least root of the search NttContext::find_primitive_root makes (math/ntt.rs:743-752),
// so the slot order matches the reference's transform.
u64 find_root(u64 order) {
  const u64 e = (Q - 1) / order;
  for (u64 g = 2; g < (1u << 16); g++) {
    u64 c = powmod(g, e);
    if (powmod(c, order) == 1 && powmod(c, order / 2) != 1) return c;
  }
  return 0;
}

// Bit-reversed power ladder f[m] (math/ntt.rs:780-804).
std::vector<u64> ladder(size_t n, u64 psi) {
  std::vector<u64> f(n, 0);
  f[1] = 1;
  for (size_t m = 1; m < n; m++) {
    if ((m & (m - 1)) == 0)
      f[m] = powmod(psi, n / (2 * m));
    else
      f[m] = mulmod(f[m & (m - 1)], f[m & (~m + 1)]);
  }
  return f;
}

void host_ntt(std::vector<u64>& x, const std::vector<u64>& tw) {
  size_t n = x.size(), t = n;
  for (size_t m = 1; m < n; m <<= 1) {
    t >>= 1;
    for (size_t i = 0; i < m; i++) {
      size_t j1 = 2 * i * t;
      for (size_t j = j1; j < j1 + t; j++) {
        u64 u = x[j], v = mulmod(x[j + t], tw[m + i]);
        x[j] = addq(u, v);
        x[j + t] = subq(u, v);
      }
    }
  }
}

struct HostChaCha {
  u32 key[8];
  u64 stream, word = 0;
  u32 blk[16];
  u64 have = ~0ULL;
  HostChaCha(const uint8_t seed[32], u64 s) : stream(s) {
    for (int i = 0; i < 8; i++) memcpy(&key[i], seed + 4 * i, 4);
  }
  u32 next_u32() {
    u64 b = word / 16;
    if (b != have) {
      chacha20_block(key, b, stream, blk);
      have = b;
    }
    return blk[word++ % 16];
  }
  u64 next_u64() {
    u64 lo = next_u32();
    return lo | ((u64)next_u32() << 32);
  }
};

// ---------------------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct CrsObj {
  u32 n = 0, logn = 0, gamma = 0, rows = 0, approx = 0;
  u64 p = 0;
  CrsDev dev{};
  CrsDev* d_self = nullptr;  // device copy of `dev`, named by the queries of mixed launches
  std::vector<void*> allocs;
  size_t bytes = 0;
};

struct ShardSlot {
  u64* cols = nullptr;
  u64* sums = nullptr;
  u64* tag_key = nullptr;
  u64* tags = nullptr;
  uint16_t* cols16 = nullptr;  // u16 copy of the columns; valid when `compact`
  bool compact = false;
  // The columns changed after the store was built and no longer give its tags
  // (shard_store.rs:247-257): responds on the shard are refused until the store is rebuilt.
  bool stale = false;
  // The device table entry of this shard.
  ShardDev dev() const { return ShardDev{cols, sums, tag_key, tags, compact ? cols16 : nullptr, stale ? 1u : 0u, 0}; }
};

struct DbObj {
  u64 crs = 0;
  u32 num_shards = 0;
  std::vector<ShardSlot> shards;
  ShardDev* d_table = nullptr;
  size_t bytes = 0;
};

struct SeatObj {
  u64 crs = 0;
  u32 n = 0, rows = 0, num_to_pack = 0;
  u64* yR = nullptr;
};

struct StoreObj {
  std::unordered_map<u64, SeatObj> seats;
};

// A client session on the device (ClientSession, session.rs): the secret's NTT in R-form
// and the sampler's acceptance thresholds.
struct ClientObj {
  u64 crs = 0;
  u64* s_R = nullptr;
  u64* accept = nullptr;
  GaussDev g{};
  u64 max_abs_s = 0;  // largest |s_k| of the centred secret
  std::vector<void*> allocs;
  size_t bytes = 0;
};

std::atomic<u64> g_next_handle{0};  // process-global, monotonic (session.rs:715-738)
std::atomic<u64> g_next_object{1};

}  // namespace

enum : u32 { IG_MAX_LANES = 8 };

struct ig_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string err;
  mutable std::mutex err_mu;  // err is written by the serving threads too
  std::unordered_map<u64, CrsObj> crs;
  std::unordered_map<u64, DbObj> dbs;
  std::unordered_map<u64, StoreObj> stores;
  std::unordered_map<u64, ClientObj> clients;
  std::unordered_map<std::string, DevBuf> scratch;
  u64* zero_key = nullptr;
  size_t zero_key_words = 0;
  size_t obj_bytes = 0;
  int force_serial = 0;
  // Per-region CUDA-event timing of the device respond path (RegionProfile of
  // respond.rs:1295-1345 on the GPU): pairs of events around each kernel launch.
  int profile = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
  std::vector<std::pair<int, size_t>> ev_used;  // (region, pool index)
  std::atomic<u64> launches{0};
  // Pinned staging ring for host->device copies issued on the stream: slot k is reused
  // only after the copy that last read it has completed.
  struct Staging {
    void* host = nullptr;
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
  };
  std::vector<Staging> staging;
  size_t staging_next = 0;
  // Batches of at most this many queries run two CTAs per query (a cluster of two), so
  // a batch smaller than the SM count still occupies most SMs. Default: half the SMs.
  u32 pair_threshold = 0;
  // Device-path lanes: with lanes > 1, consecutive ig_respond_seeded_batch_device calls
  // rotate over that many streams, each with its own scratch, so batches overlap on the
  // device; ig_ctx_join orders the context stream after all of them.
  u32 lanes = 1, lane_next = 0, sms = 0;
  // Host-side fault injection: the device allocation `fail_alloc_at` calls from now fails
  // (1 = the next one; 0 = none).
  std::atomic<u32> fail_alloc_at{0};
  // Launch shape of respond launches (CTAs per query). force_ctas != 0 fixes it; otherwise,
  // with a tuned entry for the launch's (ring, gamma), the shape whose measured launch time
  // is least at the number of queries expected in flight, else the fixed rule on
  // pair_threshold (four CTAs up to half of it, two up to it). tune[(n, gamma)] maps a batch size to the measured milliseconds of one launch of
  // that many queries under 1, 2 and 4 CTAs per query.
  u32 force_ctas = 0;
  std::map<std::pair<u32, u32>, std::map<u32, std::array<double, 3>>> tune;
  cudaStream_t lane_stream[IG_MAX_LANES] = {};
  cudaEvent_t lane_in[IG_MAX_LANES] = {}, lane_done[IG_MAX_LANES] = {};
  bool lane_used[IG_MAX_LANES] = {};
  // Host-buffer calls over lanes: a lane's mutex is held by one call from before its
  // launches until its results have left the lane's pinned buffer, so several caller
  // threads can have batches in flight while the context lock is held only to launch.
  struct HostLane {
    std::mutex mu;
    void* pin = nullptr;  // pinned status, a and b of the call in flight
    size_t pin_bytes = 0;
    cudaEvent_t done = nullptr;
  };
  HostLane hlane[IG_MAX_LANES];
  std::atomic<u32> hlane_next{0};
  // special_modulus objects (ig_sm_runtime.cu) and their destructor.
  void* sm = nullptr;
  void (*sm_destroy)(ig_ctx*, void*) = nullptr;
};

namespace {

enum Region { REGION_SCAN = 0, REGION_RESPOND = 1, REGION_FOLD = 2, REGION_COUNT = 3 };

// Starts a profiled region on the context stream; returns the pool slot or -1.
long prof_begin(ig_ctx* c, int region, cudaStream_t st = nullptr) {
  c->launches++;
  if (!c->profile) return -1;
  size_t k = c->ev_used.size();
  if (k == c->ev_pool.size()) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return -1;
    c->ev_pool.push_back({a, b});
  }
  c->ev_used.push_back({region, k});
  cudaEventRecord(c->ev_pool[k].first, st ? st : c->stream);
  return (long)k;
}
void prof_end(ig_ctx* c, long k, cudaStream_t st = nullptr) {
  if (k >= 0) cudaEventRecord(c->ev_pool[k].second, st ? st : c->stream);
}

int fail(ig_ctx* c, int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) {
    std::lock_guard<std::mutex> lk(c->err_mu);
    c->err = buf;
  }
  return code;
}

#define IG_CUDA(ctx, call)                                                                        \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? IG_ERR_NOMEM : IG_ERR_CUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                             \
  } while (0)

int dalloc(ig_ctx* c, void** p, size_t bytes, size_t* counter) {
  u32 at = c->fail_alloc_at.load();
  while (at && !c->fail_alloc_at.compare_exchange_weak(at, at - 1)) {
  }
  if (at == 1) {
    *p = nullptr;
    return fail(c, IG_ERR_NOMEM, "device allocation of %zu bytes failed: injected failure", bytes);
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(c, IG_ERR_NOMEM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  if (counter) *counter += bytes;
  c->obj_bytes += bytes;
  return IG_OK;
}

void dfree(ig_ctx* c, void* p, size_t bytes) {
  if (p) {
    cudaFree(p);
    c->obj_bytes -= bytes;
  }
}

// Grow-only scratch buffer by name.
int scratch(ig_ctx* c, const char* name, size_t bytes, void** out) {
  DevBuf& b = c->scratch[name];
  if (b.bytes < bytes) {
    if (b.p) dfree(c, b.p, b.bytes);
    b.p = nullptr;
    b.bytes = 0;
    size_t want = bytes + bytes / 4;
    int rc = dalloc(c, &b.p, want, nullptr);
    if (rc) return rc;
    b.bytes = want;
  }
  *out = b.p;
  return IG_OK;
}

// Copies `bytes` from host memory to `dst` on the context stream through a pinned slot,
// so the call returns without waiting for the device.
int stage_h2d(ig_ctx* c, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return IG_OK;
  if (c->staging.empty()) c->staging.resize(8);
  ig_ctx::Staging& sl = c->staging[c->staging_next];
  c->staging_next = (c->staging_next + 1) % c->staging.size();
  if (sl.done) IG_CUDA(c, cudaEventSynchronize(sl.done));
  if (sl.bytes < bytes) {
    if (sl.host) cudaFreeHost(sl.host);
    sl.host = nullptr;
    sl.bytes = 0;
    size_t want = bytes + bytes / 2;
    IG_CUDA(c, cudaHostAlloc(&sl.host, want, cudaHostAllocDefault));
    sl.bytes = want;
  }
  if (!sl.done) IG_CUDA(c, cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
  memcpy(sl.host, src, bytes);
  IG_CUDA(c, cudaMemcpyAsync(dst, sl.host, bytes, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, cudaEventRecord(sl.done, c->stream));
  return IG_OK;
}

int zero_key(ig_ctx* c, size_t words, u64** out) {
  if (c->zero_key_words < words) {
    if (c->zero_key) dfree(c, c->zero_key, c->zero_key_words * 8);
    c->zero_key = nullptr;
    int rc = dalloc(c, (void**)&c->zero_key, words * 8, nullptr);
    if (rc) return rc;
    c->zero_key_words = words;
    IG_CUDA(c, cudaMemset(c->zero_key, 0, words * 8));
  }
  *out = c->zero_key;
  return IG_OK;
}

template <class T>
int upload(ig_ctx* c, CrsObj& o, const std::vector<T>& v, const T** dst) {
  void* p;
  int rc = dalloc(c, &p, v.size() * sizeof(T), &o.bytes);
  if (rc) return rc;
  o.allocs.push_back(p);
  IG_CUDA(c, cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *dst = (const T*)p;
  return IG_OK;
}

CrsObj* get_crs(ig_ctx* c, u64 h) {
  auto it = c->crs.find(h);
  return it == c->crs.end() ? nullptr : &it->second;
}
DbObj* get_db(ig_ctx* c, u64 h) {
  auto it = c->dbs.find(h);
  return it == c->dbs.end() ? nullptr : &it->second;
}

// The CRS's device copy of its constants (allocated once, rewritten when they change).
int sync_crs_self(ig_ctx* c, CrsObj& o) {
  if (!o.d_self) {
    void* p = nullptr;
    int rc = dalloc(c, &p, sizeof(CrsDev), &o.bytes);
    if (rc) return rc;
    o.allocs.push_back(p);
    o.d_self = (CrsDev*)p;
  }
  IG_CUDA(c, cudaMemcpyAsync(o.d_self, &o.dev, sizeof(CrsDev), cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  return IG_OK;
}

int sync_table_entry(ig_ctx* c, DbObj& db, u32 s) {
  const ShardDev d = db.shards[s].dev();
  IG_CUDA(c, cudaMemcpyAsync(db.d_table + s, &d, sizeof d, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  return IG_OK;
}

// Folds step 1 over `cols` into `sums` (gamma x n, R-form): gamma forward transforms,
// then the per-slot DFT fold.
int fold_store(ig_ctx* c, CrsObj& o, const u64* cols, u64* sums) {
  void* H;
  int rc = scratch(c, "fold_H", (size_t)o.gamma * o.n * 8, &H);
  if (rc) return rc;
  long k = prof_begin(c, REGION_FOLD);
  c->launches++;
  IG_CUDA(c, igk::ntt_rows(o.dev, cols, (u64*)H, o.gamma, 1, shoup_companion(1), c->stream));
  IG_CUDA(c, igk::store_fold(o.dev, (const u64*)H, sums, c->stream));
  prof_end(c, k);
  return IG_OK;
}

int build_store(ig_ctx* c, DbObj& db, CrsObj& o, u32 s) {
  ShardSlot& sl = db.shards[s];
  if (!sl.cols)
    return fail(c, IG_ERR_ARG, "shard %u: no columns uploaded; precompute_packing needs the shard's columns", s);
  const size_t n = o.n, g = o.gamma;
  if (!sl.sums) {
    // All three buffers or none: a shard counts as stored when `sums` is set.
    u64 *sums = nullptr, *key = nullptr, *tags = nullptr;
    size_t got = 0;
    int rc = dalloc(c, (void**)&sums, g * n * 8, &got);
    if (!rc) rc = dalloc(c, (void**)&key, 2 * n * 8, &got);
    if (!rc) rc = dalloc(c, (void**)&tags, g * 8, &got);
    if (rc) {
      if (sums) dfree(c, sums, g * n * 8);
      if (key) dfree(c, key, 2 * n * 8);
      return rc;
    }
    db.bytes += got;
    sl.sums = sums;
    sl.tag_key = key;
    sl.tags = tags;
  }
  // Tag key: two words per column word below 2^61 - 1, drawn from OS entropy and never
  // leaving the device (shard_store.rs:127-135).
  std::random_device rd;
  uint8_t seed[32];
  for (int i = 0; i < 8; i++) {
    u32 v = rd();
    memcpy(seed + 4 * i, &v, 4);
  }
  HostChaCha rng(seed, 0);
  std::vector<u64> key(2 * n);
  for (auto& k : key) {
    u64 cand;
    do cand = rng.next_u64() >> 3;
    while (cand >= (1ULL << 61) - 1);
    k = cand;
  }
  IG_CUDA(c, cudaMemcpyAsync(sl.tag_key, key.data(), key.size() * 8, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, igk::column_tags(o.dev, sl.cols, sl.tag_key, sl.tags, nullptr, nullptr, c->stream));
  int rc = fold_store(c, o, sl.cols, sl.sums);
  if (rc) return rc;
  c->launches++;
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  sl.stale = false;
  return sync_table_entry(c, db, s);
}

// After new columns land in a shard that holds a store: the columns' tags against the
// store's (the check shard_store.rs:197-264 makes at every respond, made here once per
// change, since the library writes every column word itself). A mismatch marks the shard
// stale; columns equal to the stored ones keep it served.
int check_store_tags(ig_ctx* c, CrsObj& o, ShardSlot& sl) {
  if (!sl.sums) {
    sl.stale = false;
    return IG_OK;
  }
  void* flag;
  int rc = scratch(c, "tag_mismatch", 4, &flag);
  if (rc) return rc;
  IG_CUDA(c, cudaMemsetAsync(flag, 0, 4, c->stream));
  IG_CUDA(c, igk::column_tags(o.dev, sl.cols, sl.tag_key, nullptr, sl.tags, (u32*)flag, c->stream));
  c->launches++;
  u32 mismatch = 1;
  IG_CUDA(c, cudaMemcpyAsync(&mismatch, flag, 4, cudaMemcpyDeviceToHost, c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  sl.stale = mismatch != 0;
  return IG_OK;
}

}  // namespace

namespace igint {
int fail(ig_ctx* c, int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) {
    std::lock_guard<std::mutex> lk(c->err_mu);
    c->err = buf;
  }
  return code;
}
cudaStream_t stream(ig_ctx* c) { return c->stream; }
int device(ig_ctx* c) { return c->device; }
std::mutex& mutex(ig_ctx* c) { return c->mu; }
int dalloc(ig_ctx* c, void** p, size_t bytes) { return ::dalloc(c, p, bytes, nullptr); }
void dfree(ig_ctx* c, void* p, size_t bytes) { ::dfree(c, p, bytes); }
int scratch(ig_ctx* c, const char* name, size_t bytes, void** out) { return ::scratch(c, name, bytes, out); }
int stage_h2d(ig_ctx* c, void* dst, const void* src, size_t bytes) { return ::stage_h2d(c, dst, src, bytes); }
void add_launches(ig_ctx* c, unsigned n) { c->launches += n; }
void*& sm_slot(ig_ctx* c) { return c->sm; }
// The tuned row for `queries` in flight: the smallest measured batch size at or above it
// (the largest measured one beyond the grid), of the tuned width nearest gamma on ring n.
static const std::array<double, 3>* tuned_row(ig_ctx* c, u32 n, u32 gamma, u32 queries) {
  auto it = c->tune.find({n, gamma});
  if (it == c->tune.end()) {
    for (auto jt = c->tune.begin(); jt != c->tune.end(); ++jt) {
      if (jt->first.first != n) continue;
      const u32 dj = jt->first.second > gamma ? jt->first.second - gamma : gamma - jt->first.second;
      const u32 di = it == c->tune.end() ? ~0u
                                         : (it->first.second > gamma ? it->first.second - gamma : gamma - it->first.second);
      if (dj < di) it = jt;
    }
  }
  if (it == c->tune.end() || it->second.empty()) return nullptr;
  auto row = it->second.lower_bound(queries);
  if (row == it->second.end()) --row;
  return &row->second;
}

int launch_ctas(ig_ctx* c, u32 n, u32 gamma, u32 count, u32 in_flight) {
  if (c->force_ctas) return (int)c->force_ctas;
  const u32 queries = std::max(count, in_flight);
  const std::array<double, 3>* row = tuned_row(c, n, gamma, queries);
  if (!row) {  // the fixed rule: as many CTAs per query as the threshold leaves room for
    const u64 t = c->pair_threshold;
    return 2 * (u64)queries <= t ? 4 : (u64)queries <= t ? 2 : 1;
  }
  const int shapes[3] = {1, 2, 4};
  int best = 1;
  double best_ms = 0;
  for (int k = 0; k < 3; k++) {
    const double t = (*row)[k];
    if (!(t > 0)) continue;
    if (best_ms == 0 || t < best_ms * 0.98) {  // a shape must be 2% faster to take more SMs
      best = shapes[k];
      best_ms = t;
    }
  }
  return best;
}
int forced_ctas(ig_ctx* c) { return (int)c->force_ctas; }
int lanes(ig_ctx* c) { return (int)c->lanes; }
int lane_acquire(ig_ctx* c, cudaStream_t* s, int* lane) {
  *lane = -1;
  *s = c->stream;
  if (c->lanes <= 1) return IG_OK;
  const int k = (int)(c->lane_next++ % c->lanes);
  if (c->lane_used[k]) IG_CUDA(c, cudaStreamWaitEvent(c->stream, c->lane_done[k], 0));
  *lane = k;
  *s = c->lane_stream[k];
  return IG_OK;
}
void host_call_begin(ig_ctx* c, HostCall& hc) {
  hc.k = c->lanes > 1 ? c->hlane_next.fetch_add(1) % c->lanes : 0;
  hc.lane_lock = std::unique_lock<std::mutex>(c->hlane[hc.k].mu);
}
int host_call_pinned(ig_ctx* c, HostCall& hc, size_t bytes, void** pin) {
  ig_ctx::HostLane& hl = c->hlane[hc.k];
  if (hl.pin_bytes < bytes) {
    if (hl.pin) cudaFreeHost(hl.pin);
    hl.pin = nullptr;
    hl.pin_bytes = 0;
    IG_CUDA(c, cudaHostAlloc(&hl.pin, bytes, cudaHostAllocDefault));
    hl.pin_bytes = bytes;
  }
  if (!hl.done) IG_CUDA(c, cudaEventCreateWithFlags(&hl.done, cudaEventDisableTiming));
  *pin = hl.pin;
  return IG_OK;
}
cudaStream_t host_call_stream(ig_ctx* c, HostCall& hc) { return c->lanes > 1 ? c->lane_stream[hc.k] : c->stream; }
int host_call_enter(ig_ctx* c, HostCall& hc) {
  if (c->lanes <= 1) return IG_OK;
  IG_CUDA(c, cudaEventRecord(c->lane_in[hc.k], c->stream));
  IG_CUDA(c, cudaStreamWaitEvent(c->lane_stream[hc.k], c->lane_in[hc.k], 0));
  return IG_OK;
}
int host_call_launched(ig_ctx* c, HostCall& hc) {
  cudaStream_t s = host_call_stream(c, hc);
  IG_CUDA(c, cudaEventRecord(c->hlane[hc.k].done, s));
  if (c->lanes > 1) {
    IG_CUDA(c, cudaEventRecord(c->lane_done[hc.k], s));
    c->lane_used[hc.k] = true;
  }
  return IG_OK;
}
int host_call_wait(ig_ctx* c, HostCall& hc) {
  IG_CUDA(c, cudaEventSynchronize(c->hlane[hc.k].done));
  return IG_OK;
}
int lane_enter(ig_ctx* c, int lane) {
  if (lane < 0) return IG_OK;
  IG_CUDA(c, cudaEventRecord(c->lane_in[lane], c->stream));
  IG_CUDA(c, cudaStreamWaitEvent(c->lane_stream[lane], c->lane_in[lane], 0));
  return IG_OK;
}
int lane_release(ig_ctx* c, int lane) {
  if (lane < 0) return IG_OK;
  IG_CUDA(c, cudaEventRecord(c->lane_done[lane], c->lane_stream[lane]));
  c->lane_used[lane] = true;
  return IG_OK;
}
int sm_count(ig_ctx* c) { return (int)c->sms; }
void set_sm_destructor(ig_ctx* c, void (*fn)(ig_ctx*, void*)) { c->sm_destroy = fn; }
}  // namespace igint

// =========================================================================================
extern "C" {

int ig_ctx_create(int device, ig_ctx** out) {
  if (!out) return IG_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return IG_ERR_CUDA;
  }
  if (device < 0 || device >= count) return IG_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return IG_ERR_CUDA;
  auto* c = new ig_ctx();
  c->device = device;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  c->pair_threshold = (u32)(sms / 2);
  c->sms = (u32)sms;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return IG_ERR_CUDA;
  }
  *out = c;
  return IG_OK;
}

void ig_ctx_destroy(ig_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (u32 k = 0; k < IG_MAX_LANES; k++) {
    if (c->lane_stream[k]) {
      cudaStreamSynchronize(c->lane_stream[k]);
      cudaStreamDestroy(c->lane_stream[k]);
      cudaEventDestroy(c->lane_in[k]);
      cudaEventDestroy(c->lane_done[k]);
    }
    if (c->hlane[k].pin) cudaFreeHost(c->hlane[k].pin);
    if (c->hlane[k].done) cudaEventDestroy(c->hlane[k].done);
  }
  if (c->sm && c->sm_destroy) c->sm_destroy(c, c->sm);
  for (auto& kv : c->crs)
    for (void* p : kv.second.allocs) cudaFree(p);
  for (auto& kv : c->dbs) {
    for (auto& s : kv.second.shards) {
      cudaFree(s.cols);
      cudaFree(s.sums);
      cudaFree(s.tag_key);
      cudaFree(s.tags);
      cudaFree(s.cols16);
    }
    cudaFree(kv.second.d_table);
  }
  for (auto& kv : c->stores)
    for (auto& s : kv.second.seats) cudaFree(s.second.yR);
  for (auto& kv : c->clients)
    for (void* p : kv.second.allocs) cudaFree(p);
  for (auto& kv : c->scratch) cudaFree(kv.second.p);
  for (auto& st : c->staging) {
    if (st.host) cudaFreeHost(st.host);
    if (st.done) cudaEventDestroy(st.done);
  }
  for (auto& ev : c->ev_pool) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  cudaFree(c->zero_key);
  cudaStreamDestroy(c->stream);
  delete c;
}

int ig_last_error(const ig_ctx* c, char* buf, size_t len) {
  if (!c || !buf || len == 0) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->err_mu);
  snprintf(buf, len, "%s", c->err.c_str());
  return IG_OK;
}

void* ig_ctx_stream(ig_ctx* c) { return c ? (void*)c->stream : nullptr; }

uint64_t ig_ctx_device_bytes(const ig_ctx* c) { return c ? c->obj_bytes : 0; }

int ig_crs_create(ig_ctx* c, uint32_t n, uint64_t q, uint64_t p, uint64_t gadget_base, uint32_t glen, int approx,
                  uint32_t gamma, const uint8_t w_seed[32], uint64_t* crs_out) {
  if (!c || !w_seed || !crs_out) return fail(c, IG_ERR_ARG, "ig_crs_create: null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (q != Q)
    return fail(c, IG_ERR_UNSUPPORTED, "ciphertext modulus %llu is not served on the GPU path; only q = 2^60-2^14+1",
                (unsigned long long)q);
  if (gadget_base != (1ULL << 20) || glen != 3)
    return fail(c, IG_ERR_UNSUPPORTED, "packing gadget base %llu length %u is not served; only base 2^20 length 3",
                (unsigned long long)gadget_base, glen);
  if (n < 256 || n > 2048 || (n & (n - 1)))
    return fail(c, IG_ERR_UNSUPPORTED, "ring_dim %u is not served; the GPU path covers powers of two in [256, 2048]", n);
  if (gamma == 0 || (gamma & (gamma - 1)) || gamma > n / 2)
    return fail(c, IG_ERR_WIDTH,
                "InspiRING packing width %u is illegal at ring_dim %u: the width must be a power of two in [1, %u]",
                gamma, n, n / 2);
  if (p < 2 || p >= q) return fail(c, IG_ERR_ARG, "plaintext modulus %llu outside [2, q)", (unsigned long long)p);
  CrsObj o;
  o.n = n;
  o.logn = 0;
  while ((1u << o.logn) < n) o.logn++;
  o.gamma = gamma;
  o.approx = approx ? 1 : 0;
  o.rows = glen - o.approx;
  o.p = p;
  const u64 two_n = 2ULL * n;
  const u64 psi = find_root(two_n);
  std::vector<u64> tw = ladder(n, psi);
  std::vector<u64> twp(n);
  for (u32 m = 0; m < n; m++) twp[m] = shoup_companion(tw[m]);
  // Slot roots: slot t of the forward transform of X holds root w_t = w0^e_t.
  std::vector<u64> X(n, 0);
  X[1] = 1;
  host_ntt(X, tw);
  std::unordered_map<u64, u32> exp_of;
  u64 w0 = X[0], w0sq = mulmod(w0, w0), pw = w0;
  for (u64 e = 1; e < two_n; e += 2) {
    exp_of[pw] = (u32)e;
    pw = mulmod(pw, w0sq);
  }
  std::vector<uint16_t> slot_exp(n), exp_slot(n, 0xffff);
  for (u32 t = 0; t < n; t++) {
    auto it = exp_of.find(X[t]);
    if (it == exp_of.end()) return fail(c, IG_ERR_UNSUPPORTED, "automorphism tables are undefined at ring_dim %u", n);
    slot_exp[t] = (uint16_t)it->second;
    exp_slot[it->second / 2] = (uint16_t)t;
  }
  // Slots and odd exponents must pair one to one: the kernels index shared memory by
  // these tables.
  for (u32 e = 0; e < n; e++)
    if (exp_slot[e] >= n)
      return fail(c, IG_ERR_UNSUPPORTED, "automorphism tables are undefined at ring_dim %u: slot roots repeat", n);
  const u64 g = two_n / gamma + 1;
  u64 ginv = 1;  // g^(gamma-1) = g^-1 in Z*_2n
  for (u32 k = 0; k + 1 < gamma; k++) ginv = ginv * g % two_n;
  std::vector<u32> gpow(gamma), cpow(gamma), m_of_i(gamma);
  u64 a = 1, b = 1;
  const u64 L = two_n / gamma;
  for (u32 i = 0; i < gamma; i++) {
    gpow[i] = (u32)a;
    cpow[i] = (u32)b;
    if ((b - 1) % L != 0) return fail(c, IG_ERR_UNSUPPORTED, "generator subgroup is not 1 mod 2n/gamma");
    m_of_i[i] = (u32)((b - 1) / L);
    a = a * g % two_n;
    b = b * ginv % two_n;
  }
  std::vector<u64> pow_root_R(two_n);
  u64 acc = 1;
  for (u64 e = 0; e < two_n; e++) {
    pow_root_R[e] = mulmod(acc, R_MOD_Q);
    acc = mulmod(acc, w0);
  }
  // Offline mask rows: ChaCha20(w_seed) on stream 0 (exact) or gamma (approximate),
  // next_u64 mod q, the dropped digits' rows skipped (inspiring2.rs:839-887).
  HostChaCha rng(w_seed, o.approx ? gamma : 0);
  std::vector<u64> mask;
  for (u32 r = 0; r < glen; r++)
    for (u32 k = 0; k < n; k++) {
      u64 v = rng.next_u64() % Q;
      if (r >= o.approx) mask.push_back(v);
    }
  CrsDev& d = o.dev;
  d.n = n;
  d.logn = o.logn;
  d.gamma = gamma;
  d.rows = o.rows;
  d.approx = o.approx;
  int rc;
  if ((rc = upload(c, o, tw, &d.tw)) || (rc = upload(c, o, twp, &d.twp)) || (rc = upload(c, o, slot_exp, &d.slot_exp)) ||
      (rc = upload(c, o, exp_slot, &d.exp_slot)) || (rc = upload(c, o, gpow, &d.gpow)) ||
      (rc = upload(c, o, cpow, &d.cpow)) || (rc = upload(c, o, m_of_i, &d.m_of_i)) ||
      (rc = upload(c, o, pow_root_R, &d.pow_root_R))) {
    for (void* p2 : o.allocs) cudaFree(p2);
    c->obj_bytes -= o.bytes;
    return rc;
  }
  d.ninv = invmod(n);
  d.ninvp = shoup_companion(d.ninv);
  d.nlast = mulmod(d.ninv, negq(tw[1]));
  d.nlastp = shoup_companion(d.nlast);
  d.inv_gamma_R = mulmod(invmod(gamma), R_MOD_Q);
  d.inv_gamma_Rp = shoup_companion(d.inv_gamma_R);
  // Last exact digit: base^-2 (R - D0 - base D1) (inspiring2.rs:1094-1161). The kernels
  // fold these three factors into the key rows (fold_gadget3) rather than form the digit.
  const u64 inv = invmod(1ULL << 40);
  d.ld_inv_R = mulmod(inv, R_MOD_Q);
  d.ld_c0_R = mulmod(negq(inv), R_MOD_Q);
  d.ld_c1_R = mulmod(negq(mulmod(inv, 1ULL << 20)), R_MOD_Q);
  // Mask rows -> NTT, R-form.
  void* mraw = nullptr;
  void* wm = nullptr;
  rc = scratch(c, "mask_raw", mask.size() * 8, &mraw);
  if (!rc) rc = dalloc(c, &wm, mask.size() * 8, &o.bytes);
  if (rc) {
    for (void* p2 : o.allocs) cudaFree(p2);
    c->obj_bytes -= o.bytes;
    return rc;
  }
  o.allocs.push_back(wm);
  IG_CUDA(c, cudaMemcpyAsync(mraw, mask.data(), mask.size() * 8, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, igk::ntt_rows(d, (const u64*)mraw, (u64*)wm, o.rows, R_MOD_Q, shoup_companion(R_MOD_Q), c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  d.wmask_R = (const u64*)wm;
  if ((rc = sync_crs_self(c, o))) {
    for (void* p2 : o.allocs) cudaFree(p2);
    c->obj_bytes -= o.bytes;
    return rc;
  }
  const u64 h = g_next_object++;
  c->crs[h] = o;
  *crs_out = h;
  return IG_OK;
}

int ig_crs_destroy(ig_ctx* c, uint64_t crs) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->crs.find(crs);
  if (it == c->crs.end()) return fail(c, IG_ERR_HANDLE, "unknown CRS handle %llu", (unsigned long long)crs);
  cudaStreamSynchronize(c->stream);
  for (void* p : it->second.allocs) cudaFree(p);
  c->obj_bytes -= it->second.bytes;
  c->crs.erase(it);
  return IG_OK;
}

int ig_crs_key_rows(ig_ctx* c, uint64_t crs, uint32_t* rows) {
  if (!c || !rows) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  CrsObj* o = get_crs(c, crs);
  if (!o) return fail(c, IG_ERR_HANDLE, "unknown CRS handle %llu", (unsigned long long)crs);
  *rows = o->rows;
  return IG_OK;
}

int ig_db_create(ig_ctx* c, uint64_t crs, uint32_t num_shards, uint64_t* db_out) {
  if (!c || !db_out || num_shards == 0) return fail(c, IG_ERR_ARG, "ig_db_create: null output or zero shards");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (!get_crs(c, crs)) return fail(c, IG_ERR_HANDLE, "unknown CRS handle %llu", (unsigned long long)crs);
  DbObj db;
  db.crs = crs;
  db.num_shards = num_shards;
  db.shards.resize(num_shards);
  int rc = dalloc(c, (void**)&db.d_table, num_shards * sizeof(ShardDev), &db.bytes);
  if (rc) return rc;
  IG_CUDA(c, cudaMemset(db.d_table, 0, num_shards * sizeof(ShardDev)));
  const u64 h = g_next_object++;
  c->dbs[h] = std::move(db);
  *db_out = h;
  return IG_OK;
}

int ig_db_destroy(ig_ctx* c, uint64_t dbh) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->dbs.find(dbh);
  if (it == c->dbs.end()) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  cudaStreamSynchronize(c->stream);
  for (auto& s : it->second.shards) {
    cudaFree(s.cols);
    cudaFree(s.sums);
    cudaFree(s.tag_key);
    cudaFree(s.tags);
    cudaFree(s.cols16);
  }
  cudaFree(it->second.d_table);
  c->obj_bytes -= it->second.bytes;
  c->dbs.erase(it);
  return IG_OK;
}

// A shard's u64 columns and their u16 copy, both or neither (a shard counts as uploaded
// when `cols` is set).
static int alloc_columns(ig_ctx* c, DbObj& db, ShardSlot& sl, size_t bytes) {
  if (sl.cols && sl.cols16) return IG_OK;
  u64* cols = sl.cols;
  uint16_t* cols16 = sl.cols16;
  size_t got = 0;
  int rc = IG_OK;
  if (!cols) rc = dalloc(c, (void**)&cols, bytes, &got);
  if (!rc && !cols16) rc = dalloc(c, (void**)&cols16, bytes / 4, &got);
  if (rc) {
    if (cols && !sl.cols) dfree(c, cols, bytes);
    return rc;
  }
  db.bytes += got;
  sl.cols = cols;
  sl.cols16 = cols16;
  return IG_OK;
}

static int set_shard(ig_ctx* c, uint64_t dbh, uint32_t s, const uint64_t* cols, cudaMemcpyKind kind) {
  if (!c || !cols) return fail(c, IG_ERR_ARG, "ig_db_set_shard: null columns");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  if (s >= db->num_shards)
    return fail(c, IG_ERR_ARG, "shard %u not found at dense position %u; encoded database has %u shards", s, s,
                db->num_shards);
  CrsObj* o = get_crs(c, db->crs);
  const size_t bytes = (size_t)o->gamma * o->n * 8;
  ShardSlot& sl = db->shards[s];
  int rc = alloc_columns(c, *db, sl, bytes);
  if (rc) return rc;
  void* wide;
  rc = scratch(c, "compact_flag", 4, &wide);
  if (rc) return rc;
  IG_CUDA(c, cudaMemcpyAsync(sl.cols, cols, bytes, kind, c->stream));
  // Shards whose words all fit 16 bits (encoded records always do) are scanned from a
  // u16 copy: the same tags and folds from a quarter of the bytes.
  IG_CUDA(c, cudaMemsetAsync(wide, 0, 4, c->stream));
  IG_CUDA(c, igk::compact16(sl.cols, bytes / 8, sl.cols16, (u32*)wide, c->stream));
  c->launches++;
  u32 wide_h = 1;
  IG_CUDA(c, cudaMemcpyAsync(&wide_h, wide, 4, cudaMemcpyDeviceToHost, c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  sl.compact = wide_h == 0;
  rc = check_store_tags(c, *o, sl);
  if (rc) return rc;
  return sync_table_entry(c, *db, s);
}

int ig_db_encode_records(ig_ctx* c, uint64_t dbh, uint32_t first_shard, const uint8_t* records, size_t nbytes,
                         uint32_t entry_size, int on_device) {
  if (!c) return IG_ERR_ARG;
  if (!records || entry_size == 0) return fail(c, IG_ERR_ARG, "encode_database: null records or entry_size 0");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj& o = *get_crs(c, db->crs);
  const u32 n = o.n, g = o.gamma;
  const u32 columns = (entry_size + 1) / 2;  // num_columns (lib.rs): one column per 16 bits
  if (columns != g)
    return fail(c, IG_ERR_WIDTH,
                "encode_database: entry_size %u gives %u columns, the server packs gamma = %u (the CRS's "
                "inspiring_num_columns)",
                entry_size, columns, g);
  const size_t entries = nbytes / entry_size;
  const size_t shards = (entries + n - 1) / n;
  if ((size_t)first_shard + shards > db->num_shards)
    return fail(c, IG_ERR_ARG,
                "encode_database: %zu entries fill %zu shards of %u from shard %u; the database holds %u", entries,
                shards, n, first_shard, db->num_shards);
  const size_t shard_bytes = (size_t)n * entry_size;
  void* staging = nullptr;
  if (!on_device) {
    int rc = scratch(c, "encode_records", shard_bytes, &staging);
    if (rc) return rc;
  }
  for (size_t s = 0; s < shards; s++) {
    ShardSlot& sl = db->shards[first_shard + s];
    const size_t words = (size_t)g * n;
    {
      int rc = alloc_columns(c, *db, sl, words * 8);
      if (rc) return rc;
    }
    const size_t first = s * n;
    const u32 count = (u32)std::min<size_t>(n, entries - first);
    const uint8_t* src = records + first * entry_size;
    if (!on_device) {
      int rc = stage_h2d(c, staging, src, (size_t)count * entry_size);
      if (rc) return rc;
      src = (const uint8_t*)staging;
    }
    IG_CUDA(c, igk::encode_records(src, count, entry_size, n, g, sl.cols, sl.cols16, c->stream));
    c->launches++;
    sl.compact = true;
    // The staging buffer is reused by the next shard only after this encode has read it.
    if (!on_device) IG_CUDA(c, cudaStreamSynchronize(c->stream));
    int rc = check_store_tags(c, o, sl);
    if (rc) return rc;
    rc = sync_table_entry(c, *db, first_shard + (u32)s);
    if (rc) return rc;
  }
  return IG_OK;
}

int ig_db_set_shard(ig_ctx* c, uint64_t db, uint32_t s, const uint64_t* cols) {
  return set_shard(c, db, s, cols, cudaMemcpyHostToDevice);
}
int ig_db_set_shard_device(ig_ctx* c, uint64_t db, uint32_t s, const uint64_t* cols) {
  return set_shard(c, db, s, cols, cudaMemcpyDeviceToDevice);
}

int ig_db_precompute_packing(ig_ctx* c, uint64_t dbh, uint32_t s) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  if (s >= db->num_shards) return fail(c, IG_ERR_ARG, "shard %u out of range (%u shards)", s, db->num_shards);
  return build_store(c, *db, *get_crs(c, db->crs), s);
}

int ig_db_precompute_packing_all(ig_ctx* c, uint64_t dbh) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj* o = get_crs(c, db->crs);
  for (u32 s = 0; s < db->num_shards; s++) {
    int rc = build_store(c, *db, *o, s);
    if (rc) return rc;
  }
  return IG_OK;
}

int ig_db_drop_packing_store(ig_ctx* c, uint64_t dbh, uint32_t s) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  if (s >= db->num_shards) return fail(c, IG_ERR_ARG, "shard %u out of range", s);
  CrsObj* o = get_crs(c, db->crs);
  cudaStreamSynchronize(c->stream);
  ShardSlot& sl = db->shards[s];
  const size_t g = o->gamma, n = o->n;
  if (sl.sums) {
    cudaFree(sl.sums);
    cudaFree(sl.tag_key);
    cudaFree(sl.tags);
    const size_t freed = g * n * 8 + 2 * n * 8 + g * 8;
    db->bytes -= freed;
    c->obj_bytes -= freed;
    sl.sums = sl.tag_key = sl.tags = nullptr;
  }
  sl.stale = false;
  return sync_table_entry(c, *db, s);
}

int ig_db_has_store(ig_ctx* c, uint64_t dbh, uint32_t s, int* out) {
  if (!c || !out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  if (s >= db->num_shards) return fail(c, IG_ERR_ARG, "shard %u out of range", s);
  *out = db->shards[s].sums != nullptr;
  return IG_OK;
}

// ---- session store -------------------------------------------------------------------
int ig_session_store_create(ig_ctx* c, uint64_t* out) {
  if (!c || !out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  const u64 h = g_next_object++;
  c->stores[h] = StoreObj();
  *out = h;
  return IG_OK;
}

int ig_session_store_destroy(ig_ctx* c, uint64_t st) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->stores.find(st);
  if (it == c->stores.end()) return fail(c, IG_ERR_HANDLE, "unknown session store %llu", (unsigned long long)st);
  cudaStreamSynchronize(c->stream);
  for (auto& s : it->second.seats) dfree(c, s.second.yR, (size_t)s.second.rows * s.second.n * 8);
  c->stores.erase(it);
  return IG_OK;
}

// PackingKeySeat::build checks (session.rs:600-625, 661-697, 766-826), then the key
// body's NTT in R-form on the device.
static int make_seat(ig_ctx* c, CrsObj& o, const uint64_t* y_body, uint32_t rows, uint32_t num_to_pack, u64* dst,
                     bool y_on_device) {
  if (rows != o.rows)
    return fail(c, IG_ERR_WIDTH,
                "packing-key material mismatch: client sent %u y_body polynomials, the server decomposes into %u "
                "digits, and every digit needs its key polynomial. The client must re-derive its packing keys "
                "against the current CRS.",
                rows, o.rows);
  if (num_to_pack != o.gamma)
    return fail(c, IG_ERR_WIDTH,
                "packing-key width mismatch: client keys declare gamma = %u, server pack params use gamma = %u. "
                "The client must re-derive its packing keys against the current CRS.",
                num_to_pack, o.gamma);
  const u64* src = y_body;
  if (!y_on_device) {
    void* raw;
    int rc = scratch(c, "seat_raw", (size_t)rows * o.n * 8, &raw);
    if (rc) return rc;
    IG_CUDA(c, cudaMemcpyAsync(raw, y_body, (size_t)rows * o.n * 8, cudaMemcpyHostToDevice, c->stream));
    src = (const u64*)raw;
  }
  IG_CUDA(c, igk::ntt_rows(o.dev, src, dst, rows, R_MOD_Q, shoup_companion(R_MOD_Q), c->stream));
  return IG_OK;
}

int ig_session_register(ig_ctx* c, uint64_t st, uint64_t crs, const uint64_t* y_body, uint32_t rows,
                        uint32_t num_to_pack, uint64_t* handle_out) {
  if (!c || !y_body || !handle_out) return fail(c, IG_ERR_ARG, "ig_session_register: null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  auto it = c->stores.find(st);
  if (it == c->stores.end()) return fail(c, IG_ERR_HANDLE, "unknown session store %llu", (unsigned long long)st);
  CrsObj* o = get_crs(c, crs);
  if (!o) return fail(c, IG_ERR_HANDLE, "unknown CRS handle %llu", (unsigned long long)crs);
  SeatObj seat;
  seat.crs = crs;
  seat.n = o->n;
  seat.rows = rows;
  seat.num_to_pack = num_to_pack;
  if (rows == o->rows) {
    int rc = dalloc(c, (void**)&seat.yR, (size_t)rows * o->n * 8, nullptr);
    if (rc) return rc;
  }
  int rc = make_seat(c, *o, y_body, rows, num_to_pack, seat.yR, false);
  if (rc) {
    dfree(c, seat.yR, (size_t)rows * o->n * 8);
    return rc;
  }
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  u64 h = g_next_handle.load();
  do {
    if (h == ~0ULL) {
      dfree(c, seat.yR, (size_t)rows * o->n * 8);
      return fail(c, IG_ERR_EXHAUSTED,
                  "ServerSessionStore handle space exhausted at %llu; refusing the session handshake because "
                  "handle reuse could resolve stale clients to another client's packing keys",
                  (unsigned long long)h);
    }
  } while (!g_next_handle.compare_exchange_weak(h, h + 1));
  it->second.seats[h] = seat;
  *handle_out = h;
  return IG_OK;
}

int ig_session_remove(ig_ctx* c, uint64_t st, uint64_t handle, int* removed) {
  if (!c || !removed) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->stores.find(st);
  if (it == c->stores.end()) return fail(c, IG_ERR_HANDLE, "unknown session store %llu", (unsigned long long)st);
  auto s = it->second.seats.find(handle);
  *removed = s != it->second.seats.end();
  if (*removed) {
    cudaStreamSynchronize(c->stream);
    dfree(c, s->second.yR, (size_t)s->second.rows * s->second.n * 8);
    it->second.seats.erase(s);
  }
  return IG_OK;
}

int ig_session_len(ig_ctx* c, uint64_t st, uint64_t* len) {
  if (!c || !len) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->stores.find(st);
  if (it == c->stores.end()) return fail(c, IG_ERR_HANDLE, "unknown session store %llu", (unsigned long long)st);
  *len = it->second.seats.size();
  return IG_OK;
}

int ig_session_contains(ig_ctx* c, uint64_t st, uint64_t handle, int* present) {
  if (!c || !present) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->stores.find(st);
  if (it == c->stores.end()) return fail(c, IG_ERR_HANDLE, "unknown session store %llu", (unsigned long long)st);
  *present = it->second.seats.count(handle) ? 1 : 0;
  return IG_OK;
}

// ---- respond ---------------------------------------------------------------------------
static int resolve_seat(ig_ctx* c, CrsObj& o, uint64_t st, uint64_t handle, const uint64_t* inline_y,
                        uint32_t inline_rows, uint32_t inline_ntp, const u64** seat_out, u32 lane = 0) {
  if (inline_y) {
    // An inline key's seat lives in its caller's lane, which no concurrent call shares.
    char name[32];
    snprintf(name, sizeof name, "inline_seat%u", lane);
    void* p;
    int rc = scratch(c, name, (size_t)o.rows * o.n * 8, &p);
    if (rc) return rc;
    rc = make_seat(c, o, inline_y, inline_rows, inline_ntp, (u64*)p, false);
    if (rc) return rc;
    *seat_out = (const u64*)p;
    return IG_OK;
  }
  auto it = c->stores.find(st);
  if (it == c->stores.end())
    return fail(c, IG_ERR_HANDLE,
                "query references session_handle %llu but no ServerSessionStore was supplied to "
                "respond_*_with_session",
                (unsigned long long)handle);
  auto s = it->second.seats.find(handle);
  if (s == it->second.seats.end())
    return fail(c, IG_ERR_HANDLE, "ServerSessionStore has no entry for session_handle %llu",
                (unsigned long long)handle);
  const SeatObj& seat = s->second;
  if (seat.n != o.n || seat.rows != o.rows)
    return fail(c, IG_ERR_SHAPE,
                "packing-key seat is for another ring or gadget: it holds %u key rows on ring_dim %u, the server "
                "packs %u rows on ring_dim %u. The client must re-derive its packing keys against the current CRS.",
                seat.rows, seat.n, o.rows, o.n);
  if (seat.num_to_pack != o.gamma)
    return fail(c, IG_ERR_WIDTH,
                "packing-key width mismatch: client keys declare gamma = %u, server pack params use gamma = %u.",
                seat.num_to_pack, o.gamma);
  *seat_out = seat.yR;
  return IG_OK;
}

// The seat `handle` of `st` for a query on a database whose parameter set is `db_set`, and
// the parameter set the query runs under. The reference passes the CRS and its cache to
// respond_seeded_batch apart from the EncodedDatabase (respond.rs:1189-1202), and a shard's
// packing store depends only on the ring and the width (shard_store.rs:86-156), so a
// database serves every parameter set of its ring_dim and gamma: a seat registered under
// another such set (the other gadget, another mask seed) runs under its own set. Otherwise
// the seat must fit the database's set, with resolve_seat's refusals.
static int resolve_seat_for_db(ig_ctx* c, CrsObj& db_set, uint64_t st, uint64_t handle, const u64** seat_out,
                               CrsObj** set_out) {
  auto it = c->stores.find(st);
  if (it != c->stores.end()) {
    auto sit = it->second.seats.find(handle);
    if (sit != it->second.seats.end()) {
      CrsObj* own = get_crs(c, sit->second.crs);
      if (own && own != &db_set && own->n == db_set.n && own->gamma == db_set.gamma &&
          sit->second.rows == own->rows && sit->second.num_to_pack == own->gamma) {
        *seat_out = sit->second.yR;
        *set_out = own;
        return IG_OK;
      }
    }
  }
  *set_out = &db_set;
  return resolve_seat(c, db_set, st, handle, nullptr, 0, 0, seat_out);
}

// RAVEN_PROFILE_RESPOND is read once per process, as the reference does (respond.rs:1332-1345).
static bool env_profile() {
  static const bool on = getenv("RAVEN_PROFILE_RESPOND") != nullptr;
  return on;
}

static int respond_host(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, const uint64_t* inline_y,
                        uint32_t inline_rows, uint32_t inline_ntp, uint32_t count, const uint32_t* shard_ids,
                        const uint8_t* seeds, const uint64_t* as, const uint64_t* bs, uint64_t ms_target,
                        uint64_t* a_out, uint64_t* b_out) {
  if (!c) return IG_ERR_ARG;
  if (count && (!shard_ids || (!seeds && !as) || !bs || !a_out || !b_out))
    return fail(c, IG_ERR_ARG, "respond: null buffer");
  // The call's lane (lane 0 on the context stream when lanes == 1), held until its results
  // are copied out; the context lock is held only while the call validates and launches.
  igint::HostCall hc;
  igint::host_call_begin(c, hc);
  const u32 lanes = c->lanes, k = hc.k;
  std::unique_lock<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj& o = *get_crs(c, db->crs);
  const size_t n = o.n, g = o.gamma;
  if (ms_target && (ms_target >= Q || ms_target < o.p || ms_target % (2 * n) != 1))
    return fail(c, IG_ERR_ARG, "mod-switch target_modulus %llu must be in [p, q) and 1 mod 2d",
                (unsigned long long)ms_target);
  const u64* seat;
  int rc = resolve_seat(c, o, st, handle, inline_y, inline_rows, inline_ntp, &seat, k);
  if (rc) return rc;
  // respond_seeded_batch over no queries resolves the seat and answers nothing
  // (respond.rs:1196-1201).
  if (count == 0) return IG_OK;
  // checked_shard (respond.rs:601-611) for every query before any work.
  std::unordered_map<u32, u32> local;
  std::vector<u32> distinct;
  for (u32 i = 0; i < count; i++) {
    const u32 s = shard_ids[i];
    if (s >= db->num_shards)
      return fail(c, IG_ERR_ARG,
                  "respond_seeded_with_seat: shard %u not found at dense position %u; encoded database has %u shards",
                  s, s, db->num_shards);
    if (!db->shards[s].cols)
      return fail(c, IG_ERR_ARG, "respond_seeded_with_seat: shard %u holds no columns", s);
    if (!local.count(s)) {
      local[s] = (u32)distinct.size();
      distinct.push_back(s);
    }
  }
  // Shard table for this launch; shards without a store get a transient fold.
  std::vector<ShardDev> table(distinct.size());
  u32 transient = 0;
  for (u32 s : distinct)
    if (!db->shards[s].sums) transient++;
  void* tsums = nullptr;
  if (transient) {
    char tname[32];
    snprintf(tname, sizeof tname, "transient_sums%u", k);
    rc = scratch(c, tname, (size_t)transient * g * n * 8, &tsums);
    if (rc) return rc;
  }
  u64* zkey;
  rc = zero_key(c, 2 * n, &zkey);
  if (rc) return rc;
  u32 tk = 0;
  for (size_t k = 0; k < distinct.size(); k++) {
    const ShardSlot& sl = db->shards[distinct[k]];
    if (sl.sums) {
      table[k] = sl.dev();
    } else {
      u64* sums = (u64*)tsums + (size_t)tk++ * g * n;
      rc = fold_store(c, o, sl.cols, sums);
      if (rc) return rc;
      table[k] = ShardDev{sl.cols, sums, zkey, nullptr, sl.compact ? sl.cols16 : nullptr};
    }
  }
  void *d_table, *d_q, *d_seeds, *d_bs, *d_a, *d_b, *d_fold, *d_status;
  const size_t seed_bytes = as ? (size_t)count * n * 8 : (size_t)count * 32;
  auto lane_scratch = [&](const char* name, size_t bytes, void** out) {
    char full[48];
    snprintf(full, sizeof full, "%s%u", name, k);
    return scratch(c, full, bytes, out);
  };
  if ((rc = lane_scratch("table", table.size() * sizeof(ShardDev), &d_table)) ||
      (rc = lane_scratch("queries", count * sizeof(QueryDev), &d_q)) ||
      (rc = lane_scratch("seeds", seed_bytes, &d_seeds)) || (rc = lane_scratch("bs", count * n * 8, &d_bs)) ||
      (rc = lane_scratch("a_out", count * n * 8, &d_a)) || (rc = lane_scratch("b_out", count * n * 8, &d_b)) ||
      (rc = lane_scratch("fold", count * g * 8, &d_fold)) || (rc = lane_scratch("status", count * 4, &d_status)))
    return rc;
  // Pinned landing buffer of the lane: status words, then a, then b.
  const size_t st_bytes = ((size_t)count * 4 + 15) & ~(size_t)15;
  void* pin;
  if ((rc = igint::host_call_pinned(c, hc, st_bytes + 2 * (size_t)count * n * 8, &pin))) return rc;
  u32* h_status = (u32*)pin;
  u64* h_a = (u64*)((uint8_t*)pin + st_bytes);
  u64* h_b = h_a + (size_t)count * n;
  std::vector<QueryDev> qs(count);
  for (u32 i = 0; i < count; i++) {
    qs[i] = QueryDev{};
    qs[i].shard = local[shard_ids[i]];
    qs[i].fold_off = i * (u32)g;
    qs[i].seed = as ? nullptr : (const u32*)((const uint8_t*)d_seeds + (size_t)i * 32);
    qs[i].a = as ? (const u64*)d_seeds + (size_t)i * n : nullptr;
    qs[i].b = (const u64*)d_bs + (size_t)i * n;
    qs[i].seat_R = seat;
    qs[i].ms = ms_target;
    qs[i].row = i;
  }
  cudaStream_t s = igint::host_call_stream(c, hc);
  if ((rc = stage_h2d(c, d_table, table.data(), table.size() * sizeof(ShardDev))) ||
      (rc = stage_h2d(c, d_q, qs.data(), count * sizeof(QueryDev))) ||
      (rc = stage_h2d(c, d_seeds, as ? (const void*)as : (const void*)seeds, seed_bytes)) ||
      (rc = stage_h2d(c, d_bs, bs, (size_t)count * n * 8)) || (rc = igint::host_call_enter(c, hc)))
    return rc;
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  // RAVEN_PROFILE_RESPOND (respond.rs:1295-1345): CUDA events around the two regions of the
  // batch, printed to stderr in the reference's line format.
  cudaEvent_t env_ev[3] = {};
  const bool env_prof = env_profile();
  if (env_prof)
    for (auto& e : env_ev) cudaEventCreate(&e);
  if (env_prof) cudaEventRecord(env_ev[0], s);
  long pk = prof_begin(c, REGION_SCAN, s);
  IG_CUDA(c, igk::shard_scan(o.dev, (const QueryDev*)d_q, (const ShardDev*)d_table, count, nullptr, 0, (u64*)d_fold,
                             (u32*)d_status, s));
  prof_end(c, pk, s);
  if (env_prof) cudaEventRecord(env_ev[1], s);
  pk = prof_begin(c, REGION_RESPOND, s);
  IG_CUDA(c, igk::respond(o.dev, (const QueryDev*)d_q, (const ShardDev*)d_table, count, (const u64*)d_fold,
                          (u64*)d_a, (u64*)d_b, (u32*)d_status, c->force_serial,
                          igint::launch_ctas(c, (u32)n, (u32)g, count, count * lanes),
                          s));
  prof_end(c, pk, s);
  if (env_prof) {
    cudaEventRecord(env_ev[2], s);
    cudaEventSynchronize(env_ev[2]);
    float scan_ms = 0, pack_ms = 0;
    cudaEventElapsedTime(&scan_ms, env_ev[0], env_ev[1]);
    cudaEventElapsedTime(&pack_ms, env_ev[1], env_ev[2]);
    fprintf(stderr, "RAVEN_PROFILE num_cols=%u queries=%u column_check_us=%.0f pack_us=%.0f\n", (unsigned)g,
            (unsigned)count, 1e3 * scan_ms, 1e3 * pack_ms);
    for (auto& e : env_ev) cudaEventDestroy(e);
  }
  IG_CUDA(c, cudaMemcpyAsync(h_status, d_status, count * 4, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaMemcpyAsync(h_a, d_a, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaMemcpyAsync(h_b, d_b, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s));
  if ((rc = igint::host_call_launched(c, hc))) return rc;
  lk.unlock();  // other callers launch while this batch runs
  if ((rc = igint::host_call_wait(c, hc))) return rc;
  for (u32 i = 0; i < count; i++) {
    if (h_status[i] & DEV_TAG_MISMATCH)
      return fail(c, IG_ERR_STORE_REFUSED,
                  "shard %u: packing store refused: a column is not the column the store was built from. The shard "
                  "changed after the build; rebuild the store before serving it",
                  shard_ids[i]);
    if (h_status[i]) return fail(c, IG_ERR_DEVICE, "query %u: respond kernel status %u", i, h_status[i]);
  }
  memcpy(a_out, h_a, (size_t)count * n * 8);
  memcpy(b_out, h_b, (size_t)count * n * 8);
  return IG_OK;
}

int ig_respond_seeded_batch(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, const uint64_t* inline_y,
                            uint32_t inline_rows, uint32_t inline_ntp, uint32_t count, const uint32_t* shard_ids,
                            const uint8_t* seeds, const uint64_t* bs, uint64_t ms_target, uint64_t* a_out,
                            uint64_t* b_out) {
  if (!seeds && count && c) return fail(c, IG_ERR_ARG, "ig_respond_seeded_batch: null seeds");
  return respond_host(c, dbh, st, handle, inline_y, inline_rows, inline_ntp, count, shard_ids, seeds, nullptr, bs,
                      ms_target, a_out, b_out);
}

int ig_respond_batch(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, const uint64_t* inline_y,
                     uint32_t inline_rows, uint32_t inline_ntp, uint32_t count, const uint32_t* shard_ids,
                     const uint64_t* as, const uint64_t* bs, uint64_t ms_target, uint64_t* a_out, uint64_t* b_out) {
  if (!as && count && c) return fail(c, IG_ERR_ARG, "ig_respond_batch: null a");
  return respond_host(c, dbh, st, handle, inline_y, inline_rows, inline_ntp, count, shard_ids, nullptr, as, bs,
                      ms_target, a_out, b_out);
}

// ---- NoPacking respond -------------------------------------------------------------------
int ig_respond_nopacking_batch(ig_ctx* c, uint64_t dbh, uint32_t count, const uint32_t* shard_ids,
                               const uint8_t* seeds, const uint64_t* as, const uint64_t* bs, uint64_t* out) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !shard_ids || (!seeds && !as) || !bs || !out)
    return fail(c, IG_ERR_ARG, "respond: empty batch or null buffer");
  // As respond_seeded_batch: the call holds one lane (stream and scratch) while its batch
  // runs and takes the context lock only to validate and launch. The ciphertexts (gamma + 1
  // per query) are copied to the caller's buffer after the lock is released, so callers'
  // batches overlap on the device and on the copy engines.
  igint::HostCall hc;
  igint::host_call_begin(c, hc);
  const u32 k = hc.k;
  std::unique_lock<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj& o = *get_crs(c, db->crs);
  const size_t n = o.n, g = o.gamma;
  std::unordered_map<u32, u32> local;
  std::vector<ShardDev> table;
  for (u32 i = 0; i < count; i++) {
    const u32 s = shard_ids[i];
    if (s >= db->num_shards)
      return fail(c, IG_ERR_ARG, "respond: shard %u not found at dense position %u; encoded database has %u shards", s,
                  s, db->num_shards);
    if (!db->shards[s].cols) return fail(c, IG_ERR_ARG, "respond: shard %u holds no columns", s);
    if (!local.count(s)) {
      local[s] = (u32)table.size();
      table.push_back(db->shards[s].dev());
    }
  }
  const size_t seed_bytes = as ? (size_t)count * n * 8 : (size_t)count * 32;
  const size_t out_words = (size_t)count * (g + 1) * 2 * n;
  void *d_table, *d_q, *d_seeds, *d_bs, *d_ab, *d_out, *d_status;
  auto lane_scratch = [&](const char* name, size_t bytes, void** p) {
    char full[48];
    snprintf(full, sizeof full, "%s%u", name, k);
    return scratch(c, full, bytes, p);
  };
  int rc;
  if ((rc = lane_scratch("np_table", table.size() * sizeof(ShardDev), &d_table)) ||
      (rc = lane_scratch("np_queries", count * sizeof(QueryDev), &d_q)) ||
      (rc = lane_scratch("np_seeds", seed_bytes, &d_seeds)) ||
      (rc = lane_scratch("np_bs", (size_t)count * n * 8, &d_bs)) ||
      (rc = lane_scratch("np_ab", (size_t)count * 2 * n * 8, &d_ab)) ||
      (rc = lane_scratch("np_out", out_words * 8, &d_out)) || (rc = lane_scratch("np_status", count * 4, &d_status)))
    return rc;
  void* pin;
  if ((rc = igint::host_call_pinned(c, hc, (size_t)count * 4, &pin))) return rc;
  const u32* h_status = (const u32*)pin;
  std::vector<QueryDev> qs(count);
  for (u32 i = 0; i < count; i++) {
    qs[i] = QueryDev{};
    qs[i].shard = local[shard_ids[i]];
    qs[i].seed = as ? nullptr : (const u32*)((const uint8_t*)d_seeds + (size_t)i * 32);
    qs[i].a = as ? (const u64*)d_seeds + (size_t)i * n : nullptr;
    qs[i].b = (const u64*)d_bs + (size_t)i * n;
    qs[i].seat_R = nullptr;
  }
  if ((rc = stage_h2d(c, d_table, table.data(), table.size() * sizeof(ShardDev))) ||
      (rc = stage_h2d(c, d_q, qs.data(), count * sizeof(QueryDev))) ||
      (rc = stage_h2d(c, d_seeds, as ? (const void*)as : (const void*)seeds, seed_bytes)) ||
      (rc = stage_h2d(c, d_bs, bs, (size_t)count * n * 8)) || (rc = igint::host_call_enter(c, hc)))
    return rc;
  cudaStream_t s = igint::host_call_stream(c, hc);
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  IG_CUDA(c, igk::nopack(o.dev, (const QueryDev*)d_q, (const ShardDev*)d_table, count, R_MOD_Q, (u64*)d_ab,
                         (u64*)d_out, (u32*)d_status, s));
  c->launches += 3;
  IG_CUDA(c, cudaMemcpyAsync((void*)h_status, d_status, count * 4, cudaMemcpyDeviceToHost, s));
  if ((rc = igint::host_call_launched(c, hc))) return rc;
  lk.unlock();  // other callers launch while this batch runs and copies out
  // The lane's stream and scratch stay this call's until it returns (the lane lock).
  cudaError_t e = cudaMemcpyAsync(out, d_out, out_words * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(c, IG_ERR_CUDA, "respond: copy of the ciphertexts failed: %s", cudaGetErrorString(e));
  for (u32 i = 0; i < count; i++)
    if (h_status[i]) return fail(c, IG_ERR_DEVICE, "query %u: respond kernel status %u", i, h_status[i]);
  return IG_OK;
}

// ---- client side -------------------------------------------------------------------------
int ig_client_create(ig_ctx* c, uint64_t crs, const uint64_t* secret, double sigma, uint64_t* client_out) {
  if (!c || !secret || !client_out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  CrsObj* o = get_crs(c, crs);
  if (!o) return fail(c, IG_ERR_HANDLE, "unknown CRS handle %llu", (unsigned long long)crs);
  if (!(sigma > 0) || sigma > 1e6) return fail(c, IG_ERR_ARG, "sampler sigma %g is not served", sigma);
  const size_t n = o->n;
  ClientObj cl;
  cl.crs = crs;
  for (size_t k = 0; k < n; k++) {
    if (secret[k] >= Q) return fail(c, IG_ERR_SHAPE, "secret coefficient %zu is not a residue mod q", k);
    const u64 mag = secret[k] > Q / 2 ? Q - secret[k] : secret[k];
    cl.max_abs_s = std::max(cl.max_abs_s, mag);
  }
  // GaussianSampler::new (math/gaussian.rs:95-117): tailcut ceil(6 sigma), thresholds the
  // f64 bit patterns of exp(-x^2 / 2 sigma^2), a NaN as +0.0.
  const i64 t = (i64)std::ceil(sigma * 6.0);
  std::vector<u64> table;
  const double two_s2 = 2.0 * sigma * sigma;
  for (i64 x = -t; x <= t; x++) {
    double prob = std::exp(-(double)(x * x) / two_s2);
    if (std::isnan(prob)) prob = 0.0;
    u64 bits;
    memcpy(&bits, &prob, 8);
    table.push_back(bits);
  }
  void *raw = nullptr, *sR = nullptr, *acc = nullptr;
  int rc = scratch(c, "client_raw", n * 8, &raw);
  if (!rc) rc = dalloc(c, &sR, n * 8, &cl.bytes);
  if (!rc) {
    cl.allocs.push_back(sR);
    rc = dalloc(c, &acc, table.size() * 8, &cl.bytes);
  }
  if (rc) {
    for (void* p2 : cl.allocs) cudaFree(p2);
    c->obj_bytes -= cl.bytes;
    return rc;
  }
  cl.allocs.push_back(acc);
  IG_CUDA(c, cudaMemcpyAsync(raw, secret, n * 8, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, cudaMemcpyAsync(acc, table.data(), table.size() * 8, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, igk::ntt_rows(o->dev, (const u64*)raw, (u64*)sR, 1, R_MOD_Q, shoup_companion(R_MOD_Q), c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  cl.s_R = (u64*)sR;
  cl.accept = (u64*)acc;
  cl.g.accept = cl.accept;
  cl.g.tailcut = t;
  cl.g.range = (u64)(2 * t + 1);
  cl.g.zone = (cl.g.range << __builtin_clzll(cl.g.range)) - 1;
  const u64 h = g_next_object++;
  c->clients[h] = cl;
  *client_out = h;
  return IG_OK;
}

int ig_client_destroy(ig_ctx* c, uint64_t client) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->clients.find(client);
  if (it == c->clients.end()) return fail(c, IG_ERR_HANDLE, "unknown client handle %llu", (unsigned long long)client);
  cudaStreamSynchronize(c->stream);
  for (void* p : it->second.allocs) cudaFree(p);
  c->obj_bytes -= it->second.bytes;
  c->clients.erase(it);
  return IG_OK;
}

int ig_client_query_batch(ig_ctx* c, uint64_t client, uint32_t count, const uint64_t* indices, const uint8_t* seeds,
                          const uint8_t* sampler_key, uint64_t* sampler_word, uint32_t* shard_ids_out,
                          uint64_t* b_out) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !indices || !seeds || !sampler_key || !sampler_word || !shard_ids_out || !b_out)
    return fail(c, IG_ERR_ARG, "query_batch: empty batch or null buffer");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  auto it = c->clients.find(client);
  if (it == c->clients.end()) return fail(c, IG_ERR_HANDLE, "unknown client handle %llu", (unsigned long long)client);
  ClientObj& cl = it->second;
  CrsObj* o = get_crs(c, cl.crs);
  if (!o) return fail(c, IG_ERR_HANDLE, "the client's CRS is gone");
  const size_t n = o->n;
  const u64 S = (u64)count * n;
  const u64 P = *sampler_word;
  cudaStream_t s = c->stream;
  u32 key[8];
  for (int i = 0; i < 8; i++) memcpy(&key[i], sampler_key + 4 * i, 4);
  void *d_key, *d_samples, *d_total, *d_end;
  int rc;
  if ((rc = scratch(c, "cl_key", 32, &d_key)) || (rc = scratch(c, "cl_samples", S * 8, &d_samples)) ||
      (rc = scratch(c, "cl_total", 8, &d_total)) || (rc = scratch(c, "cl_end", 8, &d_end)))
    return rc;
  if ((rc = stage_h2d(c, d_key, key, 32))) return rc;
  // About 13 stream words per sample at sigma 6.4 (an x candidate is kept with probability
  // 0.62, a candidate x with about 0.2); the window doubles until it holds S samples.
  constexpr u32 SEG = 16;
  u64 W = 14 * S + 4096, total = 0, end = 0;
  for (int tries = 0; tries < 8 && total < S; tries++, W *= 2) {
    const u64 block0 = P / 16, base = P - 16 * block0;
    const u64 nblocks = (base + 2 * W + 2 + 15) / 16;
    const u64 T = (W + SEG - 1) / SEG;
    void *d_ks, *d_maps, *d_starts, *d_counts, *d_offsets;
    if ((rc = scratch(c, "cl_ks", nblocks * 64, &d_ks)) || (rc = scratch(c, "cl_maps", T, &d_maps)) ||
        (rc = scratch(c, "cl_starts", T, &d_starts)) || (rc = scratch(c, "cl_counts", T * 4, &d_counts)) ||
        (rc = scratch(c, "cl_offsets", T * 8, &d_offsets)))
      return rc;
    IG_CUDA(c, igk::keystream((const u32*)d_key, block0, nblocks, (u32*)d_ks, s));
    IG_CUDA(c, igk::gauss_parse(cl.g, (const u32*)d_ks, base, W, SEG, (uint8_t*)d_maps, (uint8_t*)d_starts,
                                (u32*)d_counts, (u64*)d_offsets, (u64*)d_total, S, (i64*)d_samples, (u64*)d_end, s));
    c->launches += 6;
    IG_CUDA(c, cudaMemcpyAsync(&total, d_total, 8, cudaMemcpyDeviceToHost, s));
    IG_CUDA(c, cudaMemcpyAsync(&end, d_end, 8, cudaMemcpyDeviceToHost, s));
    IG_CUDA(c, cudaStreamSynchronize(s));
  }
  if (total < S) return fail(c, IG_ERR_DEVICE, "query_batch: the sampler stream gave %llu of %llu samples",
                             (unsigned long long)total, (unsigned long long)S);
  // ShardConfig::index_to_shard (params.rs:1344-1385): ring_dim entries a shard.
  std::vector<u32> locals(count);
  for (u32 i = 0; i < count; i++) {
    shard_ids_out[i] = (u32)(indices[i] / n);
    locals[i] = (u32)(indices[i] % n);
  }
  void *d_q, *d_seeds, *d_locals, *d_b, *d_status;
  if ((rc = scratch(c, "cl_queries", count * sizeof(QueryDev), &d_q)) ||
      (rc = scratch(c, "cl_seeds", (size_t)count * 32, &d_seeds)) ||
      (rc = scratch(c, "cl_locals", (size_t)count * 4, &d_locals)) ||
      (rc = scratch(c, "cl_b", (size_t)count * n * 8, &d_b)) || (rc = scratch(c, "cl_status", count * 4, &d_status)))
    return rc;
  std::vector<QueryDev> qs(count);
  for (u32 i = 0; i < count; i++) {
    qs[i] = QueryDev{};
    qs[i].seed = (const u32*)((const uint8_t*)d_seeds + (size_t)i * 32);
  }
  if ((rc = stage_h2d(c, d_q, qs.data(), count * sizeof(QueryDev))) ||
      (rc = stage_h2d(c, d_seeds, seeds, (size_t)count * 32)) ||
      (rc = stage_h2d(c, d_locals, locals.data(), (size_t)count * 4)))
    return rc;
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  IG_CUDA(c, igk::client_query(o->dev, (const QueryDev*)d_q, count, cl.s_R, (const u32*)d_locals,
                               (const i64*)d_samples, Q / o->p, (u64*)d_b, (u32*)d_status, s));
  c->launches++;
  std::vector<u32> status(count);
  IG_CUDA(c, cudaMemcpyAsync(status.data(), d_status, count * 4, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaMemcpyAsync(b_out, d_b, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaStreamSynchronize(s));
  for (u32 i = 0; i < count; i++)
    if (status[i]) return fail(c, IG_ERR_DEVICE, "query %u: query kernel status %u", i, status[i]);
  *sampler_word = P + 2 * end;
  return IG_OK;
}

int ig_client_extract_batch(ig_ctx* c, uint64_t client, uint32_t count, const uint64_t* a, const uint64_t* b,
                            uint64_t modulus, uint32_t entry_size, int tree, uint8_t* records_out) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !a || !b || !records_out || entry_size == 0)
    return fail(c, IG_ERR_ARG, "extract: empty batch, zero entry size or null buffer");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  auto it = c->clients.find(client);
  if (it == c->clients.end()) return fail(c, IG_ERR_HANDLE, "unknown client handle %llu", (unsigned long long)client);
  ClientObj& cl = it->second;
  CrsObj* o = get_crs(c, cl.crs);
  if (!o) return fail(c, IG_ERR_HANDLE, "the client's CRS is gone");
  const size_t n = o->n;
  if (modulus == 0) modulus = Q;
  if (modulus > Q || modulus < o->p)
    return fail(c, IG_ERR_ARG, "response modulus %llu outside [p, q]", (unsigned long long)modulus);
  if (modulus != Q && (u128)n * modulus * cl.max_abs_s >= (u128)(Q / 2))
    return fail(c, IG_ERR_UNSUPPORTED,
                "extract over modulus %llu is not served: the secret's product could wrap q (n * m * max|s| >= q/2)",
                (unsigned long long)modulus);
  if ((entry_size + 1) / 2 > n) return fail(c, IG_ERR_ARG, "entry of %u bytes needs more than ring_dim columns", entry_size);
  const u64 delta = modulus / o->p;
  if (delta == 0) return fail(c, IG_ERR_ARG, "delta = modulus / p = 0; cannot decrypt");
  u64 dinv = 0;
  if (tree) {
    // extract_packed (extract.rs:184-226): d^-1 mod p, refused when gcd(d, p) != 1.
    u64 inv = 0;
    for (u64 x = 1; x < o->p; x++)
      if ((u128)x * (n % o->p) % o->p == 1) {
        inv = x;
        break;
      }
    if (!inv) return fail(c, IG_ERR_ARG, "degree %zu is not invertible mod p = %llu", n, (unsigned long long)o->p);
    dinv = inv;
  }
  const size_t words = (size_t)count * n;
  for (size_t i = 0; i < words; i++)
    if (a[i] >= modulus || b[i] >= modulus)
      return fail(c, IG_ERR_SHAPE, "response %zu coefficient is not canonical for modulus %llu", i / n,
                  (unsigned long long)modulus);
  void *d_a, *d_b, *d_out;
  int rc;
  if ((rc = scratch(c, "cx_a", words * 8, &d_a)) || (rc = scratch(c, "cx_b", words * 8, &d_b)) ||
      (rc = scratch(c, "cx_out", (size_t)count * entry_size, &d_out)))
    return rc;
  cudaStream_t s = c->stream;
  if ((rc = stage_h2d(c, d_a, a, words * 8)) || (rc = stage_h2d(c, d_b, b, words * 8))) return rc;
  IG_CUDA(c, cudaMemsetAsync(d_out, 0, (size_t)count * entry_size, s));
  IG_CUDA(c, igk::client_extract(o->dev, count, cl.s_R, (const u64*)d_a, (const u64*)d_b, modulus, delta, o->p, dinv,
                                 entry_size, (uint8_t*)d_out, s));
  c->launches++;
  IG_CUDA(c, cudaMemcpyAsync(records_out, d_out, (size_t)count * entry_size, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaStreamSynchronize(s));
  return IG_OK;
}

int ig_crs_set_galois_keys(ig_ctx* c, uint64_t crs, uint32_t count, uint32_t rows, const uint64_t* keys) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  CrsObj* o = get_crs(c, crs);
  if (!o) return fail(c, IG_ERR_HANDLE, "unknown CRS handle %llu", (unsigned long long)crs);
  // ServerCrs::require_galois_keys (pir/setup.rs:195-226).
  if (count != o->logn)
    return fail(c, IG_ERR_SHAPE,
                "respond_one_packing: %u galois keys, but ring_dim %u packs through %u tree levels; this CRS cannot "
                "drive automorphism packing",
                count, o->n, o->logn);
  if (rows != 3) return fail(c, IG_ERR_SHAPE, "respond_one_packing: galois key 0 carries %u rows for a 3-digit gadget", rows);
  if (!keys) return fail(c, IG_ERR_ARG, "ig_crs_set_galois_keys: null keys");
  const size_t words = (size_t)count * rows * 2 * o->n;
  for (size_t i = 0; i < words; i++)
    if (keys[i] >= Q)
      return fail(c, IG_ERR_SHAPE, "respond_one_packing: galois key %zu holds a coefficient that is not a residue mod q",
                  i / ((size_t)rows * 2 * o->n));
  void* raw = nullptr;
  void* dk = nullptr;
  int rc = scratch(c, "galois_raw", words * 8, &raw);
  if (!rc) rc = dalloc(c, &dk, words * 8, &o->bytes);
  if (rc) return rc;
  IG_CUDA(c, cudaMemcpyAsync(raw, keys, words * 8, cudaMemcpyHostToDevice, c->stream));
  IG_CUDA(c, igk::ntt_rows(o->dev, (const u64*)raw, (u64*)dk, (u32)(words / o->n), R_MOD_Q, shoup_companion(R_MOD_Q),
                           c->stream));
  IG_CUDA(c, igk::fold_gadget_keys(o->dev, (u64*)dk, count, c->stream));
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (o->dev.galois_R) {
    for (auto it = o->allocs.begin(); it != o->allocs.end(); ++it)
      if (*it == (void*)o->dev.galois_R) {
        cudaFree(*it);
        o->allocs.erase(it);
        o->bytes -= words * 8;
        c->obj_bytes -= words * 8;
        break;
      }
  }
  o->allocs.push_back(dk);
  o->dev.galois_R = (const u64*)dk;
  return sync_crs_self(c, *o);
}

int ig_respond_one_packing_batch(ig_ctx* c, uint64_t dbh, uint32_t count, const uint32_t* shard_ids,
                                 const uint8_t* seeds, const uint64_t* as, const uint64_t* bs, uint64_t ms_target,
                                 uint64_t* a_out, uint64_t* b_out) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !shard_ids || (!seeds && !as) || !bs || !a_out || !b_out)
    return fail(c, IG_ERR_ARG, "respond_one_packing: empty batch or null buffer");
  // As respond_seeded_batch: the call holds one lane (stream and scratch, the node stacks
  // included) while its batch runs, takes the context lock only to validate and launch, and
  // copies the responses to the caller's buffers after releasing it.
  igint::HostCall hc;
  igint::host_call_begin(c, hc);
  const u32 k = hc.k;
  std::unique_lock<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj& o = *get_crs(c, db->crs);
  const size_t n = o.n;
  if (!o.dev.galois_R)
    return fail(c, IG_ERR_SHAPE,
                "respond_one_packing: 0 galois keys, but ring_dim %u packs through %u tree levels; this CRS cannot "
                "drive automorphism packing",
                o.n, o.logn);
  if (ms_target && (ms_target >= Q || ms_target < o.p || ms_target % (2 * n) != 1))
    return fail(c, IG_ERR_ARG, "mod-switch target_modulus %llu must be in [p, q) and 1 mod 2d",
                (unsigned long long)ms_target);
  std::unordered_map<u32, u32> local;
  std::vector<ShardDev> table;
  for (u32 i = 0; i < count; i++) {
    const u32 s = shard_ids[i];
    if (s >= db->num_shards)
      return fail(c, IG_ERR_ARG,
                  "respond_one_packing: shard %u not found at dense position %u; encoded database has %u shards", s, s,
                  db->num_shards);
    if (!db->shards[s].cols) return fail(c, IG_ERR_ARG, "respond_one_packing: shard %u holds no columns", s);
    if (!local.count(s)) {
      local[s] = (u32)table.size();
      table.push_back(db->shards[s].dev());
    }
  }
  const size_t seed_bytes = as ? (size_t)count * n * 8 : (size_t)count * 32;
  void *d_table, *d_q, *d_seeds, *d_bs, *d_stack, *d_a, *d_b, *d_status;
  auto lane_scratch = [&](const char* name, size_t bytes, void** p) {
    char full[48];
    snprintf(full, sizeof full, "%s%u", name, k);
    return scratch(c, full, bytes, p);
  };
  int rc;
  if ((rc = lane_scratch("tr_table", table.size() * sizeof(ShardDev), &d_table)) ||
      (rc = lane_scratch("tr_queries", count * sizeof(QueryDev), &d_q)) ||
      (rc = lane_scratch("tr_seeds", seed_bytes, &d_seeds)) ||
      (rc = lane_scratch("tr_bs", (size_t)count * n * 8, &d_bs)) ||
      (rc = lane_scratch("tr_stack", (size_t)count * o.logn * 2 * n * 8, &d_stack)) ||
      (rc = lane_scratch("tr_a", (size_t)count * n * 8, &d_a)) ||
      (rc = lane_scratch("tr_b", (size_t)count * n * 8, &d_b)) || (rc = lane_scratch("tr_status", count * 4, &d_status)))
    return rc;
  void* pin;
  if ((rc = igint::host_call_pinned(c, hc, (size_t)count * 4, &pin))) return rc;
  const u32* h_status = (const u32*)pin;
  std::vector<QueryDev> qs(count);
  for (u32 i = 0; i < count; i++) {
    qs[i] = QueryDev{};
    qs[i].shard = local[shard_ids[i]];
    qs[i].seed = as ? nullptr : (const u32*)((const uint8_t*)d_seeds + (size_t)i * 32);
    qs[i].a = as ? (const u64*)d_seeds + (size_t)i * n : nullptr;
    qs[i].b = (const u64*)d_bs + (size_t)i * n;
    qs[i].seat_R = nullptr;
  }
  if ((rc = stage_h2d(c, d_table, table.data(), table.size() * sizeof(ShardDev))) ||
      (rc = stage_h2d(c, d_q, qs.data(), count * sizeof(QueryDev))) ||
      (rc = stage_h2d(c, d_seeds, as ? (const void*)as : (const void*)seeds, seed_bytes)) ||
      (rc = stage_h2d(c, d_bs, bs, (size_t)count * n * 8)) || (rc = igint::host_call_enter(c, hc)))
    return rc;
  cudaStream_t s = igint::host_call_stream(c, hc);
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  IG_CUDA(c, igk::tree(o.dev, (const QueryDev*)d_q, (const ShardDev*)d_table, count, R_MOD_Q, ms_target,
                       (u64*)d_stack, (u64*)d_a, (u64*)d_b, (u32*)d_status, s));
  c->launches++;
  IG_CUDA(c, cudaMemcpyAsync((void*)h_status, d_status, count * 4, cudaMemcpyDeviceToHost, s));
  if ((rc = igint::host_call_launched(c, hc))) return rc;
  lk.unlock();  // other callers launch while this batch runs and copies out
  // The lane's stream and scratch stay this call's until it returns (the lane lock).
  cudaError_t e = cudaMemcpyAsync(a_out, d_a, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b_out, d_b, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail(c, IG_ERR_CUDA, "respond_one_packing: copy of the responses failed: %s", cudaGetErrorString(e));
  for (u32 i = 0; i < count; i++)
    if (h_status[i]) return fail(c, IG_ERR_DEVICE, "query %u: tree kernel status %u", i, h_status[i]);
  return IG_OK;
}

int ig_respond_seeded_batch_device(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, uint32_t count,
                                   const uint32_t* shard_ids, const uint8_t* d_seeds, const uint64_t* d_bs,
                                   uint64_t ms_target, uint64_t* d_a, uint64_t* d_b, uint32_t* d_status) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !shard_ids || !d_seeds || !d_bs || !d_a || !d_b || !d_status)
    return fail(c, IG_ERR_ARG, "ig_respond_seeded_batch_device: empty batch or null buffer");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj& o = *get_crs(c, db->crs);
  const size_t n = o.n, g = o.gamma;
  if (ms_target && (ms_target >= Q || ms_target < o.p || ms_target % (2 * n) != 1))
    return fail(c, IG_ERR_ARG, "mod-switch target_modulus %llu must be in [p, q) and 1 mod 2d",
                (unsigned long long)ms_target);
  const u64* seat;
  int rc = resolve_seat(c, o, st, handle, nullptr, 0, 0, &seat);
  if (rc) return rc;
  for (u32 i = 0; i < count; i++) {
    const u32 s = shard_ids[i];
    if (s >= db->num_shards) return fail(c, IG_ERR_ARG, "shard %u not found; encoded database has %u shards", s, db->num_shards);
    if (!db->shards[s].sums)
      return fail(c, IG_ERR_ARG, "shard %u has no packing store; the device-resident path serves stored shards", s);
  }
  // Lane of this call (lanes > 1): its stream and scratch. The lane's scratch is reused
  // only after the lane's previous batch has finished with it.
  int lane = -1;
  cudaStream_t s = c->stream;
  if ((rc = igint::lane_acquire(c, &s, &lane))) return rc;
  char qname[32], fname[32];
  snprintf(qname, sizeof qname, "dev_queries%d", lane);
  snprintf(fname, sizeof fname, "dev_fold%d", lane);
  void *d_q, *d_fold;
  if ((rc = scratch(c, qname, count * sizeof(QueryDev), &d_q)) || (rc = scratch(c, fname, count * g * 8, &d_fold)))
    return rc;
  std::vector<QueryDev> qs(count);
  for (u32 i = 0; i < count; i++) {
    qs[i] = QueryDev{};
    qs[i].shard = shard_ids[i];
    qs[i].fold_off = i * (u32)g;
    qs[i].seed = (const u32*)(d_seeds + (size_t)i * 32);
    qs[i].b = d_bs + (size_t)i * n;
    qs[i].seat_R = seat;
    qs[i].ms = ms_target;
    qs[i].row = i;
  }
  if ((rc = stage_h2d(c, d_q, qs.data(), count * sizeof(QueryDev)))) return rc;
  if ((rc = igint::lane_enter(c, lane))) return rc;
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  long pk = prof_begin(c, REGION_SCAN, s);
  IG_CUDA(c, igk::shard_scan(o.dev, (const QueryDev*)d_q, db->d_table, count, nullptr, 0, (u64*)d_fold, d_status, s));
  prof_end(c, pk, s);
  // Several CTAs per query only while every lane's batch still leaves SMs for them.
  const int ctas = igint::launch_ctas(c, (u32)n, (u32)g, count, count * c->lanes);
  pk = prof_begin(c, REGION_RESPOND, s);
  IG_CUDA(c, igk::respond(o.dev, (const QueryDev*)d_q, db->d_table, count, (const u64*)d_fold, d_a, d_b, d_status,
                          c->force_serial, ctas, s));
  prof_end(c, pk, s);
  return igint::lane_release(c, lane);
}

// ---- mixed launches ------------------------------------------------------------------------
// Queries of several databases, parameter sets, seats and mod-switch targets in one launch
// (the reference answers one respond_seeded_batch call per key and database,
// respond.rs:1189-1202; here the calls of a server's queue share one scan and one respond
// launch). All sets must share the ring: n, q and with them the transform ladders and slot
// tables the kernels take from the launch's constants; gamma, the gadget and the mask rows
// come from each query's own set.
struct MixedPlan {
  CrsDev ring{};                 // the first query's set: the launch's ring constants
  std::vector<ShardDev> table;   // distinct (database, shard) pairs of the launch
  std::vector<QueryDev> qs;      // launch order: longest recursion (gamma) first
  std::vector<u32> work;         // scan work items, position << 12 | chunk
  size_t fold_words = 0;
  u32 max_gamma = 0;             // the longest recursion of the launch
};

// Resolves and checks every query (the caller holds the context lock). The whole batch is
// refused on the first error, with the reference's message where it has one. Seeds and b
// are left for the caller to point at its copies (query row r at row r of its arrays).
static int plan_mixed(ig_ctx* c, u32 count, const uint64_t* dbs, const uint64_t* stores, const uint64_t* handles,
                      const uint32_t* shard_ids, const uint64_t* ms_targets, MixedPlan& P) {
  std::map<std::pair<u64, u32>, u32> local;
  std::vector<std::pair<u32, u32>> order;  // (gamma, row)
  u32 n = 0;
  P.qs.resize(count);
  for (u32 i = 0; i < count; i++) {
    DbObj* db = get_db(c, dbs[i]);
    if (!db) return fail(c, IG_ERR_HANDLE, "query %u: unknown database handle %llu", i, (unsigned long long)dbs[i]);
    const u64* seat;
    CrsObj* set;
    int rc = resolve_seat_for_db(c, *get_crs(c, db->crs), stores[i], handles[i], &seat, &set);
    if (rc) return rc;
    CrsObj& o = *set;
    if (i == 0) {
      n = o.n;
      P.ring = o.dev;
    } else if (o.n != n) {
      return fail(c, IG_ERR_SHAPE, "query %u: ring_dim %u differs from the launch's ring_dim %u; one launch serves one ring",
                  i, o.n, n);
    }
    const u64 ms = ms_targets ? ms_targets[i] : 0;
    if (ms && (ms >= Q || ms < o.p || ms % (2ULL * n) != 1))
      return fail(c, IG_ERR_ARG, "query %u: mod-switch target_modulus %llu must be in [p, q) and 1 mod 2d", i,
                  (unsigned long long)ms);
    const u32 s = shard_ids[i];
    if (s >= db->num_shards)
      return fail(c, IG_ERR_ARG, "query %u: shard %u not found at dense position %u; encoded database has %u shards", i,
                  s, s, db->num_shards);
    if (!db->shards[s].sums)
      return fail(c, IG_ERR_ARG, "query %u: shard %u has no packing store; mixed launches serve stored shards", i, s);
    auto key = std::make_pair(dbs[i], s);
    auto it = local.find(key);
    if (it == local.end()) {
      it = local.emplace(key, (u32)P.table.size()).first;
      P.table.push_back(db->shards[s].dev());
    }
    QueryDev& q = P.qs[i];
    q = QueryDev{};
    q.shard = it->second;
    q.seat_R = seat;
    q.crs = o.d_self;
    q.ms = ms;
    q.row = i;
    order.emplace_back(o.gamma, i);
  }
  // Longest recursion first, so the launch's tail is its shortest queries.
  std::stable_sort(order.begin(), order.end(), [](const std::pair<u32, u32>& x, const std::pair<u32, u32>& y) {
    return x.first > y.first;
  });
  std::vector<QueryDev> sorted(count);
  for (u32 p = 0; p < count; p++) {
    sorted[p] = P.qs[order[p].second];
    sorted[p].fold_off = (u32)P.fold_words;
    const u32 gamma = order[p].first;
    for (u32 ch = 0; ch < igk::scan_chunks(gamma); ch++) P.work.push_back((p << 12) | ch);
    P.fold_words += gamma;
    P.max_gamma = std::max(P.max_gamma, gamma);
  }
  P.qs.swap(sorted);
  return IG_OK;
}

int ig_respond_mixed_batch_device(ig_ctx* c, uint32_t count, const uint64_t* dbs, const uint64_t* stores,
                                  const uint64_t* handles, const uint32_t* shard_ids, const uint8_t* d_seeds,
                                  const uint64_t* d_bs, const uint64_t* ms_targets, uint64_t* d_a, uint64_t* d_b,
                                  uint32_t* d_status) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !dbs || !stores || !handles || !shard_ids || !d_seeds || !d_bs || !d_a || !d_b || !d_status)
    return fail(c, IG_ERR_ARG, "ig_respond_mixed_batch_device: empty batch or null buffer");
  if (count >= (1u << 20)) return fail(c, IG_ERR_ARG, "ig_respond_mixed_batch_device: at most 2^20 - 1 queries a launch");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  MixedPlan P;
  int rc = plan_mixed(c, count, dbs, stores, handles, shard_ids, ms_targets, P);
  if (rc) return rc;
  const size_t n = P.ring.n;
  for (QueryDev& q : P.qs) {
    q.seed = (const u32*)(d_seeds + (size_t)q.row * 32);
    q.b = d_bs + (size_t)q.row * n;
  }
  int lane = -1;
  cudaStream_t s = c->stream;
  if ((rc = igint::lane_acquire(c, &s, &lane))) return rc;
  char nq[32], nt[32], nw[32], nf[32];
  snprintf(nq, sizeof nq, "mix_queries%d", lane);
  snprintf(nt, sizeof nt, "mix_table%d", lane);
  snprintf(nw, sizeof nw, "mix_work%d", lane);
  snprintf(nf, sizeof nf, "mix_fold%d", lane);
  void *dq, *dt, *dw, *df;
  if ((rc = scratch(c, nq, count * sizeof(QueryDev), &dq)) ||
      (rc = scratch(c, nt, P.table.size() * sizeof(ShardDev), &dt)) ||
      (rc = scratch(c, nw, P.work.size() * 4, &dw)) || (rc = scratch(c, nf, P.fold_words * 8, &df)))
    return rc;
  if ((rc = stage_h2d(c, dq, P.qs.data(), count * sizeof(QueryDev))) ||
      (rc = stage_h2d(c, dt, P.table.data(), P.table.size() * sizeof(ShardDev))) ||
      (rc = stage_h2d(c, dw, P.work.data(), P.work.size() * 4)) || (rc = igint::lane_enter(c, lane)))
    return rc;
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  long pk = prof_begin(c, REGION_SCAN, s);
  IG_CUDA(c, igk::shard_scan(P.ring, (const QueryDev*)dq, (const ShardDev*)dt, count, (const u32*)dw,
                             (u32)P.work.size(), (u64*)df, d_status, s));
  prof_end(c, pk, s);
  const int ctas = igint::launch_ctas(c, (u32)n, P.max_gamma, count, count * c->lanes);
  pk = prof_begin(c, REGION_RESPOND, s);
  IG_CUDA(c, igk::respond(P.ring, (const QueryDev*)dq, (const ShardDev*)dt, count, (const u64*)df, d_a, d_b, d_status,
                          c->force_serial, ctas, s));
  prof_end(c, pk, s);
  c->launches += 2;
  return igint::lane_release(c, lane);
}

int ig_respond_mixed_batch(ig_ctx* c, uint32_t count, const uint64_t* dbs, const uint64_t* stores,
                           const uint64_t* handles, const uint32_t* shard_ids, const uint8_t* seeds, const uint64_t* bs,
                           const uint64_t* ms_targets, uint64_t* a_out, uint64_t* b_out) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !dbs || !stores || !handles || !shard_ids || !seeds || !bs || !a_out || !b_out)
    return fail(c, IG_ERR_ARG, "ig_respond_mixed_batch: empty batch or null buffer");
  if (count >= (1u << 20)) return fail(c, IG_ERR_ARG, "ig_respond_mixed_batch: at most 2^20 - 1 queries a call");
  igint::HostCall hc;
  igint::host_call_begin(c, hc);
  const u32 k = hc.k;
  std::unique_lock<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  MixedPlan P;
  int rc = plan_mixed(c, count, dbs, stores, handles, shard_ids, ms_targets, P);
  if (rc) return rc;
  const size_t n = P.ring.n;
  void *dq, *dt, *dw, *df, *dseeds, *dbs_, *da, *db_, *dst;
  auto lane_scratch = [&](const char* name, size_t bytes, void** out) {
    char full[48];
    snprintf(full, sizeof full, "%s%u", name, k);
    return scratch(c, full, bytes, out);
  };
  if ((rc = lane_scratch("hmix_queries", count * sizeof(QueryDev), &dq)) ||
      (rc = lane_scratch("hmix_table", P.table.size() * sizeof(ShardDev), &dt)) ||
      (rc = lane_scratch("hmix_work", P.work.size() * 4, &dw)) ||
      (rc = lane_scratch("hmix_fold", P.fold_words * 8, &df)) ||
      (rc = lane_scratch("hmix_seeds", (size_t)count * 32, &dseeds)) ||
      (rc = lane_scratch("hmix_bs", (size_t)count * n * 8, &dbs_)) ||
      (rc = lane_scratch("hmix_a", (size_t)count * n * 8, &da)) ||
      (rc = lane_scratch("hmix_b", (size_t)count * n * 8, &db_)) ||
      (rc = lane_scratch("hmix_status", (size_t)count * 4, &dst)))
    return rc;
  for (QueryDev& q : P.qs) {
    q.seed = (const u32*)((const uint8_t*)dseeds + (size_t)q.row * 32);
    q.b = (const u64*)dbs_ + (size_t)q.row * n;
  }
  const size_t st_bytes = ((size_t)count * 4 + 15) & ~(size_t)15;
  void* pin;
  if ((rc = igint::host_call_pinned(c, hc, st_bytes + 2 * (size_t)count * n * 8, &pin))) return rc;
  u32* h_status = (u32*)pin;
  u64* h_a = (u64*)((uint8_t*)pin + st_bytes);
  u64* h_b = h_a + (size_t)count * n;
  cudaStream_t s = igint::host_call_stream(c, hc);
  if ((rc = stage_h2d(c, dq, P.qs.data(), count * sizeof(QueryDev))) ||
      (rc = stage_h2d(c, dt, P.table.data(), P.table.size() * sizeof(ShardDev))) ||
      (rc = stage_h2d(c, dw, P.work.data(), P.work.size() * 4)) ||
      (rc = stage_h2d(c, dseeds, seeds, (size_t)count * 32)) ||
      (rc = stage_h2d(c, dbs_, bs, (size_t)count * n * 8)) || (rc = igint::host_call_enter(c, hc)))
    return rc;
  IG_CUDA(c, cudaMemsetAsync(dst, 0, count * 4, s));
  IG_CUDA(c, igk::shard_scan(P.ring, (const QueryDev*)dq, (const ShardDev*)dt, count, (const u32*)dw,
                             (u32)P.work.size(), (u64*)df, (u32*)dst, s));
  IG_CUDA(c, igk::respond(P.ring, (const QueryDev*)dq, (const ShardDev*)dt, count, (const u64*)df, (u64*)da, (u64*)db_,
                          (u32*)dst, c->force_serial,
                          igint::launch_ctas(c, (u32)n, P.max_gamma, count, count * c->lanes),
                          s));
  c->launches += 2;
  IG_CUDA(c, cudaMemcpyAsync(h_status, dst, count * 4, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaMemcpyAsync(h_a, da, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaMemcpyAsync(h_b, db_, (size_t)count * n * 8, cudaMemcpyDeviceToHost, s));
  if ((rc = igint::host_call_launched(c, hc))) return rc;
  lk.unlock();  // other callers launch while this batch runs
  if ((rc = igint::host_call_wait(c, hc))) return rc;
  for (u32 i = 0; i < count; i++) {
    if (h_status[i] & DEV_TAG_MISMATCH)
      return fail(c, IG_ERR_STORE_REFUSED,
                  "shard %u: packing store refused: a column is not the column the store was built from. The shard "
                  "changed after the build; rebuild the store before serving it",
                  shard_ids[i]);
    if (h_status[i]) return fail(c, IG_ERR_DEVICE, "query %u: respond kernel status %u", i, h_status[i]);
  }
  memcpy(a_out, h_a, (size_t)count * n * 8);
  memcpy(b_out, h_b, (size_t)count * n * 8);
  return IG_OK;
}

int ig_ctx_set_lanes(ig_ctx* c, uint32_t lanes) {
  if (!c) return IG_ERR_ARG;
  if (lanes == 0 || lanes > IG_MAX_LANES)
    return fail(c, IG_ERR_ARG, "ig_ctx_set_lanes: lanes must be 1..%u", (unsigned)IG_MAX_LANES);
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  for (u32 k = 0; k < lanes; k++) {
    if (c->lane_stream[k]) continue;
    IG_CUDA(c, cudaStreamCreateWithFlags(&c->lane_stream[k], cudaStreamNonBlocking));
    IG_CUDA(c, cudaEventCreateWithFlags(&c->lane_in[k], cudaEventDisableTiming));
    IG_CUDA(c, cudaEventCreateWithFlags(&c->lane_done[k], cudaEventDisableTiming));
  }
  // Work already queued on lanes stays ordered before anything the context does next.
  for (u32 k = 0; k < IG_MAX_LANES; k++)
    if (c->lane_used[k]) IG_CUDA(c, cudaStreamWaitEvent(c->stream, c->lane_done[k], 0));
  c->lanes = lanes;
  c->lane_next = 0;
  return IG_OK;
}

int ig_ctx_join(ig_ctx* c) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  for (u32 k = 0; k < IG_MAX_LANES; k++)
    if (c->lane_used[k]) IG_CUDA(c, cudaStreamWaitEvent(c->stream, c->lane_done[k], 0));
  return IG_OK;
}

// ---- wire -------------------------------------------------------------------------------
static void put_u64(std::vector<uint8_t>& w, u64 v) {
  for (int i = 0; i < 8; i++) w.push_back((uint8_t)(v >> (8 * i)));
}
static void put_u32(std::vector<uint8_t>& w, u32 v) {
  for (int i = 0; i < 4; i++) w.push_back((uint8_t)(v >> (8 * i)));
}
static bool put_tight(std::vector<uint8_t>& w, const u64* c, size_t count, u64 modulus) {
  const unsigned bits = 64 - __builtin_clzll(modulus - 1);
  const size_t nbytes = (count * bits + 7) / 8;
  put_u64(w, nbytes);
  const size_t base = w.size();
  w.resize(base + nbytes, 0);
  for (size_t i = 0; i < count; i++) {
    if (c[i] >= modulus) return false;
    const size_t bit = i * bits;
    const u128 v = (u128)c[i] << (bit % 8);
    for (size_t k = 0; k < 10 && bit / 8 + k < nbytes; k++) w[base + bit / 8 + k] |= (uint8_t)(v >> (8 * k));
  }
  return true;
}

// RIMS frame (mod_switch.rs:254-345): header of 23 bytes, then coefficients at a whole
// number of bytes each.
static const size_t RIMS_HEADER = 23;
static unsigned rims_width(u64 modulus) {
  const unsigned bits = modulus <= 1 ? 1 : 64 - __builtin_clzll(modulus - 1);
  return (bits + 7) / 8;
}
// Writes "decode_response_packed: <message>" into err (when given) and refuses.
__attribute__((format(printf, 3, 4))) static int rims_refuse(char* err, size_t cap, const char* fmt, ...) {
  if (err && cap) {
    char msg[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    snprintf(err, cap, "decode_response_packed: %s", msg);
  }
  return IG_ERR_SHAPE;
}
static bool put_rims_poly(std::vector<uint8_t>& w, const u64* c, size_t count, u64 modulus, unsigned width) {
  for (size_t i = 0; i < count; i++) {
    if (c[i] >= modulus) return false;
    for (unsigned k = 0; k < width; k++) w.push_back((uint8_t)(c[i] >> (8 * k)));
  }
  return true;
}

int ig_response_encode_device(ig_ctx* c, uint32_t count, const uint64_t* d_a, const uint64_t* d_b, uint32_t n,
                              uint32_t retained, uint64_t modulus, uint8_t* d_out, size_t* len_out,
                              uint32_t* d_status) {
  if (!c) return IG_ERR_ARG;
  if (!len_out || n == 0 || modulus < 256 || retained == 0 || retained > n)
    return fail(c, IG_ERR_ARG, "ig_response_encode_device: ring_dim, retained or modulus out of range");
  // The template: the same response with zero coefficients, from the host encoder.
  std::vector<u64> za(n, 0), zb(retained, 0);
  size_t len = 0;
  int rc = ig_response_encode(za.data(), zb.data(), n, retained, modulus, nullptr, 0, &len);
  if (rc) return fail(c, rc, "ig_response_encode_device: template refused");
  *len_out = len;
  if (!d_out) return IG_OK;  // size query
  if (count == 0 || !d_a || !d_b || !d_status)
    return fail(c, IG_ERR_ARG, "ig_response_encode_device: empty batch or null buffer");
  std::vector<uint8_t> tmpl(len);
  ig_response_encode(za.data(), zb.data(), n, retained, modulus, tmpl.data(), len, &len);
  const unsigned bits = 64 - __builtin_clzll(modulus - 1);
  const u32 a_bytes = (u32)(((u64)n * bits + 7) / 8), b_bytes = (u32)(((u64)retained * bits + 7) / 8);
  const u32 a_off = 4 + 8, b_off = a_off + a_bytes + 41 + 8;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  void* d_t;
  if ((rc = scratch(c, "wire_template", len, &d_t))) return rc;
  if ((rc = stage_h2d(c, d_t, tmpl.data(), len))) return rc;
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, (size_t)count * 4, c->stream));
  IG_CUDA(c, igk::wire(d_a, d_b, count, n, retained, bits, modulus, (const uint8_t*)d_t, (u32)len, a_off, a_bytes,
                       b_off, b_bytes, d_out, d_status, c->stream));
  c->launches++;
  return IG_OK;
}

int ig_response_encode_full(const uint64_t* cts, uint32_t count, uint32_t n, uint64_t modulus, uint8_t* out,
                            size_t cap, size_t* len_out) {
  if (!cts || !len_out || n == 0 || modulus < 2 || count == 0) return IG_ERR_ARG;
  std::vector<uint8_t> w;
  auto poly = [&](const u64* c) {
    if (!put_tight(w, c, n, modulus)) return false;
    put_u64(w, 1);  // moduli
    put_u64(w, modulus);
    put_u64(w, modulus);  // q
    put_u64(w, n);        // dim
    put_u64(w, 0);        // crt_q0_inv_mod_q1
    w.push_back(0);       // is_ntt
    return true;
  };
  put_u32(w, 0);  // ResponseCiphertextWire::Full
  if (!poly(cts) || !poly(cts + n)) return IG_ERR_SHAPE;
  put_u64(w, count - 1);  // column_ciphertexts
  for (u32 j = 1; j < count; j++)
    if (!poly(cts + (size_t)2 * j * n) || !poly(cts + (size_t)(2 * j + 1) * n)) return IG_ERR_SHAPE;
  w.push_back(0);  // packing_mode: None
  *len_out = w.size();
  if (out) memcpy(out, w.data(), w.size() < cap ? w.size() : cap);
  return IG_OK;
}

int ig_response_encode(const uint64_t* a, const uint64_t* b, uint32_t n, uint32_t retained, uint64_t modulus,
                       uint8_t* out, size_t cap, size_t* len_out) {
  if (!a || !b || !len_out || n == 0 || modulus < 2 || retained == 0 || retained > n) return IG_ERR_ARG;
  std::vector<uint8_t> w;
  put_u32(w, 1);  // ResponseCiphertextWire::Packed
  if (!put_tight(w, a, n, modulus)) return IG_ERR_SHAPE;
  put_u64(w, 1);  // moduli
  put_u64(w, modulus);
  put_u64(w, modulus);  // q
  put_u64(w, n);        // dim
  put_u64(w, 0);        // crt_q0_inv_mod_q1
  w.push_back(0);       // is_ntt
  if (!put_tight(w, b, retained, modulus)) return IG_ERR_SHAPE;
  put_u32(w, retained);
  put_u64(w, 0);  // column_ciphertexts
  w.push_back(1);  // Some(
  put_u32(w, 0);   //   PackingMode::Inspiring)
  *len_out = w.size();
  if (out) memcpy(out, w.data(), w.size() < cap ? w.size() : cap);
  return IG_OK;
}

int ig_response_encode_tree(const uint64_t* a, const uint64_t* b, uint32_t n, uint32_t retained, uint64_t modulus,
                            uint8_t* out, size_t cap, size_t* len_out) {
  size_t len = 0;
  const int rc = ig_response_encode(a, b, n, retained, modulus, nullptr, 0, &len);
  if (rc) return rc;
  *len_out = len;
  if (!out) return IG_OK;
  std::vector<uint8_t> w(len);
  ig_response_encode(a, b, n, retained, modulus, w.data(), len, &len);
  w[len - 4] = 1;  // Some(PackingMode::Tree): variant 1 of query.rs:20-26
  memcpy(out, w.data(), len < cap ? len : cap);
  return IG_OK;
}

int ig_response_encode_rims(const uint64_t* a, const uint64_t* b, uint32_t n, uint32_t retained,
                            uint32_t packing_mode, const uint64_t* cts, uint32_t columns, uint64_t modulus,
                            uint8_t* out, size_t cap, size_t* len_out) {
  if (!a || !b || !len_out || n == 0 || modulus == 0 || packing_mode > 2) return IG_ERR_ARG;
  // (None, None): b whole and the column ciphertexts; (Some, Some(retained)): a b prefix
  // and no columns (mod_switch.rs:288-309).
  if (packing_mode == 0 ? (retained != 0 || (columns && !cts)) : (retained == 0 || retained > n || columns != 0))
    return IG_ERR_ARG;
  const unsigned width = rims_width(modulus);
  const u32 kept = packing_mode == 0 ? n : retained;
  std::vector<uint8_t> w;
  w.reserve(RIMS_HEADER + ((size_t)n + kept + 2 * (size_t)columns * n) * width);
  w.insert(w.end(), {'R', 'I', 'M', 'S', 2});
  put_u64(w, modulus);
  put_u32(w, n);
  w.push_back((uint8_t)width);
  w.push_back((uint8_t)packing_mode);
  put_u32(w, packing_mode == 0 ? columns : retained);
  if (!put_rims_poly(w, a, n, modulus, width) || !put_rims_poly(w, b, kept, modulus, width)) return IG_ERR_SHAPE;
  for (u32 j = 0; j < columns; j++)
    if (!put_rims_poly(w, cts + (size_t)2 * j * n, 2 * (size_t)n, modulus, width)) return IG_ERR_SHAPE;
  *len_out = w.size();
  if (out) memcpy(out, w.data(), w.size() < cap ? w.size() : cap);
  return IG_OK;
}

int ig_response_decode_rims(const uint8_t* bytes, size_t len, uint64_t* modulus_out, uint32_t* ring_dim_out,
                            uint32_t* packing_mode_out, uint32_t* retained_out, uint32_t* columns_out, uint64_t* a,
                            uint64_t* b, uint64_t* cts, char* err, size_t err_cap) {
  if (!bytes && len) return IG_ERR_ARG;
  auto le = [&](size_t off, int nb) {
    u64 v = 0;
    for (int k = 0; k < nb; k++) v |= (u64)bytes[off + k] << (8 * k);
    return v;
  };
  // Each check in the order of mod_switch.rs:368-509.
  if (len < RIMS_HEADER || memcmp(bytes, "RIMS", 4) != 0) return rims_refuse(err, err_cap, "bad magic / truncated header");
  if (bytes[4] != 2) return rims_refuse(err, err_cap, "unsupported version %u", (unsigned)bytes[4]);
  const u64 modulus = le(5, 8);
  if (modulus == 0) return rims_refuse(err, err_cap, "target_modulus must be positive");
  const u64 n = le(13, 4);
  if (n == 0) return rims_refuse(err, err_cap, "ring_dim must be positive");
  const unsigned width = bytes[17], expect = rims_width(modulus);
  if (width != expect || width > 8)
    return rims_refuse(err, err_cap, "bytes_per_coeff %u does not match modulus width %u", width, expect);
  const unsigned mode = bytes[18];
  if (mode > 2) return rims_refuse(err, err_cap, "unknown packing_mode byte %u", mode);
  const u64 shape = le(19, 4);
  u64 columns = 0, kept = n, retained = 0;
  if (mode == 0) {
    columns = shape;
  } else {
    if (shape == 0 || shape > n)
      return rims_refuse(err, err_cap, "retained count %llu outside 1..=%llu", (unsigned long long)shape, (unsigned long long)n);
    kept = retained = shape;
  }
  const u128 coeffs = (u128)n + kept + (u128)2 * columns * n;
  const u128 expected = RIMS_HEADER + coeffs * width;
  if (expected != (u128)len)
    return rims_refuse(err, err_cap, "payload length mismatch (expected %llu, got %llu)", (unsigned long long)expected,
                  (unsigned long long)len);
  size_t cur = RIMS_HEADER;
  auto read = [&](u64* dst, u64 count, u64 dim) -> bool {
    for (u64 i = 0; i < count; i++, cur += width) {
      const u64 v = le(cur, (int)width);
      if (v >= modulus) return false;
      if (dst) dst[i] = v;
    }
    if (dst)
      for (u64 i = count; i < dim; i++) dst[i] = 0;
    return true;
  };
  u64 bad = 0;
  auto check = [&](u64* dst, u64 count, u64 dim) {
    const size_t at = cur;
    if (read(dst, count, dim)) return true;
    // Find the offending word for the message.
    for (size_t p = at; p < at + count * width; p += width)
      if ((bad = le(p, (int)width)) >= modulus) break;
    return false;
  };
  const bool fill = a && b && (columns == 0 || cts);
  if (!check(fill ? a : nullptr, n, n) || !check(fill ? b : nullptr, kept, n))
    return rims_refuse(err, err_cap, "coefficient %llu is not canonical for modulus %llu", (unsigned long long)bad,
                  (unsigned long long)modulus);
  for (u64 j = 0; j < columns; j++)
    if (!check(fill ? cts + 2 * j * n : nullptr, n, n) || !check(fill ? cts + (2 * j + 1) * n : nullptr, n, n))
      return rims_refuse(err, err_cap, "coefficient %llu is not canonical for modulus %llu", (unsigned long long)bad,
                    (unsigned long long)modulus);
  if (n > 0xffffffffull || columns > 0xffffffffull) return rims_refuse(err, err_cap, "ring_dim or column count exceeds u32");
  if (modulus_out) *modulus_out = modulus;
  if (ring_dim_out) *ring_dim_out = (u32)n;
  if (packing_mode_out) *packing_mode_out = mode;
  if (retained_out) *retained_out = (u32)retained;
  if (columns_out) *columns_out = (u32)columns;
  return IG_OK;
}

int ig_response_encode_rims_device(ig_ctx* c, uint32_t count, const uint64_t* d_a, const uint64_t* d_b, uint32_t n,
                                   uint32_t retained, uint64_t modulus, uint8_t* d_out, size_t* len_out,
                                   uint32_t* d_status) {
  if (!c) return IG_ERR_ARG;
  if (!len_out || n == 0 || modulus < 2 || retained == 0 || retained > n)
    return fail(c, IG_ERR_ARG, "ig_response_encode_rims_device: ring_dim, retained or modulus out of range");
  // The template: the frame of a zero response; the coefficients fill whole bytes, so the
  // bit-packing wire kernel at 8 x width bits writes them.
  std::vector<u64> za(n, 0), zb(retained, 0);
  size_t len = 0;
  int rc = ig_response_encode_rims(za.data(), zb.data(), n, retained, 1, nullptr, 0, modulus, nullptr, 0, &len);
  if (rc) return fail(c, rc, "ig_response_encode_rims_device: template refused");
  *len_out = len;
  if (!d_out) return IG_OK;  // size query
  if (count == 0 || !d_a || !d_b || !d_status)
    return fail(c, IG_ERR_ARG, "ig_response_encode_rims_device: empty batch or null buffer");
  std::vector<uint8_t> tmpl(len);
  ig_response_encode_rims(za.data(), zb.data(), n, retained, 1, nullptr, 0, modulus, tmpl.data(), len, &len);
  const u32 width = rims_width(modulus);
  const u32 a_off = (u32)RIMS_HEADER, a_bytes = n * width, b_off = a_off + a_bytes, b_bytes = retained * width;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  void* d_t;
  if ((rc = scratch(c, "rims_template", len, &d_t))) return rc;
  if ((rc = stage_h2d(c, d_t, tmpl.data(), len))) return rc;
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, (size_t)count * 4, c->stream));
  IG_CUDA(c, igk::wire(d_a, d_b, count, n, retained, 8 * width, modulus, (const uint8_t*)d_t, (u32)len, a_off,
                       a_bytes, b_off, b_bytes, d_out, d_status, c->stream));
  c->launches++;
  return IG_OK;
}

int ig_ctx_set_launch_shape(ig_ctx* c, uint32_t ctas) {
  if (!c) return IG_ERR_ARG;
  if (ctas != 0 && ctas != 1 && ctas != 2 && ctas != 4)
    return fail(c, IG_ERR_ARG, "ig_ctx_set_launch_shape: 0 (chosen per launch), 1, 2 or 4 CTAs per query");
  std::lock_guard<std::mutex> lk(c->mu);
  c->force_ctas = ctas;
  return IG_OK;
}

// The launch-shape tuner: per width, launches of kTuneBatches queries under each shape, on a
// synthetic database, seat and queries built here and freed after; the same respond path as
// serving (scan and respond launches, device buffers), timed with CUDA events on the context
// stream.
static const u32 kTuneBatches[] = {1, 4, 16, 32, 64, 128, 256};
int ig_tune_launch_shapes(ig_ctx* c, uint32_t ring_dim, const uint32_t* gammas, uint32_t count, uint32_t reps) {
  if (!c) return IG_ERR_ARG;
  if (!gammas || count == 0 || reps == 0 || reps > 1000)
    return fail(c, IG_ERR_ARG, "ig_tune_launch_shapes: need 1.. widths and 1..1000 repetitions");
  u32 lanes0, force0;
  {
    std::lock_guard<std::mutex> lk(c->mu);
    lanes0 = c->lanes;
    force0 = c->force_ctas;
  }
  int rc = ig_ctx_set_lanes(c, 1);
  if (rc) return rc;
  const u32 n = ring_dim, maxq = kTuneBatches[sizeof kTuneBatches / sizeof kTuneBatches[0] - 1];
  const u32 shards = 8;
  std::mt19937_64 rng(0x7u);
  u64 *d_bs = nullptr, *d_a = nullptr, *d_b = nullptr;
  uint8_t* d_seeds = nullptr;
  u32* d_status = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    if (d_bs) dfree(c, d_bs, (size_t)maxq * n * 8);
    if (d_a) dfree(c, d_a, (size_t)maxq * n * 8);
    if (d_b) dfree(c, d_b, (size_t)maxq * n * 8);
    if (d_seeds) dfree(c, d_seeds, (size_t)maxq * 32);
    if (d_status) dfree(c, d_status, (size_t)maxq * 4);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    {
      std::lock_guard<std::mutex> lk(c->mu);
      c->force_ctas = force0;
    }
    ig_ctx_set_lanes(c, lanes0);
  };
  {
    std::lock_guard<std::mutex> lk(c->mu);
    cudaSetDevice(c->device);
    if ((rc = dalloc(c, (void**)&d_bs, (size_t)maxq * n * 8, nullptr)) ||
        (rc = dalloc(c, (void**)&d_a, (size_t)maxq * n * 8, nullptr)) ||
        (rc = dalloc(c, (void**)&d_b, (size_t)maxq * n * 8, nullptr)) ||
        (rc = dalloc(c, (void**)&d_seeds, (size_t)maxq * 32, nullptr)) ||
        (rc = dalloc(c, (void**)&d_status, (size_t)maxq * 4, nullptr))) {
      cleanup();
      return rc;
    }
    std::vector<u64> hb((size_t)maxq * n);
    for (auto& x : hb) x = rng() % Q;
    std::vector<uint8_t> hs((size_t)maxq * 32);
    for (auto& x : hs) x = (uint8_t)rng();
    cudaMemcpy(d_bs, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(d_seeds, hs.data(), hs.size(), cudaMemcpyHostToDevice);
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
      cleanup();
      return fail(c, IG_ERR_CUDA, "ig_tune_launch_shapes: event creation failed");
    }
  }
  for (u32 gi = 0; gi < count; gi++) {
    const u32 gamma = gammas[gi];
    uint8_t w_seed[32] = {0};
    u64 crs = 0, db = 0, store = 0, handle = 0;
    auto drop = [&]() {
      if (store) ig_session_store_destroy(c, store);
      if (db) ig_db_destroy(c, db);
      if (crs) ig_crs_destroy(c, crs);
    };
    if ((rc = ig_crs_create(c, n, Q, 65537, 1ULL << 20, 3, 0, gamma, w_seed, &crs)) ||
        (rc = ig_db_create(c, crs, shards, &db))) {
      drop();
      cleanup();
      return rc;
    }
    std::vector<u64> cols((size_t)gamma * n);
    for (auto& x : cols) x = rng() & 0xffff;
    for (u32 sh = 0; sh < shards && !rc; sh++) rc = ig_db_set_shard(c, db, sh, cols.data());
    if (!rc) rc = ig_db_precompute_packing_all(c, db);
    if (!rc) rc = ig_session_store_create(c, &store);
    std::vector<u64> y((size_t)3 * n);
    for (auto& x : y) x = rng() % Q;
    if (!rc) rc = ig_session_register(c, store, crs, y.data(), 3, gamma, &handle);
    if (rc) {
      drop();
      cleanup();
      return rc;
    }
    std::map<u32, std::array<double, 3>> rows;
    const u32 shapes[3] = {1, 2, 4};
    for (u32 batch : kTuneBatches) {
      std::array<double, 3> ms{};
      std::vector<u32> sids(batch);
      for (u32 q = 0; q < batch; q++) sids[q] = q % shards;
      for (int k = 0; k < 3 && !rc; k++) {
        {
          std::lock_guard<std::mutex> lk(c->mu);
          c->force_ctas = shapes[k];
        }
        for (u32 r = 0; r <= reps && !rc; r++) {
          if (r == 1) cudaEventRecord(e0, c->stream);  // after one untimed warm-up launch
          rc = ig_respond_seeded_batch_device(c, db, store, handle, batch, sids.data(), d_seeds, d_bs, 0, d_a, d_b,
                                              d_status);
        }
        cudaEventRecord(e1, c->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess && !rc)
          rc = fail(c, IG_ERR_CUDA, "ig_tune_launch_shapes: launch failed");
        float el = 0;
        cudaEventElapsedTime(&el, e0, e1);
        ms[k] = el / reps;
      }
      rows[batch] = ms;
    }
    drop();
    if (rc) {
      cleanup();
      return rc;
    }
    std::lock_guard<std::mutex> lk(c->mu);
    c->tune[{n, gamma}] = rows;
  }
  cleanup();
  return IG_OK;
}

int ig_tune_get(ig_ctx* c, uint32_t ring_dim, uint32_t gamma, uint32_t queries, double* ms_out) {
  if (!c || !ms_out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->tune.find({ring_dim, gamma});
  if (it == c->tune.end() || it->second.empty())
    return fail(c, IG_ERR_HANDLE, "no launch-shape entry for ring_dim %u, gamma %u", ring_dim, gamma);
  const std::array<double, 3>* row = igint::tuned_row(c, ring_dim, gamma, queries);
  for (int k = 0; k < 3; k++) ms_out[k] = (*row)[k];
  return IG_OK;
}

int ig_tune_choose(ig_ctx* c, uint32_t ring_dim, uint32_t gamma, uint32_t count, uint32_t in_flight, uint32_t* ctas) {
  if (!c || !ctas) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  *ctas = (u32)igint::launch_ctas(c, ring_dim, gamma, count, in_flight);
  return IG_OK;
}

int ig_tune_save(ig_ctx* c, const char* path) {
  if (!c || !path) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  FILE* f = fopen(path, "w");
  if (!f) return fail(c, IG_ERR_ARG, "ig_tune_save: cannot write %s", path);
  fprintf(f, "inspire_gb300 launch shapes 2\nsms %u\n", c->sms);
  for (const auto& kv : c->tune)
    for (const auto& row : kv.second)
      fprintf(f, "%u %u %u %.6f %.6f %.6f\n", kv.first.first, kv.first.second, row.first, row.second[0],
              row.second[1], row.second[2]);
  const bool ok = fclose(f) == 0;
  return ok ? IG_OK : fail(c, IG_ERR_ARG, "ig_tune_save: writing %s failed", path);
}

int ig_tune_load(ig_ctx* c, const char* path) {
  if (!c || !path) return IG_ERR_ARG;
  FILE* f = fopen(path, "r");
  if (!f) return fail(c, IG_ERR_ARG, "ig_tune_load: cannot read %s", path);
  unsigned version = 0, sms = 0;
  std::map<std::pair<u32, u32>, std::map<u32, std::array<double, 3>>> table;
  int rc = IG_OK;
  if (fscanf(f, "inspire_gb300 launch shapes %u sms %u", &version, &sms) != 2 || version != 2) {
    rc = fail(c, IG_ERR_ARG, "ig_tune_load: %s is not a launch-shape table", path);
  } else if (sms != c->sms) {
    rc = fail(c, IG_ERR_ARG, "ig_tune_load: %s was measured on %u SMs, this device has %u", path, sms, c->sms);
  } else {
    unsigned n, g, q;
    double a, b, d;
    int got;
    while ((got = fscanf(f, "%u %u %u %lf %lf %lf", &n, &g, &q, &a, &b, &d)) == 6) table[{n, g}][q] = {a, b, d};
    if (got != EOF) rc = fail(c, IG_ERR_ARG, "ig_tune_load: %s holds a malformed line", path);
  }
  fclose(f);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  for (const auto& kv : table) c->tune[kv.first] = kv.second;
  return IG_OK;
}

int ig_ctx_set_pair_threshold(ig_ctx* c, uint32_t max_queries) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  c->pair_threshold = max_queries;
  return IG_OK;
}

int ig_profile_enable(ig_ctx* c, int on) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  c->profile = on ? 1 : 0;
  return IG_OK;
}

int ig_profile_read(ig_ctx* c, double* ms, uint64_t* counts, int regions, int reset) {
  if (!c || !ms || !counts || regions <= 0) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  IG_CUDA(c, cudaStreamSynchronize(c->stream));
  for (u32 k = 0; k < IG_MAX_LANES; k++)
    if (c->lane_used[k]) IG_CUDA(c, cudaStreamSynchronize(c->lane_stream[k]));
  for (int r = 0; r < regions; r++) {
    ms[r] = 0;
    counts[r] = 0;
  }
  for (auto& u : c->ev_used) {
    if (u.first >= regions) continue;
    float t = 0;
    if (cudaEventElapsedTime(&t, c->ev_pool[u.second].first, c->ev_pool[u.second].second) == cudaSuccess) {
      ms[u.first] += t;
      counts[u.first]++;
    }
  }
  if (reset) c->ev_used.clear();
  return IG_OK;
}

uint64_t ig_launch_count(const ig_ctx* c) { return c ? c->launches.load() : 0; }

int ig_debug_force_serial_expand(ig_ctx* c, int on) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  c->force_serial = on ? 1 : 0;
  return IG_OK;
}

int ig_butterfly_peak(ig_ctx* c, int blocks_per_sm, int iters, double* per_s) {
  if (!c || !per_s || blocks_per_sm <= 0 || iters <= 0) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int sms = 0;
  IG_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  void* out;
  int rc = scratch(c, "peak_out", 8, &out);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  IG_CUDA(c, cudaEventCreate(&e0));
  IG_CUDA(c, cudaEventCreate(&e1));
  const int blocks = sms * blocks_per_sm;
  IG_CUDA(c, igk::butterfly_peak((u64*)out, blocks, iters / 8 + 1, c->stream));  // warm-up
  IG_CUDA(c, cudaEventRecord(e0, c->stream));
  IG_CUDA(c, igk::butterfly_peak((u64*)out, blocks, iters, c->stream));
  IG_CUDA(c, cudaEventRecord(e1, c->stream));
  IG_CUDA(c, cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->launches += 2;
  *per_s = (double)blocks * 256.0 * (double)iters * 8.0 / ((double)ms / 1e3);
  return IG_OK;
}

int ig_debug_fail_alloc_at(ig_ctx* c, uint32_t k) {
  if (!c) return IG_ERR_ARG;
  c->fail_alloc_at.store(k);
  return IG_OK;
}

int ig_debug_store_sums(ig_ctx* c, uint64_t dbh, uint32_t s, uint64_t* out) {
  if (!c || !out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle");
  if (s >= db->num_shards || !db->shards[s].sums) return fail(c, IG_ERR_ARG, "shard %u has no store", s);
  CrsObj* o = get_crs(c, db->crs);
  IG_CUDA(c, cudaMemcpy(out, db->shards[s].sums, (size_t)o->gamma * o->n * 8, cudaMemcpyDeviceToHost));
  return IG_OK;
}

}  // extern "C"

namespace igint {
static int resolve_request_locked(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, uint32_t shard,
                                  RequestView* out) {
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  const u64* seat;
  CrsObj* set;
  int rc = resolve_seat_for_db(c, *get_crs(c, db->crs), st, handle, &seat, &set);
  if (rc) return rc;
  CrsObj& o = *set;
  if (shard >= db->num_shards)
    return fail(c, IG_ERR_ARG, "shard %u not found at dense position %u; encoded database has %u shards", shard,
                shard, db->num_shards);
  const ShardSlot& sl = db->shards[shard];
  if (!sl.cols) return fail(c, IG_ERR_ARG, "shard %u holds no columns", shard);
  out->crs = o.dev;
  out->crs_dev = o.d_self;
  out->shard = sl.dev();
  out->seat = seat;
  out->seat_rows = o.rows;
  out->p = o.p;
  out->has_store = sl.sums != nullptr;
  return IG_OK;
}

int resolve_request(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, uint32_t shard, RequestView* out) {
  std::lock_guard<std::mutex> lk(c->mu);
  const int rc = resolve_request_locked(c, dbh, st, handle, shard, out);
  out->err[0] = 0;
  if (rc) {
    std::lock_guard<std::mutex> elk(c->err_mu);
    snprintf(out->err, sizeof out->err, "%s", c->err.c_str());
  }
  return rc;
}
}  // namespace igint

extern "C" {

// ---- allocation-free respond --------------------------------------------------------------
// Some embedders cannot let a library allocate device memory on a request path: servers
// that pre-size every device buffer at start-up and refuse growth afterwards, and
// memory-capped GPU partitions shared with other jobs, where a late allocation can fail.
// For them the batch respond has a variant whose scratch (the per-query fold of b, the
// query descriptors and the status words) lives in one file-scope device array of fixed
// size. Every GPU that loads the library holds this array until exit. The call blocks
// until its batch completes (it reads the status words back).
enum : u32 { NOALLOC_MAX_QUERIES = 64, NOALLOC_MAX_GAMMA = 1024 };
static constexpr size_t NOALLOC_FOLD_BYTES = (size_t)NOALLOC_MAX_QUERIES * NOALLOC_MAX_GAMMA * 8;
static constexpr size_t NOALLOC_QUERY_OFF = NOALLOC_FOLD_BYTES;
static constexpr size_t NOALLOC_STATUS_OFF =
    NOALLOC_QUERY_OFF + ((NOALLOC_MAX_QUERIES * sizeof(QueryDev) + 255) / 256) * 256;
static constexpr size_t NOALLOC_BYTES = NOALLOC_STATUS_OFF + 256;
static_assert(NOALLOC_BYTES == 528640, "the header states this size");
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of g_noalloc_scratch on `device` (the current device). In host code the
// array's name is only a stand-in for the symbol, never a device pointer: the address
// comes from cudaGetSymbolAddress, resolved once per device and cached.
static int noalloc_scratch(ig_ctx* c, unsigned char** out) {
  static std::mutex mu;
  static std::unordered_map<int, unsigned char*> addr;
  std::lock_guard<std::mutex> lk(mu);
  auto it = addr.find(c->device);
  if (it != addr.end()) {
    *out = it->second;
    return IG_OK;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(c, IG_ERR_CUDA, "cannot resolve the allocation-free scratch on device %d: %s", c->device,
                cudaGetErrorString(e));
  addr[c->device] = (unsigned char*)p;
  *out = (unsigned char*)p;
  return IG_OK;
}

int ig_respond_seeded_batch_noalloc(ig_ctx* c, uint64_t dbh, uint64_t st, uint64_t handle, uint32_t count,
                                    const uint32_t* shard_ids, const uint8_t* d_seeds, const uint64_t* d_bs,
                                    uint64_t ms_target, uint64_t* d_a, uint64_t* d_b) {
  if (!c) return IG_ERR_ARG;
  if (count == 0 || !shard_ids || !d_seeds || !d_bs || !d_a || !d_b)
    return fail(c, IG_ERR_ARG, "ig_respond_seeded_batch_noalloc: empty batch or null buffer");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DbObj* db = get_db(c, dbh);
  if (!db) return fail(c, IG_ERR_HANDLE, "unknown database handle %llu", (unsigned long long)dbh);
  CrsObj& o = *get_crs(c, db->crs);
  const size_t n = o.n, g = o.gamma;
  if (count > NOALLOC_MAX_QUERIES || g > NOALLOC_MAX_GAMMA)
    return fail(c, IG_ERR_ARG,
                "ig_respond_seeded_batch_noalloc serves at most %u queries of width at most %u per call (its "
                "scratch is fixed); got %u queries of width %zu. Split the batch or use ig_respond_seeded_batch",
                (u32)NOALLOC_MAX_QUERIES, (u32)NOALLOC_MAX_GAMMA, count, g);
  if (ms_target && (ms_target >= Q || ms_target < o.p || ms_target % (2 * n) != 1))
    return fail(c, IG_ERR_ARG, "mod-switch target_modulus %llu must be in [p, q) and 1 mod 2d",
                (unsigned long long)ms_target);
  const u64* seat;
  int rc = resolve_seat(c, o, st, handle, nullptr, 0, 0, &seat);
  if (rc) return rc;
  for (u32 i = 0; i < count; i++) {
    const u32 s = shard_ids[i];
    if (s >= db->num_shards)
      return fail(c, IG_ERR_ARG, "shard %u not found; encoded database has %u shards", s, db->num_shards);
    if (!db->shards[s].sums)
      return fail(c, IG_ERR_ARG, "shard %u has no packing store; the allocation-free respond serves stored shards",
                  s);
  }
  unsigned char* base = nullptr;
  if ((rc = noalloc_scratch(c, &base))) return rc;
  u64* d_fold = (u64*)base;
  QueryDev* d_q = (QueryDev*)(base + NOALLOC_QUERY_OFF);
  u32* d_status = (u32*)(base + NOALLOC_STATUS_OFF);
  QueryDev qs[NOALLOC_MAX_QUERIES];
  for (u32 i = 0; i < count; i++) {
    qs[i] = QueryDev{};
    qs[i].shard = shard_ids[i];
    qs[i].fold_off = i * (u32)g;
    qs[i].seed = (const u32*)(d_seeds + (size_t)i * 32);
    qs[i].b = d_bs + (size_t)i * n;
    qs[i].seat_R = seat;
    qs[i].ms = ms_target;
    qs[i].row = i;
  }
  cudaStream_t s = c->stream;
  IG_CUDA(c, cudaMemcpyAsync(d_q, qs, count * sizeof(QueryDev), cudaMemcpyHostToDevice, s));
  IG_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  IG_CUDA(c, igk::shard_scan(o.dev, d_q, db->d_table, count, nullptr, 0, d_fold, d_status, s));
  // The launch shape of ig_respond_seeded_batch_device for the same batch and lane count.
  IG_CUDA(c, igk::respond(o.dev, d_q, db->d_table, count, d_fold, d_a, d_b, d_status, c->force_serial,
                          igint::launch_ctas(c, (u32)n, (u32)g, count, count * c->lanes),
                          s));
  c->launches += 2;
  u32 status[NOALLOC_MAX_QUERIES];
  IG_CUDA(c, cudaMemcpyAsync(status, d_status, count * 4, cudaMemcpyDeviceToHost, s));
  IG_CUDA(c, cudaStreamSynchronize(s));
  for (u32 i = 0; i < count; i++) {
    if (status[i] & DEV_TAG_MISMATCH)
      return fail(c, IG_ERR_STORE_REFUSED,
                  "shard %u: packing store refused: a column is not the column the store was built from. The shard "
                  "changed after the build; rebuild the store before serving it",
                  shard_ids[i]);
    if (status[i]) return fail(c, IG_ERR_DEVICE, "query %u: respond kernel status %u", i, status[i]);
  }
  return IG_OK;
}

}  // extern "C"
