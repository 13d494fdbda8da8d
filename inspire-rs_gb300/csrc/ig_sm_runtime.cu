// Host runtime of the special_modulus path behind the C ABI (ig_sm_* in
// include/inspire_gb300.h): the served parameter set's constants, seats, shard tables and
// the batched respond, with the refusal rules of src/special_modulus/server.rs.
#include <cuda_runtime.h>

#include <cstdio>

#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/inspire_gb300.h"
#include "ig_arith.cuh"
#include "ig_internal.hpp"
#include "ig_sm.cuh"

using namespace igsm;
using igint::fail;

namespace {

typedef unsigned __int128 u128;

u32 powm(u64 b, u64 e, u64 m) {
  u64 acc = 1;
  b %= m;
  while (e) {
    if (e & 1) acc = (u64)((u128)acc * b % m);
    b = (u64)((u128)b * b % m);
    e >>= 1;
  }
  return (u32)acc;
}
u32 mulm(u64 a, u64 b, u64 m) { return (u32)((u128)a * b % m); }

bool is_prime(u64 n) {
  if (n < 2) return false;
  for (u64 d = 2; d * d <= n; d++)
    if (n % d == 0) return false;
  return true;
}

size_t bitrev(size_t x, unsigned bits) {
  size_t r = 0;
  for (unsigned i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}

// Host mirror of one Ntt32's constants (arith.rs:131-166): the least g with
// g^((m-1)/2n) of order exactly 2n gives psi.
struct HostNtt32 {
  u64 m;
  size_t n;
  u32 neg_minv;
  std::vector<u32> fwd_std, fwd, inv;  // standard-form ladder (host transform), Montgomery ladders
  u32 n_inv;
  u32 to_mont(u64 x) const { return (u32)(((u128)x << 32) % m); }
  HostNtt32(size_t nn, u64 mm) : m(mm), n(nn) {
    u32 inv32 = 1;
    for (int i = 0; i < 5; i++) inv32 *= 2u - (u32)m * inv32;
    neg_minv = 0u - inv32;
    u32 psi = 0;
    for (u64 g = 2; g < m; g++) {
      u32 c = powm(g, (m - 1) / (2 * n), m);
      if (powm(c, n, m) == m - 1) {
        psi = c;
        break;
      }
    }
    const u32 psi_inv = powm(psi, 2 * n - 1, m);
    unsigned bits = 0;
    while ((size_t(1) << bits) < n) bits++;
    std::vector<u32> pf(n), pi(n);
    u64 a = 1, b = 1;
    for (size_t k = 0; k < n; k++) {
      pf[k] = (u32)a;
      pi[k] = (u32)b;
      a = a * psi % m;
      b = b * psi_inv % m;
    }
    fwd_std.resize(n);
    fwd.resize(n);
    inv.resize(n);
    for (size_t k = 0; k < n; k++) {
      fwd_std[k] = pf[bitrev(k, bits)];
      fwd[k] = to_mont(pf[bitrev(k, bits)]);
      inv[k] = to_mont(pi[bitrev(k, bits)]);
    }
    n_inv = to_mont(powm(n, m - 2, m));
  }
  // Forward transform in standard form (same slot order as the device transform).
  void forward(std::vector<u32>& x) const {
    size_t t = n;
    for (size_t mm = 1; mm < n; mm <<= 1) {
      t >>= 1;
      for (size_t i = 0; i < mm; i++)
        for (size_t j = 2 * i * t; j < 2 * i * t + t; j++) {
          u32 u = x[j], v = mulm(x[j + t], fwd_std[mm + i], m);
          x[j] = (u32)((u + (u64)v) % m);
          x[j + t] = (u32)((u + m - v) % m);
        }
    }
  }
};

// Slot exponents of a transform relative to its slot-0 root.
bool slot_exponents(const HostNtt32& T, std::vector<uint16_t>& slot_exp, std::vector<uint16_t>& exp_slot,
                    std::vector<u32>& roots) {
  const size_t n = T.n;
  std::vector<u32> X(n, 0);
  X[1] = 1;
  T.forward(X);
  roots = X;
  std::unordered_map<u32, u32> exp_of;
  u64 w0 = X[0], w0sq = (u64)((u128)w0 * w0 % T.m), pw = w0;
  for (u64 e = 1; e < 2 * n; e += 2) {
    exp_of[(u32)pw] = (u32)e;
    pw = (u64)((u128)pw * w0sq % T.m);
  }
  slot_exp.assign(n, 0);
  exp_slot.assign(n, 0xffff);
  for (size_t t = 0; t < n; t++) {
    auto it = exp_of.find(X[t]);
    if (it == exp_of.end()) return false;
    slot_exp[t] = (uint16_t)it->second;
    exp_slot[it->second / 2] = (uint16_t)t;
  }
  for (size_t e = 0; e < n; e++)
    if (exp_slot[e] >= n) return false;
  return true;
}

struct HostChaChaSm {
  u32 key[8];
  u64 stream, word = 0, have = ~0ULL;
  u32 blk[16];
  HostChaChaSm(const uint8_t seed[32], u64 s) : stream(s) {
    for (int i = 0; i < 8; i++) memcpy(&key[i], seed + 4 * i, 4);
  }
  u64 next_u64() {
    u64 out = 0;
    for (int h = 0; h < 2; h++) {
      u64 b = word / 16;
      if (b != have) {
        ig::chacha20_block(key, b, stream, blk);
        have = b;
      }
      out |= (u64)blk[word++ % 16] << (32 * h);
    }
    return out;
  }
};

void expand_uniform(HostChaChaSm& r, u64 m, u32* out, size_t count) {
  const u64 zone = (~0ULL / m) * m;
  for (size_t i = 0; i < count; i++) {
    u64 u;
    do u = r.next_u64();
    while (u >= zone);
    out[i] = (u32)(u % m);
  }
}

const u64 KEY_MASK_STREAM = 0x6b6579206d61736bULL;  // b"key mask" read big-endian

struct ServerObj {
  u32 n, gamma, cell_bytes, record_bytes;
  u64 q, p;
  SmDev dev{};
  std::vector<std::pair<void*, size_t>> allocs;
};
struct TableObj {
  u64 server;
  u32 rows;
  int8_t* values = nullptr;
  u32* step1 = nullptr;
  size_t bytes = 0;
};
struct SeatObj {
  u64 server;
  u32* words = nullptr;  // key_q, key_p, w_q, w_p
  size_t bytes = 0;
};
struct SmState {
  std::unordered_map<u64, ServerObj> servers;
  std::unordered_map<u64, TableObj> tables;
  std::unordered_map<u64, SeatObj> seats;
  u64 next = 1;
};

void destroy_state(ig_ctx* c, void* p) {
  auto* st = (SmState*)p;
  for (auto& kv : st->servers)
    for (auto& a : kv.second.allocs) cudaFree(a.first);
  for (auto& kv : st->tables) {
    cudaFree(kv.second.values);
    cudaFree(kv.second.step1);
  }
  for (auto& kv : st->seats) cudaFree(kv.second.words);
  (void)c;
  delete st;
}

SmState& state(ig_ctx* c) {
  void*& slot = igint::sm_slot(c);
  if (!slot) {
    slot = new SmState();
    igint::set_sm_destructor(c, destroy_state);
  }
  return *(SmState*)slot;
}

template <class T>
int up(ig_ctx* c, ServerObj& o, const std::vector<T>& v, const T** dst) {
  void* p;
  int rc = igint::dalloc(c, &p, v.size() * sizeof(T));
  if (rc) return rc;
  o.allocs.push_back({p, v.size() * sizeof(T)});
  if (cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(c, IG_ERR_CUDA, "upload of special-modulus constants failed");
  *dst = (const T*)p;
  return IG_OK;
}

#define SM_CUDA(ctx, call)                                                                       \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail(ctx, IG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

extern "C" {

int ig_sm_server_create(ig_ctx* c, uint32_t ring_dim, uint32_t gamma, uint64_t q, uint64_t special_prime,
                        uint32_t cell_bytes, uint32_t record_bytes, uint32_t key_mask_version, uint64_t* out) {
  if (!c || !out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  cudaSetDevice(igint::device(c));
  // Params::validate (special_modulus/mod.rs:98-159).
  const u32 d = ring_dim;
  if (d != 2048)
    return fail(c, IG_ERR_UNSUPPORTED, "ring dimension %u is not served; the GPU path serves ring 2048", d);
  if ((gamma & (gamma - 1)) || gamma < 2 || gamma > d / 2)
    return fail(c, IG_ERR_ARG, "packed width %u is not a power of two in [2, d/2]", gamma);
  if (cell_bytes * 2 != gamma)
    return fail(c, IG_ERR_ARG, "a %u-byte cell fills %u nibbles, not the packed width %u", cell_bytes, cell_bytes * 2,
                gamma);
  if (record_bytes == 0 || record_bytes > cell_bytes)
    return fail(c, IG_ERR_ARG, "record of %u bytes does not fit a %u-byte cell", record_bytes, cell_bytes);
  if (2 * record_bytes > 512) return fail(c, IG_ERR_UNSUPPORTED, "body of %u coefficients is not served", 2 * record_bytes);
  for (u64 m : {q, special_prime})
    if (m >= (1ULL << 31) || !is_prime(m) || (m - 1) % (2 * d) != 0)
      return fail(c, IG_ERR_ARG, "%llu is not a prime below 2^31 that is 1 mod %u", (unsigned long long)m, 2 * d);
  if (special_prime <= q)
    return fail(c, IG_ERR_ARG, "special prime %llu is not above the ciphertext prime %llu",
                (unsigned long long)special_prime, (unsigned long long)q);
  if (q / 16 < (1u << 16)) return fail(c, IG_ERR_ARG, "ciphertext prime %llu leaves no room for noise", (unsigned long long)q);
  if (key_mask_version != 2)
    return fail(c, IG_ERR_ARG, "key-mask version %u is not the per-key-seed version 2", key_mask_version);
  ServerObj o;
  o.n = d;
  o.gamma = gamma;
  o.cell_bytes = cell_bytes;
  o.record_bytes = record_bytes;
  o.q = q;
  o.p = special_prime;
  HostNtt32 hq(d, q), hp(d, special_prime);
  std::vector<uint16_t> se, es, se_p, es_p;
  std::vector<u32> roots, roots_p;
  if (!slot_exponents(hq, se, es, roots) || !slot_exponents(hp, se_p, es_p, roots_p))
    return fail(c, IG_ERR_UNSUPPORTED, "transform is not an evaluation at %u distinct roots", d);
  if (se != se_p) return fail(c, IG_ERR_UNSUPPORTED, "the two limbs disagree on an automorphism");
  const u64 two_d = 2ULL * d, g = two_d / gamma + 1, L = two_d / gamma;
  u64 ginv = 1;
  for (u32 k = 0; k + 1 < gamma; k++) ginv = ginv * g % two_d;
  std::vector<u32> gpow(gamma), cpow(gamma), mi(gamma);
  u64 a = 1, b = 1;
  for (u32 i = 0; i < gamma; i++) {
    gpow[i] = (u32)a;
    cpow[i] = (u32)b;
    if ((b - 1) % L) return fail(c, IG_ERR_UNSUPPORTED, "generator subgroup is not 1 mod 2n/gamma");
    mi[i] = (u32)((b - 1) / L);
    a = a * g % two_d;
    b = b * ginv % two_d;
  }
  std::vector<u32> pw(two_d);
  u64 acc = 1;
  for (u64 e = 0; e < two_d; e++) {
    pw[e] = (u32)(((u128)acc << 32) % q);
    acc = (u64)((u128)acc * roots[0] % q);
  }
  SmDev& dv = o.dev;
  dv.n = d;
  dv.logn = 11;
  dv.gamma = gamma;
  dv.nb = 2 * record_bytes;
  dv.lq.p = Prime32{(u32)q, hq.neg_minv};
  dv.lp.p = Prime32{(u32)special_prime, hp.neg_minv};
  dv.lq.n_inv = hq.n_inv;
  dv.lp.n_inv = hp.n_inv;
  // last = mont(inv[1], n_inv) = inv[1] n_inv 2^-32
  dv.lq.last = dv.lq.p.mont(hq.inv[1], hq.n_inv);
  dv.lp.last = dv.lp.p.mont(hp.inv[1], hp.n_inv);
  // Standard-form Shoup pairs of the same: 1/n, and 1/n (m - fwd[1]) (the inverse's last
  // twiddle is the negated second forward one).
  for (Ntt32Dev* T : {&dv.lq, &dv.lp}) {
    const HostNtt32& H = T == &dv.lq ? hq : hp;
    const u64 m = H.m;
    const u64 ninv = powm(H.n % m, m - 2, m);
    const u64 last = ninv * ((m - H.fwd_std[1]) % m) % m;
    T->n_inv_s = (u32)ninv;
    T->n_inv_sp = (u32)((ninv << 32) / m);
    T->last_s = (u32)last;
    T->last_sp = (u32)((last << 32) / m);
  }
  // The forward ladders as (w, floor(w 2^32 / m)) pairs for Shoup products.
  auto shoup_ladder = [](const HostNtt32& T) {
    std::vector<u32> v(2 * T.n);
    for (size_t k = 0; k < T.n; k++) {
      v[2 * k] = T.fwd_std[k];
      v[2 * k + 1] = (u32)(((u64)T.fwd_std[k] << 32) / T.m);
    }
    return v;
  };
  const std::vector<u32> shq = shoup_ladder(hq), shp = shoup_ladder(hp);
  const u32* shq_dev = nullptr;
  const u32* shp_dev = nullptr;
  int rc;
  if ((rc = up(c, o, hq.fwd, &dv.lq.fwd)) || (rc = up(c, o, hq.inv, &dv.lq.inv)) || (rc = up(c, o, hp.fwd, &dv.lp.fwd)) ||
      (rc = up(c, o, hp.inv, &dv.lp.inv)) || (rc = up(c, o, shq, &shq_dev)) || (rc = up(c, o, shp, &shp_dev)) ||
      (rc = up(c, o, se, &dv.slot_exp)) || (rc = up(c, o, es, &dv.exp_slot)) ||
      (rc = up(c, o, gpow, &dv.gpow)) || (rc = up(c, o, cpow, &dv.cpow)) || (rc = up(c, o, mi, &dv.m_of_i)) ||
      (rc = up(c, o, pw, &dv.pow_root_R))) {
    for (auto& a2 : o.allocs) igint::dfree(c, a2.first, a2.second);
    return rc;
  }
  dv.lq.fwd_sh = reinterpret_cast<const uint2*>(shq_dev);
  dv.lp.fwd_sh = reinterpret_cast<const uint2*>(shp_dev);
  dv.inv_gamma_RR = (u32)((u128)powm(gamma, q - 2, q) * (u64)(((u128)1 << 64) % q) % q);
  dv.p_over_q = (u32)(special_prime / q);
  dv.neg_off = (u32)((q - special_prime % q) % q);
  dv.q_mu = (u32)((1ULL << 32) / q);
  dv.p_inv_R = (u32)(((u128)powm(special_prime % q, q - 2, q) << 32) % q);
  SmState& st = state(c);
  const u64 h = st.next++;
  st.servers[h] = o;
  *out = h;
  return IG_OK;
}

int ig_sm_server_destroy(ig_ctx* c, uint64_t server) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  SmState& st = state(c);
  auto it = st.servers.find(server);
  if (it == st.servers.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus server %llu", (unsigned long long)server);
  cudaStreamSynchronize(igint::stream(c));
  for (auto& a : it->second.allocs) igint::dfree(c, a.first, a.second);
  st.servers.erase(it);
  return IG_OK;
}

int ig_sm_seat(ig_ctx* c, uint64_t server, const uint8_t mask_seed[32], const uint32_t* key_q, const uint32_t* key_p,
               uint64_t* seat_out) {
  if (!c || !mask_seed || !key_q || !key_p || !seat_out) return fail(c, IG_ERR_ARG, "ig_sm_seat: null argument");
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  cudaSetDevice(igint::device(c));
  SmState& st = state(c);
  auto it = st.servers.find(server);
  if (it == st.servers.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus server %llu", (unsigned long long)server);
  ServerObj& o = it->second;
  const u32 d = o.n;
  for (u32 k = 0; k < d; k++)
    if (key_q[k] >= o.q || key_p[k] >= o.p) return fail(c, IG_ERR_SHAPE, "packing key coefficient is not a residue");
  // Server::seat (server.rs:177-203): both limbs and the key's own mask, NTT, R-form.
  std::vector<u32> raw(4 * (size_t)d);
  memcpy(raw.data(), key_q, d * 4);
  memcpy(raw.data() + d, key_p, d * 4);
  HostChaChaSm r(mask_seed, KEY_MASK_STREAM);
  expand_uniform(r, o.q, raw.data() + 2 * d, d);
  expand_uniform(r, o.p, raw.data() + 3 * d, d);
  SeatObj seat;
  seat.server = server;
  seat.bytes = 4 * (size_t)d * 4;
  int rc = igint::dalloc(c, (void**)&seat.words, seat.bytes);
  if (rc) return rc;
  void* tmp;
  if ((rc = igint::scratch(c, "sm_seat_raw", seat.bytes, &tmp))) {
    igint::dfree(c, seat.words, seat.bytes);
    return rc;
  }
  cudaStream_t s = igint::stream(c);
  SM_CUDA(c, cudaMemcpyAsync(tmp, raw.data(), seat.bytes, cudaMemcpyHostToDevice, s));
  const u32* tr = (const u32*)tmp;
  SM_CUDA(c, igsmk::ntt_rows(o.dev, 0, tr, seat.words, 1, 1, s));
  SM_CUDA(c, igsmk::ntt_rows(o.dev, 1, tr + d, seat.words + d, 1, 1, s));
  SM_CUDA(c, igsmk::ntt_rows(o.dev, 0, tr + 2 * (size_t)d, seat.words + 2 * (size_t)d, 1, 1, s));
  SM_CUDA(c, igsmk::ntt_rows(o.dev, 1, tr + 3 * (size_t)d, seat.words + 3 * (size_t)d, 1, 1, s));
  SM_CUDA(c, cudaStreamSynchronize(s));
  const u64 h = st.next++;
  st.seats[h] = seat;
  *seat_out = h;
  return IG_OK;
}

int ig_sm_seat_destroy(ig_ctx* c, uint64_t seat) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  SmState& st = state(c);
  auto it = st.seats.find(seat);
  if (it == st.seats.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus seat %llu", (unsigned long long)seat);
  cudaStreamSynchronize(igint::stream(c));
  igint::dfree(c, it->second.words, it->second.bytes);
  st.seats.erase(it);
  return IG_OK;
}

int ig_sm_table(ig_ctx* c, uint64_t server, const uint8_t* cells, size_t nbytes, uint64_t* table_out) {
  if (!c || !table_out || (!cells && nbytes)) return fail(c, IG_ERR_ARG, "ig_sm_table: null argument");
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  cudaSetDevice(igint::device(c));
  SmState& st = state(c);
  auto it = st.servers.find(server);
  if (it == st.servers.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus server %llu", (unsigned long long)server);
  ServerObj& o = it->second;
  // Server::table (server.rs:211-249).
  if (nbytes % o.cell_bytes || nbytes / o.cell_bytes > o.n)
    return fail(c, IG_ERR_SHAPE, "%zu bytes are not at most %u cells of %u bytes", nbytes, o.n, o.cell_bytes);
  const u32 rows = (u32)(nbytes / o.cell_bytes);
  for (u32 m = 0; m < rows; m++)
    for (u32 k = o.record_bytes; k < o.cell_bytes; k++)
      if (cells[(size_t)m * o.cell_bytes + k])
        return fail(c, IG_ERR_SHAPE, "cell %u has bytes past its %u-byte record", m, o.record_bytes);
  TableObj t;
  t.server = server;
  t.rows = rows;
  const size_t vbytes = (size_t)o.n * o.gamma, sbytes = (size_t)o.gamma * o.n * 4;
  int rc = igint::dalloc(c, (void**)&t.values, vbytes);
  if (rc) return rc;
  if ((rc = igint::dalloc(c, (void**)&t.step1, sbytes))) {
    igint::dfree(c, t.values, vbytes);
    return rc;
  }
  t.bytes = vbytes + sbytes;
  void *dcells, *colq, *H;
  if ((rc = igint::scratch(c, "sm_cells", nbytes ? nbytes : 1, &dcells)) ||
      (rc = igint::scratch(c, "sm_colq", sbytes, &colq)) || (rc = igint::scratch(c, "sm_colH", sbytes, &H))) {
    igint::dfree(c, t.values, vbytes);
    igint::dfree(c, t.step1, sbytes);
    return rc;
  }
  cudaStream_t s = igint::stream(c);
  if (nbytes) SM_CUDA(c, cudaMemcpyAsync(dcells, cells, nbytes, cudaMemcpyHostToDevice, s));
  SM_CUDA(c, igsmk::table_columns(o.dev, (const uint8_t*)dcells, rows, o.cell_bytes, t.values, (u32*)colq, s));
  SM_CUDA(c, igsmk::ntt_rows(o.dev, 0, (const u32*)colq, (u32*)H, o.gamma, 0, s));
  SM_CUDA(c, igsmk::table_fold(o.dev, (const u32*)H, t.step1, s));
  SM_CUDA(c, cudaStreamSynchronize(s));
  const u64 h = st.next++;
  st.tables[h] = t;
  *table_out = h;
  return IG_OK;
}

int ig_sm_table_destroy(ig_ctx* c, uint64_t table) {
  if (!c) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  SmState& st = state(c);
  auto it = st.tables.find(table);
  if (it == st.tables.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus table %llu", (unsigned long long)table);
  cudaStreamSynchronize(igint::stream(c));
  const ServerObj& so = st.servers[it->second.server];
  igint::dfree(c, it->second.values, (size_t)so.n * so.gamma);
  igint::dfree(c, it->second.step1, (size_t)so.gamma * so.n * 4);
  st.tables.erase(it);
  return IG_OK;
}

int ig_sm_table_step1(ig_ctx* c, uint64_t table, uint32_t* out) {
  if (!c || !out) return IG_ERR_ARG;
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  SmState& st = state(c);
  auto it = st.tables.find(table);
  if (it == st.tables.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus table %llu", (unsigned long long)table);
  const ServerObj& o = st.servers[it->second.server];
  SM_CUDA(c, cudaMemcpy(out, it->second.step1, (size_t)o.gamma * o.n * 4, cudaMemcpyDeviceToHost));
  return IG_OK;
}

// Builds the per-query descriptors after the checks of Server::respond (server.rs:252-279).
static int sm_prepare(ig_ctx* c, SmState& st, uint64_t server, uint32_t count, const uint64_t* tables,
                      const uint64_t* seats, ServerObj** so, std::vector<SmQueryDev>& qs) {
  auto it = st.servers.find(server);
  if (it == st.servers.end()) return fail(c, IG_ERR_HANDLE, "unknown special-modulus server %llu", (unsigned long long)server);
  *so = &it->second;
  qs.resize(count);
  for (u32 i = 0; i < count; i++) {
    auto t = st.tables.find(tables[i]);
    auto s = st.seats.find(seats[i]);
    if (t == st.tables.end() || s == st.seats.end())
      return fail(c, IG_ERR_HANDLE, "query %u names an unknown table or key seat", i);
    if (t->second.server != server || s->second.server != server)
      return fail(c, IG_ERR_SHAPE, "table or key seat belongs to another parameter set");
    qs[i].values = t->second.values;
    qs[i].step1_R = t->second.step1;
    qs[i].rows = t->second.rows;
    qs[i].seat = s->second.words;
    qs[i].reserved = 0;
  }
  return IG_OK;
}

int ig_sm_respond_batch(ig_ctx* c, uint64_t server, uint32_t count, const uint64_t* tables, const uint64_t* seats,
                        const uint8_t* seeds, const uint32_t* bodies, uint32_t* mask_out, uint32_t* body_out) {
  if (!c) return IG_ERR_ARG;
  if (!count || !tables || !seats || !seeds || !bodies || !mask_out || !body_out)
    return fail(c, IG_ERR_ARG, "ig_sm_respond_batch: empty batch or null buffer");
  // Lanes (ig_ctx_set_lanes) let several caller threads have batches in flight: the call
  // holds its lane until its results are copied out, the context lock only to launch.
  igint::HostCall hc;
  igint::host_call_begin(c, hc);
  std::unique_lock<std::mutex> lk(igint::mutex(c));
  cudaSetDevice(igint::device(c));
  SmState& st = state(c);
  ServerObj* o;
  std::vector<SmQueryDev> qs;
  int rc = sm_prepare(c, st, server, count, tables, seats, &o, qs);
  if (rc) return rc;
  const size_t d = o->n, nb = o->dev.nb;
  for (size_t k = 0; k < (size_t)count * d; k++)
    if (bodies[k] >= o->q) return fail(c, IG_ERR_SHAPE, "query %zu does not fit the set", k / d);
  void *dq, *dseeds, *dbodies, *dfold, *dmask, *dbody, *dstatus;
  auto lane_scratch = [&](const char* name, size_t bytes, void** out) {
    char full[48];
    snprintf(full, sizeof full, "%s%u", name, hc.k);
    return igint::scratch(c, full, bytes, out);
  };
  if ((rc = lane_scratch("sm_q", count * sizeof(SmQueryDev), &dq)) ||
      (rc = lane_scratch("sm_seeds", count * 32, &dseeds)) ||
      (rc = lane_scratch("sm_bodies", count * d * 4, &dbodies)) ||
      (rc = lane_scratch("sm_fold", count * nb * 8, &dfold)) ||
      (rc = lane_scratch("sm_mask", count * d * 4, &dmask)) ||
      (rc = lane_scratch("sm_body", count * nb * 4, &dbody)) ||
      (rc = lane_scratch("sm_status", count * 4, &dstatus)))
    return rc;
  // Pinned landing buffer: status words, mask, body.
  const size_t st_bytes = ((size_t)count * 4 + 15) & ~(size_t)15;
  void* pin;
  if ((rc = igint::host_call_pinned(c, hc, st_bytes + (size_t)count * (d + nb) * 4, &pin))) return rc;
  u32* h_status = (u32*)pin;
  u32* h_mask = (u32*)((uint8_t*)pin + st_bytes);
  u32* h_body = h_mask + (size_t)count * d;
  for (u32 i = 0; i < count; i++) {
    qs[i].seed = (const u32*)((const uint8_t*)dseeds + (size_t)i * 32);
    qs[i].body = (const u32*)dbodies + (size_t)i * d;
  }
  cudaStream_t s = igint::host_call_stream(c, hc);
  if ((rc = igint::stage_h2d(c, dq, qs.data(), count * sizeof(SmQueryDev))) ||
      (rc = igint::stage_h2d(c, dseeds, seeds, (size_t)count * 32)) ||
      (rc = igint::stage_h2d(c, dbodies, bodies, (size_t)count * d * 4)) || (rc = igint::host_call_enter(c, hc)))
    return rc;
  SM_CUDA(c, cudaMemsetAsync(dstatus, 0, count * 4, s));
  SM_CUDA(c, igsmk::body_fold(o->dev, (const SmQueryDev*)dq, count, (i64*)dfold, s));
  SM_CUDA(c, igsmk::respond(o->dev, (const SmQueryDev*)dq, count, (const i64*)dfold, (u32*)dmask, (u32*)dbody,
                            (u32*)dstatus, s));
  igint::add_launches(c, 2);
  SM_CUDA(c, cudaMemcpyAsync(h_status, dstatus, count * 4, cudaMemcpyDeviceToHost, s));
  SM_CUDA(c, cudaMemcpyAsync(h_mask, dmask, (size_t)count * d * 4, cudaMemcpyDeviceToHost, s));
  SM_CUDA(c, cudaMemcpyAsync(h_body, dbody, (size_t)count * nb * 4, cudaMemcpyDeviceToHost, s));
  if ((rc = igint::host_call_launched(c, hc))) return rc;
  lk.unlock();
  if ((rc = igint::host_call_wait(c, hc))) return rc;
  for (u32 i = 0; i < count; i++)
    if (h_status[i]) return fail(c, IG_ERR_DEVICE, "query %u: respond kernel status %u", i, h_status[i]);
  memcpy(mask_out, h_mask, (size_t)count * d * 4);
  memcpy(body_out, h_body, (size_t)count * nb * 4);
  return IG_OK;
}

int ig_sm_respond_batch_device(ig_ctx* c, uint64_t server, uint32_t count, const uint64_t* tables,
                               const uint64_t* seats, const uint8_t* d_seeds, const uint32_t* d_bodies,
                               uint32_t* d_mask_out, uint32_t* d_body_out, uint32_t* d_status) {
  if (!c) return IG_ERR_ARG;
  if (!count || !tables || !seats || !d_seeds || !d_bodies || !d_mask_out || !d_body_out || !d_status)
    return fail(c, IG_ERR_ARG, "ig_sm_respond_batch_device: empty batch or null buffer");
  std::lock_guard<std::mutex> lk(igint::mutex(c));
  cudaSetDevice(igint::device(c));
  SmState& st = state(c);
  ServerObj* o;
  std::vector<SmQueryDev> qs;
  int rc = sm_prepare(c, st, server, count, tables, seats, &o, qs);
  if (rc) return rc;
  const size_t d = o->n, nb = o->dev.nb;
  // Lanes (ig_ctx_set_lanes) apply here as on the InspiRING device path: consecutive
  // batches rotate over streams with their own scratch.
  cudaStream_t s;
  int lane;
  if ((rc = igint::lane_acquire(c, &s, &lane))) return rc;
  char qname[32], fname[32];
  snprintf(qname, sizeof qname, "smd_q%d", lane);
  snprintf(fname, sizeof fname, "smd_fold%d", lane);
  void *dq, *dfold;
  if ((rc = igint::scratch(c, qname, count * sizeof(SmQueryDev), &dq)) ||
      (rc = igint::scratch(c, fname, count * nb * 8, &dfold)))
    return rc;
  for (u32 i = 0; i < count; i++) {
    qs[i].seed = (const u32*)(d_seeds + (size_t)i * 32);
    qs[i].body = d_bodies + (size_t)i * d;
  }
  if ((rc = igint::stage_h2d(c, dq, qs.data(), count * sizeof(SmQueryDev)))) return rc;
  if ((rc = igint::lane_enter(c, lane))) return rc;
  SM_CUDA(c, cudaMemsetAsync(d_status, 0, count * 4, s));
  SM_CUDA(c, igsmk::body_fold(o->dev, (const SmQueryDev*)dq, count, (i64*)dfold, s));
  SM_CUDA(c, igsmk::respond(o->dev, (const SmQueryDev*)dq, count, (const i64*)dfold, d_mask_out, d_body_out, d_status,
                            s));
  igint::add_launches(c, 2);
  return igint::lane_release(c, lane);
}

// Response::to_bytes (special_modulus/wire.rs:120-125): mask then body, each packed at q's
// bit width, little-endian bit order.
int ig_sm_response_encode(const uint32_t* mask, uint32_t n, const uint32_t* body, uint32_t nb, uint64_t q,
                          uint8_t* out, size_t cap, size_t* len_out) {
  if (!mask || !body || !len_out || q < 2 || q > (1ULL << 32)) return IG_ERR_ARG;
  const unsigned bits = 64 - __builtin_clzll(q - 1);
  const size_t ma = ((size_t)n * bits + 7) / 8, mb = ((size_t)nb * bits + 7) / 8;
  std::vector<uint8_t> w(ma + mb, 0);
  for (int part = 0; part < 2; part++) {
    const uint32_t* v = part ? body : mask;
    const size_t count = part ? nb : n, base = part ? ma : 0, nbytes = part ? mb : ma;
    for (size_t i = 0; i < count; i++) {
      if (v[i] >= q) return IG_ERR_SHAPE;
      const size_t bit = i * bits;
      const u64 val = (u64)v[i] << (bit % 8);
      for (size_t k = 0; k < 8 && bit / 8 + k < nbytes; k++) w[base + bit / 8 + k] |= (uint8_t)(val >> (8 * k));
    }
  }
  *len_out = w.size();
  if (out) memcpy(out, w.data(), w.size() < cap ? w.size() : cap);
  return IG_OK;
}

}  // extern "C"
