// TEST INFRASTRUCTURE — the CPU oracle for the special_modulus respond path.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load this code, as the
// checker and the timed CPU baseline; the product library never links it.
//
// A from-scratch C++ restatement of raven-inspire's src/special_modulus/: arith.rs (Prime32,
// Ntt32), mod.rs (Params, Ring, key mask, lifts, nibbles), server.rs (seat, table,
// respond), client.rs (from_seed, key, query, decode) and wire.rs (packed byte forms).
// Pinned by the PINNED digests of tests/special_modulus_kat.rs:376-380 (key, query and
// response bytes of Client::from_seed([42; 32]) against cells from seed_from_u64(42)).
#include <omp.h>

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "oracle_rng.hpp"

namespace orc_sm {
using namespace orc;
typedef uint32_t u32;

// Prime32 (arith.rs:13-102): Montgomery with R = 2^32, words fully reduced.
struct Prime32 {
  u32 q, neg_qinv, r2;
  explicit Prime32(u64 qq = 3) {
    q = (u32)qq;
    u32 inv = 1;
    for (int i = 0; i < 5; i++) inv *= 2u - q * inv;
    neg_qinv = 0u - inv;
    r2 = (u32)((((u128)1) << 64) % qq);
  }
  u32 csub(u32 x) const {
    u32 r = x - q;
    return r + (q & (0u - (r >> 31)));
  }
  u32 add(u32 a, u32 b) const { return csub(a + b); }
  u32 sub(u32 a, u32 b) const { return csub(a + q - b); }
  u32 mont(u32 a, u32 b) const {
    u64 t = (u64)a * b;
    u32 m = (u32)t * neg_qinv;
    return csub((u32)((t + (u64)m * q) >> 32));
  }
  u32 to_mont(u32 a) const { return mont(a, r2); }
  u32 small(i64 x) const { return (u32)x + (q & (u32)(x >> 63)); }
  u32 residue(i64 x) const {
    i64 r = x % (i64)q;
    if (r < 0) r += q;
    return (u32)r;
  }
  i64 centred(u32 x) const { return x > (q >> 1) ? (i64)x - (i64)q : (i64)x; }
  u32 pow(u64 b, u64 e) const {
    u64 acc = 1, qq = q;
    b %= qq;
    while (e) {
      if (e & 1) acc = acc * b % qq;
      b = b * b % qq;
      e >>= 1;
    }
    return (u32)acc;
  }
};

static size_t bitrev(size_t x, unsigned bits) {
  size_t r = 0;
  for (unsigned i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}

// Ntt32 (arith.rs:109-251): standard-form in and out, Montgomery-form twiddles.
struct Ntt32 {
  size_t n;
  Prime32 p;
  std::vector<u32> fwd, inv;
  u32 n_inv, last;
  Ntt32() : n(0) {}
  Ntt32(size_t nn, u64 q) : n(nn), p(q) {
    u32 psi = 0;
    for (u64 g = 2; g < q; g++) {
      u32 c = p.pow(g, (q - 1) / (2 * n));
      if (p.pow(c, n) == p.q - 1) {
        psi = c;
        break;
      }
    }
    u32 psi_inv = p.pow(psi, 2 * n - 1);
    unsigned bits = 0;
    while ((size_t(1) << bits) < n) bits++;
    std::vector<std::pair<u32, u32>> powers(n);
    u64 a = 1, b = 1;
    for (size_t k = 0; k < n; k++) {
      powers[k] = {(u32)a, (u32)b};
      a = a * psi % q;
      b = b * psi_inv % q;
    }
    fwd.resize(n);
    inv.resize(n);
    for (size_t k = 0; k < n; k++) {
      fwd[k] = p.to_mont(powers[bitrev(k, bits)].first);
      inv[k] = p.to_mont(powers[bitrev(k, bits)].second);
    }
    n_inv = p.to_mont(p.pow(n, q - 2));
    last = p.mont(inv[1], n_inv);
  }
  void forward(u32* a) const {
    size_t t = n;
    for (size_t m = 1; m < n; m <<= 1) {
      t >>= 1;
      for (size_t i = 0; i < m; i++) {
        u32 s = fwd[m + i];
        for (size_t j = 2 * i * t; j < 2 * i * t + t; j++) {
          u32 u = a[j], v = p.mont(a[j + t], s);
          a[j] = p.add(u, v);
          a[j + t] = p.sub(u, v);
        }
      }
    }
  }
  void inverse(u32* a) const {
    size_t t = 1, m = n;
    while (m > 2) {
      size_t h = m >> 1;
      for (size_t i = 0; i < h; i++) {
        u32 s = inv[h + i];
        for (size_t j = 2 * i * t; j < 2 * i * t + t; j++) {
          u32 u = a[j], v = a[j + t];
          a[j] = p.add(u, v);
          a[j + t] = p.mont(u + p.q - v, s);
        }
      }
      t <<= 1;
      m = h;
    }
    for (size_t j = 0; j < t; j++) {
      u32 u = a[j], v = a[j + t];
      a[j] = p.mont(u + v, n_inv);
      a[j + t] = p.mont(u + p.q - v, last);
    }
  }
  // automorphism_tables (arith.rs:288-323): table[k] = slot whose root is root_k^t.
  std::vector<uint16_t> table(size_t t) const {
    std::vector<u32> x(n, 0);
    x[1] = 1;
    forward(x.data());
    std::vector<std::pair<u32, uint16_t>> slot_of;
    for (size_t k = 0; k < n; k++) slot_of.push_back({x[k], (uint16_t)k});
    std::sort(slot_of.begin(), slot_of.end());
    std::vector<u32> mono(n, 0);
    size_t e = t % (2 * n);
    if (e < n)
      mono[e] = 1;
    else
      mono[e - n] = p.q - 1;
    forward(mono.data());
    std::vector<uint16_t> out(n);
    for (size_t k = 0; k < n; k++) {
      auto it = std::lower_bound(slot_of.begin(), slot_of.end(), std::make_pair(mono[k], (uint16_t)0));
      if (it == slot_of.end() || it->first != mono[k]) throw std::runtime_error("tau leaves the evaluation points");
      out[k] = it->second;
    }
    return out;
  }
};

// Params::ring2048_cell256 (mod.rs:84-95).
struct Params {
  size_t d = 2048, gamma = 512;
  u64 q = 536813569, p = 2147389441;
  size_t cell_bytes = 256, record_bytes = 246;
  double sigma = 6.4;
  size_t body() const { return 2 * record_bytes; }
};

static const u64 KEY_MASK_STREAM = 0x6b6579206d61736bULL;  // b"key mask", big-endian
static const u64 KEY_SEED_STREAM = 0x6b65792073656564ULL;  // b"key seed", big-endian
static const u32 PLAINTEXT = 16;

// expand_uniform (mod.rs:225-237): rejection below floor(2^64 / m) * m, then u mod m.
static void expand_uniform(ChaCha20Rng& rng, u64 m, u32* out, size_t count) {
  const u64 zone = (UINT64_MAX / m) * m;
  for (size_t i = 0; i < count; i++) {
    for (;;) {
      u64 u = rng.next_u64();
      if (u < zone) {
        out[i] = (u32)(u % m);
        break;
      }
    }
  }
}

static std::vector<i64> tau_signed(const std::vector<i64>& v, size_t t) {
  size_t d = v.size();
  std::vector<i64> out(d, 0);
  for (size_t i = 0; i < d; i++) {
    size_t k = (t * i) % (2 * d);
    if (k < d)
      out[k] = v[i];
    else
      out[k - d] = -v[i];
  }
  return out;
}

// Ring (mod.rs:256-362).
struct Ring {
  Params P;
  Ntt32 lq, lp;
  size_t g;
  u32 delta, p_mod_q, neg_off, p_over_q, p_inv;
  std::vector<std::vector<uint16_t>> tables;
  explicit Ring(const Params& params, bool with_tables) : P(params), lq(params.d, params.q), lp(params.d, params.p) {
    g = 2 * P.d / P.gamma + 1;
    if (with_tables) {
      size_t v = 1;
      for (size_t i = 0; i < P.gamma; i++) {
        auto tq = lq.table(v), tp = lp.table(v);
        if (tq != tp) throw std::runtime_error("the two limbs disagree on an automorphism");
        tables.push_back(tq);
        v = v * g % (2 * P.d);
      }
    }
    delta = (u32)(P.q / PLAINTEXT);
    p_mod_q = (u32)(P.p % P.q);
    neg_off = (u32)((P.q - P.p % P.q) % P.q);
    p_over_q = (u32)(P.p / P.q);
    p_inv = lq.p.to_mont(lq.p.pow(P.p % P.q, P.q - 2));
  }
  void key_mask(const uint8_t seed[32], std::vector<u32>& w_q, std::vector<u32>& w_p) const {
    ChaCha20Rng rng = ChaCha20Rng::from_seed(seed);
    rng.set_stream(KEY_MASK_STREAM);
    w_q.assign(P.d, 0);
    w_p.assign(P.d, 0);
    expand_uniform(rng, P.q, w_q.data(), P.d);
    expand_uniform(rng, P.p, w_p.data(), P.d);
    lq.forward(w_q.data());
    lp.forward(w_p.data());
    for (auto& x : w_q) x = lq.p.to_mont(x);
    for (auto& x : w_p) x = lp.p.to_mont(x);
  }
  u32 p_to_q_centred(u32 r) const {
    u32 base = r;
    for (u32 k = 0; k < p_over_q; k++) base = lq.p.csub(base);
    return r > lp.p.q / 2 ? lq.p.add(base, neg_off) : base;
  }
  u32 q_to_p_centred(u32 c) const { return c > lq.p.q / 2 ? c + (lp.p.q - lq.p.q) : c; }
  u32 mod_down(u32 xq, u32 xp) const { return lq.p.mont(lq.p.sub(xq, p_to_q_centred(xp)), p_inv); }
};

static void nibbles(const uint8_t* cell, size_t nbytes, int8_t* out) {
  for (size_t i = 0; i < nbytes; i++) {
    uint8_t b = cell[i];
    out[2 * i] = (int8_t)((int8_t)(uint8_t)(b << 4) >> 4);
    out[2 * i + 1] = (int8_t)((int8_t)b >> 4);
  }
}

// Bit-packed coefficients at m's width, little-endian bit order (poly.rs:166-225).
static void pack(const u32* v, size_t count, u64 m, std::vector<uint8_t>& out) {
  unsigned bits = 64 - clz64(m - 1);
  size_t nbytes = (count * bits + 7) / 8, base = out.size();
  out.resize(base + nbytes, 0);
  for (size_t i = 0; i < count; i++) {
    size_t bit = i * bits;
    u64 val = (u64)v[i] << (bit % 8);
    for (size_t k = 0; k < 8 && bit / 8 + k < nbytes; k++) out[base + bit / 8 + k] |= (uint8_t)(val >> (8 * k));
  }
}

struct Key {
  uint8_t mask_seed[32];
  std::vector<u32> q, p;
};
struct Query {
  uint8_t seed[32];
  std::vector<u32> body;
};
struct Response {
  std::vector<u32> mask, body;
};

struct Client {
  Ring ring;
  std::vector<u32> s_q;  // NTT of the secret, R-form
  Key key;
  GaussianSampler noise;
  ChaCha20Rng seeds;
  Client(const Params& P, const uint8_t seed[32]) : ring(P, false) {
    // Client::from_seed (client.rs:137-143) and drawn (148-153).
    noise.build(P.sigma, ChaCha20Rng::from_seed(seed));
    seeds = ChaCha20Rng::from_seed(seed);
    seeds.set_stream(1);
    std::vector<i64> secret(P.d), key_error(P.d);
    for (auto& x : secret) x = noise.sample();
    for (auto& x : key_error) x = noise.sample();
    ChaCha20Rng ks = ChaCha20Rng::from_seed(seed);
    ks.set_stream(KEY_SEED_STREAM);
    ks.fill_bytes(key.mask_seed, 32);
    build(secret, key_error);
  }
  // Client::build (client.rs:181-243).
  void build(const std::vector<i64>& secret, const std::vector<i64>& key_error) {
    const Params& P = ring.P;
    const Prime32 &pq = ring.lq.p, &pp = ring.lp.p;
    std::vector<u32> w_q, w_p;
    ring.key_mask(key.mask_seed, w_q, w_p);
    std::vector<u32> sq(P.d), sp(P.d);
    for (size_t k = 0; k < P.d; k++) {
      sq[k] = pq.small(secret[k]);
      sp[k] = pp.small(secret[k]);
    }
    ring.lq.forward(sq.data());
    ring.lp.forward(sp.data());
    std::vector<u32> swq(P.d), swp(P.d);
    for (size_t k = 0; k < P.d; k++) {
      swq[k] = pq.mont(sq[k], w_q[k]);
      swp[k] = pp.mont(sp[k], w_p[k]);
    }
    ring.lq.inverse(swq.data());
    ring.lp.inverse(swp.data());
    auto ts = tau_signed(secret, ring.g);
    u32 pmq = pq.to_mont(ring.p_mod_q);
    key.q.resize(P.d);
    key.p.resize(P.d);
    for (size_t k = 0; k < P.d; k++) {
      u32 lead = pq.mont(pq.small(ts[k]), pmq);
      key.q[k] = pq.add(pq.sub(lead, swq[k]), pq.small(key_error[k]));
      key.p[k] = pp.sub(pp.small(key_error[k]), swp[k]);
    }
    s_q = sq;
    for (auto& x : s_q) x = pq.to_mont(x);
  }
  Query query(size_t row) {
    Query qy;
    seeds.fill_bytes(qy.seed, 32);
    std::vector<i64> err(ring.P.d);
    for (auto& x : err) x = noise.sample();
    query_with(row, qy, err);
    return qy;
  }
  // Client::query_with (client.rs:279-313).
  void query_with(size_t row, Query& qy, const std::vector<i64>& err) const {
    const Params& P = ring.P;
    const Prime32& pq = ring.lq.p;
    std::vector<u32> a(P.d);
    ChaCha20Rng r = ChaCha20Rng::from_seed(qy.seed);
    expand_uniform(r, P.q, a.data(), P.d);
    ring.lq.forward(a.data());
    for (size_t k = 0; k < P.d; k++) a[k] = pq.mont(a[k], s_q[k]);
    ring.lq.inverse(a.data());
    size_t target = (P.d - row) & (P.d - 1);
    u32 message = row == 0 ? ring.delta : pq.q - ring.delta;
    qy.body.resize(P.d);
    for (size_t k = 0; k < P.d; k++) qy.body[k] = pq.add(pq.sub(pq.small(err[k]), a[k]), k == target ? message : 0);
  }
  // Client::decode (client.rs:315-345): phase = mask * s + body, rounded to nibbles.
  std::vector<uint8_t> decode(const Response& r) const {
    const Params& P = ring.P;
    const Prime32& pq = ring.lq.p;
    std::vector<u32> ph = r.mask;
    ring.lq.forward(ph.data());
    for (size_t k = 0; k < P.d; k++) ph[k] = pq.mont(ph[k], s_q[k]);
    ring.lq.inverse(ph.data());
    std::vector<uint8_t> out;
    u64 delta = ring.delta, half = delta / 2;
    auto nib = [&](u32 x) { return (uint8_t)(((u64)x + half) / delta & (PLAINTEXT - 1)); };
    for (size_t k = 0; k + 1 < r.body.size(); k += 2) {
      u32 a = pq.add(ph[k], r.body[k]), b = pq.add(ph[k + 1], r.body[k + 1]);
      out.push_back((uint8_t)(nib(a) | (nib(b) << 4)));
    }
    return out;
  }
};

struct Seat {
  std::vector<u32> q, p, w_q, w_p;
};
struct Table {
  std::vector<u32> step1;   // gamma x d, R-form
  std::vector<int8_t> values;  // d x gamma
  size_t rows;
};

struct Server {
  Ring ring;
  explicit Server(const Params& P) : ring(P, true) {}
  // Server::seat (server.rs:177-203).
  Seat seat(const Key& key) const {
    Seat s;
    s.q = key.q;
    s.p = key.p;
    ring.lq.forward(s.q.data());
    ring.lp.forward(s.p.data());
    for (auto& x : s.q) x = ring.lq.p.to_mont(x);
    for (auto& x : s.p) x = ring.lp.p.to_mont(x);
    ring.key_mask(key.mask_seed, s.w_q, s.w_p);
    return s;
  }
  // Server::table (server.rs:211-249) with step1_row_impl (331-383).
  Table table(const uint8_t* cells, size_t nbytes) const {
    const Params& P = ring.P;
    size_t d = P.d, gamma = P.gamma;
    Table t;
    t.rows = nbytes / P.cell_bytes;
    t.values.assign(d * gamma, 0);
    for (size_t m = 0; m < t.rows; m++) nibbles(cells + m * P.cell_bytes, P.cell_bytes, &t.values[m * gamma]);
    std::vector<int8_t> columns(gamma * d, 0);
    for (size_t m = 0; m < t.rows; m++)
      for (size_t j = 0; j < gamma; j++) columns[j * d + m] = t.values[m * gamma + j];
    t.step1.assign(gamma * d, 0);
    const Prime32& pq = ring.lq.p;
    u32 inv_gamma = pq.to_mont(pq.to_mont(pq.pow(gamma, P.q - 2)));
#pragma omp parallel for schedule(dynamic, 4)
    for (long i = 0; i < (long)gamma; i++) {
      size_t two_d = 2 * d, e = 1, base = ring.g % two_d, k = (d - i) % d;
      while (k) {
        if (k & 1) e = e * base % two_d;
        base = base * base % two_d;
        k >>= 1;
      }
      std::vector<int32_t> acc(d, 0);
      for (size_t j = 0; j < gamma; j++) {
        const int8_t* col = &columns[j * d];
        size_t kk = (j * e) % two_d;
        bool flip = kk >= d;
        size_t sh = flip ? kk - d : kk;
        // acc[(sh + m) mod d] += +/- col[m], negated again on wrap (X^d = -1).
        for (size_t m = 0; m < d; m++) {
          size_t pos = sh + m;
          int32_t v = col[m];
          bool neg = flip ^ (pos >= d);
          acc[pos % d] += neg ? -v : v;
        }
      }
      std::vector<u32> poly(d);
      for (size_t m = 0; m < d; m++) poly[m] = pq.small(acc[m]);
      ring.lq.forward(poly.data());
      for (size_t m = 0; m < d; m++) t.step1[i * d + m] = pq.mont(poly[ring.tables[i][m]], inv_gamma);
    }
    return t;
  }
  // respond_impl (server.rs:386-498).
  Response respond(const Table& t, const Seat& s, const Query& qy) const {
    const Params& P = ring.P;
    size_t d = P.d, gamma = P.gamma, nb = P.body();
    const Prime32 &pq = ring.lq.p, &pp = ring.lp.p;
    std::vector<i64> fold(nb, 0);
    for (size_t m = 0; m < t.rows; m++) {
      i64 c = m == 0 ? pq.centred(qy.body[0]) : -pq.centred(qy.body[d - m]);
      for (size_t k = 0; k < nb; k++) fold[k] += c * (i64)t.values[m * gamma + k];
    }
    std::vector<u32> a(d);
    ChaCha20Rng r = ChaCha20Rng::from_seed(qy.seed);
    expand_uniform(r, P.q, a.data(), d);
    ring.lq.forward(a.data());
    std::vector<u32> cur(d), next(d), tp(d), cp(d), rq(d), acc_q(d, 0), acc_p(d, 0);
    for (size_t k = 0; k < d; k++) cur[k] = pq.mont(a[ring.tables[gamma - 1][k]], t.step1[(gamma - 1) * d + k]);
    for (long i = (long)gamma - 2; i >= 0; i--) {
      const auto& tab = ring.tables[i];
      tp = cur;
      ring.lq.inverse(tp.data());
      for (auto& x : tp) x = ring.q_to_p_centred(x);
      ring.lp.forward(tp.data());
      for (size_t k = 0; k < d; k++) cp[k] = pp.mont(tp[k], s.w_p[tab[k]]);
      ring.lp.inverse(cp.data());
      for (size_t k = 0; k < d; k++) rq[k] = ring.p_to_q_centred(cp[k]);
      ring.lq.forward(rq.data());
      const u32* s1 = &t.step1[i * d];
      for (size_t k = 0; k < d; k++) {
        size_t src = tab[k];
        u32 cq = pq.mont(cur[k], s.w_q[src]);
        next[k] = pq.add(pq.mont(a[src], s1[k]), pq.mont(pq.sub(cq, rq[k]), ring.p_inv));
        acc_q[k] = pq.add(acc_q[k], pq.mont(cur[k], s.q[src]));
        acc_p[k] = pp.add(acc_p[k], pp.mont(tp[k], s.p[src]));
      }
      std::swap(cur, next);
    }
    Response out;
    out.mask = cur;
    ring.lq.inverse(out.mask.data());
    ring.lq.inverse(acc_q.data());
    ring.lp.inverse(acc_p.data());
    out.body.resize(nb);
    for (size_t k = 0; k < nb; k++) out.body[k] = pq.add(ring.mod_down(acc_q[k], acc_p[k]), pq.residue(fold[k]));
    return out;
  }
};

static std::vector<uint8_t> key_bytes(const Params& P, const Key& k) {
  std::vector<uint8_t> out = {0, 2};  // key-mask version 2, big-endian
  out.insert(out.end(), k.mask_seed, k.mask_seed + 32);
  pack(k.q.data(), k.q.size(), P.q, out);
  pack(k.p.data(), k.p.size(), P.p, out);
  return out;
}
static std::vector<uint8_t> query_bytes(const Params& P, const Query& q) {
  std::vector<uint8_t> out(q.seed, q.seed + 32);
  pack(q.body.data(), q.body.size(), P.q, out);
  return out;
}
static std::vector<uint8_t> response_bytes(const Params& P, const Response& r) {
  std::vector<uint8_t> out;
  pack(r.mask.data(), r.mask.size(), P.q, out);
  pack(r.body.data(), r.body.size(), P.q, out);
  return out;
}

}  // namespace orc_sm

// =======================================================================================
using namespace orc_sm;

extern "C" {

void* orc_sm_server_new() { return new Server(Params()); }
void orc_sm_server_free(void* s) { delete (Server*)s; }
// The same parameter set over another ciphertext prime q (Params::validate's rules).
void* orc_sm_server_new_q(uint64_t q) {
  Params P;
  P.q = q;
  return new Server(P);
}

void* orc_sm_client_new(const uint8_t* seed) { return new Client(Params(), seed); }
void* orc_sm_client_new_q(const uint8_t* seed, uint64_t q) {
  Params P;
  P.q = q;
  return new Client(P, seed);
}
void orc_sm_client_free(void* c) { delete (Client*)c; }

// Key parts: mask_seed (32 B), q limb and p limb (d words each, coefficient form).
void orc_sm_client_key(void* cv, uint8_t* mask_seed, uint32_t* kq, uint32_t* kp) {
  auto* c = (Client*)cv;
  memcpy(mask_seed, c->key.mask_seed, 32);
  memcpy(kq, c->key.q.data(), c->key.q.size() * 4);
  memcpy(kp, c->key.p.data(), c->key.p.size() * 4);
}
uint64_t orc_sm_client_key_bytes(void* cv, uint8_t* out, uint64_t cap) {
  auto v = key_bytes(((Client*)cv)->ring.P, ((Client*)cv)->key);
  if (out) memcpy(out, v.data(), std::min<uint64_t>(cap, v.size()));
  return v.size();
}
void orc_sm_client_query(void* cv, uint64_t row, uint8_t* seed, uint32_t* body) {
  auto q = ((Client*)cv)->query(row);
  memcpy(seed, q.seed, 32);
  memcpy(body, q.body.data(), q.body.size() * 4);
}
// Decodes (mask d words, body 2*record words) to the record bytes; returns their count.
uint64_t orc_sm_client_decode(void* cv, const uint32_t* mask, const uint32_t* body, uint8_t* out) {
  auto* c = (Client*)cv;
  Response r;
  r.mask.assign(mask, mask + c->ring.P.d);
  r.body.assign(body, body + c->ring.P.body());
  auto v = c->decode(r);
  memcpy(out, v.data(), v.size());
  return v.size();
}

void* orc_sm_table_new(void* sv, const uint8_t* cells, uint64_t nbytes) {
  return new Table(((Server*)sv)->table(cells, nbytes));
}
void orc_sm_table_free(void* t) { delete (Table*)t; }
void orc_sm_table_step1(void* tv, uint32_t* out) {
  auto* t = (Table*)tv;
  memcpy(out, t->step1.data(), t->step1.size() * 4);
}

void* orc_sm_seat_new(void* sv, const uint8_t* mask_seed, const uint32_t* kq, const uint32_t* kp) {
  auto* s = (Server*)sv;
  Key k;
  memcpy(k.mask_seed, mask_seed, 32);
  k.q.assign(kq, kq + s->ring.P.d);
  k.p.assign(kp, kp + s->ring.P.d);
  return new Seat(s->seat(k));
}
void orc_sm_seat_free(void* s) { delete (Seat*)s; }

void orc_sm_respond(void* sv, void* tv, void* seatv, const uint8_t* seed, const uint32_t* body, uint32_t* mask_out,
                    uint32_t* body_out) {
  auto* s = (Server*)sv;
  Query q;
  memcpy(q.seed, seed, 32);
  q.body.assign(body, body + s->ring.P.d);
  Response r = s->respond(*(Table*)tv, *(Seat*)seatv, q);
  memcpy(mask_out, r.mask.data(), r.mask.size() * 4);
  memcpy(body_out, r.body.data(), r.body.size() * 4);
}

uint64_t orc_sm_query_bytes(const uint8_t* seed, const uint32_t* body, uint8_t* out, uint64_t cap) {
  Params P;
  Query q;
  memcpy(q.seed, seed, 32);
  q.body.assign(body, body + P.d);
  auto v = query_bytes(P, q);
  if (out) memcpy(out, v.data(), std::min<uint64_t>(cap, v.size()));
  return v.size();
}
uint64_t orc_sm_response_bytes(const uint32_t* mask, const uint32_t* body, uint8_t* out, uint64_t cap) {
  Params P;
  Response r;
  r.mask.assign(mask, mask + P.d);
  r.body.assign(body, body + P.body());
  auto v = response_bytes(P, r);
  if (out) memcpy(out, v.data(), std::min<uint64_t>(cap, v.size()));
  return v.size();
}

// Cells of the KAT: `rows` cells, each with fill_bytes of record_bytes from
// ChaCha20Rng::seed_from_u64(seed), bytes past the record zero
// (tests/special_modulus_kat.rs:37-46).
void orc_sm_kat_cells(uint64_t seed, uint64_t rows, uint8_t* out) {
  Params P;
  ChaCha20Rng rng = ChaCha20Rng::seed_from_u64(seed);
  memset(out, 0, rows * P.cell_bytes);
  for (uint64_t m = 0; m < rows; m++) rng.fill_bytes(out + m * P.cell_bytes, P.record_bytes);
}

}  // extern "C"
