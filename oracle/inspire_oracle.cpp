// TEST INFRASTRUCTURE — the CPU oracle for the InspiRING respond path.
//
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may
// load this library, as the checker and as the timed CPU baseline. The product library
// (inspire-rs_gb300/) never links or calls it.
//
// A from-scratch C++ restatement of the reference crate raven-inspire (hisoka-io/inspire-rs)
// for single-prime parameter sets. File:line citations point into the reference:
//   math/ntt.rs            NTT (Montgomery R=2^64, bit-reversed twiddle ladder, CT/GS)
//   math/poly.rs           ring ops, seed expansion, tight coefficient codec
//   inspiring/inspiring2.rs  PackParams, offline keys, rotation sums, backward recursion,
//                            online gather, client key body
//   inspiring/shard_store.rs packing store: step-1 sums, tags, scan + b fold, gather
//   pir/respond.rs         pack_shard (both branches), ServerResponse wire
//   pir/mod_switch.rs      response mod switch
//   pir/setup.rs, pir/session.rs, rgsw/types.rs, pir/encode_db.rs, params.rs
//                          client-side regeneration of the KAT inputs
// Parity pins: tests/fixtures/respond_byte_identity_d256.bin (FNV 0x796a80ca60d31a52) and
// the single-prime lines of tests/fixtures/packing_seat_response_kat.txt, replayed by
// tests/test_oracle_pins.py.
#include <omp.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "oracle_rng.hpp"

namespace orc {

typedef std::vector<u64> Vec;

static inline u64 mulmod(u64 a, u64 b, u64 q) { return (u64)((u128)a * b % q); }
static inline u64 powmod(u64 b, u64 e, u64 m) {
  u64 r = 1;
  b %= m;
  while (e) {
    if (e & 1) r = mulmod(r, b, m);
    b = mulmod(b, b, m);
    e >>= 1;
  }
  return r;
}
static inline u64 addmod(u64 a, u64 b, u64 q) {
  u64 s = a + b;
  return s >= q ? s - q : s;
}
static inline u64 submod(u64 a, u64 b, u64 q) { return a >= b ? a - b : a + q - b; }

// Extended-gcd inverse (inspiring2.rs:1853-1860); 0 when none exists.
static u64 mod_inverse(u64 a, u64 m) {
  __int128 t = 0, nt = 1, r = m, nr = a % m;
  while (nr != 0) {
    __int128 qq = r / nr;
    __int128 tmp = t - qq * nt;
    t = nt;
    nt = tmp;
    tmp = r - qq * nr;
    r = nr;
    nr = tmp;
  }
  if (r != 1) return 0;
  if (t < 0) t += m;
  return (u64)t;
}

// ---------------------------------------------------------------------------------------
// NTT context: math/ntt.rs:35-146 (construction), 247-349 (butterflies), 688-694 (REDC),
// 743-752 (root search), 806-833 (Montgomery twiddle ladder).
struct Ntt {
  size_t n;
  unsigned logn;
  u64 q, qinv_neg, r2;
  Vec psi_pow, psi_inv_pow;
  u64 n_inv_mont;

  u64 mont(u64 a, u64 b) const {
    u128 ab = (u128)a * b;
    u64 m = (u64)ab * qinv_neg;
    u64 t = (u64)((ab + (u128)m * q) >> 64);
    return t >= q ? t - q : t;
  }
  u64 to_mont(u64 a) const { return mont(a, r2); }
  u64 from_mont(u64 a) const { return mont(a, 1); }

  static u64 find_root(u64 order, u64 q) {
    u64 e = (q - 1) / order;
    for (u64 g = 2; g < (1ull << 16) && g < q; g++) {
      u64 c = powmod(g, e, q);
      if (powmod(c, order, q) == 1 && powmod(c, order / 2, q) != 1) return c;
    }
    throw std::runtime_error("no primitive root");
  }

  Vec ladder(u64 psi_m) const {
    Vec f(n, 0);
    f[1] = to_mont(1);
    for (size_t m = 1; m < n; m++) {
      if ((m & (m - 1)) == 0) {
        size_t e = n / (2 * m);
        u64 p = to_mont(1);
        for (size_t k = 0; k < e; k++) p = mont(p, psi_m);
        f[m] = p;
      } else {
        f[m] = mont(f[m & (m - 1)], f[m & (~m + 1)]);
      }
    }
    return f;
  }

  Ntt(size_t n_, u64 q_) : n(n_), q(q_) {
    if ((q - 1) % (2 * n) != 0) throw std::runtime_error("q != 1 mod 2n");
    logn = 0;
    while ((size_t(1) << logn) < n) logn++;
    u64 y = 1;
    for (int i = 1; i < 64; i++) y |= (y * q) & (1ull << i);
    qinv_neg = (u64)0 - y;
    u64 rmod = (u64)(((u128)1 << 64) % q);
    r2 = mulmod(rmod, rmod, q);
    u64 psi = find_root(2 * n, q);
    psi_pow = ladder(to_mont(psi));
    psi_inv_pow = ladder(to_mont(powmod(psi, q - 2, q)));
    n_inv_mont = to_mont(powmod(n, q - 2, q));
  }

  // Forward: standard-form coefficients in, Montgomery-form evaluations out.
  void forward(u64* c) const {
    for (size_t i = 0; i < n; i++) c[i] = to_mont(c[i]);
    size_t t = n;
    for (size_t m = 1; m < n; m <<= 1) {
      t >>= 1;
      for (size_t i = 0; i < m; i++) {
        size_t j1 = 2 * i * t;
        u64 w = psi_pow[m + i];
        for (size_t j = j1; j < j1 + t; j++) {
          u64 u = c[j], v = mont(c[j + t], w);
          c[j] = addmod(u, v, q);
          c[j + t] = submod(u, v, q);
        }
      }
    }
  }
  // Inverse: Montgomery-form evaluations in, standard-form coefficients out.
  void inverse(u64* c) const {
    size_t t = 1;
    for (size_t m = n; m > 1;) {
      m >>= 1;
      for (size_t i = 0; i < m; i++) {
        size_t j2 = i * 2 * t;
        u64 w = psi_inv_pow[m + i];
        for (size_t j = j2; j < j2 + t; j++) {
          u64 u = c[j], v = c[j + t];
          c[j] = addmod(u, v, q);
          c[j + t] = mont(submod(u, v, q), w);
        }
      }
      t <<= 1;
    }
    for (size_t i = 0; i < n; i++) c[i] = mont(mont(c[i], n_inv_mont), 1);
  }
  Vec fwd(Vec v) const {
    forward(v.data());
    return v;
  }
  Vec inv(Vec v) const {
    inverse(v.data());
    return v;
  }
  // mul_acc_ntt_domain scalar loop (poly.rs:1032-1040).
  void mul_acc(u64* acc, const u64* a, const u64* b) const {
    for (size_t i = 0; i < n; i++) {
      u64 s = acc[i] + mont(a[i], b[i]);
      acc[i] = s >= q ? s - q : s;
    }
  }
  // Negacyclic product through the transform (poly.rs:900-928).
  Vec mul(const Vec& a, const Vec& b) const {
    Vec x = fwd(a), y = fwd(b), r(n);
    for (size_t i = 0; i < n; i++) r[i] = mont(x[i], y[i]);
    inverse(r.data());
    return r;
  }
};

// ---------------------------------------------------------------------------------------
// Parameter set (params.rs:137-196) restricted to one prime.
struct Params {
  size_t n;
  u64 q;
  u64 p;
  double sigma;
  u64 gadget_base;
  size_t gadget_len;  // packing_gadget_len (== query_gadget_len in every shipped set)
  bool approx;        // approximate_packing_gadget
  size_t dropped() const { return approx ? 1 : 0; }
  size_t key_rows() const { return gadget_len - dropped(); }
  u64 delta() const { return q / p; }
};

static u64 gadget_power(const Params& P, size_t i) {
  u128 r = 1;
  for (size_t k = 0; k < i; k++) r = r * P.gadget_base % P.q;
  return (u64)r;
}

// ---------------------------------------------------------------------------------------
// PackParams (inspiring2.rs:209-286) and derive_automorph_tables (330-379).
struct PackParams {
  Params P;
  std::shared_ptr<Ntt> ntt;
  size_t gamma;
  u64 generator;
  std::vector<u64> gen_pows;
  u64 mod_inv_gamma;
  Vec mod_inv_poly_ntt;
  std::vector<Vec> mono_ntt, neg_mono_ntt;
  // tables[(t-1)/2][i]: source slot of slot i under tau_t, built for the odd t the path
  // reads (the generator powers); every other entry stays empty.
  std::vector<std::vector<uint32_t>> tables;

  const std::vector<uint32_t>& table(u64 t) const { return tables[(t - 1) / 2]; }
};

static std::shared_ptr<PackParams> make_pack_params(const Params& P, size_t gamma) {
  auto pp = std::make_shared<PackParams>();
  size_t n = P.n;
  if (gamma == 0 || (gamma & (gamma - 1)) || gamma > n / 2) throw std::runtime_error("illegal width");
  pp->P = P;
  pp->ntt = std::make_shared<Ntt>(n, P.q);
  pp->gamma = gamma;
  pp->generator = 2 * n / gamma + 1;
  u64 two_n = 2 * n, v = 1;
  for (size_t i = 0; i < n; i++) {
    pp->gen_pows.push_back(v);
    v = v * pp->generator % two_n;
  }
  pp->mod_inv_gamma = mod_inverse(gamma, P.q);
  Vec c(n, 0);
  c[0] = pp->mod_inv_gamma;
  pp->mod_inv_poly_ntt = pp->ntt->fwd(c);
  pp->mono_ntt.resize(n);
  pp->neg_mono_ntt.resize(n);
#pragma omp parallel for schedule(static)
  for (long j = 0; j < (long)n; j++) {
    Vec m(n, 0);
    m[j] = 1;
    pp->mono_ntt[j] = pp->ntt->fwd(m);
    m[j] = P.q - 1;
    pp->neg_mono_ntt[j] = pp->ntt->fwd(m);
  }
  // Slot j of NTT(X^k) for k in [0, 2n), via X^(k+n) = -X^k.
  auto slot_value = [&](size_t k, size_t j) -> u64 {
    if (k < n) return pp->mono_ntt[k][j];
    u64 v = pp->mono_ntt[k - n][j];
    return (P.q - v) % P.q;
  };
  std::vector<std::pair<u64, u64>> powers;  // (value, odd exponent) of w_0
  for (size_t e = 1; e < two_n; e += 2) powers.push_back({slot_value(e, 0), e});
  std::sort(powers.begin(), powers.end());
  for (size_t i = 1; i < powers.size(); i++)
    if (powers[i].first == powers[i - 1].first) throw std::runtime_error("tables underivable");
  std::vector<u64> exps(n);
  std::vector<size_t> slot_of_exp(n, SIZE_MAX);
  for (size_t j = 0; j < n; j++) {
    u64 root = slot_value(1, j);
    auto it = std::lower_bound(powers.begin(), powers.end(), std::make_pair(root, (u64)0));
    if (it == powers.end() || it->first != root) throw std::runtime_error("tables underivable");
    u64 e = it->second;
    slot_of_exp[e / 2] = j;
    exps[j] = e;
  }
  pp->tables.resize(n);
  for (size_t i = 0; i < n && i < gamma; i++) {
    u64 t = pp->gen_pows[i];
    auto& tb = pp->tables[(t - 1) / 2];
    if (!tb.empty()) continue;
    tb.resize(n);
    for (size_t j = 0; j < n; j++) tb[j] = (uint32_t)slot_of_exp[((t * exps[j]) % two_n) / 2];
  }
  return pp;
}

// ---------------------------------------------------------------------------------------
// Offline packing keys (inspiring2.rs:537-598, 839-887).
struct OfflineKeys {
  std::vector<std::vector<Vec>> w_all_ntt;  // [gamma-1][key_rows]
  std::vector<Vec> w_mask;                  // coefficient form, key_rows polys
};

static std::vector<Vec> expand_mask(const uint8_t seed[32], u64 stream, size_t n, u64 q, size_t count) {
  ChaCha20Rng rng = ChaCha20Rng::from_seed(seed);
  rng.set_stream(stream);
  std::vector<Vec> out;
  for (size_t k = 0; k < count; k++) {
    Vec c(n);
    for (size_t i = 0; i < n; i++) c[i] = rng.next_u64() % q;
    out.push_back(c);
  }
  return out;
}

static std::vector<Vec> kept_mask_rows(const uint8_t seed[32], const Params& P, size_t gamma) {
  u64 stream = P.dropped() == 0 ? 0 : (u64)gamma;
  auto all = expand_mask(seed, stream, P.n, P.q, P.gadget_len);
  return std::vector<Vec>(all.begin() + P.dropped(), all.end());
}

static Vec permute(const Vec& src, const std::vector<uint32_t>& tb) {
  Vec r(src.size());
  for (size_t i = 0; i < src.size(); i++) r[i] = src[tb[i]];
  return r;
}

static OfflineKeys make_offline_keys(const PackParams& pp, const uint8_t w_seed[32]) {
  OfflineKeys k;
  k.w_mask = kept_mask_rows(w_seed, pp.P, pp.gamma);
  std::vector<Vec> w_mask_ntt;
  for (auto& w : k.w_mask) w_mask_ntt.push_back(pp.ntt->fwd(w));
  for (size_t i = 0; i + 1 < pp.gamma; i++) {
    const auto& tb = pp.table(pp.gen_pows[i]);
    std::vector<Vec> row;
    for (auto& w : w_mask_ntt) row.push_back(permute(w, tb));
    k.w_all_ntt.push_back(row);
  }
  return k;
}

// ---------------------------------------------------------------------------------------
// rotation_sums (inspiring2.rs:964-1004).
static std::vector<Vec> rotation_sums(const PackParams& pp, const std::vector<Vec>& inputs_ntt) {
  size_t n = pp.P.n, gamma = pp.gamma;
  std::vector<Vec> out(gamma);
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = 0; i < (long)gamma; i++) {
    Vec r(n, 0);
    size_t exp_index = (n - (size_t)i) % n;
    for (size_t j = 0; j < inputs_ntt.size(); j++) {
      size_t index = (j * pp.gen_pows[exp_index]) % (2 * n);
      const Vec& mono = index < n ? pp.mono_ntt[index % n] : pp.neg_mono_ntt[index % n];
      pp.ntt->mul_acc(r.data(), mono.data(), inputs_ntt[j].data());
    }
    Vec scaled(n);
    for (size_t t = 0; t < n; t++) scaled[t] = pp.ntt->mont(r[t], pp.mod_inv_poly_ntt[t]);
    out[i] = permute(scaled, pp.table(pp.gen_pows[i]));
  }
  return out;
}

// Gadget decomposition (rgsw/external_product.rs:30-99) and its rounded variant
// (inspiring2.rs:1167-1225).
static std::vector<Vec> gadget_decompose(const Params& P, const Vec& coeffs) {
  std::vector<Vec> d(P.gadget_len, Vec(P.n));
  for (size_t j = 0; j < P.n; j++) {
    u64 val = coeffs[j];
    for (size_t k = 0; k < P.gadget_len; k++) {
      d[k][j] = (val % P.gadget_base) % P.q;
      val /= P.gadget_base;
    }
  }
  return d;
}

static std::vector<Vec> gadget_decompose_rounded(const Params& P, const Vec& coeffs, size_t dropped) {
  size_t rows = P.gadget_len - dropped;
  std::vector<Vec> d(rows, Vec(P.n, 0));
  u128 base = P.gadget_base, unit = 1;
  for (size_t k = 0; k < dropped; k++) unit *= base;
  for (size_t j = 0; j < P.n; j++) {
    u128 rounded = ((u128)coeffs[j] + unit / 2) / unit;
    for (size_t r = 0; r + 1 < rows; r++) {
      d[r][j] = (u64)(rounded % base);
      rounded /= base;
    }
    d[rows - 1][j] = (u64)rounded;
  }
  // Poly::from_coeffs_moduli reduces each digit row mod q.
  for (auto& row : d)
    for (auto& x : row) x %= P.q;
  return d;
}

struct Precomp {
  Vec a_hat;                              // coefficient form
  std::vector<std::vector<Vec>> bold_t_ntt;  // [gamma-1][key_rows]
};

// fold_rotations_backward (inspiring2.rs:1014-1085) with LastDigitNtt (1094-1161).
static Precomp fold_rotations_backward(const PackParams& pp, const OfflineKeys& keys, std::vector<Vec> r_all) {
  const Params& P = pp.P;
  const Ntt& ntt = *pp.ntt;
  size_t gamma = pp.gamma, n = P.n;
  bool use_last = false;
  Vec of_sum;
  std::vector<Vec> of_digit;
  if (gamma > P.gadget_len + 1 && P.dropped() == 0) {
    u128 q = P.q, base = P.gadget_base, span = 1, power = 1;
    std::vector<u128> powers;
    bool ok = base >= 2;
    for (size_t k = 0; k < P.gadget_len; k++) {
      powers.push_back(power);
      power = power * (base % q) % q;
      span = span > (((u128)1 << 120) / base) ? ((u128)1 << 120) : span * base;
    }
    if (ok && span >= q) {
      u64 inverse = mod_inverse((u64)powers.back(), P.q);
      if (inverse != 0) {
        use_last = true;
        auto constant = [&](u64 v) {
          Vec c(n, 0);
          c[0] = v;
          return ntt.fwd(c);
        };
        of_sum = constant(inverse);
        for (size_t k = 0; k + 1 < P.gadget_len; k++)
          of_digit.push_back(constant((u64)((q - (u128)inverse * powers[k] % q) % q)));
      }
    }
  }
  Precomp pc;
  pc.bold_t_ntt.resize(gamma - 1);
  for (long i = (long)gamma - 2; i >= 0; i--) {
    Vec r_coeff = ntt.inv(r_all[i + 1]);
    std::vector<Vec> digits = P.dropped() == 0 ? gadget_decompose(P, r_coeff)
                                               : gadget_decompose_rounded(P, r_coeff, P.dropped());
    size_t transformed = use_last ? digits.size() - 1 : digits.size();
    std::vector<Vec> dn;
    for (size_t k = 0; k < transformed; k++) dn.push_back(ntt.fwd(digits[k]));
    if (use_last) {
      Vec last(n, 0);
      ntt.mul_acc(last.data(), r_all[i + 1].data(), of_sum.data());
      for (size_t k = 0; k < dn.size() && k < of_digit.size(); k++)
        ntt.mul_acc(last.data(), dn[k].data(), of_digit[k].data());
      dn.push_back(last);
    }
    for (size_t k = 0; k < dn.size() && k < keys.w_all_ntt[i].size(); k++)
      ntt.mul_acc(r_all[i].data(), dn[k].data(), keys.w_all_ntt[i][k].data());
    pc.bold_t_ntt[i] = dn;
  }
  pc.a_hat = ntt.inv(r_all[0]);
  return pc;
}

// packing_online_gather (inspiring2.rs:1393-1485), returning the final b.
static Vec packing_online_gather(const PackParams& pp, const Precomp& pc, const std::vector<Vec>& y_body_ntt,
                                 const Vec& b_poly) {
  size_t n = pp.P.n;
  const Ntt& ntt = *pp.ntt;
  Vec acc(n, 0);
  for (size_t i = 0; i + 1 < pp.gamma; i++) {
    const auto& tb = pp.table(pp.gen_pows[i]);
    for (size_t k = 0; k < y_body_ntt.size(); k++) {
      const Vec& y = y_body_ntt[k];
      const Vec& t = pc.bold_t_ntt[i][k];
      for (size_t j = 0; j < n; j++) acc[j] = addmod(acc[j], ntt.mont(y[tb[j]], t[j]), pp.P.q);
    }
  }
  Vec sum_b = ntt.inv(acc);
  Vec out(n);
  for (size_t j = 0; j < n; j++) out[j] = addmod(b_poly[j], sum_b[j], pp.P.q);
  return out;
}

// ---------------------------------------------------------------------------------------
// Packing store (shard_store.rs:86-156, 197-264, 282-342, 378-427).
static const u64 TAG_PRIME = (1ull << 61) - 1;

struct Store {
  std::vector<Vec> column_sums_ntt;
  Vec tag_key;
  std::vector<u64> column_tags;
};

static u64 column_tag(const u64* words, size_t n, const u64* key) {
  u128 sum = 0;
  for (size_t k = 0; k < n; k++) sum += (u128)(words[k] & 0xffffffffull) * key[2 * k] + (u128)(words[k] >> 32) * key[2 * k + 1];
  return (u64)(sum % TAG_PRIME);
}

static Store build_store(const PackParams& pp, const std::vector<Vec>& columns, u64 key_seed) {
  Store s;
  size_t n = pp.P.n;
  // The reference keys the tags from OS entropy; any key in [0, 2^61-1) serves.
  ChaCha20Rng rng = ChaCha20Rng::seed_from_u64(key_seed);
  for (size_t i = 0; i < 2 * n; i++) {
    u64 c;
    do c = rng.next_u64() >> 3;
    while (c >= TAG_PRIME);
    s.tag_key.push_back(c);
  }
  for (auto& col : columns) s.column_tags.push_back(column_tag(col.data(), n, s.tag_key.data()));
  std::vector<Vec> cols_ntt(columns.size());
#pragma omp parallel for
  for (long j = 0; j < (long)columns.size(); j++) cols_ntt[j] = pp.ntt->fwd(columns[j]);
  s.column_sums_ntt = rotation_sums(pp, cols_ntt);
  return s;
}

// check_columns_and_fold_b: returns false on a tag mismatch.
static bool check_and_fold_b(const PackParams& pp, const Store& s, const std::vector<Vec>& columns, const Vec& b,
                             Vec& b_poly) {
  size_t n = pp.P.n;
  u64 q = pp.P.q;
  Vec b_rev(n);
  for (size_t k = 0; k < n; k++) b_rev[k] = k == 0 ? b[0] % q : (q - b[n - k] % q) % q;
  b_poly.assign(n, 0);
  std::vector<u64> tags(columns.size());
#pragma omp parallel for
  for (long j = 0; j < (long)columns.size(); j++) {
    const Vec& col = columns[j];
    u128 tag = 0, low = 0, high = 0;
    for (size_t k = 0; k < n; k++) {
      tag += (u128)(col[k] & 0xffffffffull) * s.tag_key[2 * k] + (u128)(col[k] >> 32) * s.tag_key[2 * k + 1];
      u128 prod = (u128)col[k] * b_rev[k];
      low += (u64)prod;
      high += (u64)(prod >> 64);
    }
    u128 qq = q;
    u128 coeff0 = ((high % qq) * ((((u128)1) << 64) % qq) + low % qq) % qq;
    tags[j] = (u64)(tag % TAG_PRIME);
    b_poly[j] = (u64)coeff0;
  }
  for (size_t j = 0; j < columns.size(); j++)
    if (tags[j] != s.column_tags[j]) return false;
  return true;
}

static Precomp store_packing_offline(const PackParams& pp, const Store& s, const OfflineKeys& keys, const Vec& a) {
  size_t n = pp.P.n;
  Vec a_ntt = pp.ntt->fwd(a);
  std::vector<Vec> r_all(pp.gamma, Vec(n));
#pragma omp parallel for
  for (long i = 0; i < (long)pp.gamma; i++) {
    const auto& tb = pp.table(pp.gen_pows[i]);
    for (size_t k = 0; k < n; k++) r_all[i][k] = pp.ntt->mont(a_ntt[tb[k]], s.column_sums_ntt[i][k]);
  }
  return fold_rotations_backward(pp, keys, r_all);
}

// ---------------------------------------------------------------------------------------
// pack_shard (respond.rs:770-863): returns (a_hat, b).
struct Packed {
  Vec a, b;
};

static Packed pack_per_query(const PackParams& pp, const OfflineKeys& keys, const std::vector<Vec>& columns,
                             const Vec& a, const Vec& b, const std::vector<Vec>& y_body) {
  size_t n = pp.P.n, gamma = pp.gamma;
  const Ntt& ntt = *pp.ntt;
  // plaintext_multiply_columns + sample_extract_coeff0 + b_poly assembly.
  std::vector<Vec> a_ct(gamma);
  Vec b_poly(n, 0);
#pragma omp parallel for
  for (long j = 0; j < (long)gamma; j++) {
    a_ct[j] = ntt.mul(a, columns[j]);
    Vec bj = ntt.mul(b, columns[j]);
    b_poly[j] = bj[0];
  }
  std::vector<Vec> a_ntt(gamma);
#pragma omp parallel for
  for (long j = 0; j < (long)gamma; j++) a_ntt[j] = ntt.fwd(a_ct[j]);
  auto r_all = rotation_sums(pp, a_ntt);
  Precomp pc = fold_rotations_backward(pp, keys, r_all);
  std::vector<Vec> y_ntt;
  for (auto& y : y_body) y_ntt.push_back(ntt.fwd(y));
  Packed out;
  out.a = pc.a_hat;
  out.b = packing_online_gather(pp, pc, y_ntt, b_poly);
  return out;
}

static bool pack_with_store(const PackParams& pp, const OfflineKeys& keys, const Store& s,
                            const std::vector<Vec>& columns, const Vec& a, const Vec& b,
                            const std::vector<Vec>& y_body, Packed& out) {
  Vec b_poly;
  if (!check_and_fold_b(pp, s, columns, b, b_poly)) return false;
  Precomp pc = store_packing_offline(pp, s, keys, a);
  std::vector<Vec> y_ntt;
  for (auto& y : y_body) y_ntt.push_back(pp.ntt->fwd(y));
  out.a = pc.a_hat;
  out.b = packing_online_gather(pp, pc, y_ntt, b_poly);
  return true;
}

// mod_switch_poly (mod_switch.rs:148-176).
static Vec mod_switch(const Vec& c, u64 q_old, u64 q_new) {
  Vec o(c.size());
  for (size_t i = 0; i < c.size(); i++) {
    u128 scaled = (u128)c[i] * q_new + q_old / 2;
    o[i] = (u64)((scaled / q_old) % q_new);
  }
  return o;
}

// ---------------------------------------------------------------------------------------
// bincode 1.3 fixint little-endian writer and the tight coefficient codec (poly.rs:166-225).
struct Bin {
  std::vector<uint8_t> b;
  void u8(uint8_t v) { b.push_back(v); }
  void u32(uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void u64_(u64 v) {
    for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void bytes(const std::vector<uint8_t>& v) {
    u64_(v.size());
    b.insert(b.end(), v.begin(), v.end());
  }
};

static std::vector<uint8_t> pack_tight(const u64* c, size_t count, u64 modulus) {
  unsigned bits = 64 - clz64(modulus - 1);
  size_t nbytes = (count * bits + 7) / 8;
  std::vector<uint8_t> out(nbytes, 0);
  for (size_t i = 0; i < count; i++) {
    size_t bit = i * bits;
    u128 v = (u128)c[i] << (bit % 8);
    size_t by = bit / 8;
    for (size_t k = 0; k < 10 && by + k < nbytes; k++) out[by + k] |= (uint8_t)(v >> (8 * k));
  }
  return out;
}

static void write_poly(Bin& w, const Vec& c, u64 modulus) {
  w.bytes(pack_tight(c.data(), c.size(), modulus));
  w.u64_(1);
  w.u64_(modulus);
  w.u64_(modulus);  // q = product of the one modulus
  w.u64_(c.size());
  w.u64_(0);  // crt_q0_inv_mod_q1
  w.u8(0);    // is_ntt
}

// ServerResponse tight wire (respond.rs:111-176): Packed{a, b_prefix, retained}, no
// column ciphertexts, Some(PackingMode::Inspiring).
// `variant`: the PackingMode index (query.rs:20-26), 0 Inspiring, 1 Tree.
static std::vector<uint8_t> response_bytes(const Vec& a, const Vec& b, size_t retained, u64 modulus,
                                           uint32_t variant = 0) {
  Bin w;
  w.u32(1);
  write_poly(w, a, modulus);
  w.bytes(pack_tight(b.data(), retained, modulus));
  w.u32((uint32_t)retained);
  w.u64_(0);
  w.u8(1);
  w.u32(variant);
  return w.b;
}

static std::vector<uint8_t> key_bytes(const std::vector<Vec>& y_body, size_t gamma, u64 modulus) {
  Bin w;
  w.u64_(y_body.size());
  for (auto& y : y_body) write_poly(w, y, modulus);
  w.u64_(0);
  w.u8(0);
  w.u64_(gamma);
  return w.b;
}

// ---------------------------------------------------------------------------------------
// Client-side regeneration of KAT inputs.

static Vec sample_gaussian_poly(GaussianSampler& g, size_t n, u64 q) {
  Vec c(n);
  for (size_t i = 0; i < n; i++) c[i] = from_signed(g.sample(), q);
  return c;
}

// apply_automorphism in the coefficient domain (rlwe/galois.rs:12-45).
static Vec automorphism_coeff(const Vec& p, u64 g, u64 q) {
  size_t d = p.size();
  Vec r(d, 0);
  for (size_t i = 0; i < d; i++) {
    size_t idx = (size_t)((g * i) % (2 * d));
    if (idx < d)
      r[idx] = addmod(r[idx], p[i], q);
    else
      r[idx - d] = submod(r[idx - d], p[i], q);
  }
  return r;
}

// inverse_monomial (encode_db.rs:43-70): X^(-k) in Z_q[X]/(X^d + 1).
static Vec inverse_monomial(size_t k, size_t d, u64 q) {
  Vec c(d, 0);
  k %= 2 * d;
  if (k == 0)
    c[0] = 1;
  else if (k <= d)
    c[d - k] = q - 1;
  else
    c[2 * d - k] = 1;
  return c;
}

// Poly::from_seed_moduli (poly.rs:657-686): ChaCha20 from the seed, gen_range(0..q) per coeff.
static Vec expand_seed(const uint8_t seed[32], size_t n, u64 q) {
  ChaCha20Rng rng = ChaCha20Rng::from_seed(seed);
  Vec c(n);
  for (size_t i = 0; i < n; i++) c[i] = gen_range_u64(rng, 0, q);
  return c;
}

struct Cell {
  Params P;
  size_t entry_size, gamma, num_shards;
  std::vector<uint8_t> db;
  uint8_t w_seed[32];
  std::shared_ptr<PackParams> pp;
  OfflineKeys keys;
  std::vector<std::vector<Vec>> shards;  // [shard][column] coefficient form
  Vec sk;
  std::vector<Vec> y_body;
  GaussianSampler sampler;
  ChaCha20Rng rng;
  std::vector<std::unique_ptr<Store>> stores;
};

static size_t num_columns(size_t entry) { return entry == 0 ? 1 : (entry + 1) / 2; }

// setup_with_rng (pir/setup.rs:408-495) draws, once the cell's records, sampler and rng are
// in place: the setup secret key, then one error polynomial per Galois-key row (their `a`
// come from OS entropy and never reach a response), then the two public seeds. Returns the
// setup secret.
static Vec cell_setup_draws(Cell* c) {
  const Params& P = c->P;
  size_t n = P.n;
  Vec sk = sample_gaussian_poly(c->sampler, n, P.q);
  size_t log_d = 0;
  while ((size_t(1) << (log_d + 1)) <= n) log_d++;
  for (size_t i = 0; i < log_d; i++)
    for (size_t r = 0; r < P.gadget_len; r++)
      for (size_t k = 0; k < n; k++) c->sampler.sample();
  c->rng.fill_bytes(c->w_seed, 32);
  uint8_t v_seed[32];
  c->rng.fill_bytes(v_seed, 32);
  return sk;
}

// The rest of a cell once its secret c->sk is set: pack params, offline keys,
// encode_database (encode_db.rs:74-134: one record per coefficient, 16-bit columns) and the
// session's packing keys, ClientPackingKeys::generate_once (inspiring2.rs:764-791) and
// generate_ksk_body (893-929), errors from the sampler.
static void cell_finish(Cell* c) {
  const Params& P = c->P;
  size_t n = P.n, entry_size = c->entry_size;
  c->gamma = num_columns(entry_size);
  c->pp = make_pack_params(P, c->gamma);
  c->keys = make_offline_keys(*c->pp, c->w_seed);
  size_t total = c->db.size() / entry_size;
  c->num_shards = (total + n - 1) / n;
  for (size_t s = 0; s < c->num_shards; s++) {
    std::vector<Vec> cols(c->gamma, Vec(n, 0));
    for (size_t col = 0; col < c->gamma; col++)
      for (size_t l = 0; l < n && s * n + l < total; l++) {
        const uint8_t* e = &c->db[(s * n + l) * entry_size];
        size_t off = col * 2;
        u64 v = 0;
        if (off + 1 < entry_size)
          v = (u64)e[off] | ((u64)e[off + 1] << 8);
        else if (off < entry_size)
          v = e[off];
        cols[col][l] = v % P.q;
      }
    c->shards.push_back(cols);
  }
  const Ntt& ntt = *c->pp->ntt;
  u64 gen = c->pp->generator % (2 * n);
  Vec tau_s = automorphism_coeff(c->sk, gen, P.q);
  for (size_t row = 0; row < c->keys.w_mask.size(); row++) {
    u64 gp = gadget_power(P, P.dropped() + row);
    Vec s_w = ntt.mul(c->sk, c->keys.w_mask[row]);
    Vec e = sample_gaussian_poly(c->sampler, n, P.q);
    Vec y(n);
    for (size_t i = 0; i < n; i++) y[i] = addmod(addmod(mulmod(tau_s[i], gp, P.q), (P.q - s_w[i]) % P.q, P.q), e[i], P.q);
    c->y_body.push_back(y);
  }
  c->stores.resize(c->num_shards);
}

// The KAT cell of tests/packing_key_fixture/mod.rs:65-146: the fixture's database formula,
// the session built on the setup secret (ClientSession::new), and the probe query the
// fixture makes before its recorded ones.
static Cell* cell_build(const Params& P, size_t entry_size, u64 seed, size_t entries) {
  auto* c = new Cell();
  c->P = P;
  c->entry_size = entry_size;
  size_t n = P.n;
  // tests/packing_key_fixture/mod.rs:65-69 database formula.
  c->db.resize(entries * entry_size);
  for (size_t i = 0; i < c->db.size(); i++) c->db[i] = (uint8_t)(((u64)i * 0x9E3779B9ull + seed) >> 7);
  c->sampler = GaussianSampler::with_seed(P.sigma, seed);
  c->rng = ChaCha20Rng::seed_from_u64(seed ^ 0x5eed);
  c->sk = cell_setup_draws(c);
  cell_finish(c);
  // The probe query_seeded(0): its `a` seed is OS entropy, its error draws n samples.
  for (size_t k = 0; k < n; k++) c->sampler.sample();
  return c;
}

// The plain method as the reference's public API runs it: `entries` records of entry_size
// uniform bytes from ChaCha20Rng::seed_from_u64(seed).fill_bytes; setup_with_rng under
// GaussianSampler::with_seed(sigma, seed) and ChaCha20Rng::seed_from_u64(seed); then
// ClientSession::with_seeded_secret (pir/session.rs:141-145), which draws the session's own
// secret (RlweSecretKey::generate, rlwe/enc.rs:48-51) and its packing-key errors from the
// same sampler. Queries follow with cell_next_query: the index and the `a` seed (OS entropy
// in the reference, here the next 32 bytes of setup's rng) from the rng, the error from
// the sampler.
static Cell* cell_build_seeded(const Params& P, size_t entry_size, u64 seed, size_t entries) {
  auto* c = new Cell();
  c->P = P;
  c->entry_size = entry_size;
  c->db.resize(entries * entry_size);
  {
    ChaCha20Rng records = ChaCha20Rng::seed_from_u64(seed);
    records.fill_bytes(c->db.data(), c->db.size());
  }
  c->sampler = GaussianSampler::with_seed(P.sigma, seed);
  c->rng = ChaCha20Rng::seed_from_u64(seed);
  (void)cell_setup_draws(c);  // the setup secret stays the server's; the session draws its own
  c->sk = sample_gaussian_poly(c->sampler, P.n, P.q);
  cell_finish(c);
  return c;
}

// Cell::next_query (tests/packing_key_fixture/mod.rs:126-146) with
// SeededRgswCiphertext::encrypt_with_rng (rgsw/types.rs:345-388).
static void cell_next_query(Cell* c, u64 index, uint32_t* shard_id, uint8_t seed[32], u64* b_out) {
  const Params& P = c->P;
  size_t n = P.n;
  *shard_id = (uint32_t)(index / n);
  size_t local = (size_t)(index % n);
  Vec scaled = inverse_monomial(local, n, P.q);
  for (auto& x : scaled) x = mulmod(x, P.delta(), P.q);
  c->rng.fill_bytes(seed, 32);
  Vec a = expand_seed(seed, n, P.q);
  Vec e = sample_gaussian_poly(c->sampler, n, P.q);
  Vec as = c->pp->ntt->mul(a, c->sk);
  for (size_t i = 0; i < n; i++) b_out[i] = addmod(addmod((P.q - as[i]) % P.q, e[i], P.q), scaled[i], P.q);
}

// extract_inspiring (pir/extract.rs:229-263): decrypt, round, reassemble the record.
static bool cell_decode(const Cell* c, u64 index, const u64* a, const u64* b, uint8_t* record_out) {
  const Params& P = c->P;
  size_t n = P.n;
  Vec av(a, a + n);
  Vec as = c->pp->ntt->mul(av, c->sk);
  u64 delta = P.delta();
  std::vector<u64> vals;
  for (size_t col = 0; col < c->gamma; col++) {
    u64 noisy = addmod(as[col], b[col], P.q);
    u128 num = (u128)noisy + delta / 2;
    vals.push_back((u64)(num / delta) % P.p);
  }
  std::vector<uint8_t> entry(c->entry_size, 0);
  for (size_t col = 0; col < vals.size(); col++) {
    size_t off = col * 2;
    if (off < c->entry_size) entry[off] = (uint8_t)(vals[col] & 0xff);
    if (off + 1 < c->entry_size) entry[off + 1] = (uint8_t)((vals[col] >> 8) & 0xff);
  }
  memcpy(record_out, entry.data(), entry.size());
  return memcmp(entry.data(), &c->db[index * c->entry_size], c->entry_size) == 0;
}

// ---------------------------------------------------------------------------------------
// OnePacking: respond_one_packing (pir/respond.rs:696-729) over the Galois-automorphism tree
// of inspiring/automorph_pack.rs.

// One key-switching matrix (ks/setup.rs:12-20): a row (a, b) per gadget power, coefficient
// form.
struct KsMatrix {
  std::vector<Vec> a, b;
};

// homomorphic_automorph (automorph_pack.rs:15-43): tau_t on both parts, then the a part's
// base-2^20 digits times the key rows, each product through the transform.
static void hom_automorph(const Params& P, const Ntt& ntt, const Vec& ca, const Vec& cb, u64 t, const KsMatrix& ks,
                          Vec& ra, Vec& rb) {
  const u64 q = P.q;
  const Vec aa = automorphism_coeff(ca, t, q);
  rb = automorphism_coeff(cb, t, q);
  ra.assign(P.n, 0);
  const auto digits = gadget_decompose(P, aa);
  for (size_t i = 0; i < digits.size(); i++) {
    if (i >= ks.a.size()) continue;
    const Vec ta = ntt.mul(digits[i], ks.a[i]), tb = ntt.mul(digits[i], ks.b[i]);
    for (size_t k = 0; k < P.n; k++) {
      ra[k] = addmod(ra[k], ta[k], q);
      rb[k] = addmod(rb[k], tb[k], q);
    }
  }
}

// pack_lwes_inner (automorph_pack.rs:96-163): the 2^ell ciphertexts reachable from `start`
// (b parts zero at the leaves) combined as (even + y odd) + tau_t(even - y odd) with
// y = X^(d >> ell), t = 2^ell + 1 and key index log d - ell. Leaves past the inputs are the
// zero ciphertexts of the padding.
static void pack_inner(const Params& P, const Ntt& ntt, size_t ell, size_t start, const std::vector<Vec>& leaf_a,
                       const std::vector<KsMatrix>& keys, size_t log_n, Vec& ra, Vec& rb) {
  const size_t d = P.n;
  const u64 q = P.q;
  if (ell == 0) {
    ra = start < leaf_a.size() ? leaf_a[start] : Vec(d, 0);
    rb.assign(d, 0);
    return;
  }
  const size_t step = (size_t)1 << (log_n - ell);
  Vec ea, eb, oa, ob;
  pack_inner(P, ntt, ell - 1, start, leaf_a, keys, log_n, ea, eb);
  pack_inner(P, ntt, ell - 1, start + step, leaf_a, keys, log_n, oa, ob);
  Vec y(d, 0), ny(d, 0);  // YConstants (automorph_pack.rs:55-83), level ell - 1
  y[d >> ell] = 1;
  ny[d >> ell] = q - 1;
  const Vec ya = ntt.mul(oa, y), yb = ntt.mul(ob, y), na = ntt.mul(oa, ny), nb = ntt.mul(ob, ny);
  Vec s0a(d), s0b(d), s1a(d), s1b(d);
  for (size_t k = 0; k < d; k++) {
    s0a[k] = addmod(ea[k], ya[k], q);
    s0b[k] = addmod(eb[k], yb[k], q);
    s1a[k] = addmod(ea[k], na[k], q);
    s1b[k] = addmod(eb[k], nb[k], q);
  }
  const u64 t = ((u64)1 << ell) + 1;
  const size_t ks_idx = keys.size() - ell;
  Vec ha, hb;
  hom_automorph(P, ntt, s1a, s1b, t, keys[ks_idx], ha, hb);
  ra.resize(d);
  rb.resize(d);
  for (size_t k = 0; k < d; k++) {
    ra[k] = addmod(s0a[k], ha[k], q);
    rb[k] = addmod(s0b[k], hb[k], q);
  }
}

// respond_one_packing: the column products (plaintext_multiply_columns, respond.rs:585-599),
// their coefficient-0 LWEs (rlwe/enc.rs:161-174), whose a vectors prep_pack_lwes turns back
// into the products' a polynomials (automorph_pack.rs:238-268), then pack_lwes
// (automorph_pack.rs:270-341): one input skips the tree and its scaling; otherwise the
// tree over d padded leaves, and b_k += d b-value_k.
static void respond_one_packing(const PackParams& pp, const std::vector<Vec>& columns, const Vec& a, const Vec& b,
                                const std::vector<KsMatrix>& keys, Vec& out_a, Vec& out_b) {
  const Params& P = pp.P;
  const Ntt& ntt = *pp.ntt;
  const size_t d = P.n, gamma = columns.size();
  const u64 q = P.q;
  std::vector<Vec> leaf_a(gamma);
  Vec bvals(gamma);
#pragma omp parallel for
  for (long j = 0; j < (long)gamma; j++) {
    leaf_a[j] = ntt.mul(a, columns[j]);
    bvals[j] = ntt.mul(b, columns[j])[0];
  }
  if (gamma == 1) {
    out_a = leaf_a[0];
    out_b.assign(d, 0);
    out_b[0] = bvals[0];
    return;
  }
  size_t log_d = 0;
  while (((size_t)1 << log_d) < d) log_d++;
  pack_inner(P, ntt, log_d, 0, leaf_a, keys, log_d, out_a, out_b);
  for (size_t z = 0; z < gamma; z++) out_b[z] = addmod(out_b[z], mulmod(bvals[z], d % q, q), q);
}

// Test-only Galois keys for secret s, in the shape setup_with_rng makes them
// (pir/setup.rs:435-445, ks/setup.rs:101-153): key i switches tau_t(s) to s for
// t = d / 2^i + 1, rows (a_r, -a_r s + e_r + tau_t(s) base^r). The reference draws a_r from
// the OS entropy source, so its keys cannot be regenerated; here a_r is uniform from
// ChaCha20(seed) on stream i * rows + r and e_r uniform in [-4, 4] from the same stream.
static std::vector<KsMatrix> test_galois_keys(const Params& P, const Ntt& ntt, const Vec& sk, const uint8_t seed[32]) {
  const size_t d = P.n;
  const u64 q = P.q;
  size_t log_d = 0;
  while (((size_t)1 << log_d) < d) log_d++;
  std::vector<KsMatrix> keys(log_d);
  for (size_t i = 0; i < log_d; i++) {
    const Vec sa = automorphism_coeff(sk, (d >> i) + 1, q);
    for (size_t r = 0; r < P.gadget_len; r++) {
      ChaCha20Rng rng = ChaCha20Rng::from_seed(seed);
      rng.set_stream(i * P.gadget_len + r);
      Vec a(d), e(d);
      for (size_t k = 0; k < d; k++) a[k] = gen_range_u64(rng, 0, q);
      for (size_t k = 0; k < d; k++) e[k] = from_signed((i64)(rng.next_u64() % 9) - 4, q);
      const Vec as = ntt.mul(a, sk);
      const u64 pw = gadget_power(P, r);
      Vec bb(d);
      for (size_t k = 0; k < d; k++) bb[k] = addmod(submod(e[k], as[k], q), mulmod(sa[k], pw, q), q);
      keys[i].a.push_back(a);
      keys[i].b.push_back(bb);
    }
  }
  return keys;
}

static std::vector<KsMatrix> unpack_keys(const u64* keys, size_t count, size_t rows, size_t n) {
  std::vector<KsMatrix> out(count);
  for (size_t i = 0; i < count; i++)
    for (size_t r = 0; r < rows; r++) {
      const u64* row = keys + (i * rows + r) * 2 * n;
      out[i].a.emplace_back(row, row + n);
      out[i].b.emplace_back(row + n, row + 2 * n);
    }
  return out;
}

// extract_packed for a tree response (pir/extract.rs:184-226): decrypt, round by delta,
// then multiply by d^-1 mod p.
static bool cell_decode_tree(const Cell* c, u64 index, const u64* a, const u64* b, uint8_t* record_out) {
  const Params& P = c->P;
  const size_t n = P.n;
  Vec av(a, a + n);
  const Vec as = c->pp->ntt->mul(av, c->sk);
  const u64 delta = P.delta();
  const u64 d_inv = powmod(n % P.p, P.p - 2, P.p);
  std::vector<uint8_t> entry(c->entry_size, 0);
  for (size_t col = 0; col < c->gamma; col++) {
    const u64 noisy = addmod(as[col], b[col], P.q);
    const u64 m = (u64)(((u128)noisy + delta / 2) / delta) % P.p;
    const u64 v = mulmod(m, d_inv, P.p);
    const size_t off = col * 2;
    if (off < c->entry_size) entry[off] = (uint8_t)(v & 0xff);
    if (off + 1 < c->entry_size) entry[off + 1] = (uint8_t)((v >> 8) & 0xff);
  }
  memcpy(record_out, entry.data(), entry.size());
  return memcmp(entry.data(), &c->db[index * c->entry_size], c->entry_size) == 0;
}

}  // namespace orc

// =======================================================================================
// C API for the Python test harness (ctypes).
using namespace orc;

struct OrcCache {
  std::shared_ptr<PackParams> pp;
  OfflineKeys keys;
};

static Params make_params(u64 n, u64 q, u64 p, double sigma, u64 base, u64 glen, int approx) {
  Params P;
  P.n = n;
  P.q = q;
  P.p = p;
  P.sigma = sigma;
  P.gadget_base = base;
  P.gadget_len = glen;
  P.approx = approx != 0;
  return P;
}

static thread_local std::string g_err;

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void orc_set_threads(int t) { omp_set_num_threads(t); }
int orc_max_threads() { return omp_get_max_threads(); }

u64 orc_fnv1a(const uint8_t* p, size_t n) { return fnv1a(p, n); }

// FNV-1a of `count` Gaussian samples (i64 LE) from GaussianSampler::with_seed(sigma, seed):
// the reference pins these streams in src/math/gaussian.rs:335-351.
u64 orc_gaussian_stream_fnv(double sigma, u64 seed, u64 count) {
  GaussianSampler g = GaussianSampler::with_seed(sigma, seed);
  u64 h = 0xcbf29ce484222325ULL;
  for (u64 i = 0; i < count; i++) {
    i64 x = g.sample();
    for (int k = 0; k < 8; k++) {
      h ^= (uint8_t)((u64)x >> (8 * k));
      h *= 0x00000100000001b3ULL;
    }
  }
  return h;
}

void orc_expand_seed(const uint8_t* seed, u64 n, u64 q, u64* out) {
  Vec a = expand_seed(seed, n, q);
  memcpy(out, a.data(), n * 8);
}

void orc_chacha_u64s(const uint8_t* seed, u64 stream, u64 count, u64* out) {
  ChaCha20Rng r = ChaCha20Rng::from_seed(seed);
  r.set_stream(stream);
  for (u64 i = 0; i < count; i++) out[i] = r.next_u64();
}

// NTT of one polynomial, Montgomery-form output, exactly as NttContext::forward.
int orc_ntt_forward(u64 n, u64 q, u64* c) {
  try {
    Ntt ntt(n, q);
    ntt.forward(c);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
int orc_ntt_inverse(u64 n, u64 q, u64* c) {
  try {
    Ntt ntt(n, q);
    ntt.inverse(c);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

void* orc_cache_new(u64 n, u64 q, u64 p, double sigma, u64 base, u64 glen, int approx, u64 gamma,
                    const uint8_t* w_seed) {
  try {
    auto* c = new OrcCache();
    c->pp = make_pack_params(make_params(n, q, p, sigma, base, glen, approx), gamma);
    c->keys = make_offline_keys(*c->pp, w_seed);
    return c;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void orc_cache_free(void* c) { delete (OrcCache*)c; }

// Slot tables the path reads: out[i*n + t] = source slot of t under tau_{g^i}, i < gamma.
void orc_cache_tables(void* cv, uint32_t* out) {
  auto* c = (OrcCache*)cv;
  size_t n = c->pp->P.n;
  for (size_t i = 0; i < c->pp->gamma; i++) {
    const auto& tb = c->pp->table(c->pp->gen_pows[i]);
    memcpy(out + i * n, tb.data(), n * 4);
  }
}

// Offline key rotations in Montgomery NTT form: out[((i*rows)+k)*n + t].
void orc_cache_w_all_ntt(void* cv, u64* out) {
  auto* c = (OrcCache*)cv;
  size_t n = c->pp->P.n, rows = c->pp->P.key_rows();
  for (size_t i = 0; i + 1 < c->pp->gamma; i++)
    for (size_t k = 0; k < rows; k++) memcpy(out + (i * rows + k) * n, c->keys.w_all_ntt[i][k].data(), n * 8);
}

static std::vector<Vec> unpack_polys(const u64* p, size_t count, size_t n) {
  std::vector<Vec> v;
  for (size_t i = 0; i < count; i++) v.push_back(Vec(p + i * n, p + (i + 1) * n));
  return v;
}

// pack_shard on the per-query branch (no store). a is the expanded query `a` (coefficient
// form); columns gamma x n; y_body key_rows x n (coefficient form).
int orc_respond_per_query(void* cv, const u64* columns, const u64* a, const u64* b, const u64* y_body,
                          u64* a_out, u64* b_out) {
  auto* c = (OrcCache*)cv;
  size_t n = c->pp->P.n;
  try {
    Packed r = pack_per_query(*c->pp, c->keys, unpack_polys(columns, c->pp->gamma, n), Vec(a, a + n), Vec(b, b + n),
                              unpack_polys(y_body, c->pp->P.key_rows(), n));
    memcpy(a_out, r.a.data(), n * 8);
    memcpy(b_out, r.b.data(), n * 8);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

struct OrcStore {
  Store s;
  std::vector<Vec> columns;  // the columns as the shard holds them now
};

void* orc_store_build(void* cv, const u64* columns, u64 key_seed) {
  auto* c = (OrcCache*)cv;
  auto* st = new OrcStore();
  st->columns = unpack_polys(columns, c->pp->gamma, c->pp->P.n);
  st->s = build_store(*c->pp, st->columns, key_seed);
  return st;
}
void orc_store_free(void* s) { delete (OrcStore*)s; }

// Step-1 sums in Montgomery NTT form: out[i*n + t].
void orc_store_sums(void* cv, void* sv, u64* out) {
  auto* c = (OrcCache*)cv;
  auto* st = (OrcStore*)sv;
  size_t n = c->pp->P.n;
  for (size_t i = 0; i < c->pp->gamma; i++) memcpy(out + i * n, st->s.column_sums_ntt[i].data(), n * 8);
}

// Store branch of pack_shard against `columns` (the live columns). Returns 1 when the tag
// check refuses the columns.
int orc_respond_store(void* cv, void* sv, const u64* columns, const u64* a, const u64* b, const u64* y_body,
                      u64* a_out, u64* b_out) {
  auto* c = (OrcCache*)cv;
  auto* st = (OrcStore*)sv;
  size_t n = c->pp->P.n;
  Packed r;
  if (!pack_with_store(*c->pp, c->keys, st->s, unpack_polys(columns, c->pp->gamma, n), Vec(a, a + n),
                       Vec(b, b + n), unpack_polys(y_body, c->pp->P.key_rows(), n), r))
    return 1;
  memcpy(a_out, r.a.data(), n * 8);
  memcpy(b_out, r.b.data(), n * 8);
  return 0;
}

// Scan only: tags check + b fold. Returns 1 on a tag mismatch.
int orc_store_scan(void* cv, void* sv, const u64* columns, const u64* b, u64* b_poly_out) {
  auto* c = (OrcCache*)cv;
  auto* st = (OrcStore*)sv;
  size_t n = c->pp->P.n;
  Vec bp;
  bool ok = check_and_fold_b(*c->pp, st->s, unpack_polys(columns, c->pp->gamma, n), Vec(b, b + n), bp);
  memcpy(b_poly_out, bp.data(), n * 8);
  return ok ? 0 : 1;
}

void orc_mod_switch(const u64* c, u64 count, u64 q_old, u64 q_new, u64* out) {
  Vec r = mod_switch(Vec(c, c + count), q_old, q_new);
  memcpy(out, r.data(), count * 8);
}

// ServerResponse bytes for coefficient-form (a, b) over `modulus`; returns the length and
// writes at most `cap` bytes.
u64 orc_response_bytes(const u64* a, const u64* b, u64 n, u64 retained, u64 modulus, uint8_t* out, u64 cap) {
  auto v = response_bytes(Vec(a, a + n), Vec(b, b + n), retained, modulus);
  if (out) memcpy(out, v.data(), std::min<u64>(cap, v.size()));
  return v.size();
}
// The same bytes for a tree-packed response (packing_mode Some(Tree)).
u64 orc_response_bytes_tree(const u64* a, const u64* b, u64 n, u64 retained, u64 modulus, uint8_t* out, u64 cap) {
  auto v = response_bytes(Vec(a, a + n), Vec(b, b + n), retained, modulus, 1);
  if (out) memcpy(out, v.data(), std::min<u64>(cap, v.size()));
  return v.size();
}

// respond (respond.rs:614-643), the NoPacking variant: one RLWE ciphertext (a h_j, b h_j)
// per column from plaintext_multiply_columns (respond.rs:585-599), and their sum as the
// response ciphertext. out: (gamma + 1) ciphertexts of (a, b), n words each, the sum first.
int orc_respond_nopacking(void* cv, const u64* columns, const u64* a, const u64* b, u64* out) {
  auto* c = (OrcCache*)cv;
  const size_t n = c->pp->P.n, gamma = c->pp->gamma;
  const u64 q = c->pp->P.q;
  try {
    const Ntt& ntt = *c->pp->ntt;
    auto cols = unpack_polys(columns, gamma, n);
    Vec av(a, a + n), bv(b, b + n);
    std::vector<Vec> ca(gamma), cb(gamma);
#pragma omp parallel for
    for (long j = 0; j < (long)gamma; j++) {
      ca[j] = ntt.mul(av, cols[j]);
      cb[j] = ntt.mul(bv, cols[j]);
    }
    Vec sa = ca[0], sb = cb[0];
    for (size_t j = 1; j < gamma; j++)
      for (size_t k = 0; k < n; k++) {
        sa[k] = (sa[k] + ca[j][k]) % q;
        sb[k] = (sb[k] + cb[j][k]) % q;
      }
    memcpy(out, sa.data(), n * 8);
    memcpy(out + n, sb.data(), n * 8);
    for (size_t j = 0; j < gamma; j++) {
      memcpy(out + (2 + 2 * j) * n, ca[j].data(), n * 8);
      memcpy(out + (3 + 2 * j) * n, cb[j].data(), n * 8);
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// respond_one_packing for one query: columns gamma x n, a and b n words (coefficient form),
// keys log d x rows x (a, b) x n words; writes the packed (a, b).
int orc_respond_one_packing(void* cv, const u64* columns, const u64* a, const u64* b, const u64* keys, u64 nkeys,
                            u64* out_a, u64* out_b) {
  auto* c = (OrcCache*)cv;
  const size_t n = c->pp->P.n, gamma = c->pp->gamma;
  try {
    auto cols = unpack_polys(columns, gamma, n);
    const auto ks = unpack_keys(keys, nkeys, c->pp->P.gadget_len, n);
    Vec av(a, a + n), bv(b, b + n), ra, rb;
    respond_one_packing(*c->pp, cols, av, bv, ks, ra, rb);
    memcpy(out_a, ra.data(), n * 8);
    memcpy(out_b, rb.data(), n * 8);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// ServerResponse tight wire of an unpacked response (respond.rs:111-176): Full(ciphertext),
// the column ciphertexts, packing_mode None. cts: `count` ciphertexts of (a, b), the
// response ciphertext first, then count - 1 column ciphertexts.
u64 orc_response_bytes_full(const u64* cts, u64 count, u64 n, u64 modulus, uint8_t* out, u64 cap) {
  Bin w;
  w.u32(0);
  write_poly(w, Vec(cts, cts + n), modulus);
  write_poly(w, Vec(cts + n, cts + 2 * n), modulus);
  w.u64_(count - 1);
  for (u64 j = 1; j < count; j++) {
    write_poly(w, Vec(cts + 2 * j * n, cts + (2 * j + 1) * n), modulus);
    write_poly(w, Vec(cts + (2 * j + 1) * n, cts + (2 * j + 2) * n), modulus);
  }
  w.u8(0);
  if (out) memcpy(out, w.b.data(), std::min<u64>(cap, w.b.size()));
  return w.b.size();
}

// -- KAT cells --------------------------------------------------------------------------
void* orc_cell_build(u64 n, u64 q, u64 p, double sigma, u64 base, u64 glen, int approx, u64 entry_size, u64 seed,
                     u64 entries) {
  try {
    return cell_build(make_params(n, q, p, sigma, base, glen, approx), entry_size, seed, entries);
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void* orc_cell_build_seeded(u64 n, u64 q, u64 p, double sigma, u64 base, u64 glen, int approx, u64 entry_size,
                            u64 seed, u64 entries) {
  try {
    return cell_build_seeded(make_params(n, q, p, sigma, base, glen, approx), entry_size, seed, entries);
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
// rand's gen_range(0..bound) on the cell's rng (the query index of the plain method).
u64 orc_cell_draw_index(void* cv, u64 bound) { return gen_range_u64(((Cell*)cv)->rng, 0, bound); }
void orc_cell_free(void* c) { delete (Cell*)c; }
void orc_cell_info(void* cv, u64* gamma, u64* num_shards, u64* key_rows, uint8_t* w_seed) {
  auto* c = (Cell*)cv;
  *gamma = c->gamma;
  *num_shards = c->num_shards;
  *key_rows = c->P.key_rows();
  memcpy(w_seed, c->w_seed, 32);
}
void orc_cell_columns(void* cv, u64 shard, u64* out) {
  auto* c = (Cell*)cv;
  for (size_t j = 0; j < c->gamma; j++) memcpy(out + j * c->P.n, c->shards[shard][j].data(), c->P.n * 8);
}
void orc_cell_keys(void* cv, u64* out) {
  auto* c = (Cell*)cv;
  for (size_t k = 0; k < c->y_body.size(); k++) memcpy(out + k * c->P.n, c->y_body[k].data(), c->P.n * 8);
}
void orc_cell_secret(void* cv, u64* out) {
  auto* c = (Cell*)cv;
  memcpy(out, c->sk.data(), c->P.n * 8);
}
u64 orc_cell_key_bytes(void* cv, uint8_t* out, u64 cap) {
  auto* c = (Cell*)cv;
  auto v = key_bytes(c->y_body, c->gamma, c->P.q);
  if (out) memcpy(out, v.data(), std::min<u64>(cap, v.size()));
  return v.size();
}
void orc_cell_next_query(void* cv, u64 index, uint32_t* shard_id, uint8_t* seed, u64* b_out) {
  cell_next_query((Cell*)cv, index, shard_id, seed, b_out);
}
int orc_cell_decode(void* cv, u64 index, const u64* a, const u64* b, uint8_t* record_out) {
  return cell_decode((const Cell*)cv, index, a, b, record_out) ? 1 : 0;
}
// Test Galois keys of the cell's secret: out = log d x rows x (a, b) x n words.
void orc_cell_galois_keys(void* cv, const uint8_t* seed, u64* out) {
  auto* c = (Cell*)cv;
  const auto keys = test_galois_keys(c->P, *c->pp->ntt, c->sk, seed);
  size_t k = 0;
  for (auto& m : keys)
    for (size_t r = 0; r < m.a.size(); r++) {
      memcpy(out + k * c->P.n, m.a[r].data(), c->P.n * 8);
      memcpy(out + (k + 1) * c->P.n, m.b[r].data(), c->P.n * 8);
      k += 2;
    }
}
int orc_cell_decode_tree(void* cv, u64 index, const u64* a, const u64* b, uint8_t* record_out) {
  return cell_decode_tree((const Cell*)cv, index, a, b, record_out) ? 1 : 0;
}
// The cell's Gaussian sampler stream: its ChaCha20 key and the 32-bit words consumed so far.
void orc_cell_sampler_state(void* cv, uint8_t* key_out, u64* word_pos) {
  auto* c = (Cell*)cv;
  const ChaCha20Rng& r = c->sampler.rng;
  memcpy(key_out, r.key, 32);
  *word_pos = r.idx >= 64 ? r.block * 16 : (r.block - 4) * 16 + r.idx;
}
// The cell's whole database (entries x entry_size bytes); returns its length.
u64 orc_cell_db(void* cv, uint8_t* out, u64 cap) {
  auto* c = (Cell*)cv;
  if (out) memcpy(out, c->db.data(), std::min<u64>(cap, c->db.size()));
  return c->db.size();
}
void orc_cell_record(void* cv, u64 index, uint8_t* out) {
  auto* c = (Cell*)cv;
  memcpy(out, &c->db[index * c->entry_size], c->entry_size);
}

}  // extern "C"
