// TEST INFRASTRUCTURE — part of the CPU oracle. Only tests/, __graft_entry__.smoke() and
// bench.py's cpu_baseline leg may load it, as the checker / CPU baseline; the product
// library never links it.
//
// Restatement, from their published specifications, of the third-party generators the
// reference draws from (the reference pins them in Cargo.lock):
//   * rand_chacha 0.3.1  ChaCha20Rng: 20-round ChaCha block function, 64-bit block
//     counter in state words 12-13, 64-bit stream id in words 14-15, results buffered
//     four blocks (64 words) at a time; next_u64 = two consecutive words, low first;
//     fill_bytes consumes whole words.
//   * rand_core 0.6.4    SeedableRng::seed_from_u64: PCG32 output words fill the seed.
//   * rand 0.8.6         gen_range over integer ranges (widening-multiply rejection with
//     the "zone" shortcut) and over an f64 half-open range (52 random mantissa bits).
// Call sites in the reference: src/math/poly.rs:657-686 (query `a` expansion),
// src/inspiring/inspiring2.rs:866-887 (mask expansion), src/math/gaussian.rs:210-224
// (sampler), src/special_modulus/mod.rs:216-237 (key mask).
// Pinned by the reference's sampler stream hashes (src/math/gaussian.rs:335-351) and by
// every byte-identity KAT replayed in tests/.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

typedef uint64_t u64;
typedef int64_t i64;
typedef unsigned __int128 u128;

static inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

struct ChaCha20Rng {
  uint32_t key[8];
  u64 block = 0;   // next block counter to generate
  u64 stream = 0;  // nonce words 14-15
  uint32_t buf[64];
  uint32_t idx = 64;  // 64 = buffer exhausted

  static ChaCha20Rng from_seed(const uint8_t seed[32]) {
    ChaCha20Rng r;
    for (int i = 0; i < 8; i++)
      r.key[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) |
                 ((uint32_t)seed[4 * i + 2] << 16) | ((uint32_t)seed[4 * i + 3] << 24);
    r.block = 0;
    r.stream = 0;
    r.idx = 64;
    return r;
  }

  // rand_core 0.6.4: PCG32 (MUL 6364136223846793005, INC 11634580027462260723),
  // state advanced before each output, XSH-RR output, little-endian words.
  static ChaCha20Rng seed_from_u64(u64 state) {
    uint8_t seed[32];
    for (int c = 0; c < 8; c++) {
      state = state * 6364136223846793005ULL + 11634580027462260723ULL;
      uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
      uint32_t rot = (uint32_t)(state >> 59);
      uint32_t x = (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
      memcpy(seed + 4 * c, &x, 4);
    }
    return from_seed(seed);
  }

  static void block_fn(const uint32_t key[8], u64 counter, u64 stream, uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                      key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                      (uint32_t)counter, (uint32_t)(counter >> 32),
                      (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    memcpy(x, s, sizeof x);
#define ORC_QR(a, b, c, d)             \
  x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16); \
  x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12); \
  x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);  \
  x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
    for (int i = 0; i < 10; i++) {
      ORC_QR(0, 4, 8, 12) ORC_QR(1, 5, 9, 13) ORC_QR(2, 6, 10, 14) ORC_QR(3, 7, 11, 15)
      ORC_QR(0, 5, 10, 15) ORC_QR(1, 6, 11, 12) ORC_QR(2, 7, 8, 13) ORC_QR(3, 4, 9, 14)
    }
#undef ORC_QR
    for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
  }

  void refill() {
    for (int b = 0; b < 4; b++) block_fn(key, block + b, stream, buf + 16 * b);
    block += 4;
  }

  // rand_chacha set_stream right after construction (the only way the reference uses
  // it): the buffer is empty, so only the nonce changes.
  void set_stream(u64 s) {
    if (idx != 64) {
      // Re-seek to the same word position under the new stream.
      u64 word_pos = (block - 4) * 16 + idx;
      stream = s;
      block = word_pos / 16;
      refill();
      idx = (uint32_t)(word_pos % 16);
      return;
    }
    stream = s;
  }

  uint32_t next_u32() {
    if (idx >= 64) {
      refill();
      idx = 0;
    }
    return buf[idx++];
  }

  u64 next_u64() {
    if (idx < 63) {
      u64 v = (u64)buf[idx] | ((u64)buf[idx + 1] << 32);
      idx += 2;
      return v;
    } else if (idx >= 64) {
      refill();
      idx = 2;
      return (u64)buf[0] | ((u64)buf[1] << 32);
    } else {
      u64 lo = buf[63];
      refill();
      idx = 1;
      return lo | ((u64)buf[0] << 32);
    }
  }

  void fill_bytes(uint8_t* dst, size_t len) {
    size_t done = 0;
    while (done < len) {
      if (idx >= 64) {
        refill();
        idx = 0;
      }
      size_t avail_words = 64 - idx;
      size_t want = len - done;
      size_t bytes = avail_words * 4 < want ? avail_words * 4 : want;
      for (size_t b = 0; b < bytes; b++) dst[done + b] = (uint8_t)(buf[idx + b / 4] >> (8 * (b % 4)));
      idx += (uint32_t)((bytes + 3) / 4);
      done += bytes;
    }
  }
};

static inline int clz64(u64 x) { return x ? __builtin_clzll(x) : 64; }

// rand 0.8: UniformInt::sample_single_inclusive over a 64-bit type. `range` is
// high - low + 1 computed in the unsigned type; 0 means the full domain.
static inline u64 uniform_u64_offset(ChaCha20Rng& rng, u64 range) {
  if (range == 0) return rng.next_u64();
  u64 zone = (range << clz64(range)) - 1;
  for (;;) {
    u64 v = rng.next_u64();
    u128 m = (u128)v * range;
    if ((u64)m <= zone) return (u64)(m >> 64);
  }
}

// gen_range(low..high) for u64 (half-open).
static inline u64 gen_range_u64(ChaCha20Rng& rng, u64 low, u64 high) {
  return low + uniform_u64_offset(rng, high - low);
}

// gen_range(low..=high) for i64.
static inline i64 gen_range_i64_inclusive(ChaCha20Rng& rng, i64 low, i64 high) {
  u64 range = (u64)high - (u64)low + 1;
  return (i64)((u64)low + uniform_u64_offset(rng, range));
}

// gen_range(0.0..1.0) for f64: 52 high bits of a u64 as the mantissa of [1,2), minus 1.
static inline double gen_f64_unit(ChaCha20Rng& rng) {
  for (;;) {
    u64 bits = (rng.next_u64() >> 12) | 0x3FF0000000000000ULL;
    double v;
    memcpy(&v, &bits, 8);
    double res = (v - 1.0) * 1.0 + 0.0;
    if (res < 1.0) return res;
  }
}

// Discrete Gaussian by rejection, restating src/math/gaussian.rs:34-36,100-117,210-224:
// tailcut = ceil(6 sigma); x uniform in [-tailcut, tailcut]; accept when the f64 bit
// pattern of exp(-x^2 / 2 sigma^2) exceeds that of a uniform u in [0,1).
struct GaussianSampler {
  double sigma;
  i64 tailcut;
  std::vector<u64> accept_bits;
  ChaCha20Rng rng;

  void build(double s, const ChaCha20Rng& r) {
    sigma = s;
    tailcut = (i64)std::ceil(s * 6.0);
    double two_s2 = 2.0 * s * s;
    accept_bits.clear();
    for (i64 x = -tailcut; x <= tailcut; x++) {
      double x_sq = (double)(x * x);
      double prob = std::exp(-x_sq / two_s2);
      u64 b;
      if (std::isnan(prob)) prob = 0.0;
      memcpy(&b, &prob, 8);
      accept_bits.push_back(b);
    }
    rng = r;
  }
  static GaussianSampler with_seed(double s, u64 seed) {
    GaussianSampler g;
    g.build(s, ChaCha20Rng::seed_from_u64(seed));
    return g;
  }
  i64 sample() {
    for (;;) {
      i64 x = gen_range_i64_inclusive(rng, -tailcut, tailcut);
      u64 threshold = accept_bits[(size_t)(x + tailcut)];
      double u = gen_f64_unit(rng);
      u64 ub;
      memcpy(&ub, &u, 8);
      if (threshold > ub) return x;
    }
  }
};

static inline u64 from_signed(i64 v, u64 q) {
  __int128 r = (__int128)v % (__int128)q;
  if (r < 0) r += q;
  return (u64)r;
}

static inline u64 fnv1a(const uint8_t* p, size_t n) {
  u64 h = 0xcbf29ce484222325ULL;
  for (size_t i = 0; i < n; i++) {
    h ^= p[i];
    h *= 0x00000100000001b3ULL;
  }
  return h;
}

}  // namespace orc
