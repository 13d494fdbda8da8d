// Exact arithmetic shared by the device kernels and the host-side set-up code.
//
// Modulus: q = 2^60 - 2^14 + 1 (DEFAULT_Q of the reference, src/math/mod_q.rs:7), the
// only ciphertext modulus of the d2048 parameter sets the respond path serves.
//
// Two product forms are used, both exact and canonical ([0, q) in, [0, q) out):
//   * Shoup (a * w mod q for a fixed w with companion w' = floor(w * 2^64 / q)): NTT
//     twiddles and scalar constants.
//   * Montgomery (a * b * 2^-64 mod q): products of a value in standard form with an
//     operand stored pre-multiplied by 2^64 ("R-form"). The packing store, the offline
//     key mask and the seated keys are held in R-form, so a product needs no conversion.
// NTT-domain values that vary per query stay in standard form.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define IG_HD __host__ __device__ __forceinline__
#else
#define IG_HD inline
#endif

namespace ig {

typedef uint64_t u64;
typedef uint32_t u32;
typedef unsigned __int128 u128;
typedef int64_t i64;

static constexpr u64 Q = 1152921504606830593ULL;  // 2^60 - 2^14 + 1
// -q^-1 mod 2^64
static constexpr u64 QINV_NEG = []() constexpr {
  u64 y = 1;
  for (int i = 1; i < 64; i++) y |= (y * Q) & (1ULL << i);
  return (u64)0 - y;
}();

IG_HD u64 mulhi(u64 a, u64 b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (u64)(((u128)a * b) >> 64);
#endif
}

IG_HD u64 csub(u64 x) { return x >= Q ? x - Q : x; }
IG_HD u64 addq(u64 a, u64 b) { return csub(a + b); }
IG_HD u64 subq(u64 a, u64 b) { return a >= b ? a - b : a + Q - b; }
IG_HD u64 negq(u64 a) { return a == 0 ? 0 : Q - a; }

// hi * q mod 2^64 with q's shape: (hi << 60) - (hi << 14) + hi.
IG_HD u64 mul_q_lo(u64 hi) { return (hi << 60) - (hi << 14) + hi; }

// q held in a register the compiler cannot see through, so est * q issues as an integer
// multiply (FMA pipe) rather than shifts and adds (ALU pipe).
IG_HD u64 q_opaque() {
#ifdef __CUDA_ARCH__
  u64 r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "l"(Q));
  return r;
#else
  return Q;
#endif
}

// a * w mod q up to one q: in [0, 2q) for any a < 2^64 (Shoup, w' = floor(w 2^64 / q)).
IG_HD u64 shoup_lazy(u64 a, u64 w, u64 wp) {
  const u64 est = mulhi(a, wp);
  return a * w - est * q_opaque();
}

// a * w mod q, w < q; any a < 2^64.
IG_HD u64 shoup(u64 a, u64 w, u64 wp) { return csub(shoup_lazy(a, w, wp)); }

IG_HD u32 mulhi32(u32 a, u32 b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (u32)(((u64)a * b) >> 32);
#endif
}

// a * w mod q up to three q: in [0, 4q) for any a < 2^64. The quotient estimate takes the
// high word of a * w' from three of its four 32-bit partial products: the high one whole
// and the high halves of the two middle ones; the low one is dropped. The three dropped
// fractions are each below one unit, so the estimate undershoots floor(a w' / 2^64) by
// at most 2, and a w - est q exceeds the exact Shoup remainder (below 2q) by at most 2q.
IG_HD u64 shoup_lazy4(u64 a, u64 w, u64 wp) {
  const u32 ah = (u32)(a >> 32), al = (u32)a, wh = (u32)(wp >> 32), wl = (u32)wp;
  const u64 est = (u64)ah * wh + mulhi32(ah, wl) + mulhi32(al, wh);
  return a * w - est * q_opaque();
}

// a * w mod q up to three q for a below 2^32 (a gadget digit). The quotient estimate is
// floor(a wh / 2^32), wh the high word of w'; the exact floor(a w' / 2^64) adds a wl / 2^64
// (below one unit, wl the low word) to a wh / 2^32, so the estimate undershoots it by at
// most 1 and a w - est q lies in [0, 3q).
IG_HD u64 shoup_digit(u32 a, u64 w, u64 wp) {
  const u64 est = mulhi32(a, (u32)(wp >> 32));
  return (u64)a * w - est * q_opaque();
}

// x - 2q when x >= 2q.
IG_HD u64 csub2(u64 x) { return x >= 2 * Q ? x - 2 * Q : x; }
// x - 4q when x >= 4q.
IG_HD u64 csub4(u64 x) { return x >= 4 * Q ? x - 4 * Q : x; }

// a * b * 2^-64 mod q for a, b < q.
IG_HD u64 mont(u64 a, u64 b) {
  u64 lo = a * b;
  u64 hi = mulhi(a, b);
  u64 m = lo * QINV_NEG;
  // (a*b + m*q) / 2^64; the low halves sum to 0 mod 2^64, carrying 1 unless both are 0.
  u64 t = hi + mulhi(m, Q) + (lo != 0 ? 1 : 0);
  return csub(t);
}

// Montgomery reduction of a 128-bit sum of products: x * 2^-64 mod q for x < q * 2^64
// (any sum of up to 15 products of words below q).
IG_HD u64 redc(u128 x) {
  const u64 lo = (u64)x, hi = (u64)(x >> 64);
  const u64 m = lo * QINV_NEG;
  return csub(hi + mulhi(m, Q) + (lo != 0 ? 1 : 0));
}

// The same for x < 2q * 2^64 (sums of products whose factors run up to 8q, such as
// transforms kept below 8q times words below q): the quotient lands below 3q.
IG_HD u64 redc_wide(u128 x) {
  const u64 lo = (u64)x, hi = (u64)(x >> 64);
  const u64 m = lo * QINV_NEG;
  return csub(csub2(hi + mulhi(m, Q) + (lo != 0 ? 1 : 0)));
}

IG_HD u128 wide(u64 a, u64 b) { return (u128)a * b; }

// Shoup companion floor(w * 2^64 / q).
IG_HD u64 shoup_companion(u64 w) { return (u64)(((u128)w << 64) / Q); }

// x mod q for any 128-bit x, using 2^60 == 2^14 - 1 (mod q).
IG_HD u64 reduce128(u128 x) {
  const u128 M60 = (((u128)1) << 60) - 1;
  x = (x >> 60) * ((((u128)1) << 14) - 1) + (x & M60);  // < 2^83
  x = (x >> 60) * ((((u128)1) << 14) - 1) + (x & M60);  // < 2^61
  u64 r = (u64)x;
  r = csub(r);
  return csub(r);
}

// ChaCha20 block (RFC 7539 quarter rounds, 64-bit counter in words 12-13 and 64-bit
// stream id in words 14-15), the keystream rand_chacha's ChaCha20Rng draws from.
IG_HD u32 rotl(u32 x, int r) { return (x << r) | (x >> (32 - r)); }

IG_HD void chacha20_block(const u32 key[8], u64 counter, u64 stream, u32 out[16]) {
  u32 s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
               key[4], key[5], key[6], key[7], (u32)counter, (u32)(counter >> 32), (u32)stream,
               (u32)(stream >> 32)};
  u32 x[16];
#pragma unroll
  for (int i = 0; i < 16; i++) x[i] = s[i];
#define IG_QR(a, b, c, d)                      \
  x[a] += x[b]; x[d] = rotl(x[d] ^ x[a], 16); \
  x[c] += x[d]; x[b] = rotl(x[b] ^ x[c], 12); \
  x[a] += x[b]; x[d] = rotl(x[d] ^ x[a], 8);  \
  x[c] += x[d]; x[b] = rotl(x[b] ^ x[c], 7);
#pragma unroll
  for (int i = 0; i < 10; i++) {
    IG_QR(0, 4, 8, 12) IG_QR(1, 5, 9, 13) IG_QR(2, 6, 10, 14) IG_QR(3, 7, 11, 15)
    IG_QR(0, 5, 10, 15) IG_QR(1, 6, 11, 12) IG_QR(2, 7, 8, 13) IG_QR(3, 4, 9, 14)
  }
#undef IG_QR
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}

// rand 0.8 gen_range(0..q) acceptance for u64: v * q = hi:lo, accept when lo <= zone,
// zone = (q << clz(q)) - 1.
static constexpr u64 RANGE_ZONE = (Q << 4) - 1;

}  // namespace ig
