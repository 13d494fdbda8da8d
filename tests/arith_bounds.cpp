// Host check of the lazy bounds the recursion kernels rely on, against exact 128-bit
// arithmetic (compiled and run by test_arith_cpu.py):
//   shoup_lazy4(a, w, w')  in [0, 4q) and = a w mod q, for any a < 2^64, w < q;
//   shoup_digit(a, w, w')  in [0, 3q) and = a w mod q, for any a < 2^32, w < q;
//   the butterflies built on it keep the forward's words below 8q and the inverse's
//   below 4q, and stay congruent to the exact butterflies;
//   redc_wide(x)           canonical and = x 2^-64 mod q, for x < 2q 2^64;
//   Prime32::shoupl(a, w, w') in [0, 2m) and = a w mod m, for the special_modulus primes.
#include <cstdio>
#include <cstdlib>

#include "ig_arith.cuh"
#include "ig_sm.cuh"

using namespace ig;

static u64 rng_state = 0x9E3779B97F4A7C15ULL;
static u64 next() {
  rng_state ^= rng_state << 13;
  rng_state ^= rng_state >> 7;
  rng_state ^= rng_state << 17;
  return rng_state;
}
static u64 mulmod(u64 a, u64 b) { return (u64)((u128)a * b % Q); }
static u64 powmod(u64 a, u64 e) {
  u64 r = 1;
  for (; e; e >>= 1, a = mulmod(a, a))
    if (e & 1) r = mulmod(r, a);
  return r;
}

static int fails = 0;
static void fail(const char* what, unsigned long long a, unsigned long long b) {
  if (fails++ < 5) std::printf("FAIL %s: %llx %llx\n", what, a, b);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  const u64 R_INV = powmod((u64)(((u128)1 << 64) % Q), Q - 2);  // 2^-64 mod q
  const u64 edges[] = {0, 1, Q - 1, Q, 2 * Q - 1, 4 * Q - 1, 8 * Q - 1, ~0ULL, ~0ULL - Q};
  for (long i = 0; i < n; i++) {
    const u64 w = i < 3 ? (u64)i : (i == 3 ? Q - 1 : next() % Q);
    const u64 wp = shoup_companion(w);
    const u64 a = i < 9 ? edges[i] : (i & 1 ? next() : next() % (8 * Q));
    const u64 v = shoup_lazy4(a, w, wp);
    if (v >= 4 * Q || v % Q != mulmod(a % Q, w)) fail("shoup_lazy4", a, w);
    // Digits: below 2^20 (exact gadget), below 2^24 (rounded), and any 32-bit word.
    const u32 dg = i < 4 ? (u32)(i == 0 ? 0 : i == 1 ? 0xFFFFFu : i == 2 ? 0xFFFFFFu : 0xFFFFFFFFu)
                         : (u32)(next() >> (i % 3 == 0 ? 44 : i % 3 == 1 ? 40 : 32));
    const u64 vd = shoup_digit(dg, w, wp);
    if (vd >= 3 * Q || vd % Q != mulmod(dg, w)) fail("shoup_digit", dg, w);

    // Forward butterfly on words below 8q (bf_fwd8), inverse on words below 4q (bf_inv4).
    const u64 X = next() % (8 * Q), Y = next() % (8 * Q);
    const u64 x = csub4(X), t = shoup_lazy4(Y, w, wp);
    const u64 X1 = x + t, Y1 = x - t + 4 * Q;
    if (X1 >= 8 * Q || Y1 >= 8 * Q) fail("bf_fwd8 bound", X, Y);
    if (X1 % Q != (X % Q + mulmod(Y % Q, w)) % Q || Y1 % Q != (X % Q + Q - mulmod(Y % Q, w)) % Q)
      fail("bf_fwd8 value", X, Y);
    const u64 U = next() % (4 * Q), V = next() % (4 * Q);
    const u64 u = csub4(U + V), d = shoup_lazy4(U - V + 4 * Q, w, wp);
    if (u >= 4 * Q || d >= 4 * Q) fail("bf_inv4 bound", U, V);
    if (u % Q != (U + V) % Q || d % Q != mulmod((U % Q + Q - V % Q) % Q, w)) fail("bf_inv4 value", U, V);

    // redc_wide over sums below 2q 2^64 (e.g. three products of words below 8q by words
    // below q, plus one below q^2).
    const u128 xw = ((u128)(next() % (2 * Q)) << 64) | next();
    const u64 r = redc_wide(xw);
    if (r >= Q || r != mulmod((u64)(xw % Q), R_INV)) fail("redc_wide", (u64)(xw >> 64), (u64)xw);
  }
  const uint32_t primes[] = {536813569u, 2147389441u, 536903681u, 1073750017u};
  for (uint32_t m : primes) {
    igsm::Prime32 P{m, 0};
    for (long i = 0; i < n / 4; i++) {
      const uint32_t w = i == 0 ? m - 1 : (uint32_t)(next() % m);
      const uint32_t wp = (uint32_t)(((u64)w << 32) / m);
      const uint32_t a = i == 1 ? 0xFFFFFFFFu : (uint32_t)next();
      const uint32_t v = P.shoupl(a, w, wp);
      if (v >= 2 * m || v % m != (uint32_t)((u64)a * w % m)) fail("Prime32::shoupl", a, w);
    }
  }
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
