// special_modulus respond path (reference src/special_modulus/): 32-bit words, ciphertext
// prime q below the special prime p < 2^31, Montgomery with R = 2^32 throughout.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace igsm {

typedef uint32_t u32;
typedef uint64_t u64;
typedef int64_t i64;

// x - k where x >= k, else x, for any 32-bit x and k: when x < k the difference wraps
// above x, so the smaller of the two is the answer.
__host__ __device__ __forceinline__ u32 csub_by(u32 x, u32 k) {
  const u32 d = x - k;
  return d < x ? d : x;
}

// Prime32 (arith.rs:13-102): canonical words, mont(a, b) = a b 2^-32 mod m.
struct Prime32 {
  u32 m, neg_minv;
  __host__ __device__ __forceinline__ u32 csub(u32 x) const { return csub_by(x, m); }
  __host__ __device__ __forceinline__ u32 add(u32 a, u32 b) const { return csub(a + b); }
  __host__ __device__ __forceinline__ u32 sub(u32 a, u32 b) const { return csub(a + m - b); }
  // a b 2^-32 mod m in [0, 2m), for any 32-bit a and b < m: a b + k m < 2^33 m.
  __host__ __device__ __forceinline__ u32 montl(u32 a, u32 b) const {
    const u64 t = (u64)a * b;
    const u32 k = (u32)t * neg_minv;
    return (u32)((t + (u64)k * m) >> 32);
  }
  __host__ __device__ __forceinline__ u32 mont(u32 a, u32 b) const { return csub(montl(a, b)); }
  // a w mod m in [0, 2m) for any 32-bit a and w < m, with w' = floor(w 2^32 / m) (Shoup):
  // one high and two low 32-bit multiplies, where montl takes two wide ones and a low one.
  __host__ __device__ __forceinline__ u32 shoupl(u32 a, u32 w, u32 wp) const {
#ifdef __CUDA_ARCH__
    const u32 est = __umulhi(a, wp);
#else
    const u32 est = (u32)(((u64)a * wp) >> 32);
#endif
    return a * w - est * m;
  }
  __host__ __device__ __forceinline__ u32 shoup(u32 a, u32 w, u32 wp) const { return csub(shoupl(a, w, wp)); }
  __host__ __device__ __forceinline__ u32 small(i64 x) const { return (u32)x + (m & (u32)(x >> 63)); }
  __host__ __device__ __forceinline__ i64 centred(u32 x) const { return x > (m >> 1) ? (i64)x - (i64)m : (i64)x; }
};

// One transform's constants: bit-reversed Montgomery-form powers of psi and psi^-1, and the
// two factors of the inverse's fused last stage (arith.rs:131-166).
struct Ntt32Dev {
  Prime32 p;
  const u32* fwd;
  const u32* inv;
  const uint2* fwd_sh;  // the forward ladder in standard form with Shoup companions (w, w')
  u32 n_inv, last;      // Montgomery form: 1/n, and 1/n times the inverse's last twiddle
  u32 n_inv_s, n_inv_sp, last_s, last_sp;  // the same two in standard form with companions
};

struct SmDev {
  u32 n, logn, gamma, nb;  // ring, packed width, body coefficients (2 * record bytes)
  Ntt32Dev lq, lp;
  const uint16_t* slot_exp;  // odd exponent of slot t's root relative to slot 0's (q transform)
  const uint16_t* exp_slot;  // slot of odd exponent e, at e / 2
  const u32* gpow;           // g^i mod 2n
  const u32* cpow;           // g^-i mod 2n
  const u32* m_of_i;         // (g^-i - 1) / (2n / gamma)
  const u32* pow_root_R;     // w0^e * 2^32 mod q, e < 2n (store fold)
  u32 inv_gamma_RR;          // gamma^-1 * 2^64 mod q: mont(x, .) = x gamma^-1 2^32
  u32 p_over_q, neg_off, p_inv_R;  // lifts between the limbs and 1/p mod q (R-form)
  u32 q_mu;                        // floor(2^32 / q), the Barrett factor of the lazy lift
};

struct SmQueryDev {
  const u32* seed;     // 8 ChaCha20 key words
  const u32* body;     // n words mod q
  const int8_t* values;  // the shard's nibbles, [row][gamma]
  const u32* step1_R;    // the shard's step-1 table, gamma x n, R-form
  const u32* seat;       // 4 x n: key_q, key_p, w_q, w_p (NTT, R-form)
  u32 rows;              // cells in the shard
  u32 reserved;
};

}  // namespace igsm

namespace igsmk {
using namespace igsm;

// Forward transforms of `rows` rows (mod q when which == 0, mod p when 1); with to_mont
// the outputs are multiplied by 2^32. Inputs are reduced mod the prime first.
cudaError_t ntt_rows(const SmDev& c, int which, const u32* in, u32* out, u32 rows, int to_mont, cudaStream_t s);
// Nibble columns (signed, low first) of `rows` cells of cell_bytes into values[row][gamma]
// and the columns' q-limb words colq[gamma][n] (rows past `rows` are zero).
cudaError_t table_columns(const SmDev& c, const uint8_t* cells, u32 rows, u32 cell_bytes, int8_t* values, u32* colq,
                          cudaStream_t s);
// Step-1 table from the columns' transforms (H: gamma x n standard form): per-slot DFT.
cudaError_t table_fold(const SmDev& c, const u32* H, u32* step1_R, cudaStream_t s);
// Body fold: fold[q][k] = sum_m c_m values[m][k] (c_0 = centred b_0, c_m = -centred b_{n-m}).
cudaError_t body_fold(const SmDev& c, const SmQueryDev* queries, u32 nq, i64* fold, cudaStream_t s);
// The 2n-step recursion and the final transforms; one CTA per query.
cudaError_t respond(const SmDev& c, const SmQueryDev* queries, u32 nq, const i64* fold, u32* mask_out, u32* body_out,
                    u32* status, cudaStream_t s);
}  // namespace igsmk
