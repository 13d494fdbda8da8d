// Kernels of the InspiRING respond path on sm_103a.
//
// Work map (reference call sites in src/):
//   ntt_rows      negacyclic forward NTT of many rows: the seat's key body
//                 (pir/session.rs:600-625), the offline mask rows
//                 (inspiring/inspiring2.rs:537-598) and a shard's columns before its
//                 store is folded (inspiring/shard_store.rs:139-144).
//   store_fold    step 1 of the offline phase folded over one shard's columns
//                 (inspiring/inspiring2.rs:964-1004 via shard_store.rs:145), computed per
//                 slot as a length-gamma cyclic DFT instead of gamma^2 monomial products.
//   shard_scan    the store's column check and b fold (shard_store.rs:197-264): one HBM
//                 pass over the queried shard's columns per query.
//   respond       one CTA per query: the query's `a` expansion (math/poly.rs:657-686),
//                 the store gather (shard_store.rs:282-342), the backward recursion
//                 (inspiring2.rs:1014-1085) with the online gather fused into each link
//                 (inspiring2.rs:1393-1485), the final inverse transforms and the 36-bit
//                 mod switch (pir/mod_switch.rs:148-176).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "ig_kernels.cuh"

namespace igk {
using namespace ig;

// ------------------------------------------------------------------------------------
// Negacyclic transforms in shared memory. Forward: Cooley-Tukey over the bit-reversed
// ladder psi^brv(m) (math/ntt.rs:600-623 order); inverse: Gentleman-Sande over the
// inverse ladder (math/ntt.rs:626-654) without the final n^-1, which consumers fold into
// their first use. Both are linear in standard form.
//
// Radix-4 transforms: each thread carries one 4-element unit through two
// consecutive stages in registers (N/4 threads), halving shared-memory round trips and
// barriers against a stage-per-barrier radix-2 schedule. Odd log n adds one radix-2 stage
// (first in the forward, last in the inverse). The butterflies are Harvey's lazy ones: the
// forward keeps words in [0, 4q) and the inverse in [0, 2q) (inputs canonical), reducing
// only where the bound requires; results agree with the reference transform mod q. The
// recursion kernels' per-link transforms use bf_fwd8 / bf_inv4 instead, whose products
// take one 32-bit multiply fewer and whose words stay below 8q and 4q.

// Forward CT butterfly on lazy words: X, Y < 4q in, both outputs < 4q.
__device__ __forceinline__ void bf_fwd(u64& X, u64& Y, u64 w, u64 wp) {
  const u64 x = csub2(X);
  const u64 t = shoup_lazy(Y, w, wp);
  X = x + t;
  Y = x - t + 2 * Q;
}

// Inverse GS butterfly: X, Y < 2q in, both outputs < 2q.
__device__ __forceinline__ void bf_inv(u64& X, u64& Y, u64 w, u64 wp) {
  const u64 u = csub2(X + Y);
  Y = shoup_lazy(X - Y + 2 * Q, w, wp);
  X = u;
}

// The same butterflies on shoup_lazy4 (one 32-bit multiply fewer per product), with the
// bounds doubled: the forward keeps words below 8q, the inverse below 4q.
__device__ __forceinline__ void bf_fwd8(u64& X, u64& Y, u64 w, u64 wp) {
  const u64 x = csub4(X);
  const u64 t = shoup_lazy4(Y, w, wp);
  X = x + t;
  Y = x - t + 4 * Q;
}
__device__ __forceinline__ void bf_inv4(u64& X, u64& Y, u64 w, u64 wp) {
  const u64 u = csub4(X + Y);
  Y = shoup_lazy4(X - Y + 4 * Q, w, wp);
  X = u;
}

template <int LOGN, int NT, int NB>
__device__ __forceinline__ void ntt_fwd_r4(u64* const (&x)[NB], const u64* tw, const u64* twp) {
  constexpr int N = 1 << LOGN, UPT = N / 4 / NT;
  static_assert(UPT >= 1 && (N / 4) % NT == 0, "whole radix-4 units per thread");
  const int tid = threadIdx.x;
  int s = 0;
  if (LOGN & 1) {
    constexpr int t = N / 2;
    const u64 w = tw[1], wp = twp[1];
#pragma unroll
    for (int r = 0; r < 2 * UPT; r++) {
      const int b = tid + r * NT;
#pragma unroll
      for (int k = 0; k < NB; k++) {
        u64 a = x[k][b], c = x[k][b + t];
        bf_fwd(a, c, w, wp);
        x[k][b] = a;
        x[k][b + t] = c;
      }
    }
    __syncthreads();
    s = 1;
  }
#pragma unroll 1
  for (; s < LOGN; s += 2) {
    const int t = N >> (s + 1), m = 1 << s, h = t >> 1;
#pragma unroll
    for (int uu = 0; uu < UPT; uu++) {
      const int u = tid + uu * NT;
      const int i = u / h, o = u - i * h;
      const int e0 = i * 2 * t + o;
      const u64 wa = tw[m + i], wap = twp[m + i];
      const u64 wb = tw[2 * m + 2 * i], wbp = twp[2 * m + 2 * i];
      const u64 wc = tw[2 * m + 2 * i + 1], wcp = twp[2 * m + 2 * i + 1];
#pragma unroll
      for (int k = 0; k < NB; k++) {
        u64 a0 = x[k][e0], a1 = x[k][e0 + h], a2 = x[k][e0 + t], a3 = x[k][e0 + t + h];
        bf_fwd(a0, a2, wa, wap);
        bf_fwd(a1, a3, wa, wap);
        bf_fwd(a0, a1, wb, wbp);
        bf_fwd(a2, a3, wc, wcp);
        x[k][e0] = a0;
        x[k][e0 + h] = a1;
        x[k][e0 + t] = a2;
        x[k][e0 + t + h] = a3;
      }
    }
    __syncthreads();
  }
}

// Inverse ladder entry m from the forward one: psi^-brv(m) = q - f[3*2^s - 1 - m] for m in
// [2^s, 2^(s+1)), and the Shoup companion of q - w is the bitwise complement of w's.
__device__ __forceinline__ void inv_twiddle(const u64* tw, const u64* twp, int m, u64& w, u64& wp) {
  const int s = 31 - __clz(m);
  const int mp = 3 * (1 << s) - 1 - m;
  w = Q - tw[mp];
  wp = ~twp[mp];
}

template <int LOGN, int NT, int NB>
__device__ __forceinline__ void ntt_inv_r4(u64* const (&x)[NB], const u64* tw, const u64* twp) {
  constexpr int N = 1 << LOGN, UPT = N / 4 / NT;
  static_assert(UPT >= 1 && (N / 4) % NT == 0, "whole radix-4 units per thread");
  const int tid = threadIdx.x;
  int s = 0;
#pragma unroll 1
  for (; s + 1 < LOGN; s += 2) {
    const int t = 1 << s, m = N >> (s + 1);
#pragma unroll
    for (int uu = 0; uu < UPT; uu++) {
      const int u = tid + uu * NT;
      const int B = u >> s, o = u & (t - 1);
      const int e0 = B * 4 * t + o;
      u64 w0, w0p, w1, w1p, w2, w2p;
      inv_twiddle(tw, twp, m + 2 * B, w0, w0p);
      inv_twiddle(tw, twp, m + 2 * B + 1, w1, w1p);
      inv_twiddle(tw, twp, (m >> 1) + B, w2, w2p);
#pragma unroll
      for (int k = 0; k < NB; k++) {
        u64 a0 = x[k][e0], a1 = x[k][e0 + t], a2 = x[k][e0 + 2 * t], a3 = x[k][e0 + 3 * t];
        bf_inv(a0, a1, w0, w0p);
        bf_inv(a2, a3, w1, w1p);
        bf_inv(a0, a2, w2, w2p);
        bf_inv(a1, a3, w2, w2p);
        x[k][e0] = a0;
        x[k][e0 + t] = a1;
        x[k][e0 + 2 * t] = a2;
        x[k][e0 + 3 * t] = a3;
      }
    }
    __syncthreads();
  }
  if (LOGN & 1) {
    constexpr int t = N / 2;
    u64 w, wp;
    inv_twiddle(tw, twp, 1, w, wp);
#pragma unroll
    for (int r = 0; r < 2 * UPT; r++) {
      const int b = tid + r * NT;
#pragma unroll
      for (int k = 0; k < NB; k++) {
        u64 a = x[k][b], c = x[k][b + t];
        bf_inv(a, c, w, wp);
        x[k][b] = a;
        x[k][b + t] = c;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------
// Batched forward NTT: one CTA per row.
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4) k_ntt_rows(CrsDev c, const u64* in, u64* out, u64 scale,
                                                              u64 scalep) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  extern __shared__ __align__(16) u64 sm[];
  u64* x = sm;
  u64* tw = sm + N;
  u64* twp = sm + 2 * N;
  const u64* row = in + (size_t)blockIdx.x * N;
  for (int k = threadIdx.x; k < N; k += NT) {
    x[k] = reduce128(row[k]);
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
  }
  __syncthreads();
  {
    u64* const bufs[1] = {x};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  u64* o = out + (size_t)blockIdx.x * N;
  for (int k = threadIdx.x; k < N; k += NT) o[k] = shoup(x[k], scale, scalep);
}

// ------------------------------------------------------------------------------------
// Store fold. For slot t with root w_t = w0^e_t, step 1 at rotation i reads
//   acc_i[t] = sum_j w_t^(j * c_i) H_j[t],  c_i = g^-i mod 2n = 1 + m_i * (2n/gamma),
// so with u_j = w0^(e_t j) H_j[t] and zeta = w0^(2n/gamma) (order gamma),
//   acc_i[t] = DFT_zeta(u)[(e_t * m_i) mod gamma].
// The sum lands at S_i[t'] with table_i[t'] = t, i.e. t' = slot of exponent c_i * e_t,
// scaled by gamma^-1 and stored in R-form.
constexpr int FOLD_TILE = 2048;
constexpr int FOLD_THREADS = 256;

template <int LOGN>
__global__ void __launch_bounds__(FOLD_THREADS) k_store_fold(CrsDev c, const u64* H, u64* sums_R, u32 SL) {
  constexpr int N = 1 << LOGN;
  constexpr u32 M2N = 2 * N - 1;
  extern __shared__ __align__(16) u64 sm[];
  const u32 gamma = c.gamma;
  const u32 tile = SL * gamma;   // SL slots per CTA, tile <= FOLD_TILE words
  u64* x = sm;                   // [slot][j]
  u64* pw = sm + FOLD_TILE;      // w0^e R-form, 2N words
  const u32 t0 = blockIdx.x * SL;
  u32 lg = 0;
  while ((1u << lg) < gamma) lg++;
  for (int k = threadIdx.x; k < 2 * N; k += FOLD_THREADS) pw[k] = c.pow_root_R[k];
  __syncthreads();
  for (u32 idx = threadIdx.x; idx < tile; idx += FOLD_THREADS) {
    const u32 j = idx / SL, s = idx % SL;
    const u32 t = t0 + s;
    const u32 e = c.slot_exp[t];
    const u64 h = H[(size_t)j * N + t];
    x[s * gamma + j] = mont(h, pw[(e * j) & M2N]);
  }
  __syncthreads();
  // Gentleman-Sande DFT of length gamma per slot, bit-reversed output.
  for (u32 len = gamma >> 1; len >= 1; len >>= 1) {
    const u32 half_total = SL * (gamma >> 1);
    for (u32 b = threadIdx.x; b < half_total; b += FOLD_THREADS) {
      const u32 s = b / (gamma >> 1);
      const u32 bb = b % (gamma >> 1);
      const u32 blk = bb / len, j = bb % len;
      const u32 i0 = s * gamma + blk * 2 * len + j;
      const u64 u = x[i0], v = x[i0 + len];
      x[i0] = addq(u, v);
      x[i0 + len] = mont(subq(u, v), pw[(j * (N / len)) & M2N]);
    }
    __syncthreads();
  }
  for (u32 idx = threadIdx.x; idx < tile; idx += FOLD_THREADS) {
    const u32 i = idx / SL, s = idx % SL;
    const u32 t = t0 + s;
    const u32 e = c.slot_exp[t];
    const u32 k = (e * c.m_of_i[i]) & (gamma - 1);
    const u32 kr = lg ? (__brev(k) >> (32 - lg)) : 0;
    const u64 val = x[s * gamma + kr];
    const u32 tp = c.exp_slot[((c.cpow[i] * e) & M2N) >> 1];
    sums_R[(size_t)i * N + tp] = shoup(val, c.inv_gamma_R, c.inv_gamma_Rp);
  }
}

// ------------------------------------------------------------------------------------
// Shard scan (shard_store.rs:197-264), split in two.
//
// Column tags (k_column_tags). Per word w_k of column j:
//   tag = sum_k lo32(w_k) key[2k] + hi32(w_k) key[2k+1]   (mod 2^61 - 1)
// The reference recomputes the tags from the caller's columns at every respond and refuses
// a shard whose columns no longer give the stored tags. Here the columns live in device
// memory the library owns and change only through its own calls (a shard upload or an
// encode), so the tags are recomputed once, at each such change, and compared with the
// stored ones: a mismatch marks the shard stale, and every later respond on it is refused
// with the reference's message until the store is rebuilt. The refusal stays at respond
// time; the tag check leaves the per-query scan.
//
// b fold (k_scan), per query and column j of its shard:
//   fold_j = sum_k w_k * b_rev[k],  b_rev[0] = b_0, b_rev[k] = -b_{n-k}   (mod q)
// = coeff0(b * h_j). Compact shards (every word below 2^16, kept as a u16 copy): the fold
// is a matrix-vector product of the column words with b_rev, whose words are split into
// two 32-bit limbs and staged once per CTA in shared memory. Every product w * limb is
// below 2^48, so a lane's 64-bit accumulators hold its 64 products per column exactly, and
// the limbs recombine into a 128-bit sum at the end: two 32x32->64 multiply-adds per
// 16-bit word. The vector layout V[k & 7][k >> 3] lets lane l read positions 8m..8m+7
// (m = l + 32 it) conflict-free while it reads the same positions of a column as one
// 16-byte word. Other shards take an exact 128-bit path over the u64 words.
//
// Work items: a CTA takes SCAN_COLS consecutive columns of one query (SCAN_ROWS per warp),
// item = query << 12 | chunk from a per-launch list, so queries of different widths share
// a launch; without a list CTA b takes query b / chunks, chunk b % chunks.
constexpr int SCAN_WARPS = 16;
constexpr int SCAN_ROWS = 4;
constexpr int SCAN_COLS = SCAN_WARPS * SCAN_ROWS;
constexpr int SCAN_STAGES = 2;
constexpr u64 TAG_PRIME = (1ULL << 61) - 1;

__device__ __forceinline__ u128 shfl_xor_u128(u128 v, int m) {
  u64 lo = (u64)v, hi = (u64)(v >> 64);
  lo = __shfl_xor_sync(0xffffffffu, lo, m);
  hi = __shfl_xor_sync(0xffffffffu, hi, m);
  return ((u128)hi << 64) | lo;
}

// Tags of `gamma` columns: one warp per column. With `expect` set, a tag that differs sets
// *mismatch instead of being written.
template <int LOGN>
__global__ void __launch_bounds__(256) k_column_tags(u32 gamma, const u64* cols, const u64* key, u64* tags_out,
                                                     const u64* expect, u32* mismatch) {
  constexpr int N = 1 << LOGN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const u32 j = blockIdx.x * (blockDim.x >> 5) + warp;
  if (j >= gamma) return;
  const u64* col = cols + (size_t)j * N;
  u128 tag = 0;
#pragma unroll 4
  for (int k = lane; k < N; k += 32) {
    const u64 w = col[k];
    const ulonglong2 kk = *reinterpret_cast<const ulonglong2*>(key + 2 * k);
    tag += (u128)(w & 0xffffffffULL) * kk.x + (u128)(w >> 32) * kk.y;
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) tag += shfl_xor_u128(tag, m);
  if (lane == 0) {
    u128 t = (tag & TAG_PRIME) + (tag >> 61);
    t = (t & TAG_PRIME) + (t >> 61);
    u64 tv = (u64)t;
    while (tv >= TAG_PRIME) tv -= TAG_PRIME;
    if (expect) {
      if (tv != expect[j]) atomicOr(mismatch, 1u);
    } else {
      tags_out[j] = tv;
    }
  }
}

// Shared memory of the compact path: the vector V, then per warp a ring of SCAN_STAGES
// steps of column chunks its lanes copy ahead (cp.async), so the next steps' loads are in
// flight while the current step's products run.
__host__ __device__ constexpr size_t scan_smem_bytes(int n) {
  return (size_t)n * 8 + (size_t)SCAN_WARPS * SCAN_STAGES * SCAN_ROWS * 32 * 16;
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned addr = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(addr), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// Sums eight per-lane values over the warp in nine 64-bit exchanges instead of forty:
// each step halves the values a lane keeps and doubles the lanes summed into them. On
// return, lane l holds the warp total of value ((l >> 4) & 1) * 4 + ((l >> 3) & 1) * 2 +
// ((l >> 2) & 1) in v[0].
__device__ __forceinline__ void warp_reduce8(u64 (&v)[8], int lane) {
  {
    const bool up = lane & 16;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const u64 send = up ? v[k] : v[k + 4];
      const u64 got = __shfl_xor_sync(0xffffffffu, send, 16);
      v[k] = (up ? v[k + 4] : v[k]) + got;
    }
  }
  {
    const bool up = lane & 8;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const u64 send = up ? v[k] : v[k + 2];
      const u64 got = __shfl_xor_sync(0xffffffffu, send, 8);
      v[k] = (up ? v[k + 2] : v[k]) + got;
    }
  }
  {
    const bool up = lane & 4;
    const u64 send = up ? v[0] : v[1];
    const u64 got = __shfl_xor_sync(0xffffffffu, send, 4);
    v[0] = (up ? v[1] : v[0]) + got;
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

template <int LOGN>
__global__ void __launch_bounds__(SCAN_WARPS * 32, 2) k_scan(CrsDev c, const QueryDev* queries, const ShardDev* shards,
                                                          const u32* work, u32 chunks, u64* b_fold, u32* status) {
  constexpr int N = 1 << LOGN, M = N / 8, ITER = M / 32;
  extern __shared__ __align__(16) uint4 scan_sm[];
  uint2* V = reinterpret_cast<uint2*>(scan_sm);  // [8][M]: b_rev[k] lo, hi
  u32 qi, chunk;
  if (work) {
    const u32 w = work[blockIdx.x];
    qi = w >> 12;
    chunk = w & 0xfff;
  } else {
    qi = blockIdx.x / chunks;
    chunk = blockIdx.x - qi * chunks;
  }
  const QueryDev qd = queries[qi];
  // b_rev in 32-bit limbs: every thread's loads of b issued first, beside the shard entry's.
  constexpr int PER = (N + SCAN_WARPS * 32 - 1) / (SCAN_WARPS * 32);
  u64 braw[PER];
#pragma unroll
  for (int j = 0; j < PER; j++) {
    const int k = threadIdx.x + j * SCAN_WARPS * 32;
    if (k < N) braw[j] = qd.b[k == 0 ? 0 : N - k];
  }
  const ShardDev sh = shards[qd.shard];
  const u32 gamma = qd.crs ? qd.crs->gamma : c.gamma;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const u32 j0 = chunk * SCAN_COLS + warp * SCAN_ROWS;
  const u64* b = qd.b;
  u64* fold_out = b_fold + qd.fold_off;
  if (chunk == 0 && threadIdx.x == 0 && sh.stale) atomicOr(status + qd.row, (u32)DEV_TAG_MISMATCH);
  const int rows = j0 < gamma ? min(SCAN_ROWS, (int)(gamma - j0)) : 0;

  if (sh.cols16) {
    const uint16_t* col = sh.cols16 + (size_t)j0 * N;
    uint4* ring = scan_sm + N / 2 + (size_t)warp * SCAN_STAGES * SCAN_ROWS * 32;
    // Lane l copies, for step it, the 16-byte chunk at positions 8m..8m+7 (m = l + 32 it)
    // of each of the warp's rows into its own ring slots.
    auto issue = [&](int it) {
      if (it < ITER) {
        uint4* dst = ring + (it % SCAN_STAGES) * SCAN_ROWS * 32 + lane;
        const int m = lane + 32 * it;
        for (int r = 0; r < rows; r++) cp_async16(dst + r * 32, col + (size_t)r * N + 8 * m);
      }
      cp_async_commit();
    };
#pragma unroll
    for (int it = 0; it < SCAN_STAGES - 1; it++) issue(it);
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int k = threadIdx.x + j * SCAN_WARPS * 32;
      if (k >= N) break;
      const u64 bv = k == 0 ? reduce128(braw[j]) : negq(reduce128(braw[j]));
      V[(k & 7) * M + (k >> 3)] = make_uint2((u32)bv, (u32)(bv >> 32));
    }
    __syncthreads();
    if (rows == 0) {
      asm volatile("cp.async.wait_all;\n" ::: "memory");
      return;
    }
    u64 acc[8];  // acc[2r] = low-limb sum of row r, acc[2r + 1] = high-limb sum
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = 0;
#pragma unroll 1
    for (int it = 0; it < ITER; it++) {
      issue(it + SCAN_STAGES - 1);
      cp_async_wait<SCAN_STAGES - 1>();  // step it's copies have landed
      const int m = lane + 32 * it;
      const uint4* src = ring + (it % SCAN_STAGES) * SCAN_ROWS * 32 + lane;
      uint4 w[SCAN_ROWS];
#pragma unroll
      for (int r = 0; r < SCAN_ROWS; r++) w[r] = r < rows ? src[r * 32] : make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int p = 0; p < 8; p++) {
        const uint2 v = V[p * M + m];
#pragma unroll
        for (int r = 0; r < SCAN_ROWS; r++) {
          const u32 word = p & 1 ? (((&w[r].x)[p >> 1]) >> 16) : (((&w[r].x)[p >> 1]) & 0xffffu);
          acc[2 * r] += (u64)word * v.x;
          acc[2 * r + 1] += (u64)word * v.y;
        }
      }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    warp_reduce8(acc, lane);
    // Lane l holds value x = ((l >> 4) & 1) 4 + ((l >> 3) & 1) 2 + ((l >> 2) & 1): row x / 2,
    // limb x & 1; a row's high limb sits four lanes above its low limb.
    const u64 hi = __shfl_down_sync(0xffffffffu, acc[0], 4);
    const int r = ((lane >> 4) & 1) * 2 + ((lane >> 3) & 1);
    if ((lane & 7) == 0 && r < rows) fold_out[j0 + r] = reduce128((u128)acc[0] + ((u128)hi << 32));
    return;
  }

#pragma unroll 1
  for (int r = 0; r < rows; r++) {
    const u32 j = j0 + r;
    const u64* col = sh.columns + (size_t)j * N;
    u128 flo = 0, fhi = 0;
#pragma unroll 4
    for (int k0 = lane * 2; k0 < N; k0 += 64) {
      const ulonglong2 w = *reinterpret_cast<const ulonglong2*>(col + k0);
      const u64 r0 = k0 == 0 ? reduce128(b[0]) : negq(reduce128(b[N - k0]));
      const u64 r1 = negq(reduce128(b[N - k0 - 1]));
      const u128 p0 = (u128)w.x * r0, p1 = (u128)w.y * r1;
      flo += (u128)(u64)p0 + (u64)p1;
      fhi += (p0 >> 64) + (p1 >> 64);
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      flo += shfl_xor_u128(flo, m);
      fhi += shfl_xor_u128(fhi, m);
    }
    if (lane == 0) {
      // fold = fhi * 2^64 + flo (mod q)
      const u64 r64 = (u64)((((u128)1) << 64) % Q);
      const u64 hq = reduce128(fhi), lq = reduce128(flo);
      fold_out[j] = reduce128((u128)hq * r64 + lq);
    }
  }
}

// ServerResponse wire on the device (respond.rs:111-176, tight codec poly.rs:166-225):
// `tmpl` is the response with zero coefficients (header, lengths and trailer already in
// place); byte k of a packed region takes bits [8k, 8k+8) of the coefficients laid end to
// end at `bits` each, least significant first. One thread per output byte; a coefficient at
// or above the modulus sets status bit 1 of its response.
__global__ void k_wire(const u64* a, const u64* b, u32 n, u32 retained, u32 bits, u64 modulus, const uint8_t* tmpl,
                       u32 len, u32 a_off, u32 a_bytes, u32 b_off, u32 b_bytes, uint8_t* out, u32* status) {
  const u32 r = blockIdx.y;
  const u32 k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= len) return;
  u32 v = tmpl[k];
  const u64* c = nullptr;
  u32 count = 0, byte = 0;
  if (k >= a_off && k < a_off + a_bytes) {
    c = a + (size_t)r * n, count = n, byte = k - a_off;
  } else if (k >= b_off && k < b_off + b_bytes) {
    c = b + (size_t)r * n, count = retained, byte = k - b_off;
  }
  if (c) {
    const u64 bit = (u64)byte * 8;
    const u32 i0 = (u32)(bit / bits), sh = (u32)(bit - (u64)i0 * bits);
    u64 x = c[i0] >> sh;
    if (c[i0] >= modulus) atomicOr(status + r, 1u);
    if (sh + 8 > bits && i0 + 1 < count) x |= c[i0 + 1] << (bits - sh);
    v |= (u32)(x & 0xff);
  }
  out[(size_t)r * len + k] = (uint8_t)v;
}

// encode_database's column split (pir/encode_db.rs:74-168) for one shard: column j, row k
// holds bytes 2j and 2j+1 of entry k little-endian (one byte when the entry ends there,
// zero past it), rows past `entries` are zero. Writes the u64 words and their u16 copy.
__global__ void k_encode_records(const uint8_t* rec, u32 entries, u32 entry_size, u32 n, u32 gamma, u64* cols,
                                 uint16_t* cols16) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)gamma * n) return;
  const u32 j = (u32)(idx / n), k = (u32)(idx % n);
  u32 v = 0;
  if (k < entries) {
    const uint8_t* e = rec + (size_t)k * entry_size;
    const u32 off = 2 * j;
    if (off + 1 < entry_size)
      v = (u32)e[off] | ((u32)e[off + 1] << 8);
    else if (off < entry_size)
      v = e[off];
  }
  cols[idx] = v;
  cols16[idx] = (uint16_t)v;
}

// Compact copy of a shard's columns: out[k] = w[k] when every word is below 2^16; any
// larger word sets *wide. Eight words per thread.
__global__ void k_compact16(const u64* cols, size_t groups, uint16_t* out, u32* wide) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= groups) return;
  const ulonglong2* src = reinterpret_cast<const ulonglong2*>(cols + 8 * g);
  u64 w[8];
  bool big = false;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const ulonglong2 v = src[k];
    w[2 * k] = v.x;
    w[2 * k + 1] = v.y;
    big |= (v.x | v.y) >> 16 != 0;
  }
  if (big) atomicOr(wide, 1u);
  uint4 o;
  o.x = (u32)w[0] | ((u32)w[1] << 16);
  o.y = (u32)w[2] | ((u32)w[3] << 16);
  o.z = (u32)w[4] | ((u32)w[5] << 16);
  o.w = (u32)w[6] | ((u32)w[7] << 16);
  reinterpret_cast<uint4*>(out)[g] = o;
}

// ------------------------------------------------------------------------------------
// Mod switch c' = floor((c q' + floor(q/2)) / q) mod q' (exact; q' < 2^62).
__device__ __forceinline__ u64 mod_switch_word(u64 cv, u64 qn) {
  const u128 x = (u128)cv * qn + (Q >> 1);
  u64 quo = (u64)(x >> 60);
  u128 r = x - (u128)quo * Q;
  while (r >= Q) {
    r -= Q;
    quo++;
  }
  return quo % qn;
}

// Rows X_0, X_1, X_2 (R-form, `stride` words apart) of a 3-digit gadget key, folded for
// digits whose third transform is derived, D_2 = base^-2 (R - D_0 - base D_1):
//   sum_k X_k D_k = D_0 (X_0 - base^-2 X_2) + D_1 (X_1 - base^-1 X_2) + R base^-2 X_2.
// The folded rows are R-form too; a consumer then needs neither D_2 nor its reduction.
// Every read precedes every write, so src may equal dst.
__device__ __forceinline__ void fold_gadget3(u64 ld_inv_R, u64 ld_c0_R, u64 ld_c1_R, const u64* src, u64* dst,
                                             int stride) {
  const u64 x0 = src[0], x1 = src[stride], x2 = src[2 * stride];
  const u64 f0 = addq(x0, mont(x2, ld_c0_R));
  const u64 f1 = addq(x1, mont(x2, ld_c1_R));
  const u64 f2 = mont(x2, ld_inv_R);
  dst[0] = f0;
  dst[stride] = f1;
  dst[2 * stride] = f2;
}

// The Galois keys ([key][digit][part][n], R-form NTT) folded in place by fold_gadget3.
__global__ void k_fold_gadget_keys(CrsDev c, u64* keys, u32 count) {
  const u32 n = c.n;
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;  // (key, part, coefficient)
  if (i >= count * 2 * n) return;
  const u32 key = i / (2 * n), r = i - key * 2 * n;
  u64* x = keys + (size_t)key * 6 * n + r;
  fold_gadget3(c.ld_inv_R, c.ld_c0_R, c.ld_c1_R, x, x, (int)(2 * n));
}

// Per-query constants into shared memory: forward ladder and slot tables of the ring (c),
// the mask rows of the query's parameter set (v) and the seat's key rows (both R-form NTT;
// with the exact gadget, folded by fold_gadget3).
template <int N, int NT>
__device__ __forceinline__ void stage_constants(const CrsDev& c, const SetView& v, const u64* yR, u64* tw, u64* twp,
                                                u64* Wm, u64* Y, uint16_t* e_tab, uint16_t* s_tab) {
  for (int k = threadIdx.x; k < N; k += NT) {
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
    e_tab[k] = c.slot_exp[k];
    s_tab[k] = c.exp_slot[k];
  }
  if (v.approx == 0) {
    for (int k = threadIdx.x; k < N; k += NT) {
      fold_gadget3(v.ld_inv_R, v.ld_c0_R, v.ld_c1_R, v.wmask_R + k, Wm + k, N);
      fold_gadget3(v.ld_inv_R, v.ld_c0_R, v.ld_c1_R, yR + k, Y + k, N);
    }
  } else {
    for (u32 k = threadIdx.x; k < v.rows * N; k += NT) {
      Wm[k] = v.wmask_R[k];
      Y[k] = yR[k];
    }
  }
}

// The query's `a` in coefficient form: the ChaCha20 keystream of its seed as u64 words
// in order, each accepted by rand's gen_range(0..q) rule (math/poly.rs:657-671). Block b
// of the stream yields words 8b..8b+7; a rejected word (probability ~2^-46) shifts every
// later coefficient, and the walk is then redone word by word. Ends with a barrier.
template <int N, int NT>
__device__ __forceinline__ void expand_a(const QueryDev& qd, u64* a, u32* status, u32 qi, int force_serial) {
  const int tid = threadIdx.x;
  bool rejected = false;
  if (qd.a) {
    for (int k = tid; k < N; k += NT) a[k] = reduce128(qd.a[k]);
  } else if (tid < N / 8) {
    u32 blk[16], key[8];
#pragma unroll
    for (int k = 0; k < 8; k++) key[k] = qd.seed[k];
    chacha20_block(key, (u64)tid, 0, blk);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const u64 v = (u64)blk[2 * k] | ((u64)blk[2 * k + 1] << 32);
      if (v * Q > RANGE_ZONE) rejected = true;
      a[tid * 8 + k] = mulhi(v, Q);
    }
  }
  if (__syncthreads_or(rejected || (force_serial && !qd.a))) {
    if (tid == 0) {
      u32 blk[16], key[8];
      for (int k = 0; k < 8; k++) key[k] = qd.seed[k];
      u64 have = ~0ULL, cand = 0;
      int filled = 0;
      const u64 limit = (u64)N + 65536;
      while (filled < N && cand < limit) {
        const u64 bi = cand >> 3;
        if (bi != have) {
          chacha20_block(key, bi, 0, blk);
          have = bi;
        }
        const int k = (int)(cand & 7);
        const u64 v = (u64)blk[2 * k] | ((u64)blk[2 * k + 1] << 32);
        if (v * Q <= RANGE_ZONE) a[filled++] = mulhi(v, Q);
        cand++;
      }
      if (filled < N) {
        atomicOr(status + qi, (u32)DEV_EXPAND_EXHAUSTED);
        for (; filled < N; filled++) a[filled] = 0;
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ u64 finish_a(const CrsDev& c, u64 x, u64 ms) {
  const u64 v = shoup(x, c.ninv, c.ninvp);
  return ms ? mod_switch_word(v, ms) : v;
}
__device__ __forceinline__ u64 finish_b(const CrsDev& c, u64 x, u32 t, u32 gamma, const u64* fold, u64 ms) {
  u64 v = shoup(x, c.ninv, c.ninvp);
  if (t < gamma) v = addq(v, fold[t]);
  return ms ? mod_switch_word(v, ms) : v;
}

// ------------------------------------------------------------------------------------
// Shared-memory position of word e of the one-CTA kernel's per-link transform buffers
// (8-byte words, 16 to a 128-byte bank row): bits 4 and 5 of e are XORed into bits 2 and 3,
// which puts every half-warp of the small-stride radix-4 passes (t = 4, 16 in the inverse;
// h = 4, 16 in the forward) on 16 distinct bank pairs. 2-word pairs stay contiguous and
// 16-byte aligned, and each 16-word row maps onto itself.
__device__ __forceinline__ int sw(int e) { return e ^ (((e >> 4) & 3) << 2); }

// ------------------------------------------------------------------------------------
// One CTA per query (batches that fill the GPU). Thread u owns slots 4u..4u+3 of every
// NTT-domain vector (one transform unit). Each link of the recursion (i from gamma-2 down
// to 0) holds R_{i+1} in NTT form (`cur`, in registers):
//   r = INTT(R_{i+1});  d_k = base-2^20 digits of r (rounded, top carry kept, when the
//   lowest digit is dropped);  D_k = NTT(d_k);
//   sum_b += sum_k Y_k[tau_i(t)] D_k[t];
//   R_i[t] = a_ntt[tau_i(t)] S_i[t] + sum_k W_k[tau_i(t)] D_k[t]
// with tau_i the slot permutation of the automorphism X -> X^(g^i), S the packing store,
// W the mask rows and Y the seat. Each sum of products takes one Montgomery reduction.
// The inverse's first two stages and the forward's last two act within each thread's unit
// and run in registers; the inverse's last stage, n^-1, the digit split and the forward's
// first stage fuse into one pass. Digits 0 and 1 are transformed; with the exact gadget
// digit 2's transform is D_2 = base^-2 (R_{i+1} - D_0 - base D_1) (inspiring2.rs:1094-1161),
// a fixed linear combination, so the key rows are folded at staging (fold_gadget3) and
// R_{i+1} takes digit 2's place in the sums.
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4, 1)
    k_respond(CrsDev c, const QueryDev* queries, const ShardDev* shards, const u64* b_fold, u64* a_out, u64* b_out,
              u32* status, int force_serial) {
  constexpr int N = 1 << LOGN, NT = N / 4, H = N / 2;
  constexpr u32 M2N = 2 * N - 1;
  constexpr u64 DMASK = (1ULL << 20) - 1;
  extern __shared__ __align__(16) u64 sm[];
  u64* X = sm;       // N: the inverse in progress
  u64* D = sm + N;   // 2N: digits 0 and 1 (forward in progress)
  u64* a_ntt = D + 2 * N;
  u64* tw = a_ntt + N;
  u64* twp = tw + N;
  // Room for three key rows whatever the query's gadget, so queries of different sets
  // share a launch.
  u64* Wm = twp + N;
  u64* Y = Wm + 3 * N;
  uint16_t* e_tab = reinterpret_cast<uint16_t*>(Y + 3 * N);
  uint16_t* s_tab = e_tab + N;

  const int tid = threadIdx.x;
  const QueryDev qd = queries[blockIdx.x];
  const u32 qi = qd.row;  // output and status row
  const ShardDev sh = shards[qd.shard];
  const SetView ps = set_view(c, qd.crs);
  const u32 gamma = ps.gamma;
  const bool exact = ps.approx == 0;
  const int l0 = 4 * tid;

  stage_constants<N, NT>(c, ps, qd.seat_R, tw, twp, Wm, Y, e_tab, s_tab);
  expand_a<N, NT>(qd, a_ntt, status, qi, force_serial);
  {
    u64* const bufs[1] = {a_ntt};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }

  u64 cur[4], sb[4];
  u32 et[4];
#pragma unroll
  for (int k = 0; k < 4; k++) et[k] = e_tab[l0 + k];
  {
    const u32 gp = ps.gpow[gamma - 1];
    const u64* Srow = sh.sums_R + (size_t)(gamma - 1) * N;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const u32 tb = s_tab[((gp * et[k]) & M2N) >> 1];
      cur[k] = mont(a_ntt[tb], Srow[l0 + k]);
      sb[k] = 0;
    }
  }
  constexpr int MF = 1 << (LOGN - 2);
  const u64 wf = tw[1], wfp = twp[1];
#pragma unroll 1
  for (int i = (int)gamma - 2; i >= 0; i--) {
    const u64* Srow = sh.sums_R + (size_t)i * N + l0;
    const ulonglong2 sv01 = *reinterpret_cast<const ulonglong2*>(Srow);
    const ulonglong2 sv23 = *reinterpret_cast<const ulonglong2*>(Srow + 2);
    const u32 gp = ps.gpow[i];
    {
      // Inverse stages 0-1 of unit tid (block B = tid, m = N/2).
      u64 w0, w0p, w1, w1p, w2, w2p;
      inv_twiddle(tw, twp, H + 2 * tid, w0, w0p);
      inv_twiddle(tw, twp, H + 2 * tid + 1, w1, w1p);
      inv_twiddle(tw, twp, H / 2 + tid, w2, w2p);
      u64 a0 = cur[0], a1 = cur[1], a2 = cur[2], a3 = cur[3];
      bf_inv4(a0, a1, w0, w0p);
      bf_inv4(a2, a3, w1, w1p);
      bf_inv4(a0, a2, w2, w2p);
      bf_inv4(a1, a3, w2, w2p);
      *reinterpret_cast<ulonglong2*>(X + sw(l0)) = make_ulonglong2(a0, a1);
      *reinterpret_cast<ulonglong2*>(X + sw(l0 + 2)) = make_ulonglong2(a2, a3);
    }
    __syncthreads();
    // Inverse stages 2 .. logn-2 (radix-4 pairs, a radix-2 stage last when logn is even).
    int s = 2;
#pragma unroll 1
    for (; s + 1 <= LOGN - 2; s += 2) {
      const int t = 1 << s, m = N >> (s + 1);
      const int B = tid >> s, o = tid & (t - 1);
      const int e0 = B * 4 * t + o;
      u64 w0, w0p, w1, w1p, w2, w2p;
      inv_twiddle(tw, twp, m + 2 * B, w0, w0p);
      inv_twiddle(tw, twp, m + 2 * B + 1, w1, w1p);
      inv_twiddle(tw, twp, (m >> 1) + B, w2, w2p);
      u64 a0 = X[sw(e0)], a1 = X[sw(e0 + t)], a2 = X[sw(e0 + 2 * t)], a3 = X[sw(e0 + 3 * t)];
      bf_inv4(a0, a1, w0, w0p);
      bf_inv4(a2, a3, w1, w1p);
      bf_inv4(a0, a2, w2, w2p);
      bf_inv4(a1, a3, w2, w2p);
      X[sw(e0)] = a0;
      X[sw(e0 + t)] = a1;
      X[sw(e0 + 2 * t)] = a2;
      X[sw(e0 + 3 * t)] = a3;
      __syncthreads();
    }
    if (s == LOGN - 2) {
      const int t = 1 << s, m = N >> (s + 1);
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int v = tid + r * NT;
        const int B = v >> s, o = v & (t - 1);
        const int e = B * 2 * t + o;
        u64 w, wp;
        inv_twiddle(tw, twp, m + B, w, wp);
        u64 a = X[sw(e)], b = X[sw(e + t)];
        bf_inv4(a, b, w, wp);
        X[sw(e)] = a;
        X[sw(e + t)] = b;
      }
      __syncthreads();
    }
    // Inverse stage logn-1, n^-1, digit split and forward stage 0, per pair (b, b + N/2).
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int b = tid + j * NT;
      const u64 x0 = X[sw(b)], x1 = X[sw(b + H)];
      // The inverse's last stage and n^-1 as one product per output: n^-1 on the sum,
      // n^-1 times the stage's twiddle on the difference.
      const u64 r0 = shoup(x0 + x1, c.ninv, c.ninvp), r1 = shoup(x0 - x1 + 4 * Q, c.nlast, c.nlastp);
      u64 p0, p1, q0, q1;  // digits 0 and 1 of coefficients b and b + N/2
      if (exact) {
        p0 = r0 & DMASK;
        p1 = (r0 >> 20) & DMASK;
        q0 = r1 & DMASK;
        q1 = (r1 >> 20) & DMASK;
      } else {
        const u64 rr0 = (r0 + (1ULL << 19)) >> 20, rr1 = (r1 + (1ULL << 19)) >> 20;
        p0 = rr0 & DMASK;
        p1 = rr0 >> 20;
        q0 = rr1 & DMASK;
        q1 = rr1 >> 20;
      }
      const u64 t0 = shoup_digit((u32)q0, wf, wfp), t1 = shoup_digit((u32)q1, wf, wfp);
      D[sw(b)] = p0 + t0;
      D[sw(b + H)] = p0 + 4 * Q - t0;
      D[N + sw(b)] = p1 + t1;
      D[N + sw(b + H)] = p1 + 4 * Q - t1;
    }
    __syncthreads();
    // Forward stages 1 .. logn-3 (a radix-2 stage first when logn is even), both digits.
    s = 1;
    if (!(LOGN & 1)) {
      const int lt = LOGN - 2, t = 1 << lt;
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int v = tid + r * NT;
        const int ib = v >> lt, o = v & (t - 1);
        const int e = ib * 2 * t + o;
        const u64 w = tw[2 + ib], wp = twp[2 + ib];
#pragma unroll
        for (int k = 0; k < 2; k++) {
          u64* x = D + k * N;
          u64 a = x[sw(e)], b = x[sw(e + t)];
          bf_fwd8(a, b, w, wp);
          x[sw(e)] = a;
          x[sw(e + t)] = b;
        }
      }
      __syncthreads();
      s = 2;
    }
#pragma unroll 1
    for (; s < LOGN - 2; s += 2) {
      const int t = N >> (s + 1), m = 1 << s, h = t >> 1;
      const int ib = tid / h, o = tid - ib * h;
      const int e0 = ib * 2 * t + o;
      const u64 wa = tw[m + ib], wap = twp[m + ib];
      const u64 wb = tw[2 * m + 2 * ib], wbp = twp[2 * m + 2 * ib];
      const u64 wc = tw[2 * m + 2 * ib + 1], wcp = twp[2 * m + 2 * ib + 1];
      const int i0 = sw(e0), i1 = sw(e0 + h), i2 = sw(e0 + t), i3 = sw(e0 + t + h);
      u64* x0 = D;
      u64* x1 = D + N;
      u64 a0 = x0[i0], a1 = x0[i1], a2 = x0[i2], a3 = x0[i3];
      u64 c0 = x1[i0], c1 = x1[i1], c2 = x1[i2], c3 = x1[i3];
      bf_fwd8(a0, a2, wa, wap);
      bf_fwd8(c0, c2, wa, wap);
      bf_fwd8(a1, a3, wa, wap);
      bf_fwd8(c1, c3, wa, wap);
      bf_fwd8(a0, a1, wb, wbp);
      bf_fwd8(c0, c1, wb, wbp);
      bf_fwd8(a2, a3, wc, wcp);
      bf_fwd8(c2, c3, wc, wcp);
      x0[i0] = a0;
      x0[i1] = a1;
      x0[i2] = a2;
      x0[i3] = a3;
      x1[i0] = c0;
      x1[i1] = c1;
      x1[i2] = c2;
      x1[i3] = c3;
      __syncthreads();
    }
    // Forward stages logn-2, logn-1 of unit tid, both digits, in registers.
    u64 d0[4], d1[4];
    {
      const u64 fa = tw[MF + tid], fap = twp[MF + tid];
      const u64 fb = tw[2 * MF + 2 * tid], fbp = twp[2 * MF + 2 * tid];
      const u64 fc = tw[2 * MF + 2 * tid + 1], fcp = twp[2 * MF + 2 * tid + 1];
      const ulonglong2 v01 = *reinterpret_cast<const ulonglong2*>(D + sw(l0));
      const ulonglong2 v23 = *reinterpret_cast<const ulonglong2*>(D + sw(l0 + 2));
      const ulonglong2 g01 = *reinterpret_cast<const ulonglong2*>(D + N + sw(l0));
      const ulonglong2 g23 = *reinterpret_cast<const ulonglong2*>(D + N + sw(l0 + 2));
      d0[0] = v01.x, d0[1] = v01.y, d0[2] = v23.x, d0[3] = v23.y;
      d1[0] = g01.x, d1[1] = g01.y, d1[2] = g23.x, d1[3] = g23.y;
      bf_fwd8(d0[0], d0[2], fa, fap);
      bf_fwd8(d1[0], d1[2], fa, fap);
      bf_fwd8(d0[1], d0[3], fa, fap);
      bf_fwd8(d1[1], d1[3], fa, fap);
      bf_fwd8(d0[0], d0[1], fb, fbp);
      bf_fwd8(d1[0], d1[1], fb, fbp);
      bf_fwd8(d0[2], d0[3], fc, fcp);
      bf_fwd8(d1[2], d1[3], fc, fcp);
    }
    const u64 sv[4] = {sv01.x, sv01.y, sv23.x, sv23.y};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const u32 tb = s_tab[((gp * et[k]) & M2N) >> 1];
      u128 nb = wide(d0[k], Y[tb]) + wide(d1[k], Y[N + tb]);
      u128 nc = wide(a_ntt[tb], sv[k]) + wide(d0[k], Wm[tb]) + wide(d1[k], Wm[N + tb]);
      if (exact) {  // the rows are folded: R_{i+1} stands in for digit 2
        nb += wide(cur[k], Y[2 * N + tb]);
        nc += wide(cur[k], Wm[2 * N + tb]);
      }
      sb[k] = addq(sb[k], redc_wide(nb));
      cur[k] = redc_wide(nc);
    }
  }
  __syncthreads();  // every thread is past its last read of D
#pragma unroll
  for (int k = 0; k < 4; k++) {
    D[l0 + k] = cur[k];
    D[N + l0 + k] = sb[k];
  }
  __syncthreads();
  {
    u64* const bufs[2] = {D, D + N};
    ntt_inv_r4<LOGN, NT, 2>(bufs, tw, twp);
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int t = tid + k * NT;
    a_out[(size_t)qi * N + t] = finish_a(c, D[t], qd.ms);
    b_out[(size_t)qi * N + t] = finish_b(c, D[N + t], t, gamma, b_fold + qd.fold_off, qd.ms);
  }
}

// ------------------------------------------------------------------------------------
// Split transforms for the two-CTA kernel. The inverse (Gentleman-Sande, from t = 1
// upward) combines indices within blocks of growing size: its stages 0 .. logn-2 stay
// inside each half of N/2 words, and only the last stage (t = N/2) mixes the halves. The
// forward (Cooley-Tukey, from t = N/2 downward) mixes the halves in its first stage only.
// So each CTA of a pair runs the local stages on the half of the slots it owns, and the
// two cross stages run once per link, fused with the digit split. Unit and butterfly
// numbering is the full transform's, so the twiddles are the full transform's.

// The same split holds for R parts of N/R words: the inverse's stages 0 .. logn-1-log R and
// the forward's stages log R .. logn-1 stay inside a part. The helpers below run a local
// pass on the part of rank `rank` of a cluster of R CTAs (R = 2 or 4).

// Inverse radix-4 pass (stages s, s+1) over this CTA's part xp (N/R words, local index);
// threads below N/(4R) carry one unit each. Ends with a barrier.
template <int LOGN, int R>
__device__ __forceinline__ void inv_part_r4(u64* xp, int s, int rank, const u64* tw, const u64* twp) {
  constexpr int N = 1 << LOGN, P = N / R, PU = P / 4;
  const int tid = threadIdx.x;
  if (tid < PU) {
    const int u = rank * PU + tid;
    const int t = 1 << s, m = N >> (s + 1);
    const int B = u >> s, o = u & (t - 1);
    const int e0 = B * 4 * t + o - rank * P;
    u64 w0, w0p, w1, w1p, w2, w2p;
    inv_twiddle(tw, twp, m + 2 * B, w0, w0p);
    inv_twiddle(tw, twp, m + 2 * B + 1, w1, w1p);
    inv_twiddle(tw, twp, (m >> 1) + B, w2, w2p);
    u64 a0 = xp[sw(e0)], a1 = xp[sw(e0 + t)], a2 = xp[sw(e0 + 2 * t)], a3 = xp[sw(e0 + 3 * t)];
    bf_inv4(a0, a1, w0, w0p);
    bf_inv4(a2, a3, w1, w1p);
    bf_inv4(a0, a2, w2, w2p);
    bf_inv4(a1, a3, w2, w2p);
    xp[sw(e0)] = a0;
    xp[sw(e0 + t)] = a1;
    xp[sw(e0 + 2 * t)] = a2;
    xp[sw(e0 + 3 * t)] = a3;
  }
  __syncthreads();
}

// Inverse radix-2 stage s over this CTA's part (the last local stage when their count is
// odd); one butterfly per thread below N/(2R). Ends with a barrier.
template <int LOGN, int R>
__device__ __forceinline__ void inv_part_r2(u64* xp, int s, int rank, const u64* tw, const u64* twp) {
  constexpr int N = 1 << LOGN, P = N / R;
  if ((int)threadIdx.x < P / 2) {
    const int v = rank * (P / 2) + (int)threadIdx.x;
    const int t = 1 << s, m = N >> (s + 1);
    const int B = v >> s, o = v & (t - 1);
    const int e = B * 2 * t + o - rank * P;
    u64 w, wp;
    inv_twiddle(tw, twp, m + B, w, wp);
    u64 a = xp[sw(e)], b = xp[sw(e + t)];
    bf_inv4(a, b, w, wp);
    xp[sw(e)] = a;
    xp[sw(e + t)] = b;
  }
  __syncthreads();
}

// Forward radix-4 pass (stages s, s+1; s >= log R) over this CTA's part of two buffers
// D[0..P) and D[P..2P), P = N/R; one unit per thread below N/(2R). Ends with a barrier.
template <int LOGN, int R>
__device__ __forceinline__ void fwd_part_r4(u64* D, int s, int rank, const u64* tw, const u64* twp) {
  constexpr int N = 1 << LOGN, P = N / R, PU = P / 4;
  const int tid = threadIdx.x;
  if (tid < 2 * PU) {
    u64* x = D + (tid >= PU ? P : 0);
    const int u = rank * PU + (tid & (PU - 1));
    const int lt = LOGN - s - 1;  // log2 t
    const int t = 1 << lt, m = 1 << s, h = t >> 1;
    const int i = u >> (lt - 1), o = u & (h - 1);
    const int e0 = i * 2 * t + o - rank * P;
    const u64 wa = tw[m + i], wap = twp[m + i];
    const u64 wb = tw[2 * m + 2 * i], wbp = twp[2 * m + 2 * i];
    const u64 wc = tw[2 * m + 2 * i + 1], wcp = twp[2 * m + 2 * i + 1];
    u64 a0 = x[sw(e0)], a1 = x[sw(e0 + h)], a2 = x[sw(e0 + t)], a3 = x[sw(e0 + t + h)];
    bf_fwd8(a0, a2, wa, wap);
    bf_fwd8(a1, a3, wa, wap);
    bf_fwd8(a0, a1, wb, wbp);
    bf_fwd8(a2, a3, wc, wcp);
    x[sw(e0)] = a0;
    x[sw(e0 + h)] = a1;
    x[sw(e0 + t)] = a2;
    x[sw(e0 + t + h)] = a3;
  }
  __syncthreads();
}

// Forward radix-2 stage s over this CTA's part of both buffers (when the local stages are
// odd in number); one butterfly per buffer per thread below N/(2R). Ends with a barrier.
template <int LOGN, int R>
__device__ __forceinline__ void fwd_part_r2(u64* D, int s, int rank, const u64* tw, const u64* twp) {
  constexpr int N = 1 << LOGN, P = N / R;
  if ((int)threadIdx.x < P / 2) {
    const int v = rank * (P / 2) + (int)threadIdx.x;
    const int lt = LOGN - s - 1;
    const int t = 1 << lt, m = 1 << s;
    const int i = v >> lt, o = v & (t - 1);
    const int e = i * 2 * t + o - rank * P;
    const u64 w = tw[m + i], wp = twp[m + i];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      u64* x = D + k * P;
      u64 a = x[sw(e)], b = x[sw(e + t)];
      bf_fwd8(a, b, w, wp);
      x[sw(e)] = a;
      x[sw(e + t)] = b;
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------
// Two CTAs per query (a thread-block cluster), for batches that leave SMs idle with one
// CTA each. CTA r owns slots [r N/2, (r+1) N/2) of every NTT-domain vector. Per link:
//   own half of R_{i+1} -> local inverse stages -> cluster barrier -> cross stage over
//   (own half, peer's half read through distributed shared memory), n^-1, digit split and
//   the forward cross stage, keeping this CTA's half of digits 0 and 1 -> local forward
//   stages -> pointwise at own slots.
// Thread pair (2u, 2u+1) owns local slots 4u..4u+3, two each: the first inverse pass
// (stages 0 and 1, one 4-slot unit) and the last forward pass (same units, one digit per
// lane) run in registers with one lane exchange, next to the pointwise link.
// One cluster barrier per link: the exchange buffer X alternates between two halves by
// link parity, so a CTA rewrites the half its peer read at link i only at link i-2, after
// both passed the barrier of link i-1. With the exact gadget the third digit's transform
// comes from the other two: D_2 = base^-2 (R_{i+1} - D_0 - base D_1)
// (inspiring2.rs:1094-1161).
template <int LOGN>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__((1 << LOGN) / 4, 1)
    k_respond_pair(CrsDev c, const QueryDev* queries, const ShardDev* shards, const u64* b_fold, u64* a_out,
                   u64* b_out, u32* status, int force_serial) {
  namespace cg = cooperative_groups;
  constexpr int N = 1 << LOGN, NT = N / 4, H = N / 2, HU = N / 8;
  constexpr u32 M2N = 2 * N - 1;
  constexpr u64 DMASK = (1ULL << 20) - 1;
  extern __shared__ __align__(16) u64 sm[];
  u64* X = sm;      // [2][H] own half of the inverse, by link parity
  u64* D = sm + N;  // [2][H] own half of the transformed digits 0 and 1; N words at the end
  u64* a_ntt = D + N;
  u64* tw = a_ntt + N;
  u64* twp = tw + N;
  u64* Wm = twp + N;  // room for three key rows, as in k_respond
  u64* Y = Wm + 3 * N;
  uint16_t* e_tab = reinterpret_cast<uint16_t*>(Y + 3 * N);
  uint16_t* s_tab = e_tab + N;

  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const u64* peerX = cluster.map_shared_rank(X, rank ^ 1);
  const int tid = threadIdx.x;
  const QueryDev qd = queries[blockIdx.x >> 1];
  const u32 qi = qd.row;  // output and status row
  const ShardDev sh = shards[qd.shard];
  const SetView ps = set_view(c, qd.crs);
  const u32 gamma = ps.gamma;
  const bool exact = ps.approx == 0;
  const int own = rank * H, other = (rank ^ 1) * H;
  const int u = tid >> 1, dg = tid & 1;
  const int ls = 4 * u + 2 * dg;  // local slots ls, ls + 1
  const int ug = rank * HU + u;   // global unit index of slots 4u..4u+3

  stage_constants<N, NT>(c, ps, qd.seat_R, tw, twp, Wm, Y, e_tab, s_tab);
  expand_a<N, NT>(qd, a_ntt, status, qi, force_serial);
  {
    u64* const bufs[1] = {a_ntt};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  u64 cur[2], sb[2];
  u32 et[2];
#pragma unroll
  for (int k = 0; k < 2; k++) et[k] = e_tab[own + ls + k];
  {
    const u32 gp = ps.gpow[gamma - 1];
    const u64* Srow = sh.sums_R + (size_t)(gamma - 1) * N;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const u32 tb = s_tab[((gp * et[k]) & M2N) >> 1];
      cur[k] = mont(a_ntt[tb], Srow[own + ls + k]);
      sb[k] = 0;
    }
  }
  // Twiddles of the register passes: inverse stages 0-1 of unit ug, forward stages
  // logn-2, logn-1 of unit ug (fixed per thread).
  u64 wl1, wl1p, wl2, wl2p;
  inv_twiddle(tw, twp, H + 2 * ug + dg, wl1, wl1p);
  inv_twiddle(tw, twp, H / 2 + ug, wl2, wl2p);
  constexpr int MF = 1 << (LOGN - 2);
  const u64 fa = tw[MF + ug], fap = twp[MF + ug];
  const u64 fb = tw[2 * MF + 2 * ug], fbp = twp[2 * MF + 2 * ug];
  const u64 fc = tw[2 * MF + 2 * ug + 1], fcp = twp[2 * MF + 2 * ug + 1];
  const u64 wf = tw[1], wfp = twp[1];
#pragma unroll 1
  for (int i = (int)gamma - 2; i >= 0; i--) {
    const u64* Srow = sh.sums_R + (size_t)i * N;
    const ulonglong2 sv = *reinterpret_cast<const ulonglong2*>(Srow + own + ls);
    const u32 gp = ps.gpow[i];
    const int par = (i & 1) * H;
    u64* xh = X + par;
    {
      // Inverse stages 0-1 of unit ug: lane dg holds slots 4u + 2dg, +1.
      u64 p = cur[0], q = cur[1];
      bf_inv4(p, q, wl1, wl1p);
      const u64 recv = __shfl_xor_sync(0xffffffffu, dg == 0 ? q : p, 1);
      u64 x0 = dg == 0 ? p : recv, x1 = dg == 0 ? recv : q;  // (slot 4u, 4u+2) or (4u+1, 4u+3)
      bf_inv4(x0, x1, wl2, wl2p);
      xh[sw(4 * u + dg)] = x0;
      xh[sw(4 * u + dg + 2)] = x1;
    }
    __syncthreads();
    int s = 2;
#pragma unroll 1
    for (; s + 1 <= LOGN - 2; s += 2) inv_part_r4<LOGN, 2>(xh, s, rank, tw, twp);
    if (s == LOGN - 2) inv_part_r2<LOGN, 2>(xh, s, rank, tw, twp);
    cluster.sync();
    {
      // Elements [0, H) of the inverse live in rank 0's X, elements [H, N) in rank 1's.
      const u64* lo = (rank == 0 ? (const u64*)X : peerX) + par;
      const u64* hi = (rank == 0 ? peerX : (const u64*)X) + par;
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int b = tid + j * NT;
        const u64 x0 = lo[sw(b)], x1 = hi[sw(b)];
        // The inverse's last stage and n^-1 as one product per output: n^-1 on the sum,
        // n^-1 times the stage's twiddle on the difference.
        const u64 r0 = shoup(x0 + x1, c.ninv, c.ninvp), r1 = shoup(x0 - x1 + 4 * Q, c.nlast, c.nlastp);
        u64 p0, p1, q0, q1;  // digits 0 and 1 of coefficients b and b + H
        if (exact) {
          p0 = r0 & DMASK;
          p1 = (r0 >> 20) & DMASK;
          q0 = r1 & DMASK;
          q1 = (r1 >> 20) & DMASK;
        } else {
          const u64 rr0 = (r0 + (1ULL << 19)) >> 20, rr1 = (r1 + (1ULL << 19)) >> 20;
          p0 = rr0 & DMASK;
          p1 = rr0 >> 20;
          q0 = rr1 & DMASK;
          q1 = rr1 >> 20;
        }
        // Forward cross stage: slot b gets p + w q, slot b + H gets p - w q.
        const u64 t0 = shoup_digit((u32)q0, wf, wfp), t1 = shoup_digit((u32)q1, wf, wfp);
        D[sw(b)] = rank == 0 ? p0 + t0 : p0 + 4 * Q - t0;
        D[H + sw(b)] = rank == 0 ? p1 + t1 : p1 + 4 * Q - t1;
      }
    }
    __syncthreads();
    s = 1;
    if (!(LOGN & 1)) {
      fwd_part_r2<LOGN, 2>(D, 1, rank, tw, twp);
      s = 2;
    }
#pragma unroll 1
    for (; s < LOGN - 2; s += 2) fwd_part_r4<LOGN, 2>(D, s, rank, tw, twp);
    // Forward stages logn-2, logn-1 of unit ug for digit dg, then each lane takes the other
    // digit at its own two slots from its partner.
    u64 d0[2], d1[2];
    {
      const u64* x = D + dg * H;
      const ulonglong2 v01 = *reinterpret_cast<const ulonglong2*>(x + sw(4 * u));
      const ulonglong2 v23 = *reinterpret_cast<const ulonglong2*>(x + sw(4 * u + 2));
      u64 a0 = v01.x, a1 = v01.y, a2 = v23.x, a3 = v23.y;
      bf_fwd8(a0, a2, fa, fap);
      bf_fwd8(a1, a3, fa, fap);
      bf_fwd8(a0, a1, fb, fbp);
      bf_fwd8(a2, a3, fc, fcp);
      const u64 g0 = __shfl_xor_sync(0xffffffffu, dg == 0 ? a2 : a0, 1);
      const u64 g1 = __shfl_xor_sync(0xffffffffu, dg == 0 ? a3 : a1, 1);
      const u64 m0 = dg == 0 ? a0 : a2, m1 = dg == 0 ? a1 : a3;
      d0[0] = dg == 0 ? m0 : g0;
      d0[1] = dg == 0 ? m1 : g1;
      d1[0] = dg == 0 ? g0 : m0;
      d1[1] = dg == 0 ? g1 : m1;
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const u32 tb = s_tab[((gp * et[k]) & M2N) >> 1];
      u128 nb = wide(d0[k], Y[tb]) + wide(d1[k], Y[N + tb]);
      u128 nc = wide(a_ntt[tb], k == 0 ? sv.x : sv.y) + wide(d0[k], Wm[tb]) + wide(d1[k], Wm[N + tb]);
      if (exact) {  // the rows are folded: R_{i+1} stands in for digit 2
        nb += wide(cur[k], Y[2 * N + tb]);
        nc += wide(cur[k], Wm[2 * N + tb]);
      }
      sb[k] = addq(sb[k], redc_wide(nb));
      cur[k] = redc_wide(nc);
    }
  }
  // Final transforms: rank 0 assembles R_0 (-> a), rank 1 the online sum (-> b), each
  // from its own half and the peer's half (exchanged through the half of X that link 0
  // did not use; the peer read it last at link 1, before the barrier of link 0).
  __syncthreads();  // every lane is past its last read of D
  u64* xf = X + H;
  const u64* pf = peerX + H;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    xf[ls + k] = rank == 0 ? sb[k] : cur[k];
    D[own + ls + k] = rank == 0 ? cur[k] : sb[k];
  }
  cluster.sync();
#pragma unroll
  for (int k = 0; k < 2; k++) D[other + tid + k * NT] = pf[tid + k * NT];
  cluster.sync();  // each CTA's X stays alive until its peer has read it
  {
    u64* const bufs[1] = {D};
    ntt_inv_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int t = tid + k * NT;
    if (rank == 0)
      a_out[(size_t)qi * N + t] = finish_a(c, D[t], qd.ms);
    else
      b_out[(size_t)qi * N + t] = finish_b(c, D[t], t, gamma, b_fold + qd.fold_off, qd.ms);
  }
}

// ------------------------------------------------------------------------------------
// Four CTAs per query (a cluster of 4), for small batches whose latency sets the tail: a
// query's recursion spread over four SMs. CTA r owns quarter r, slots [r N/4, (r+1) N/4), of
// every NTT-domain vector, two slots per thread (N/8 threads: the quarter-local passes keep
// half of them busy or all, where N/4 threads left three quarters or half idle at every
// barrier). The inverse's stages 0 .. logn-3 and the
// forward's stages 2 .. logn-1 stay inside a quarter (the part helpers above); the two
// stages on each side that mix quarters combine the four elements b, b + N/4, b + N/2,
// b + 3N/4 of each b < N/4, so they run as one radix-4 cross pass per link: thread b reads
// its four elements (three through distributed shared memory), takes the inverse's last two
// stages with n^-1 folded into the last (n^-1 on the sum, n^-1 times the stage's twiddle on
// the difference), splits the four coefficients into digits and runs the forward's first
// two stages, of which it keeps its own quarter's output (three products a digit). One
// cluster barrier per link: the inverse's exchange buffer alternates between two quarters
// by link parity, so a CTA rewrites what its peers read at link i only at link i-2, after
// all passed the barrier of link i-1. With the exact gadget the third digit's transform
// comes from the other two (inspiring2.rs:1094-1161), folded into the key rows as in
// k_respond.
template <int LOGN>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__((1 << LOGN) / 8, 1)
    k_respond_quad(CrsDev c, const QueryDev* queries, const ShardDev* shards, const u64* b_fold, u64* a_out,
                   u64* b_out, u32* status, int force_serial) {
  namespace cg = cooperative_groups;
  constexpr int N = 1 << LOGN, NT = N / 8, P = N / 4, SPT = P / NT;  // two slots a thread
  constexpr u32 M2N = 2 * N - 1;
  constexpr u64 DMASK = (1ULL << 20) - 1;
  extern __shared__ __align__(16) u64 sm[];
  u64* X = sm;          // [2][P] own quarter of the inverse, by link parity
  u64* D = sm + 2 * P;  // [2][P] own quarter of digits 0 and 1; N words for the last transform
  u64* a_ntt = D + N;
  u64* tw = a_ntt + N;
  u64* twp = tw + N;
  u64* Wm = twp + N;  // room for three key rows, as in k_respond
  u64* Y = Wm + 3 * N;
  uint16_t* e_tab = reinterpret_cast<uint16_t*>(Y + 3 * N);
  uint16_t* s_tab = e_tab + N;

  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const u64* peer[4];
#pragma unroll
  for (int k = 0; k < 4; k++) peer[k] = cluster.map_shared_rank(X, k);
  const int tid = threadIdx.x;
  const QueryDev qd = queries[blockIdx.x >> 2];
  const u32 qi = qd.row;  // output and status row
  const ShardDev sh = shards[qd.shard];
  const SetView ps = set_view(c, qd.crs);
  const u32 gamma = ps.gamma;
  const bool exact = ps.approx == 0;
  // This thread's slots: rank P + tid + j NT, j < SPT.

  stage_constants<N, NT>(c, ps, qd.seat_R, tw, twp, Wm, Y, e_tab, s_tab);
  expand_a<N, NT>(qd, a_ntt, status, qi, force_serial);
  {
    u64* const bufs[1] = {a_ntt};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  u32 et[SPT];
  u64 cur[SPT], sb[SPT];
#pragma unroll
  for (int j = 0; j < SPT; j++) {
    const int slot = rank * P + tid + j * NT;
    et[j] = e_tab[slot];
    const u32 gp = ps.gpow[gamma - 1];
    const u32 tb = s_tab[((gp * et[j]) & M2N) >> 1];
    cur[j] = mont(a_ntt[tb], sh.sums_R[(size_t)(gamma - 1) * N + slot]);
    sb[j] = 0;
  }
  // Twiddles of the cross pass: the inverse's stage logn-2 (indices 2 and 3), the forward's
  // stage 0 (index 1) and stage 1 (index 2 for the first half, 3 for the second).
  u64 wi2, wi2p, wi3, wi3p;
  inv_twiddle(tw, twp, 2, wi2, wi2p);
  inv_twiddle(tw, twp, 3, wi3, wi3p);
  const u64 wf1 = tw[1], wf1p = twp[1];
  const u64 wfs = tw[2 + (rank >> 1)], wfsp = twp[2 + (rank >> 1)];
#pragma unroll 1
  for (int i = (int)gamma - 2; i >= 0; i--) {
    u64 sv[SPT];
#pragma unroll
    for (int j = 0; j < SPT; j++) sv[j] = sh.sums_R[(size_t)i * N + rank * P + tid + j * NT];
    const u32 gp = ps.gpow[i];
    const int par = (i & 1) * P;
    u64* xq = X + par;
#pragma unroll
    for (int j = 0; j < SPT; j++) xq[sw(tid + j * NT)] = cur[j];
    __syncthreads();
    int s = 0;
#pragma unroll 1
    for (; s + 1 <= LOGN - 3; s += 2) inv_part_r4<LOGN, 4>(xq, s, rank, tw, twp);
    if (s == LOGN - 3) inv_part_r2<LOGN, 4>(xq, s, rank, tw, twp);
    cluster.sync();
#pragma unroll
    for (int j = 0; j < SPT; j++) {
      const int b = tid + j * NT;
      u64 x0 = peer[0][par + sw(b)], x1 = peer[1][par + sw(b)];
      u64 x2 = peer[2][par + sw(b)], x3 = peer[3][par + sw(b)];
      bf_inv4(x0, x1, wi2, wi2p);  // (b, b + N/4), block 0 of stage logn-2
      bf_inv4(x2, x3, wi3, wi3p);  // (b + N/2, b + 3N/4), block 1
      u64 cf[4];                   // coefficients b, b + N/4, b + N/2, b + 3N/4
      cf[0] = shoup(x0 + x2, c.ninv, c.ninvp);
      cf[2] = shoup(x0 - x2 + 4 * Q, c.nlast, c.nlastp);
      cf[1] = shoup(x1 + x3, c.ninv, c.ninvp);
      cf[3] = shoup(x1 - x3 + 4 * Q, c.nlast, c.nlastp);
      u64 g0[4], g1[4];  // digits 0 and 1
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (exact) {
          g0[k] = cf[k] & DMASK;
          g1[k] = (cf[k] >> 20) & DMASK;
        } else {
          const u64 rr = (cf[k] + (1ULL << 19)) >> 20;
          g0[k] = rr & DMASK;
          g1[k] = rr >> 20;
        }
      }
      // Forward stage 0 (b with b + N/2, b + N/4 with b + 3N/4), then stage 1 on this
      // quarter's half: a bf_fwd8 whose output r & 1 is the quarter's word.
      auto fwd = [&](const u64(&g)[4]) -> u64 {
        const u64 t2 = shoup_digit((u32)g[2], wf1, wf1p), t3 = shoup_digit((u32)g[3], wf1, wf1p);
        u64 lo, hi;
        if (rank < 2) {
          lo = g[0] + t2;
          hi = g[1] + t3;
        } else {
          lo = g[0] + 4 * Q - t2;
          hi = g[1] + 4 * Q - t3;
        }
        bf_fwd8(lo, hi, wfs, wfsp);
        return (rank & 1) ? hi : lo;
      };
      D[sw(b)] = fwd(g0);
      D[P + sw(b)] = fwd(g1);
    }
    __syncthreads();
    s = 2;
    if ((LOGN - 2) & 1) {
      fwd_part_r2<LOGN, 4>(D, 2, rank, tw, twp);
      s = 3;
    }
#pragma unroll 1
    for (; s < LOGN; s += 2) fwd_part_r4<LOGN, 4>(D, s, rank, tw, twp);
#pragma unroll
    for (int j = 0; j < SPT; j++) {
      const u64 d0 = D[sw(tid + j * NT)], d1 = D[P + sw(tid + j * NT)];
      const u32 tb = s_tab[((gp * et[j]) & M2N) >> 1];
      u128 nb = wide(d0, Y[tb]) + wide(d1, Y[N + tb]);
      u128 nc = wide(a_ntt[tb], sv[j]) + wide(d0, Wm[tb]) + wide(d1, Wm[N + tb]);
      if (exact) {  // the rows are folded: R_{i+1} stands in for digit 2
        nb += wide(cur[j], Y[2 * N + tb]);
        nc += wide(cur[j], Wm[2 * N + tb]);
      }
      sb[j] = addq(sb[j], redc_wide(nb));
      cur[j] = redc_wide(nc);
    }
  }
  // Final transforms: rank 0 assembles R_0 (-> a), rank 1 the online sum (-> b), each from
  // the four quarters exchanged through X once every peer is past its last cross-pass read.
  cluster.sync();
#pragma unroll
  for (int j = 0; j < SPT; j++) {
    X[tid + j * NT] = cur[j];
    X[P + tid + j * NT] = sb[j];
  }
  cluster.sync();
  if (rank < 2) {
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < SPT; j++) D[k * P + tid + j * NT] = peer[k][rank * P + tid + j * NT];
  }
  cluster.sync();  // each CTA's X stays alive until ranks 0 and 1 have read it
  if (rank >= 2) return;
  __syncthreads();
  {
    u64* const bufs[1] = {D};
    ntt_inv_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
#pragma unroll
  for (int k = 0; k < N / NT; k++) {
    const int t = tid + k * NT;
    if (rank == 0)
      a_out[(size_t)qi * N + t] = finish_a(c, D[t], qd.ms);
    else
      b_out[(size_t)qi * N + t] = finish_b(c, D[t], t, gamma, b_fold + qd.fold_off, qd.ms);
  }
}

// ------------------------------------------------------------------------------------
// NoPacking respond (respond.rs:614-643): one RLWE ciphertext (a h_j, b h_j) per column j
// (plaintext_multiply_columns, respond.rs:585-599) and their sum.
//   nopack_prep: per query, NTT(a) and NTT(b) in R-form (a expanded from the seed);
//   nopack_cols: per (query, column), NTT(h_j), the two products (one Montgomery product
//                each against the R-form operands) and their inverse transforms, written
//                as ciphertext 1 + j of the query;
//   nopack_sum:  ciphertext 0 = the sum of the column ciphertexts mod q.
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4) k_nopack_prep(CrsDev c, const QueryDev* queries, u64 r_mod_q,
                                                                 u64 r_mod_qp, u64* AB_R, u32* status) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  extern __shared__ __align__(16) u64 sm[];
  u64* xa = sm;
  u64* xb = sm + N;
  u64* tw = sm + 2 * N;
  u64* twp = sm + 3 * N;
  const u32 qi = blockIdx.x;
  const QueryDev qd = queries[qi];
  for (int k = threadIdx.x; k < N; k += NT) {
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
    xb[k] = reduce128(qd.b[k]);
  }
  expand_a<N, NT>(qd, xa, status, qi, 0);  // ends with a barrier
  {
    u64* const bufs[2] = {xa, xb};
    ntt_fwd_r4<LOGN, NT, 2>(bufs, tw, twp);
  }
  u64* o = AB_R + (size_t)qi * 2 * N;
  for (int k = threadIdx.x; k < N; k += NT) {
    o[k] = shoup(xa[k], r_mod_q, r_mod_qp);
    o[N + k] = shoup(xb[k], r_mod_q, r_mod_qp);
  }
}

template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4) k_nopack_cols(CrsDev c, const QueryDev* queries,
                                                                 const ShardDev* shards, const u64* AB_R, u64* out) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  extern __shared__ __align__(16) u64 sm[];
  u64* x = sm;
  u64* ya = sm + N;
  u64* yb = sm + 2 * N;
  u64* tw = sm + 3 * N;
  u64* twp = sm + 4 * N;
  const u32 j = blockIdx.x, qi = blockIdx.y;
  const QueryDev qd = queries[qi];
  const u64* col = shards[qd.shard].columns + (size_t)j * N;
  for (int k = threadIdx.x; k < N; k += NT) {
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
    x[k] = reduce128(col[k]);
  }
  __syncthreads();
  {
    u64* const bufs[1] = {x};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  const u64* A = AB_R + (size_t)qi * 2 * N;
  for (int k = threadIdx.x; k < N; k += NT) {
    const u64 h = csub(csub2(x[k]));
    ya[k] = mont(A[k], h);
    yb[k] = mont(A[N + k], h);
  }
  __syncthreads();
  {
    u64* const bufs[2] = {ya, yb};
    ntt_inv_r4<LOGN, NT, 2>(bufs, tw, twp);
  }
  u64* o = out + ((size_t)qi * (c.gamma + 1) + 1 + j) * 2 * N;
  for (int k = threadIdx.x; k < N; k += NT) {
    o[k] = shoup(ya[k], c.ninv, c.ninvp);
    o[N + k] = shoup(yb[k], c.ninv, c.ninvp);
  }
}

__global__ void k_nopack_sum(u32 n, u32 gamma, u64* out) {
  const u32 qi = blockIdx.y;
  const u32 k = blockIdx.x * blockDim.x + threadIdx.x;  // over 2n words of a ciphertext
  if (k >= 2 * n) return;
  u64* base = out + (size_t)qi * (gamma + 1) * 2 * n;
  u64 acc = 0;
  for (u32 j = 1; j <= gamma; j++) acc = addq(acc, base[(size_t)j * 2 * n + k]);
  base[k] = acc;
}

// ------------------------------------------------------------------------------------
// OnePacking: respond_one_packing (pir/respond.rs:696-729), the Galois-automorphism tree of
// inspiring/automorph_pack.rs, one CTA per query. Leaf j (j < gamma) is the column product's
// a part a h_j (b part zero) and b-value_j = coeff0(b h_j); leaves past gamma are the
// padding's zero ciphertexts. Node (ell, start) = (E + y O) + keyswitch(tau_t(E - y O)) with
// E, O its children (start, start + n/2^ell), y = X^(n >> ell), t = 2^ell + 1 and Galois key
// log n - ell (pack_lwes_inner, automorph_pack.rs:96-163). Every node whose start is at or
// past gamma is exactly zero, so only those below gamma are computed.
//
// Nodes live in the NTT domain: y O is a product by NTT(X^s), tau_t a slot permutation,
// and only the key switch's digit split needs coefficients: a = INTT(tau_t(...).a), digits
// 0 and 1 (base 2^20) transformed, digit 2's transform base^-2 (a - D0 - base D1) (the
// unsigned split of rgsw/external_product.rs:58-99 leaves a = D0 + base D1 + base^2 D2
// exactly), which the keys' folded rows (fold_gadget_keys) take from a itself. Key rows
// are R-form NTT, so each sum of three products takes one reduction.
//
// The walk is the recursion's depth-first order: leaf k of the walk is start = bitrev(k),
// and a binary-counter carry combines each finished node with its waiting sibling; the
// waiting nodes sit in a per-query stack of log n node slots in global memory.
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4, 1)
    k_tree(CrsDev c, const QueryDev* queries, const ShardDev* shards, u64 r_mod_q, u64 r_mod_qp, u64 ms_target,
           u64* stack, u64* a_out, u64* b_out, u32* status) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  constexpr u32 M2N = 2 * N - 1;
  constexpr u64 DMASK = (1ULL << 20) - 1;
  extern __shared__ __align__(16) u64 sm[];
  u64* tw = sm;
  u64* twp = tw + N;
  u64* aR = twp + N;     // NTT(a) in R-form
  u64* S1a = aR + N;     // E - y O, permuted by the automorphism
  u64* S1b = S1a + N;
  u64* X = S1b + N;      // the inverse in progress, then a leaf column
  u64* D = X + N;        // digits 0 and 1
  u64* bval = D + 2 * N; // b-values of the leaves (gamma <= n/2)
  u64* red = bval + N / 2;  // per-warp partial sums
  uint16_t* e_tab = reinterpret_cast<uint16_t*>(red + 32);
  uint16_t* s_tab = e_tab + N;
  const int tid = threadIdx.x;
  const u32 qi = blockIdx.x;
  const QueryDev qd = queries[qi];
  const ShardDev sh = shards[qd.shard];
  const u32 gamma = c.gamma;
  u64* stk = stack + (size_t)qi * LOGN * 2 * N;

  for (int k = tid; k < N; k += NT) {
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
    e_tab[k] = c.slot_exp[k];
    s_tab[k] = c.exp_slot[k];
  }
  expand_a<N, NT>(qd, aR, status, qi, 0);  // ends with a barrier
  {
    u64* const bufs[1] = {aR};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  for (int k = tid; k < N; k += NT) aR[k] = shoup(aR[k], r_mod_q, r_mod_qp);
  __syncthreads();

  const int l0 = 4 * tid;
  u64 ca[4], cb[4];  // the current node at slots l0..l0+3 (thread tid's transform unit)
  bool cur_zero = true;
  const u64 wf = tw[1], wfp = twp[1];
  constexpr int H = N / 2, MF = 1 << (LOGN - 2);
  // Leaf `start`: the column through the transform times NTT(a); its b-value on the side.
  auto leaf = [&](u32 start) {
    u128 acc = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int k = tid + j * NT;
      const u64 h = sh.cols16 ? (u64)sh.cols16[(size_t)start * N + k] : reduce128(sh.columns[(size_t)start * N + k]);
      const u64 br = k == 0 ? reduce128(qd.b[0]) : negq(reduce128(qd.b[N - k]));
      acc += wide(h, br);
      X[k] = h;
    }
    u64 v = reduce128(acc);
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v = addq(v, __shfl_xor_sync(0xffffffffu, v, m));
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      u64 t = 0;
      for (int w = 0; w < NT / 32; w++) t = addq(t, red[w]);
      bval[start] = t;
    }
    {
      u64* const bufs[1] = {X};
      ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);  // ends with a barrier
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      ca[j] = mont(csub(csub2(X[l0 + j])), aR[l0 + j]);
      cb[j] = 0;
    }
    __syncthreads();  // X is rewritten next
  };
  // The current node becomes (E + y O) + keyswitch(tau_t(E - y O)) at level ell, E from the
  // stack slot ell - 1; the current node is O (zero when odd_zero). The transforms follow
  // k_respond's link: the inverse's first two stages in registers, its last stage fused with
  // n^-1, the digit split and the forward's first stage, the forward's last two stages in
  // registers, X and D under the sw() layout.
  auto combine = [&](int ell, bool odd_zero) {
    const u64* E = stk + (size_t)(ell - 1) * 2 * N + l0;
    const u32 sy = (u32)(N >> ell), t = (1u << ell) + 1;
    const u64* key = c.galois_R + (size_t)(LOGN - ell) * 6 * N + l0;
    u64 s0a[4], s0b[4], aa[4], ab[4];
    {
      const ulonglong2 e01 = *reinterpret_cast<const ulonglong2*>(E);
      const ulonglong2 e23 = *reinterpret_cast<const ulonglong2*>(E + 2);
      const ulonglong2 f01 = *reinterpret_cast<const ulonglong2*>(E + N);
      const ulonglong2 f23 = *reinterpret_cast<const ulonglong2*>(E + N + 2);
      const u64 ea[4] = {e01.x, e01.y, e23.x, e23.y}, eb[4] = {f01.x, f01.y, f23.x, f23.y};
      u64 da[4], db[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        u64 ya = 0, yb = 0;
        if (!odd_zero) {
          const u64 y = c.pow_root_R[(e_tab[l0 + j] * sy) & M2N];
          ya = mont(ca[j], y);
          yb = mont(cb[j], y);
        }
        s0a[j] = addq(ea[j], ya);
        s0b[j] = addq(eb[j], yb);
        da[j] = subq(ea[j], ya);
        db[j] = subq(eb[j], yb);
      }
      *reinterpret_cast<ulonglong2*>(S1a + l0) = make_ulonglong2(da[0], da[1]);
      *reinterpret_cast<ulonglong2*>(S1a + l0 + 2) = make_ulonglong2(da[2], da[3]);
      *reinterpret_cast<ulonglong2*>(S1b + l0) = make_ulonglong2(db[0], db[1]);
      *reinterpret_cast<ulonglong2*>(S1b + l0 + 2) = make_ulonglong2(db[2], db[3]);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const u32 src = s_tab[((t * e_tab[l0 + j]) & M2N) >> 1];
      aa[j] = S1a[src];
      ab[j] = S1b[src];
    }
    {
      // Inverse stages 0-1 of unit tid (block B = tid, m = N/2).
      u64 w0, w0p, w1, w1p, w2, w2p;
      inv_twiddle(tw, twp, H + 2 * tid, w0, w0p);
      inv_twiddle(tw, twp, H + 2 * tid + 1, w1, w1p);
      inv_twiddle(tw, twp, H / 2 + tid, w2, w2p);
      u64 a0 = aa[0], a1 = aa[1], a2 = aa[2], a3 = aa[3];
      bf_inv4(a0, a1, w0, w0p);
      bf_inv4(a2, a3, w1, w1p);
      bf_inv4(a0, a2, w2, w2p);
      bf_inv4(a1, a3, w2, w2p);
      *reinterpret_cast<ulonglong2*>(X + sw(l0)) = make_ulonglong2(a0, a1);
      *reinterpret_cast<ulonglong2*>(X + sw(l0 + 2)) = make_ulonglong2(a2, a3);
    }
    __syncthreads();
    // Inverse stages 2 .. logn-2 (radix-4 pairs, a radix-2 stage last when logn is even).
    int s = 2;
#pragma unroll 1
    for (; s + 1 <= LOGN - 2; s += 2) {
      const int tt = 1 << s, m = N >> (s + 1);
      const int B = tid >> s, o = tid & (tt - 1);
      const int e0 = B * 4 * tt + o;
      u64 w0, w0p, w1, w1p, w2, w2p;
      inv_twiddle(tw, twp, m + 2 * B, w0, w0p);
      inv_twiddle(tw, twp, m + 2 * B + 1, w1, w1p);
      inv_twiddle(tw, twp, (m >> 1) + B, w2, w2p);
      u64 a0 = X[sw(e0)], a1 = X[sw(e0 + tt)], a2 = X[sw(e0 + 2 * tt)], a3 = X[sw(e0 + 3 * tt)];
      bf_inv4(a0, a1, w0, w0p);
      bf_inv4(a2, a3, w1, w1p);
      bf_inv4(a0, a2, w2, w2p);
      bf_inv4(a1, a3, w2, w2p);
      X[sw(e0)] = a0;
      X[sw(e0 + tt)] = a1;
      X[sw(e0 + 2 * tt)] = a2;
      X[sw(e0 + 3 * tt)] = a3;
      __syncthreads();
    }
    if (s == LOGN - 2) {
      const int tt = 1 << s, m = N >> (s + 1);
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int v = tid + r * NT;
        const int B = v >> s, o = v & (tt - 1);
        const int e = B * 2 * tt + o;
        u64 w, wp;
        inv_twiddle(tw, twp, m + B, w, wp);
        u64 a = X[sw(e)], b = X[sw(e + tt)];
        bf_inv4(a, b, w, wp);
        X[sw(e)] = a;
        X[sw(e + tt)] = b;
      }
      __syncthreads();
    }
    // Inverse stage logn-1, n^-1, digit split and forward stage 0, per pair (b, b + N/2).
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int b = tid + j * NT;
      const u64 x0 = X[sw(b)], x1 = X[sw(b + H)];
      // The inverse's last stage and n^-1 as one product per output: n^-1 on the sum,
      // n^-1 times the stage's twiddle on the difference.
      const u64 r0 = shoup(x0 + x1, c.ninv, c.ninvp), r1 = shoup(x0 - x1 + 4 * Q, c.nlast, c.nlastp);
      const u64 p0 = r0 & DMASK, p1 = (r0 >> 20) & DMASK, q0 = r1 & DMASK, q1 = (r1 >> 20) & DMASK;
      const u64 t0 = shoup_digit((u32)q0, wf, wfp), t1 = shoup_digit((u32)q1, wf, wfp);
      D[sw(b)] = p0 + t0;
      D[sw(b + H)] = p0 + 4 * Q - t0;
      D[N + sw(b)] = p1 + t1;
      D[N + sw(b + H)] = p1 + 4 * Q - t1;
    }
    __syncthreads();
    // Forward stages 1 .. logn-3 (a radix-2 stage first when logn is even), both digits.
    s = 1;
    if (!(LOGN & 1)) {
      const int lt = LOGN - 2, tt = 1 << lt;
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int v = tid + r * NT;
        const int ib = v >> lt, o = v & (tt - 1);
        const int e = ib * 2 * tt + o;
        const u64 w = tw[2 + ib], wp = twp[2 + ib];
#pragma unroll
        for (int k = 0; k < 2; k++) {
          u64* x = D + k * N;
          u64 a = x[sw(e)], b = x[sw(e + tt)];
          bf_fwd8(a, b, w, wp);
          x[sw(e)] = a;
          x[sw(e + tt)] = b;
        }
      }
      __syncthreads();
      s = 2;
    }
#pragma unroll 1
    for (; s < LOGN - 2; s += 2) {
      const int tt = N >> (s + 1), m = 1 << s, h = tt >> 1;
      const int ib = tid / h, o = tid - ib * h;
      const int e0 = ib * 2 * tt + o;
      const u64 wa = tw[m + ib], wap = twp[m + ib];
      const u64 wb = tw[2 * m + 2 * ib], wbp = twp[2 * m + 2 * ib];
      const u64 wc = tw[2 * m + 2 * ib + 1], wcp = twp[2 * m + 2 * ib + 1];
      const int i0 = sw(e0), i1 = sw(e0 + h), i2 = sw(e0 + tt), i3 = sw(e0 + tt + h);
      u64* x0 = D;
      u64* x1 = D + N;
      u64 a0 = x0[i0], a1 = x0[i1], a2 = x0[i2], a3 = x0[i3];
      u64 c0 = x1[i0], c1 = x1[i1], c2 = x1[i2], c3 = x1[i3];
      bf_fwd8(a0, a2, wa, wap);
      bf_fwd8(c0, c2, wa, wap);
      bf_fwd8(a1, a3, wa, wap);
      bf_fwd8(c1, c3, wa, wap);
      bf_fwd8(a0, a1, wb, wbp);
      bf_fwd8(c0, c1, wb, wbp);
      bf_fwd8(a2, a3, wc, wcp);
      bf_fwd8(c2, c3, wc, wcp);
      x0[i0] = a0;
      x0[i1] = a1;
      x0[i2] = a2;
      x0[i3] = a3;
      x1[i0] = c0;
      x1[i1] = c1;
      x1[i2] = c2;
      x1[i3] = c3;
      __syncthreads();
    }
    // Forward stages logn-2, logn-1 of unit tid, both digits, in registers.
    u64 d0[4], d1[4];
    {
      const u64 fa = tw[MF + tid], fap = twp[MF + tid];
      const u64 fb = tw[2 * MF + 2 * tid], fbp = twp[2 * MF + 2 * tid];
      const u64 fc = tw[2 * MF + 2 * tid + 1], fcp = twp[2 * MF + 2 * tid + 1];
      const ulonglong2 v01 = *reinterpret_cast<const ulonglong2*>(D + sw(l0));
      const ulonglong2 v23 = *reinterpret_cast<const ulonglong2*>(D + sw(l0 + 2));
      const ulonglong2 g01 = *reinterpret_cast<const ulonglong2*>(D + N + sw(l0));
      const ulonglong2 g23 = *reinterpret_cast<const ulonglong2*>(D + N + sw(l0 + 2));
      d0[0] = v01.x, d0[1] = v01.y, d0[2] = v23.x, d0[3] = v23.y;
      d1[0] = g01.x, d1[1] = g01.y, d1[2] = g23.x, d1[3] = g23.y;
      bf_fwd8(d0[0], d0[2], fa, fap);
      bf_fwd8(d1[0], d1[2], fa, fap);
      bf_fwd8(d0[1], d0[3], fa, fap);
      bf_fwd8(d1[1], d1[3], fa, fap);
      bf_fwd8(d0[0], d0[1], fb, fbp);
      bf_fwd8(d1[0], d1[1], fb, fbp);
      bf_fwd8(d0[2], d0[3], fc, fcp);
      bf_fwd8(d1[2], d1[3], fc, fcp);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      // The keys' digit rows are folded (fold_gadget3): aa stands in for digit 2.
      const u64 na = redc_wide(wide(d0[j], key[j]) + wide(d1[j], key[2 * N + j]) + wide(aa[j], key[4 * N + j]));
      const u64 nb = redc_wide(wide(d0[j], key[N + j]) + wide(d1[j], key[3 * N + j]) + wide(aa[j], key[5 * N + j]));
      ca[j] = addq(s0a[j], na);
      cb[j] = addq(s0b[j], addq(ab[j], nb));
    }
    __syncthreads();  // S1, X and D are rewritten next
  };

  if (gamma == 1) {
    // pack_lwes with one input returns it untouched: no tree and no d scaling.
    leaf(0);
    cur_zero = false;
  } else {
    u32 zero_slots = 0;  // bit L: the waiting node at level L is zero
#pragma unroll 1
    for (u32 k = 0; k < (u32)N; k++) {
      const u32 start = __brev(k) >> (32 - LOGN);
      cur_zero = start >= gamma;
      if (!cur_zero) leaf(start);
      int L = 0;
      while ((k >> L) & 1) {
        if ((zero_slots >> L) & 1) {
          cur_zero = true;  // an even child at or past gamma makes its sibling zero too
        } else {
          combine(L + 1, cur_zero);
          cur_zero = false;
        }
        L++;
      }
      if (L < LOGN) {
        if (cur_zero) {
          zero_slots |= 1u << L;
        } else {
          zero_slots &= ~(1u << L);
          u64* slot = stk + (size_t)L * 2 * N + l0;
          *reinterpret_cast<ulonglong2*>(slot) = make_ulonglong2(ca[0], ca[1]);
          *reinterpret_cast<ulonglong2*>(slot + 2) = make_ulonglong2(ca[2], ca[3]);
          *reinterpret_cast<ulonglong2*>(slot + N) = make_ulonglong2(cb[0], cb[1]);
          *reinterpret_cast<ulonglong2*>(slot + N + 2) = make_ulonglong2(cb[2], cb[3]);
        }
      }
    }
  }
  // The root to coefficients; b_z += n b-value_z for z < gamma (pack_lwes, automorph_pack.rs
  // 327-338), except for a single input.
#pragma unroll
  for (int j = 0; j < 4; j++) {
    X[l0 + j] = ca[j];
    D[l0 + j] = cb[j];
  }
  __syncthreads();
  {
    u64* const bufs[2] = {X, D};
    ntt_inv_r4<LOGN, NT, 2>(bufs, tw, twp);
  }
  const u64 scale = gamma == 1 ? 1 : (u64)N;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int k = tid + j * NT;
    u64 av = shoup(X[k], c.ninv, c.ninvp);
    u64 bv = gamma == 1 ? (k == 0 ? bval[0] : 0) : shoup(D[k], c.ninv, c.ninvp);
    if (gamma > 1 && (u32)k < gamma) bv = addq(bv, reduce128(wide(bval[k], scale)));
    if (ms_target) {
      av = mod_switch_word(av, ms_target);
      bv = mod_switch_word(bv, ms_target);
    }
    a_out[(size_t)qi * N + k] = av;
    b_out[(size_t)qi * N + k] = bv;
  }
}

// ------------------------------------------------------------------------------------
// Client side (ClientSession::query_batch, session.rs:377-434; extract_inspiring and
// extract_packed, extract.rs:184-263): queries and record decoding for many queries at once.
//
// The query error comes from the session's Gaussian sampler (math/gaussian.rs:210-224),
// one stream shared by the whole batch in order: each sample draws x uniform in
// [-tailcut, tailcut] (rand's widening-multiply rejection: a 64-bit word whose low product
// half exceeds the zone is skipped) and then u uniform in [0, 1) from one 64-bit word, and
// keeps x when threshold(x) > bits(u). Read as a machine over the stream's 64-bit words it
// has two states, A (next word is an x candidate) and B (next word is the u of an accepted
// x), so the stream is parsed in parallel: each thread composes the state maps of a segment
// of words, a scan gives every segment its start state, and a second walk counts and places
// the samples.

// Word i of the stream: u32 words base + 2i, base + 2i + 1 of the keystream buffer.
__device__ __forceinline__ u64 ks_word(const u32* ks, u64 base, u64 i) {
  return (u64)ks[base + 2 * i] | ((u64)ks[base + 2 * i + 1] << 32);
}
// x of candidate word w, or false when rand rejects it.
__device__ __forceinline__ bool gauss_x(const GaussDev& g, u64 w, i64& x) {
  const u128 m = (u128)w * g.range;
  if ((u64)m > g.zone) return false;
  x = -g.tailcut + (i64)(u64)(m >> 64);
  return true;
}
// rand's f64 in [0, 1) from w (52 high bits as the mantissa of [1, 2), minus 1, exact), and
// the acceptance of x: threshold bits above the bits of u.
__device__ __forceinline__ bool gauss_keep(const GaussDev& g, i64 x, u64 w) {
  const double v = __longlong_as_double((long long)((w >> 12) | 0x3FF0000000000000ULL)) - 1.0;
  return g.accept[x + g.tailcut] > (u64)__double_as_longlong(v);
}

// The sampler's keystream: ChaCha20 blocks block0 .. block0 + nblocks - 1 of stream 0.
__global__ void k_keystream(const u32* key, u64 block0, u64 nblocks, u32* ks) {
  const u64 b = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  u32 k[8], out[16];
#pragma unroll
  for (int i = 0; i < 8; i++) k[i] = key[i];
  chacha20_block(k, block0 + b, 0, out);
#pragma unroll
  for (int i = 0; i < 16; i++) ks[b * 16 + i] = out[i];
}

// Segment t (words [t seg, t seg + seg) of W): bit 0 = end state from A, bit 1 = from B.
__global__ void k_gauss_maps(GaussDev g, const u32* ks, u64 base, u64 W, u32 seg, uint8_t* maps, u64 T) {
  const u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  u32 sa = 0, sb = 1;
  const u64 e = min(W, (t + 1) * seg);
  for (u64 i = t * seg; i < e; i++) {
    i64 x;
    const u32 next_a = gauss_x(g, ks_word(ks, base, i), x) ? 1u : 0u;
    sa = sa ? 0u : next_a;
    sb = sb ? 0u : next_a;
  }
  maps[t] = (uint8_t)(sa | (sb << 1));
}

// One block: exclusive scan of T segment maps from state A (start states), or, with
// counts, exclusive prefix sums of T counts (offsets) and their total.
__global__ void __launch_bounds__(1024) k_gauss_scan(const uint8_t* maps, uint8_t* starts, const u32* counts,
                                                     u64* offsets, u64* total, u64 T) {
  __shared__ u64 part[1024];
  const u64 per = (T + 1023) / 1024;
  const u64 b = threadIdx.x * per, e = min(T, b + per);
  if (maps) {
    // Composite map of this thread's range, as the pair (image of A, image of B).
    u32 fa = 0, fb = 1;
    for (u64 i = b; i < e; i++) {
      const u32 m = maps[i];
      fa = (m >> fa) & 1;
      fb = (m >> fb) & 1;
    }
    part[threadIdx.x] = fa | (fb << 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      u32 st = 0;
      for (int c = 0; c < 1024; c++) {
        const u32 m = (u32)part[c];
        part[c] = st;
        st = (m >> st) & 1;
      }
    }
    __syncthreads();
    u32 st = (u32)part[threadIdx.x];
    for (u64 i = b; i < e; i++) {
      starts[i] = (uint8_t)st;
      st = (maps[i] >> st) & 1;
    }
  } else {
    u64 sum = 0;
    for (u64 i = b; i < e; i++) sum += counts[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
      u64 acc = 0;
      for (int c = 0; c < 1024; c++) {
        const u64 v = part[c];
        part[c] = acc;
        acc += v;
      }
      *total = acc;
    }
    __syncthreads();
    u64 acc = part[threadIdx.x];
    for (u64 i = b; i < e; i++) {
      offsets[i] = acc;
      acc += counts[i];
    }
  }
}

// Walk of segment t from its start state: counts its samples (offsets null), or writes
// sample k to out[k] for k < S and, at the S-th, the word index after it to *end.
__global__ void k_gauss_walk(GaussDev g, const u32* ks, u64 base, u64 W, u32 seg, const uint8_t* starts, u64 T,
                             u32* counts, const u64* offsets, u64 S, i64* out, u64* end) {
  const u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  u64 i = t * seg;
  const u64 e = min(W, i + seg);
  u32 st = starts[t];
  i64 x = 0;
  if (st == 1) gauss_x(g, ks_word(ks, base, i - 1), x);  // the pending x is the previous word's
  u64 k = offsets ? offsets[t] : 0;
  u32 n = 0;
  for (; i < e; i++) {
    const u64 w = ks_word(ks, base, i);
    if (st == 0) {
      st = gauss_x(g, w, x) ? 1u : 0u;
    } else {
      st = 0;
      if (gauss_keep(g, x, w)) {
        if (offsets) {
          if (k < S) out[k] = x;
          if (k == S - 1) *end = i + 1;
          k++;
        } else {
          n++;
        }
      }
    }
  }
  if (!offsets) counts[t] = n;
}

// One CTA per query: b = Delta X^-local - a s + e (SeededRgswCiphertext::encrypt_with_rng,
// rgsw/types.rs:345-388, one gadget row of power 1), a from the query's seed.
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4) k_client_query(CrsDev c, const QueryDev* queries,
                                                                  const u64* s_R, const u32* locals,
                                                                  const i64* samples, u64 delta, u64* b_out,
                                                                  u32* status) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  extern __shared__ __align__(16) u64 sm[];
  u64* x = sm;
  u64* tw = sm + N;
  u64* twp = tw + N;
  const u32 qi = blockIdx.x;
  const QueryDev qd = queries[qi];
  for (int k = threadIdx.x; k < N; k += NT) {
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
  }
  expand_a<N, NT>(qd, x, status, qi, 0);  // ends with a barrier
  {
    u64* const bufs[1] = {x};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  for (int k = threadIdx.x; k < N; k += NT) x[k] = mont(csub(csub2(x[k])), s_R[k]);
  __syncthreads();
  {
    u64* const bufs[1] = {x};
    ntt_inv_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  const u32 local = locals[qi];
  const int pos = local == 0 ? 0 : N - (int)local;
  const u64 mono = local == 0 ? delta : Q - delta;  // Delta X^-local (encode_db.rs:43-70)
  for (int k = threadIdx.x; k < N; k += NT) {
    const u64 as = shoup(x[k], c.ninv, c.ninvp);
    const i64 ev = samples[(size_t)qi * N + k];
    u64 b = addq(negq(as), ev < 0 ? Q - (u64)(-ev) : (u64)ev);
    if (k == pos) b = addq(b, mono);
    b_out[(size_t)qi * N + k] = b;
  }
}

// One CTA per response: (a s + b) mod the response modulus, rounded by delta and taken mod p
// (PlaintextRounding, rlwe/enc.rs:14-44); times d^-1 mod p for a tree response; the first
// ceil(entry/2) values are the record's 16-bit columns (encode_db.rs:152-168). The product
// is taken mod q: a switched modulus m keeps |a s| below n m max|s| < q/2, so the centred
// residue is the integer product (the host checks the bound).
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4) k_client_extract(CrsDev c, const u64* s_R, const u64* a,
                                                                    const u64* b, u64 modulus, u64 delta, u64 p,
                                                                    u64 dinv, u32 entry_size, uint8_t* out) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  extern __shared__ __align__(16) u64 sm[];
  u64* x = sm;
  u64* tw = sm + N;
  u64* twp = tw + N;
  const u32 qi = blockIdx.x;
  for (int k = threadIdx.x; k < N; k += NT) {
    tw[k] = c.tw[k];
    twp[k] = c.twp[k];
    x[k] = a[(size_t)qi * N + k];
  }
  __syncthreads();
  {
    u64* const bufs[1] = {x};
    ntt_fwd_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  for (int k = threadIdx.x; k < N; k += NT) x[k] = mont(csub(csub2(x[k])), s_R[k]);
  __syncthreads();
  {
    u64* const bufs[1] = {x};
    ntt_inv_r4<LOGN, NT, 1>(bufs, tw, twp);
  }
  const u32 cols = (entry_size + 1) / 2;
  for (u32 k = threadIdx.x; k < cols && k < (u32)N; k += NT) {
    u64 as = shoup(x[k], c.ninv, c.ninvp);
    if (modulus != Q) {
      const bool neg = as > (Q >> 1);
      const u64 mag = (neg ? Q - as : as) % modulus;
      as = neg && mag ? modulus - mag : mag;
    }
    const u64 bv = b[(size_t)qi * N + k];
    u64 noisy = as + bv;
    if (noisy >= modulus) noisy -= modulus;
    u64 m = ((noisy + delta / 2) / delta) % p;
    if (dinv) m = (u64)((u128)m * dinv % p);
    uint8_t* rec = out + (size_t)qi * entry_size;
    rec[2 * k] = (uint8_t)(m & 0xff);
    if (2 * k + 1 < entry_size) rec[2 * k + 1] = (uint8_t)((m >> 8) & 0xff);
  }
}

// ------------------------------------------------------------------------------------
// Integer roofline probe: the recursion kernels' lazy forward butterflies (bf_fwd8: one
// Shoup product, two 64-bit adds and a conditional subtraction each, the transforms' unit
// of work) on values held in registers, eight independent chains per thread, no memory
// traffic. Its rate is the ceiling the respond kernels' butterflies are measured against.
__global__ void __launch_bounds__(256) k_butterfly_peak(u64* out, int iters, u64 w, u64 wp) {
  u64 x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (u64)(blockIdx.x * 8191u + threadIdx.x * 131u + k) * 0x9E3779B97F4A7C15ULL % Q;
#pragma unroll 1
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k += 2) bf_fwd8(x[k], x[k + 1], w, wp);
#pragma unroll
    for (int k = 0; k < 4; k++) bf_fwd8(x[k], x[k + 4], w, wp);
  }
  u64 acc = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) acc ^= x[k];
  if (acc == 0x123456789ULL) out[0] = acc;  // keeps the chains live; practically never taken
}

// ------------------------------------------------------------------------------------
// Launchers.

#define IG_DISPATCH_LOGN(logn, ...)                   \
  switch (logn) {                                     \
    case 8: { constexpr int L = 8; __VA_ARGS__; } break;   \
    case 9: { constexpr int L = 9; __VA_ARGS__; } break;   \
    case 10: { constexpr int L = 10; __VA_ARGS__; } break; \
    case 11: { constexpr int L = 11; __VA_ARGS__; } break; \
    default: return cudaErrorInvalidValue;                 \
  }

cudaError_t fold_gadget_keys(const CrsDev& c, u64* keys, u32 count, cudaStream_t s) {
  const u32 total = count * 2 * c.n;
  if (total == 0) return cudaSuccess;
  k_fold_gadget_keys<<<(total + 255) / 256, 256, 0, s>>>(c, keys, count);
  return cudaGetLastError();
}

cudaError_t ntt_rows(const CrsDev& c, const u64* in, u64* out, u32 rows, u64 scale, u64 scalep, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  const size_t smem = 3 * (size_t)c.n * 8;
  IG_DISPATCH_LOGN(c.logn, {
    auto k = k_ntt_rows<L>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<rows, (1 << L) / 4, smem, s>>>(c, in, out, scale, scalep);
  });
  return cudaGetLastError();
}

cudaError_t store_fold(const CrsDev& c, const u64* H, u64* sums_R, cudaStream_t s) {
  if (c.gamma > (u32)FOLD_TILE || c.gamma == 0 || c.gamma > c.n) return cudaErrorInvalidValue;
  u32 SL = FOLD_TILE / c.gamma;
  if (SL > c.n) SL = c.n;
  if (c.n % SL) return cudaErrorInvalidValue;
  const u32 blocks = c.n / SL;
  const size_t smem = (FOLD_TILE + 2 * (size_t)c.n) * 8;
  IG_DISPATCH_LOGN(c.logn, {
    auto k = k_store_fold<L>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<blocks, FOLD_THREADS, smem, s>>>(c, H, sums_R, SL);
  });
  return cudaGetLastError();
}

u32 scan_chunks(u32 gamma) { return (gamma + SCAN_COLS - 1) / SCAN_COLS; }

cudaError_t shard_scan(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq, const u32* work,
                       u32 nwork, u64* b_fold, u32* status, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  const u32 chunks = scan_chunks(c.gamma);
  const u32 blocks = work ? nwork : nq * chunks;
  if (blocks == 0) return cudaSuccess;
  const size_t smem = scan_smem_bytes((int)c.n);
  IG_DISPATCH_LOGN(c.logn, {
    auto k = k_scan<L>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<blocks, SCAN_WARPS * 32, smem, s>>>(c, queries, shards, work, chunks, b_fold, status);
  });
  return cudaGetLastError();
}

cudaError_t column_tags(const CrsDev& c, const u64* cols, const u64* key, u64* tags_out, const u64* expect,
                        u32* mismatch, cudaStream_t s) {
  if (c.gamma == 0) return cudaSuccess;
  constexpr u32 per_cta = 8;  // warps of 256 threads, one column each
  IG_DISPATCH_LOGN(c.logn, {
    k_column_tags<L><<<(c.gamma + per_cta - 1) / per_cta, per_cta * 32, 0, s>>>(c.gamma, cols, key, tags_out,
                                                                              expect, mismatch);
  });
  return cudaGetLastError();
}

cudaError_t encode_records(const uint8_t* rec, u32 entries, u32 entry_size, u32 n, u32 gamma, u64* cols,
                           uint16_t* cols16, cudaStream_t s) {
  const size_t words = (size_t)gamma * n;
  k_encode_records<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(rec, entries, entry_size, n, gamma, cols, cols16);
  return cudaGetLastError();
}

cudaError_t wire(const u64* a, const u64* b, u32 count, u32 n, u32 retained, u32 bits, u64 modulus,
                 const uint8_t* tmpl, u32 len, u32 a_off, u32 a_bytes, u32 b_off, u32 b_bytes, uint8_t* out,
                 u32* status, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  dim3 grid((len + 255) / 256, count);
  k_wire<<<grid, 256, 0, s>>>(a, b, n, retained, bits, modulus, tmpl, len, a_off, a_bytes, b_off, b_bytes, out,
                              status);
  return cudaGetLastError();
}

cudaError_t compact16(const u64* cols, size_t words, uint16_t* out, u32* wide, cudaStream_t s) {
  if (words == 0 || words % 8) return cudaErrorInvalidValue;
  const size_t groups = words / 8;
  const unsigned threads = 256;
  k_compact16<<<(unsigned)((groups + threads - 1) / threads), threads, 0, s>>>(cols, groups, out, wide);
  return cudaGetLastError();
}

cudaError_t nopack(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq, u64 r_mod_q,
                   u64* AB_R, u64* out, u32* status, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  IG_DISPATCH_LOGN(c.logn, {
    constexpr int N = 1 << L;
    {
      auto k = k_nopack_prep<L>;
      const size_t smem = 4 * (size_t)N * 8;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      k<<<nq, N / 4, smem, s>>>(c, queries, r_mod_q, shoup_companion(r_mod_q), AB_R, status);
    }
    {
      auto k = k_nopack_cols<L>;
      const size_t smem = 5 * (size_t)N * 8;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      k<<<dim3(c.gamma, nq), N / 4, smem, s>>>(c, queries, shards, AB_R, out);
    }
    k_nopack_sum<<<dim3((2 * N + 255) / 256, nq), 256, 0, s>>>(N, c.gamma, out);
  });
  return cudaGetLastError();
}

cudaError_t keystream(const u32* key, u64 block0, u64 nblocks, u32* ks, cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  k_keystream<<<(unsigned)((nblocks + 255) / 256), 256, 0, s>>>(key, block0, nblocks, ks);
  return cudaGetLastError();
}

cudaError_t gauss_parse(const GaussDev& g, const u32* ks, u64 base, u64 W, u32 seg, uint8_t* maps, uint8_t* starts,
                        u32* counts, u64* offsets, u64* total, u64 S, i64* out, u64* end, cudaStream_t s) {
  const u64 T = (W + seg - 1) / seg;
  const unsigned blocks = (unsigned)((T + 255) / 256);
  k_gauss_maps<<<blocks, 256, 0, s>>>(g, ks, base, W, seg, maps, T);
  k_gauss_scan<<<1, 1024, 0, s>>>(maps, starts, nullptr, nullptr, nullptr, T);
  k_gauss_walk<<<blocks, 256, 0, s>>>(g, ks, base, W, seg, starts, T, counts, nullptr, S, out, end);
  k_gauss_scan<<<1, 1024, 0, s>>>(nullptr, nullptr, counts, offsets, total, T);
  k_gauss_walk<<<blocks, 256, 0, s>>>(g, ks, base, W, seg, starts, T, nullptr, offsets, S, out, end);
  return cudaGetLastError();
}

cudaError_t client_query(const CrsDev& c, const QueryDev* queries, u32 nq, const u64* s_R, const u32* locals,
                         const i64* samples, u64 delta, u64* b_out, u32* status, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  const size_t smem = 3 * (size_t)c.n * 8;
  IG_DISPATCH_LOGN(c.logn, {
    auto k = k_client_query<L>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<nq, (1 << L) / 4, smem, s>>>(c, queries, s_R, locals, samples, delta, b_out, status);
  });
  return cudaGetLastError();
}

cudaError_t client_extract(const CrsDev& c, u32 count, const u64* s_R, const u64* a, const u64* b, u64 modulus,
                           u64 delta, u64 p, u64 dinv, u32 entry_size, uint8_t* out, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  const size_t smem = 3 * (size_t)c.n * 8;
  IG_DISPATCH_LOGN(c.logn, {
    auto k = k_client_extract<L>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<count, (1 << L) / 4, smem, s>>>(c, s_R, a, b, modulus, delta, p, dinv, entry_size, out);
  });
  return cudaGetLastError();
}

size_t tree_smem_bytes(const CrsDev& c) { return ((size_t)8 * c.n + c.n / 2 + 32) * 8 + 2 * (size_t)c.n * 2; }

cudaError_t tree(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq, u64 r_mod_q, u64 ms_target,
                 u64* stack, u64* a_out, u64* b_out, u32* status, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  if (!c.galois_R || c.gamma > c.n / 2) return cudaErrorInvalidValue;
  const size_t smem = tree_smem_bytes(c);
  IG_DISPATCH_LOGN(c.logn, {
    auto k = k_tree<L>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<nq, (1 << L) / 4, smem, s>>>(c, queries, shards, r_mod_q, shoup_companion(r_mod_q), ms_target, stack, a_out,
                                      b_out, status);
  });
  return cudaGetLastError();
}

cudaError_t butterfly_peak(u64* out, int blocks, int iters, cudaStream_t s) {
  const u64 w = 0x0123456789ABCDEULL % Q;
  k_butterfly_peak<<<blocks, 256, 0, s>>>(out, iters, w, shoup_companion(w));
  return cudaGetLastError();
}

size_t respond_smem_bytes(const CrsDev& c, int ctas) {
  // X, D and a_ntt, the two ladders, three key rows of W and Y, two u16 slot tables.
  const size_t n = c.n;
  const size_t words = ctas == 4 ? n / 2 + 4 * n : ctas == 2 ? 5 * n : 6 * n;
  return (words + 2 * (size_t)3 * n) * 8 + 2 * n * 2;
}

cudaError_t respond(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq,
                    const u64* b_fold, u64* a_out, u64* b_out, u32* status,
                    int force_serial_expand, int ctas, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  if (ctas != 1 && ctas != 2 && ctas != 4) return cudaErrorInvalidValue;
  const size_t smem = respond_smem_bytes(c, ctas);
  IG_DISPATCH_LOGN(c.logn, {
    if (ctas == 4) {
      auto k = k_respond_quad<L>;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      k<<<4 * nq, (1 << L) / 8, smem, s>>>(c, queries, shards, b_fold, a_out, b_out, status, force_serial_expand);
    } else if (ctas == 2) {
      auto k = k_respond_pair<L>;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      k<<<2 * nq, (1 << L) / 4, smem, s>>>(c, queries, shards, b_fold, a_out, b_out, status, force_serial_expand);
    } else {
      auto k = k_respond<L>;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      k<<<nq, (1 << L) / 4, smem, s>>>(c, queries, shards, b_fold, a_out, b_out, status, force_serial_expand);
    }
  });
  return cudaGetLastError();
}


}  // namespace igk
