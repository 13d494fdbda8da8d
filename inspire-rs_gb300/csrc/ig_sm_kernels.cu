// Kernels of the special_modulus respond path (reference src/special_modulus/server.rs).
//
//   ntt_rows      forward Ntt32 of many rows (seat limbs, key mask, table columns)
//   table_columns nibble decode of a shard's cells (mod.rs:366-371, server.rs:211-249)
//   table_fold    step 1 folded over the columns (server.rs:331-383) as a per-slot DFT
//   body_fold     the response body's column fold over the shard's nibbles (server.rs:401-411)
//   respond       the 2n-link two-prime recursion and final transforms (server.rs:386-498)
//
// Every word is a canonical residue; products are Montgomery with R = 2^32 as in Prime32.
#include <cuda_runtime.h>

#include "ig_arith.cuh"
#include "ig_sm.cuh"

namespace igsmk {
using namespace igsm;

// ------------------------------------------------------------------------------------
// Ntt32 in shared memory, radix-4 (one 4-word unit per thread, N/4 threads). The stage
// schedule and twiddle indices are those of arith.rs:169-251: forward Cooley-Tukey over
// fwd[m + i], inverse Gentleman-Sande over inv[h + i] with the last stage carrying 1/n.
template <int LOGN>
__device__ __forceinline__ void fwd32(u32* x, const Ntt32Dev& T, const u32* tw) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  static_assert(LOGN & 1, "odd log n: one radix-2 stage then radix-4 pairs");
  const Prime32 P = T.p;
  const int tid = threadIdx.x;
  {
    constexpr int t = N / 2;
    const u32 w = tw[1];
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int b = tid + r * NT;
      const u32 u = x[b], v = P.mont(x[b + t], w);
      x[b] = P.add(u, v);
      x[b + t] = P.sub(u, v);
    }
    __syncthreads();
  }
#pragma unroll 1
  for (int s = 1; s < LOGN; s += 2) {
    const int t = N >> (s + 1), m = 1 << s, h = t >> 1;
    const int i = tid / h, o = tid - i * h;
    const int e0 = i * 2 * t + o;
    const u32 wa = tw[m + i], wb = tw[2 * m + 2 * i], wc = tw[2 * m + 2 * i + 1];
    u32 a0 = x[e0], a1 = x[e0 + h], a2 = x[e0 + t], a3 = x[e0 + t + h];
    u32 v = P.mont(a2, wa);
    a2 = P.sub(a0, v);
    a0 = P.add(a0, v);
    v = P.mont(a3, wa);
    a3 = P.sub(a1, v);
    a1 = P.add(a1, v);
    v = P.mont(a1, wb);
    x[e0] = P.add(a0, v);
    x[e0 + h] = P.sub(a0, v);
    v = P.mont(a3, wc);
    x[e0 + t] = P.add(a2, v);
    x[e0 + t + h] = P.sub(a2, v);
    __syncthreads();
  }
}

template <int LOGN>
__device__ __forceinline__ void inv32(u32* x, const Ntt32Dev& T, const u32* itw) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  static_assert(LOGN & 1, "odd log n: radix-4 pairs then the fused radix-2 stage");
  const Prime32 P = T.p;
  const int tid = threadIdx.x;
#pragma unroll 1
  for (int s = 0; s + 1 < LOGN; s += 2) {
    const int t = 1 << s, m = N >> (s + 1);
    const int B = tid >> s, o = tid & (t - 1);
    const int e0 = B * 4 * t + o;
    const u32 w0 = itw[m + 2 * B], w1 = itw[m + 2 * B + 1], w2 = itw[(m >> 1) + B];
    u32 a0 = x[e0], a1 = x[e0 + t], a2 = x[e0 + 2 * t], a3 = x[e0 + 3 * t];
    const u32 d01 = P.mont(a0 + P.m - a1, w0);
    a0 = P.add(a0, a1);
    const u32 d23 = P.mont(a2 + P.m - a3, w1);
    a2 = P.add(a2, a3);
    x[e0] = P.add(a0, a2);
    x[e0 + 2 * t] = P.mont(a0 + P.m - a2, w2);
    x[e0 + t] = P.add(d01, d23);
    x[e0 + 3 * t] = P.mont(d01 + P.m - d23, w2);
    __syncthreads();
  }
  {
    constexpr int t = N / 2;
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int b = tid + r * NT;
      const u32 u = x[b], v = x[b + t];
      x[b] = P.mont(u + v, T.n_inv);
      x[b + t] = P.mont(u + P.m - v, T.last);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------
template <int LOGN>
__global__ void __launch_bounds__((1 << LOGN) / 4) k_sm_ntt_rows(SmDev c, int which, const u32* in, u32* out,
                                                                 int to_mont) {
  constexpr int N = 1 << LOGN, NT = N / 4;
  __shared__ u32 x[N];
  __shared__ u32 tw[N];
  const Ntt32Dev& T = which ? c.lp : c.lq;
  const u32* row = in + (size_t)blockIdx.x * N;
  for (int k = threadIdx.x; k < N; k += NT) {
    x[k] = row[k] % T.p.m;
    tw[k] = T.fwd[k];
  }
  __syncthreads();
  fwd32<LOGN>(x, T, tw);
  // to_mont: mont(x, 2^64 mod m) = x 2^32 mod m.
  const u32 r2 = (u32)((((unsigned __int128)1) << 64) % T.p.m);
  u32* o = out + (size_t)blockIdx.x * N;
  for (int k = threadIdx.x; k < N; k += NT) o[k] = to_mont ? T.p.mont(x[k], r2) : x[k];
}

// values[m][j] for m < n (zero past `rows`), colq[j][m] = the nibble as a residue mod q.
__global__ void k_sm_columns(SmDev c, const uint8_t* cells, u32 rows, u32 cell_bytes, int8_t* values, u32* colq) {
  const u32 idx = blockIdx.x * blockDim.x + threadIdx.x;  // over n rows x gamma/2 bytes
  const u32 half = c.gamma / 2;
  if (idx >= c.n * half) return;
  const u32 m = idx / half, byte = idx % half;
  const uint8_t b = m < rows && byte < cell_bytes ? cells[(size_t)m * cell_bytes + byte] : 0;
  const int8_t lo = (int8_t)((int8_t)(uint8_t)(b << 4) >> 4);
  const int8_t hi = (int8_t)((int8_t)b >> 4);
  values[(size_t)m * c.gamma + 2 * byte] = lo;
  values[(size_t)m * c.gamma + 2 * byte + 1] = hi;
  colq[(size_t)(2 * byte) * c.n + m] = c.lq.p.small(lo);
  colq[(size_t)(2 * byte + 1) * c.n + m] = c.lq.p.small(hi);
}

// Step 1 per slot t (root w_t = w0^e_t): acc_i[t] = sum_j w_t^(j c_i) H_j[t] with
// c_i = g^-i = 1 + m_i (2n/gamma), i.e. a length-gamma DFT of u_j = w0^(e_t j) H_j[t] read
// at (e_t m_i) mod gamma; then S_i[t'] = gamma^-1 acc_i[t] at the slot t' whose image under
// tau_{g^i} is t, in R-form.
constexpr int SM_FOLD_TILE = 2048;
constexpr int SM_FOLD_THREADS = 256;

template <int LOGN>
__global__ void __launch_bounds__(SM_FOLD_THREADS) k_sm_fold(SmDev c, const u32* H, u32* step1_R, u32 SL) {
  constexpr int N = 1 << LOGN;
  constexpr u32 M2N = 2 * N - 1;
  __shared__ u32 x[SM_FOLD_TILE];
  __shared__ u32 pw[2 * N];
  const u32 gamma = c.gamma, tile = SL * gamma, t0 = blockIdx.x * SL;
  const Prime32 P = c.lq.p;
  u32 lg = 0;
  while ((1u << lg) < gamma) lg++;
  for (int k = threadIdx.x; k < 2 * N; k += SM_FOLD_THREADS) pw[k] = c.pow_root_R[k];
  __syncthreads();
  for (u32 idx = threadIdx.x; idx < tile; idx += SM_FOLD_THREADS) {
    const u32 j = idx / SL, s = idx % SL;
    const u32 e = c.slot_exp[t0 + s];
    x[s * gamma + j] = P.mont(H[(size_t)j * N + t0 + s], pw[(e * j) & M2N]);
  }
  __syncthreads();
  for (u32 len = gamma >> 1; len >= 1; len >>= 1) {
    for (u32 b = threadIdx.x; b < SL * (gamma >> 1); b += SM_FOLD_THREADS) {
      const u32 s = b / (gamma >> 1), bb = b % (gamma >> 1);
      const u32 blk = bb / len, j = bb % len;
      const u32 i0 = s * gamma + blk * 2 * len + j;
      const u32 u = x[i0], v = x[i0 + len];
      x[i0] = P.add(u, v);
      x[i0 + len] = P.mont(P.sub(u, v), pw[(j * (N / len)) & M2N]);
    }
    __syncthreads();
  }
  for (u32 idx = threadIdx.x; idx < tile; idx += SM_FOLD_THREADS) {
    const u32 i = idx / SL, s = idx % SL;
    const u32 e = c.slot_exp[t0 + s];
    const u32 k = (e * c.m_of_i[i]) & (gamma - 1);
    const u32 kr = lg ? (__brev(k) >> (32 - lg)) : 0;
    const u32 tp = c.exp_slot[((c.cpow[i] * e) & M2N) >> 1];
    step1_R[(size_t)i * N + tp] = P.mont(x[s * gamma + kr], c.inv_gamma_RR);
  }
}

// ------------------------------------------------------------------------------------
// Body fold: thread k < nb sums c_m values[m][k] over the shard's rows (exact in i64).
__global__ void __launch_bounds__(512) k_sm_body_fold(SmDev c, const SmQueryDev* queries, i64* fold) {
  const SmQueryDev qd = queries[blockIdx.x];
  const u32 k = threadIdx.x;
  if (k >= c.nb) return;
  const Prime32 P = c.lq.p;
  i64 acc = 0;
#pragma unroll 8
  for (u32 m = 0; m < qd.rows; m++) {
    const u32 bw = qd.body[m == 0 ? 0 : c.n - m];
    const i64 cm = m == 0 ? P.centred(bw) : -P.centred(bw);
    acc += cm * (i64)qd.values[(size_t)m * c.gamma + k];
  }
  fold[(size_t)blockIdx.x * c.nb + k] = acc;
}

// Inverse twiddle m of a ladder (Gentleman-Sande, psi^-brv(m)) from the forward ladder's
// Shoup pairs: for 2^s <= m < 2^(s+1), brv(3 2^s - 1 - m) = n - brv(m), so
// psi^-brv(m) = -psi^brv(3 2^s - 1 - m); and the companion of pm - w is the complement of
// w's (w != 0, pm prime above w).
__device__ __forceinline__ uint2 inv_tw(const uint2* fs, u32 pm, int m) {
  const int s = 31 - __clz(m);
  const uint2 f = fs[3 * (1 << s) - 1 - m];
  return make_uint2(pm - f.x, ~f.y);
}

// ------------------------------------------------------------------------------------
// expand_uniform (mod.rs:225-237) on the query seed's stream 0: accept u < floor(2^64/q) q,
// take u mod q. Word w of the stream is keystream words 2w, 2w+1. A rejection (probability
// below 2^-35 per word) shifts the rest, and the walk is redone word by word.
template <int N, int NT>
__device__ __forceinline__ void sm_expand(const SmQueryDev& qd, u32 q, u32* a, u32* status, u32 qi) {
  const int tid = threadIdx.x;
  const u64 zone = (~0ULL / q) * q;
  bool rejected = false;
  u32 key[8];
#pragma unroll
  for (int k = 0; k < 8; k++) key[k] = qd.seed[k];
  if (tid < N / 8) {
    u32 blk[16];
    ig::chacha20_block(key, (u64)tid, 0, blk);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const u64 v = (u64)blk[2 * k] | ((u64)blk[2 * k + 1] << 32);
      if (v >= zone) rejected = true;
      a[tid * 8 + k] = (u32)(v % q);
    }
  }
  if (__syncthreads_or(rejected)) {
    if (tid == 0) {
      u32 blk[16];
      u64 have = ~0ULL, cand = 0;
      int filled = 0;
      const u64 limit = (u64)N + 65536;
      while (filled < N && cand < limit) {
        const u64 bi = cand >> 3;
        if (bi != have) {
          ig::chacha20_block(key, bi, 0, blk);
          have = bi;
        }
        const int k = (int)(cand & 7);
        const u64 v = (u64)blk[2 * k] | ((u64)blk[2 * k + 1] << 32);
        if (v < zone) a[filled++] = (u32)(v % q);
        cand++;
      }
      if (filled < N) {
        atomicOr(status + qi, 2u);
        for (; filled < N; filled++) a[filled] = 0;
      }
    }
    __syncthreads();
  }
}

// p_to_q_centred / q_to_p_centred (mod.rs:334-355).
__device__ __forceinline__ u32 p_to_q(const SmDev& c, u32 r) {
  const Prime32 Q = c.lq.p;
  u32 base = r;
  for (u32 k = 0; k < c.p_over_q; k++) base = Q.csub(base);
  return r > (c.lp.p.m >> 1) ? Q.add(base, c.neg_off) : base;
}
// The same lift left in [0, 3q) for the lazy q passes: one Barrett step (the quotient
// estimate from floor(2^32 / q) is the true quotient or one less, r being below 2^32)
// leaves r mod q plus at most q, and the centred offset adds less than q.
__device__ __forceinline__ u32 p_to_q_lazy(const SmDev& c, u32 r) {
  const u32 base = r - __umulhi(r, c.q_mu) * c.lq.p.m;
  return r > (c.lp.p.m >> 1) ? base + c.neg_off : base;
}
__device__ __forceinline__ u32 q_to_p(const SmDev& c, u32 x) {
  return x > (c.lq.p.m >> 1) ? x + (c.lp.p.m - c.lq.p.m) : x;
}

// One CTA per query. Each link i = gamma-2 .. 0 (server.rs:434-487):
//   tp = NTT_p(lift(INTT_q(R_{i+1})));  cp = INTT_p(tp . w_p[tau_i]);  rq = NTT_q(lift(cp));
//   R_i = a[tau_i] S_i + (R_{i+1} w_q[tau_i] - rq) / p;
//   acc_q += R_{i+1} key_q[tau_i];  acc_p += tp key_p[tau_i].
// Thread u owns slots 4u..4u+3 (one transform unit), so the passes that act within a unit
// run in registers beside the pointwise steps: the first inverse pass of INTT_q, the last
// forward pass of NTT_p with the products by key_p and w_p and the first inverse pass of
// INTT_p, and the last forward pass of NTT_q with the link's update. Each inverse's last
// stage (t = n/2, carrying 1/n), the limb lift and the next forward's first stage (the
// same index pairs) run as one pass in place.
//
// Twiddle products are Shoup products against the forward ladders' (w, w') pairs (the
// inverse ladders derived from them by inv_tw); products by R-form operands are
// Montgomery products.
//
// LAZY (q below 2^29, so 8q < 2^32): the q-limb passes skip most reductions. montl and
// shoupl leave [0, 2q) for any 32-bit left operand, and the values between passes stay in [0, 4q)
// through INTT_q and in [0, 6q) through NTT_q; every sum and every difference (offset by
// 2q or 4q) stays below 8q. Values are brought to [0, q) where the arithmetic needs a
// residue: before the lift to p and at the end of the chain. The p limb (near 2^31) has
// no headroom and stays reduced.
template <int LOGN, bool LAZY>
__global__ void __launch_bounds__((1 << LOGN) / 4, 2)
    k_sm_respond(SmDev c, const SmQueryDev* queries, const i64* fold, u32* mask_out, u32* body_out, u32* status) {
  constexpr int N = 1 << LOGN, NT = N / 4, H = N / 2;
  constexpr u32 M2N = 2 * N - 1;
  extern __shared__ __align__(16) u32 smw[];
  u32* buf = smw;
  u32* a = smw + N;
  u32* kq = smw + 2 * N;
  u32* kp = smw + 3 * N;
  u32* wq = smw + 4 * N;
  u32* wp = smw + 5 * N;
  uint2* fqs = reinterpret_cast<uint2*>(smw + 6 * N);  // forward ladders with Shoup companions
  uint2* fps = reinterpret_cast<uint2*>(smw + 8 * N);
  uint16_t* e_tab = reinterpret_cast<uint16_t*>(smw + 10 * N);
  uint16_t* s_tab = e_tab + N;
  const int tid = threadIdx.x;
  const u32 qi = blockIdx.x;
  const SmQueryDev qd = queries[qi];
  const Prime32 PQ = c.lq.p, PP = c.lp.p;
  for (int k = tid; k < N; k += NT) {
    kq[k] = qd.seat[k];
    kp[k] = qd.seat[N + k];
    wq[k] = qd.seat[2 * N + k];
    wp[k] = qd.seat[3 * N + k];
    fqs[k] = c.lq.fwd_sh[k];
    fps[k] = c.lp.fwd_sh[k];
    e_tab[k] = c.slot_exp[k];
    s_tab[k] = c.exp_slot[k];
  }
  sm_expand<N, NT>(qd, PQ.m, a, status, qi);
  fwd32<LOGN>(a, c.lq, c.lq.fwd);

  const int l0 = 4 * tid;
  u32 cur[4], accq[4], accp[4], et[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    et[k] = e_tab[l0 + k];
    const u32 tb = s_tab[((c.gpow[c.gamma - 1] * et[k]) & M2N) >> 1];
    cur[k] = PQ.mont(a[tb], qd.step1_R[(size_t)(c.gamma - 1) * N + l0 + k]);
    accq[k] = 0;
    accp[k] = 0;
  }
  // Inverse stages 0-1 of unit tid (t = 1, block tid), in registers, to buf[l0..l0+3].
  auto inv_first = [&](const Prime32& P, const uint2* fs, u32 a0, u32 a1, u32 a2, u32 a3) {
    const uint2 w0 = inv_tw(fs, P.m, H + 2 * tid), w1 = inv_tw(fs, P.m, H + 2 * tid + 1),
                w2 = inv_tw(fs, P.m, H / 2 + tid);
    const u32 d01 = P.shoup(a0 + P.m - a1, w0.x, w0.y);
    a0 = P.add(a0, a1);
    const u32 d23 = P.shoup(a2 + P.m - a3, w1.x, w1.y);
    a2 = P.add(a2, a3);
    *reinterpret_cast<uint4*>(buf + l0) = make_uint4(P.add(a0, a2), P.add(d01, d23), P.shoup(a0 + P.m - a2, w2.x, w2.y),
                                                     P.shoup(d01 + P.m - d23, w2.x, w2.y));
  };
  // Inverse stages 2 .. logn-2 over buf (radix-4 pairs; logn is odd).
  auto inv_middle = [&](const Prime32& P, const uint2* fs) {
#pragma unroll 1
    for (int s = 2; s + 1 < LOGN; s += 2) {
      const int t = 1 << s, m = N >> (s + 1);
      const int B = tid >> s, o = tid & (t - 1);
      const int e0 = B * 4 * t + o;
      const uint2 w0 = inv_tw(fs, P.m, m + 2 * B), w1 = inv_tw(fs, P.m, m + 2 * B + 1),
                  w2 = inv_tw(fs, P.m, (m >> 1) + B);
      u32 a0 = buf[e0], a1 = buf[e0 + t], a2 = buf[e0 + 2 * t], a3 = buf[e0 + 3 * t];
      const u32 d01 = P.shoup(a0 + P.m - a1, w0.x, w0.y);
      a0 = P.add(a0, a1);
      const u32 d23 = P.shoup(a2 + P.m - a3, w1.x, w1.y);
      a2 = P.add(a2, a3);
      buf[e0] = P.add(a0, a2);
      buf[e0 + 2 * t] = P.shoup(a0 + P.m - a2, w2.x, w2.y);
      buf[e0 + t] = P.add(d01, d23);
      buf[e0 + 3 * t] = P.shoup(d01 + P.m - d23, w2.x, w2.y);
      __syncthreads();
    }
  };
  // Forward stages 1 .. logn-3 over buf.
  auto fwd_middle = [&](const Prime32& P, const uint2* fs) {
#pragma unroll 1
    for (int s = 1; s < LOGN - 2; s += 2) {
      const int t = N >> (s + 1), m = 1 << s, h = t >> 1;
      const int i = tid / h, o = tid - i * h;
      const int e0 = i * 2 * t + o;
      const uint2 wa = fs[m + i], wb = fs[2 * m + 2 * i], wc = fs[2 * m + 2 * i + 1];
      u32 a0 = buf[e0], a1 = buf[e0 + h], a2 = buf[e0 + t], a3 = buf[e0 + t + h];
      u32 v = P.shoup(a2, wa.x, wa.y);
      a2 = P.sub(a0, v);
      a0 = P.add(a0, v);
      v = P.shoup(a3, wa.x, wa.y);
      a3 = P.sub(a1, v);
      a1 = P.add(a1, v);
      v = P.shoup(a1, wb.x, wb.y);
      buf[e0] = P.add(a0, v);
      buf[e0 + h] = P.sub(a0, v);
      v = P.shoup(a3, wc.x, wc.y);
      buf[e0 + t] = P.add(a2, v);
      buf[e0 + t + h] = P.sub(a2, v);
      __syncthreads();
    }
  };
  // Forward stages logn-2, logn-1 of unit tid, in registers, from buf[l0..l0+3].
  auto fwd_last = [&](const Prime32& P, const uint2* fs, u32 (&x)[4]) {
    constexpr int MF = 1 << (LOGN - 2);
    const uint2 wa = fs[MF + tid], wb = fs[2 * MF + 2 * tid], wc = fs[2 * MF + 2 * tid + 1];
    const uint4 v4 = *reinterpret_cast<const uint4*>(buf + l0);
    u32 a0 = v4.x, a1 = v4.y, a2 = v4.z, a3 = v4.w;
    u32 v = P.shoup(a2, wa.x, wa.y);
    a2 = P.sub(a0, v);
    a0 = P.add(a0, v);
    v = P.shoup(a3, wa.x, wa.y);
    a3 = P.sub(a1, v);
    a1 = P.add(a1, v);
    v = P.shoup(a1, wb.x, wb.y);
    x[0] = P.add(a0, v);
    x[1] = P.sub(a0, v);
    v = P.shoup(a3, wc.x, wc.y);
    x[2] = P.add(a2, v);
    x[3] = P.sub(a2, v);
  };
  const u32 Q2 = 2 * PQ.m, Q4 = 4 * PQ.m, Q6 = 6 * PQ.m;
  // Lazy INTT_q passes: inputs below 4q, outputs below 4q (three reductions per unit).
  auto inv_unit_lazy = [&](uint2 w0, uint2 w1, uint2 w2, u32& a0, u32& a1, u32& a2, u32& a3) {
    const u32 d01 = PQ.shoupl(a0 + Q4 - a1, w0.x, w0.y);
    const u32 s01 = csub_by(a0 + a1, Q4);
    const u32 d23 = PQ.shoupl(a2 + Q4 - a3, w1.x, w1.y);
    const u32 s23 = csub_by(a2 + a3, Q4);
    a0 = csub_by(s01 + s23, Q4);
    a2 = PQ.shoupl(s01 + Q4 - s23, w2.x, w2.y);
    a1 = d01 + d23;
    a3 = PQ.shoupl(d01 + Q2 - d23, w2.x, w2.y);
  };
  auto inv_first_lazy = [&](u32 a0, u32 a1, u32 a2, u32 a3) {
    inv_unit_lazy(inv_tw(fqs, PQ.m, H + 2 * tid), inv_tw(fqs, PQ.m, H + 2 * tid + 1), inv_tw(fqs, PQ.m, H / 2 + tid), a0,
                  a1, a2, a3);
    *reinterpret_cast<uint4*>(buf + l0) = make_uint4(a0, a1, a2, a3);
  };
  auto inv_middle_lazy = [&]() {
#pragma unroll 1
    for (int s = 2; s + 1 < LOGN; s += 2) {
      const int t = 1 << s, m = N >> (s + 1);
      const int B = tid >> s, o = tid & (t - 1);
      const int e0 = B * 4 * t + o;
      u32 a0 = buf[e0], a1 = buf[e0 + t], a2 = buf[e0 + 2 * t], a3 = buf[e0 + 3 * t];
      inv_unit_lazy(inv_tw(fqs, PQ.m, m + 2 * B), inv_tw(fqs, PQ.m, m + 2 * B + 1), inv_tw(fqs, PQ.m, (m >> 1) + B), a0,
                    a1, a2, a3);
      buf[e0] = a0;
      buf[e0 + t] = a1;
      buf[e0 + 2 * t] = a2;
      buf[e0 + 3 * t] = a3;
      __syncthreads();
    }
  };
  // Lazy NTT_q passes: inputs below 6q, outputs below 6q (two reductions per unit).
  auto fwd_unit_lazy = [&](uint2 wa, uint2 wb, uint2 wc, u32& a0, u32& a1, u32& a2, u32& a3) {
    u32 v = PQ.shoupl(a2, wa.x, wa.y);
    a2 = a0 + Q2 - v;  // below 8q
    a0 = a0 + v;
    v = PQ.shoupl(a3, wa.x, wa.y);
    a3 = a1 + Q2 - v;
    a1 = a1 + v;
    a0 = csub_by(a0, Q4);  // below 4q
    v = PQ.shoupl(a1, wb.x, wb.y);
    a1 = a0 + Q2 - v;
    a0 = a0 + v;
    a2 = csub_by(a2, Q4);
    v = PQ.shoupl(a3, wc.x, wc.y);
    a3 = a2 + Q2 - v;
    a2 = a2 + v;
  };
  auto fwd_middle_lazy = [&]() {
#pragma unroll 1
    for (int s = 1; s < LOGN - 2; s += 2) {
      const int t = N >> (s + 1), m = 1 << s, h = t >> 1;
      const int i = tid / h, o = tid - i * h;
      const int e0 = i * 2 * t + o;
      u32 a0 = buf[e0], a1 = buf[e0 + h], a2 = buf[e0 + t], a3 = buf[e0 + t + h];
      fwd_unit_lazy(fqs[m + i], fqs[2 * m + 2 * i], fqs[2 * m + 2 * i + 1], a0, a1, a2, a3);
      buf[e0] = a0;
      buf[e0 + h] = a1;
      buf[e0 + t] = a2;
      buf[e0 + t + h] = a3;
      __syncthreads();
    }
  };
#pragma unroll 1
  for (int i = (int)c.gamma - 2; i >= 0; i--) {
    const uint4 sv4 = *reinterpret_cast<const uint4*>(qd.step1_R + (size_t)i * N + l0);
    const u32 sv[4] = {sv4.x, sv4.y, sv4.z, sv4.w};
    u32 tb[4];
    const u32 gp = c.gpow[i];
#pragma unroll
    for (int k = 0; k < 4; k++) tb[k] = s_tab[((gp * et[k]) & M2N) >> 1];
    if constexpr (LAZY) {
      inv_first_lazy(cur[0], cur[1], cur[2], cur[3]);
      __syncthreads();
      inv_middle_lazy();
    } else {
      inv_first(PQ, fqs, cur[0], cur[1], cur[2], cur[3]);
      __syncthreads();
      inv_middle(PQ, fqs);
    }
    // INTT_q's last stage with 1/n, the lift to p, and NTT_p's first stage, pair (b, b + n/2).
    // The lift takes residues, so both products are reduced fully here.
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int b = tid + r * NT;
      const u32 u = buf[b], v = buf[b + H];
      const u32 y0 = q_to_p(c, PQ.shoup(u + v, c.lq.n_inv_s, c.lq.n_inv_sp));
      const u32 y1 = q_to_p(c, PQ.shoup(u + (LAZY ? Q4 : PQ.m) - v, c.lq.last_s, c.lq.last_sp));
      const u32 z = PP.shoup(y1, fps[1].x, fps[1].y);
      buf[b] = PP.add(y0, z);
      buf[b + H] = PP.sub(y0, z);
    }
    __syncthreads();
    fwd_middle(PP, fps);
    {
      u32 tp[4], y[4];
      fwd_last(PP, fps, tp);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        accp[k] = PP.add(accp[k], PP.mont(tp[k], kp[tb[k]]));
        y[k] = PP.mont(tp[k], wp[tb[k]]);
      }
      inv_first(PP, fps, y[0], y[1], y[2], y[3]);
    }
    __syncthreads();
    inv_middle(PP, fps);
    // INTT_p's last stage with 1/n, the lift to q, and NTT_q's first stage.
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int b = tid + r * NT;
      const u32 u = buf[b], v = buf[b + H];
      const u32 xp0 = PP.shoup(u + v, c.lp.n_inv_s, c.lp.n_inv_sp);
      const u32 xp1 = PP.shoup(u + PP.m - v, c.lp.last_s, c.lp.last_sp);
      if constexpr (LAZY) {
        const u32 y0 = p_to_q_lazy(c, xp0);  // below 3q
        const u32 z = PQ.shoupl(p_to_q_lazy(c, xp1), fqs[1].x, fqs[1].y);
        buf[b] = y0 + z;  // below 5q
        buf[b + H] = y0 + Q2 - z;
      } else {
        const u32 y0 = p_to_q(c, xp0), y1 = p_to_q(c, xp1);
        const u32 z = PQ.shoup(y1, fqs[1].x, fqs[1].y);
        buf[b] = PQ.add(y0, z);
        buf[b + H] = PQ.sub(y0, z);
      }
    }
    __syncthreads();
    u32 rq[4];
    if constexpr (LAZY) {
      fwd_middle_lazy();
      constexpr int MF = 1 << (LOGN - 2);
      const uint4 v4 = *reinterpret_cast<const uint4*>(buf + l0);
      rq[0] = v4.x, rq[1] = v4.y, rq[2] = v4.z, rq[3] = v4.w;
      fwd_unit_lazy(fqs[MF + tid], fqs[2 * MF + 2 * tid], fqs[2 * MF + 2 * tid + 1], rq[0], rq[1], rq[2], rq[3]);
      // cur below 4q, rq below 6q: R_i = a S_i + (cur w_q - rq) / p lands below 4q, acc_q
      // stays below 2q.
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const u32 cq = PQ.montl(cur[k], wq[tb[k]]);
        accq[k] = csub_by(accq[k] + PQ.montl(cur[k], kq[tb[k]]), Q2);
        cur[k] = PQ.montl(a[tb[k]], sv[k]) + PQ.montl(cq + Q6 - rq[k], c.p_inv_R);
      }
    } else {
      fwd_middle(PQ, fqs);
      fwd_last(PQ, fqs, rq);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const u32 cq = PQ.mont(cur[k], wq[tb[k]]);
        accq[k] = PQ.add(accq[k], PQ.mont(cur[k], kq[tb[k]]));
        cur[k] = PQ.add(PQ.mont(a[tb[k]], sv[k]), PQ.mont(PQ.sub(cq, rq[k]), c.p_inv_R));
      }
    }
  }
  if constexpr (LAZY) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      cur[k] = PQ.csub(csub_by(cur[k], Q2));
      accq[k] = PQ.csub(accq[k]);
    }
  }
  // mask = INTT_q(R_0); body = mod_down(INTT_q(acc_q), INTT_p(acc_p)) + fold.
  __syncthreads();  // every thread is past its last read of buf
#pragma unroll
  for (int k = 0; k < 4; k++) buf[l0 + k] = cur[k];
  __syncthreads();
  inv32<LOGN>(buf, c.lq, c.lq.inv);
#pragma unroll
  for (int k = 0; k < 4; k++) mask_out[(size_t)qi * N + tid + k * NT] = buf[tid + k * NT];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; k++) buf[l0 + k] = accq[k];
  __syncthreads();
  inv32<LOGN>(buf, c.lq, c.lq.inv);
  u32 xq[4];
#pragma unroll
  for (int k = 0; k < 4; k++) xq[k] = buf[tid + k * NT];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; k++) buf[l0 + k] = accp[k];
  __syncthreads();
  inv32<LOGN>(buf, c.lp, c.lp.inv);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int t = tid + k * NT;
    if ((u32)t < c.nb) {
      const u32 down = PQ.mont(PQ.sub(xq[k], p_to_q(c, buf[t])), c.p_inv_R);
      i64 f = fold[(size_t)qi * c.nb + t] % (i64)PQ.m;
      if (f < 0) f += PQ.m;
      body_out[(size_t)qi * c.nb + t] = PQ.add(down, (u32)f);
    }
  }
}

// ------------------------------------------------------------------------------------
cudaError_t ntt_rows(const SmDev& c, int which, const u32* in, u32* out, u32 rows, int to_mont, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  if (c.logn != 11) return cudaErrorInvalidValue;
  k_sm_ntt_rows<11><<<rows, 512, 0, s>>>(c, which, in, out, to_mont);
  return cudaGetLastError();
}

cudaError_t table_columns(const SmDev& c, const uint8_t* cells, u32 rows, u32 cell_bytes, int8_t* values, u32* colq,
                          cudaStream_t s) {
  const u32 total = c.n * (c.gamma / 2);
  k_sm_columns<<<(total + 255) / 256, 256, 0, s>>>(c, cells, rows, cell_bytes, values, colq);
  return cudaGetLastError();
}

cudaError_t table_fold(const SmDev& c, const u32* H, u32* step1_R, cudaStream_t s) {
  if (c.logn != 11 || c.gamma == 0 || c.gamma > (u32)SM_FOLD_TILE) return cudaErrorInvalidValue;
  u32 SL = SM_FOLD_TILE / c.gamma;
  if (SL > c.n) SL = c.n;
  k_sm_fold<11><<<c.n / SL, SM_FOLD_THREADS, 0, s>>>(c, H, step1_R, SL);
  return cudaGetLastError();
}

cudaError_t body_fold(const SmDev& c, const SmQueryDev* queries, u32 nq, i64* fold, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  if (c.nb > 512) return cudaErrorInvalidValue;
  k_sm_body_fold<<<nq, 512, 0, s>>>(c, queries, fold);
  return cudaGetLastError();
}

cudaError_t respond(const SmDev& c, const SmQueryDev* queries, u32 nq, const i64* fold, u32* mask_out, u32* body_out,
                    u32* status, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  if (c.logn != 11) return cudaErrorInvalidValue;
  const size_t smem = (10 * (size_t)c.n) * 4 + 2 * (size_t)c.n * 2;
  // The lazy q-limb passes need every value below 8q to fit 32 bits.
  const bool lazy = (u64)c.lq.p.m * 8 <= (1ULL << 32);
  auto kern = lazy ? k_sm_respond<11, true> : k_sm_respond<11, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<nq, 512, smem, s>>>(c, queries, fold, mask_out, body_out, status);
  return cudaGetLastError();
}

}  // namespace igsmk
