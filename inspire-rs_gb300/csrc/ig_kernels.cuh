// Device-side structures shared by the kernels and the runtime.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ig_arith.cuh"

namespace ig {

// Status words a kernel writes for the host; 0 = ok.
enum DeviceStatus : u32 {
  DEV_OK = 0,
  DEV_TAG_MISMATCH = 1,     // a column is not the column the store was built from
  DEV_EXPAND_EXHAUSTED = 2  // query `a` expansion ran past its candidate budget
};

// Per parameter-set constants, resident in device memory.
struct CrsDev {
  u32 n, logn, gamma, rows, approx;
  const u64 *tw, *twp;    // forward ladder psi^brv(m), Shoup companions (index m in [1, n))
  u64 ninv, ninvp;        // n^-1 mod q, Shoup
  u64 nlast, nlastp;      // n^-1 times the inverse's last twiddle (q - tw[1]), Shoup
  const uint16_t* slot_exp;  // odd exponent e_t of slot t's root relative to slot 0's
  const uint16_t* exp_slot;  // slot holding exponent e, indexed e/2
  const u32* gpow;           // g^i mod 2n, i < gamma
  const u32* cpow;           // g^-i mod 2n, i < gamma
  const u32* m_of_i;         // (g^-i - 1) / (2n/gamma)
  const u64* pow_root_R;     // w0^e * 2^64 mod q for e < 2n (w0 = slot 0's root)
  u64 inv_gamma_R, inv_gamma_Rp;  // gamma^-1 * 2^64 mod q, Shoup
  const u64* wmask_R;        // rows x n: NTT of the kept mask rows, R-form
  // The last exact-gadget digit's factors (D2 = base^-2 (R - D0 - base D1)) in R-form:
  // base^-2, -base^-2 and -base^-1, by which the key rows are folded (fold_gadget3).
  u64 ld_inv_R, ld_c0_R, ld_c1_R;
  // Galois keys of the automorphism tree (OnePacking), null when the CRS carries none:
  // key i (t = n / 2^i + 1) as 3 rows of (a, b), each n words, R-form NTT, folded at
  // upload (fold_gadget_keys) so the node stands in for the third digit.
  const u64* galois_R;
};

// One query of a launch.
struct QueryDev {
  u32 shard;          // index into the launch's shard table
  u32 fold_off;       // first of the query's gamma words in the launch's b_fold
  const u32* seed;    // 8 ChaCha20 key words of the query's `a` seed
  const u64* b;       // coefficient-form b of the query (n words)
  const u64* seat_R;  // rows x n key body in R-form NTT (the packing-key seat)
  const u64* a;       // explicit coefficient-form `a` (unseeded query), or null
  // The query's parameter set (a device copy of its CrsDev), or null for the launch's. Every
  // set of one launch shares the ring: n, q, the transform ladders and the slot tables;
  // gamma, the gadget, the key rows and the mask may differ per query.
  const CrsDev* crs;
  u64 ms;             // mod-switch target of the response (0: none)
  u32 row;            // the query's row of the launch's outputs and status words
  u32 pad;
};

// The parts of a parameter set that may differ between the queries of one respond launch.
struct SetView {
  u32 gamma, rows, approx;
  const u32* gpow;
  const u64* wmask_R;
  u64 ld_inv_R, ld_c0_R, ld_c1_R;
};

__device__ __forceinline__ SetView set_view(const CrsDev& c, const CrsDev* own) {
  if (own)
    return SetView{own->gamma, own->rows, own->approx, own->gpow, own->wmask_R, own->ld_inv_R, own->ld_c0_R,
                   own->ld_c1_R};
  return SetView{c.gamma, c.rows, c.approx, c.gpow, c.wmask_R, c.ld_inv_R, c.ld_c0_R, c.ld_c1_R};
}

// The client's Gaussian sampler (math/gaussian.rs:95-224): acceptance thresholds (f64 bit
// patterns of exp(-x^2 / 2 sigma^2), x = -tailcut .. tailcut) and rand's integer range.
struct GaussDev {
  const u64* accept;
  i64 tailcut;
  u64 range, zone;  // 2 tailcut + 1 and (range << clz(range)) - 1
};

struct ShardDev {
  const u64* columns;        // gamma x n raw column words
  const u64* sums_R;         // gamma x n step-1 sums, R-form NTT (the packing store)
  const u64* tag_key;        // 2n key words
  const u64* tags;           // gamma column tags
  const uint16_t* cols16;    // the same words as u16 when all are below 2^16, else null
  // 1 when the columns no longer give the store's tags (checked whenever the columns
  // change): a respond on the shard is refused with DEV_TAG_MISMATCH.
  u32 stale;
  u32 pad;
};

}  // namespace ig

// Launchers (ig_kernels.cu). Every launcher enqueues on `stream` and returns the
// launch status.
namespace igk {
using namespace ig;

// The Galois keys ([key][3 digits][2 parts][n], R-form NTT) folded in place for consumers
// that take R in place of the derived third digit.
cudaError_t fold_gadget_keys(const CrsDev& c, u64* keys, u32 count, cudaStream_t s);
// Forward NTT of `rows` polynomials: out[r] = scale * NTT(in[r] mod q), scale given with
// its Shoup companion (scale = 1 for standard form, 2^64 mod q for R-form).
cudaError_t ntt_rows(const CrsDev& c, const u64* in, u64* out, u32 rows, u64 scale, u64 scalep,
                     cudaStream_t s);

// Shard scan over `nq` queries: for query q and column j < gamma_q,
// b_fold[fold_off_q + j] = coeff0(b_q * column_j); a query on a stale shard gets
// DEV_TAG_MISMATCH. The work list (nwork entries, query << 12 | chunk, chunk < scan_chunks
// of the query's gamma) lets queries of different widths share a launch; without one, every
// query has c's gamma.
u32 scan_chunks(u32 gamma);
cudaError_t shard_scan(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq, const u32* work,
                       u32 nwork, u64* b_fold, u32* status, cudaStream_t s);

// Keyed tags of a shard's gamma columns (u64 words, key: 2n words below 2^61 - 1) into
// tags_out; with `expect` set, *mismatch gets 1 when a tag differs from expect instead.
cudaError_t column_tags(const CrsDev& c, const u64* cols, const u64* key, u64* tags_out, const u64* expect,
                        u32* mismatch, cudaStream_t s);

// One shard's columns from its records (entries of entry_size bytes, at most n of them):
// the gamma x n u64 words and their u16 copy.
cudaError_t encode_records(const uint8_t* rec, u32 entries, u32 entry_size, u32 n, u32 gamma, u64* cols,
                           uint16_t* cols16, cudaStream_t s);

// ServerResponse bytes of `count` responses into out[len * r ..] from the zero-coefficient
// template (a: n coefficients at a_off, b: `retained` at b_off, `bits` each).
cudaError_t wire(const u64* a, const u64* b, u32 count, u32 n, u32 retained, u32 bits, u64 modulus,
                 const uint8_t* tmpl, u32 len, u32 a_off, u32 a_bytes, u32 b_off, u32 b_bytes, uint8_t* out,
                 u32* status, cudaStream_t s);

// Compact u16 copy of `words` column words (a multiple of 8); sets *wide when a word is
// 2^16 or above (the copy is then unusable).
cudaError_t compact16(const u64* cols, size_t words, uint16_t* out, u32* wide, cudaStream_t s);

// Step-1 sums of one shard from the NTTs of its columns (H: gamma x n standard form).
cudaError_t store_fold(const CrsDev& c, const u64* H, u64* sums_R, cudaStream_t s);

// Fused per-query respond: expansion of `a`, store gather, backward recursion with the
// online gather, final transforms, the mod switch to each query's target (QueryDev::ms).
// `ctas` CTAs per query: 1, or a cluster of 2 or 4 that splits each query's transforms
// over as many SMs (shorter latency, more SM time). Queries may carry their own parameter
// set (QueryDev::crs) on c's ring.
cudaError_t respond(const CrsDev& c, const QueryDev* queries, const ShardDev* shards,
                    u32 nq, const u64* b_fold, u64* a_out, u64* b_out, u32* status, int force_serial_expand,
                    int ctas, cudaStream_t s);

size_t respond_smem_bytes(const CrsDev& c, int ctas);

// NoPacking respond of `nq` queries: out[q] holds gamma + 1 ciphertexts of (a, b), n words
// each in coefficient form, the column sum first (respond.rs:614-643). AB_R: nq x 2n words
// of scratch. r_mod_q = 2^64 mod q.
cudaError_t nopack(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq, u64 r_mod_q,
                   u64* AB_R, u64* out, u32* status, cudaStream_t s);

// OnePacking (respond_one_packing): one CTA per query walks the automorphism tree; stack
// holds nq x logn x 2n words of waiting nodes. Outputs coefficient-form (a, b), switched to
// ms_target when nonzero.
size_t tree_smem_bytes(const CrsDev& c);

// Client side: the sampler's keystream (ChaCha20 blocks of stream 0), the parallel parse of
// W stream words from u32 offset `base` of ks into the first S samples (out) and the word
// index after the S-th (*end; *total counts every sample in the window), the queries' b
// and the records of responses.
cudaError_t keystream(const u32* key, u64 block0, u64 nblocks, u32* ks, cudaStream_t s);
cudaError_t gauss_parse(const GaussDev& g, const u32* ks, u64 base, u64 W, u32 seg, uint8_t* maps, uint8_t* starts,
                        u32* counts, u64* offsets, u64* total, u64 S, i64* out, u64* end, cudaStream_t s);
cudaError_t client_query(const CrsDev& c, const QueryDev* queries, u32 nq, const u64* s_R, const u32* locals,
                         const i64* samples, u64 delta, u64* b_out, u32* status, cudaStream_t s);
cudaError_t client_extract(const CrsDev& c, u32 count, const u64* s_R, const u64* a, const u64* b, u64 modulus,
                           u64 delta, u64 p, u64 dinv, u32 entry_size, uint8_t* out, cudaStream_t s);
cudaError_t tree(const CrsDev& c, const QueryDev* queries, const ShardDev* shards, u32 nq, u64 r_mod_q, u64 ms_target,
                 u64* stack, u64* a_out, u64* b_out, u32* status, cudaStream_t s);

// Integer roofline probe: blocks x 256 threads x iters x 8 lazy butterflies in registers.
cudaError_t butterfly_peak(u64* out, int blocks, int iters, cudaStream_t s);
}  // namespace igk
