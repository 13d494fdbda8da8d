/* inspire_gb300.h — C ABI of the GB300-native InsPIRe respond path.
 *
 * One shared library (libinspire_gb300.so) exposes the server respond path of
 * raven-inspire (hisoka-io/inspire-rs) to any host language over plain pointers and
 * sizes. Each entry point names the reference interface it replaces (file:line in the
 * reference crate). All polynomials are arrays of ring_dim u64 coefficients in
 * coefficient form; multi-polynomial arguments are row-major (row r at offset r*ring_dim).
 *
 * Errors: every call returns IG_OK (0) or an IG_ERR_* code, and stores an actionable
 * message retrievable with ig_last_error(). A refused batch produces no partial output
 * (respond.rs:1187). Device faults are never used to signal refusals: kernels report
 * through status words the host reads back.
 *
 * Threading: a context serialises its calls internally; distinct contexts may be used
 * from distinct threads. Handles (CRS, database, session store, seat) are owned by the
 * context that made them and freed with the matching *_destroy / ig_seat_remove.
 */
#ifndef INSPIRE_GB300_H
#define INSPIRE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum ig_status {
  IG_OK = 0,
  IG_ERR_ARG = 1,           /* null pointer, zero count, bad size */
  IG_ERR_SHAPE = 2,         /* wire shape refused: ring, moduli, row count (respond.rs:409-611) */
  IG_ERR_WIDTH = 3,         /* packing width / key width mismatch (session.rs:766-826) */
  IG_ERR_HANDLE = 4,        /* unknown CRS/db/store/seat handle (respond.rs:1117-1134) */
  IG_ERR_STORE_REFUSED = 5, /* columns differ from the store's (shard_store.rs:247-257) */
  IG_ERR_CUDA = 6,          /* CUDA runtime error */
  IG_ERR_UNSUPPORTED = 7,   /* parameter set outside what the GPU path serves */
  IG_ERR_NOMEM = 8,         /* device allocation failed (admission refused) */
  IG_ERR_DEVICE = 9,        /* a kernel reported an internal status */
  IG_ERR_EXHAUSTED = 10,    /* handle space exhausted (session.rs:722-737) */
  IG_ERR_PENDING = 11       /* serving ticket not finished within the wait's timeout */
};

typedef struct ig_ctx ig_ctx;

/* ---- context ------------------------------------------------------------------------ */
int ig_ctx_create(int device, ig_ctx** out);
void ig_ctx_destroy(ig_ctx* ctx);
/* Copies the last error message of this context (NUL-terminated, truncated to len). */
int ig_last_error(const ig_ctx* ctx, char* buf, size_t len);
/* The CUDA stream (cudaStream_t) every kernel of this context is launched on. */
void* ig_ctx_stream(ig_ctx* ctx);
/* Device bytes held by this context's objects (stores, shards, seats, scratch). */
uint64_t ig_ctx_device_bytes(const ig_ctx* ctx);
/* Launch-shape knob of the fixed rule, used when the context holds no tuned table for the
 * launch's width (ig_tune_launch_shapes): with q the queries expected on the device (the
 * batch times the lanes, or the queries in flight), a launch runs four CTAs per query (a
 * thread-block cluster) while 2q <= max_queries, two while q <= max_queries, else one, so
 * small batches still occupy most SMs. Default: half the device's SM count; 0 runs one CTA
 * per query always. Responses are identical under every shape. */
int ig_ctx_set_pair_threshold(ig_ctx* ctx, uint32_t max_queries);
/* Launch shapes and their tuner. A respond launch runs 1, 2 or 4 CTAs per query: one CTA
 * per SM is the most work per SM-second; a cluster of 2 or 4 splits each query's
 * transforms over as many SMs and answers a small batch sooner. No counterpart in the
 * reference (its respond is CPU code).
 * ig_ctx_set_launch_shape fixes the shape of every later respond launch (1, 2 or 4), or
 * with 0 lets each launch choose: from the tuned table when it holds the launch's ring (the
 * tuned gamma nearest the launch's), else by the pair-threshold rule above.
 * ig_tune_launch_shapes measures the table for `count` packing widths on ring_dim: for each
 * width, each batch size of the grid 1, 4, 16, 32, 64, 128, 256 and each shape, the mean
 * milliseconds of `reps` launches (after one warm-up) on a synthetic database of 8 shards,
 * a synthetic seat and queries, built and freed inside. A launch then takes the shape whose
 * time is least (by at least 2% for more CTAs) in the table's row for the queries expected
 * in flight with it: the smallest tuned batch size at or above that number, the largest
 * beyond the grid. The device path expects count x lanes queries in flight, the serving
 * loop its batch and the CTAs of its batches in flight. Responses are identical under
 * every shape.
 * ig_tune_get copies the row of (ring_dim, gamma) for `queries` in flight (ms_out[0..2]: 1,
 * 2, 4 CTAs per query); ig_tune_choose gives the shape a launch of `count` queries with
 * `in_flight` queries expected would take. ig_tune_save writes the table to a text file
 * with the device's SM count, and ig_tune_load merges a saved table, refusing one measured
 * on another SM count. */
int ig_ctx_set_launch_shape(ig_ctx* ctx, uint32_t ctas);
int ig_tune_launch_shapes(ig_ctx* ctx, uint32_t ring_dim, const uint32_t* gammas, uint32_t count, uint32_t reps);
int ig_tune_get(ig_ctx* ctx, uint32_t ring_dim, uint32_t gamma, uint32_t queries, double* ms_out);
int ig_tune_choose(ig_ctx* ctx, uint32_t ring_dim, uint32_t gamma, uint32_t count, uint32_t in_flight,
                   uint32_t* ctas);
int ig_tune_save(ig_ctx* ctx, const char* path);
int ig_tune_load(ig_ctx* ctx, const char* path);
/* Device-path lanes (1..8, default 1). With lanes > 1, consecutive
 * ig_respond_seeded_batch_device calls rotate over that many streams, each with its own
 * scratch, so a batch's scan and recursion overlap the batches before it and batches of
 * fewer queries than SMs still fill the GPU. Each call's work starts after everything
 * queued on the context stream before it; call ig_ctx_join before reading a lane's
 * outputs on the context stream. The host-buffer calls (ig_respond_seeded_batch,
 * ig_respond_one_packing_batch, ig_respond_nopacking_batch, ig_sm_respond_batch) each hold
 * one lane while their batch runs and take the context lock only to validate and launch,
 * so calls from several threads overlap on the device. Responses are identical for any
 * lane count. */
int ig_ctx_set_lanes(ig_ctx* ctx, uint32_t lanes);
/* Orders the context stream after all work queued on the lanes. */
int ig_ctx_join(ig_ctx* ctx);

/* ---- CRS / ServerInspiringCache ------------------------------------------------------
 * Replaces ServerInspiringCache::new (respond.rs:926-941) = PackParams::try_new
 * (inspiring2.rs:171-183, 209-286) + OfflinePackingKeys::generate (537-598): builds the
 * twiddle ladders, slot tables and the w_seed mask rows on the device once per
 * (params, gamma, w_seed). Supported: q = 2^60-2^14+1 single prime, gadget base 2^20,
 * packing gadget length 3, ring_dim 256..2048, gamma a power of two <= ring_dim/2. */
int ig_crs_create(ig_ctx* ctx, uint32_t ring_dim, uint64_t q, uint64_t p, uint64_t gadget_base,
                  uint32_t packing_gadget_len, int approximate_packing_gadget, uint32_t gamma,
                  const uint8_t w_seed[32], uint64_t* crs_out);
int ig_crs_destroy(ig_ctx* ctx, uint64_t crs);
/* Packing-key rows the CRS expects: InspireParams::packing_key_rows (params.rs:484-487). */
int ig_crs_key_rows(ig_ctx* ctx, uint64_t crs, uint32_t* rows_out);

/* ---- EncodedDatabase / ShardData ----------------------------------------------------
 * A device-resident database of num_shards shards of gamma column polynomials
 * (EncodedDatabase, setup.rs:272-289). Columns hold raw u64 words as encode_database
 * produced them (encode_db.rs:74-134); words >= q are served as their residue. */
int ig_db_create(ig_ctx* ctx, uint64_t crs, uint32_t num_shards, uint64_t* db_out);
int ig_db_destroy(ig_ctx* ctx, uint64_t db);
/* Uploads (or replaces) shard `shard_id`'s gamma x ring_dim columns. Replacing columns
 * keeps any store. The new columns' keyed tags are checked against the store's at once
 * (the check ShardPackingStore::check_columns_and_fold_b makes at every respond,
 * shard_store.rs:197-264, made here once per change because the library writes every
 * column word itself): when they differ, every respond on the shard is refused
 * (IG_ERR_STORE_REFUSED, shard_store.rs:247-257) until its store is rebuilt. */
int ig_db_set_shard(ig_ctx* ctx, uint64_t db, uint32_t shard_id, const uint64_t* columns);
/* Same, from a device pointer (columns already in HBM). */
int ig_db_set_shard_device(ig_ctx* ctx, uint64_t db, uint32_t shard_id, const uint64_t* d_columns);
/* encode_database (pir/encode_db.rs:74-134) on the GPU: `nbytes` of concatenated entries
 * of entry_size bytes, split into shards of ring_dim entries (the last may be partial) and
 * into ceil(entry_size / 2) columns of 16-bit little-endian words (encode_db.rs:152-168),
 * written straight into shards first_shard.. of the database (a large database is encoded
 * in pieces of whole shards). entry_size must give the CRS's gamma; the entries must fit
 * the database's shards. records is a host pointer, or a device pointer when
 * on_device != 0. Existing stores are kept, as with ig_db_set_shard. */
int ig_db_encode_records(ig_ctx* ctx, uint64_t db, uint32_t first_shard, const uint8_t* records, size_t nbytes,
                         uint32_t entry_size, int on_device);
/* ShardData::precompute_packing (setup.rs:335-340) -> ShardPackingStore::build
 * (shard_store.rs:86-156): step-1 sums in HBM plus keyed column tags. */
int ig_db_precompute_packing(ig_ctx* ctx, uint64_t db, uint32_t shard_id);
/* All shards at once (the serving bring-up). */
int ig_db_precompute_packing_all(ig_ctx* ctx, uint64_t db);
/* ShardData::drop_packing_store (setup.rs:372-375). */
int ig_db_drop_packing_store(ig_ctx* ctx, uint64_t db, uint32_t shard_id);
/* 1 when the shard has a store (ShardData::packing_store, setup.rs:367-369). */
int ig_db_has_store(ig_ctx* ctx, uint64_t db, uint32_t shard_id, int* out);

/* ---- ServerSessionStore ---------------------------------------------------------------
 * session.rs:700-895. Handles come from one process-global monotonic counter and are
 * never reissued. A seat keeps y_body in NTT form on the device (49,152 B at 3 rows,
 * 32,768 B under the approximate gadget). */
int ig_session_store_create(ig_ctx* ctx, uint64_t* store_out);
int ig_session_store_destroy(ig_ctx* ctx, uint64_t store);
/* ServerSessionStore::register_server_side (session.rs:848-856) via
 * PackingKeySeat::from_wire (592-625): y_body is key_rows x ring_dim coefficient-form. */
int ig_session_register(ig_ctx* ctx, uint64_t store, uint64_t crs, const uint64_t* y_body, uint32_t rows,
                        uint32_t num_to_pack, uint64_t* handle_out);
/* ServerSessionStore::remove (879-886); *removed = 1 when the handle was present. */
int ig_session_remove(ig_ctx* ctx, uint64_t store, uint64_t handle, int* removed);
/* ServerSessionStore::len (888-890). */
int ig_session_len(ig_ctx* ctx, uint64_t store, uint64_t* len_out);
/* ServerSessionStore::get (858-866) as a presence test; *present = 0/1. */
int ig_session_contains(ig_ctx* ctx, uint64_t store, uint64_t handle, int* present);

/* ---- respond ---------------------------------------------------------------------------
 * Packing key of a call: seat `handle` from `store` (PackingKeySource::Registered), or an
 * inline key body (PackingKeySource::Inline) when inline_y_body != NULL, which is checked
 * into a request-scoped seat (resolve_packing_seat, respond.rs:1144-1157).
 *
 * ig_respond_seeded_batch replaces respond_seeded_batch (respond.rs:1189-1202): queries
 * answered in order, all or nothing. A one-query call is respond_seeded_inspiring
 * (respond.rs:1218-1226). Per query: shard_ids[i], seeds[32*i..] (the SeededRlweCiphertext
 * seed of the one RGSW row) and bs[i*ring_dim..] (its b). Outputs: the packed ciphertext's
 * a (a_out[i*ring_dim..]) and b (b_out[i*ring_dim..], the first gamma coefficients are the
 * response's b prefix). mod_switch_target != 0 applies mod_switch_response_checked
 * (mod_switch.rs:178-186) to both, e.g. 68718428161 (MOD_SWITCH_TARGET_36BIT). A call with
 * count 0 resolves the packing key (refused as above) and answers nothing; its buffers may
 * be NULL. */
int ig_respond_seeded_batch(ig_ctx* ctx, uint64_t db, uint64_t store, uint64_t handle, const uint64_t* inline_y_body,
                            uint32_t inline_rows, uint32_t inline_num_to_pack, uint32_t count,
                            const uint32_t* shard_ids, const uint8_t* seeds, const uint64_t* bs,
                            uint64_t mod_switch_target, uint64_t* a_out, uint64_t* b_out);

/* The unseeded form: respond_inspiring_cached_with_session over ClientQuery rows whose
 * `a` travels in full (respond.rs:1053-1091); as[i*ring_dim..] replaces the seed. */
int ig_respond_batch(ig_ctx* ctx, uint64_t db, uint64_t store, uint64_t handle, const uint64_t* inline_y_body,
                     uint32_t inline_rows, uint32_t inline_num_to_pack, uint32_t count, const uint32_t* shard_ids,
                     const uint64_t* as, const uint64_t* bs, uint64_t mod_switch_target, uint64_t* a_out,
                     uint64_t* b_out);

/* Same batch with every input and output already in device memory (d_* pointers); the
 * call only enqueues work on the context stream and returns. Per-query status words land
 * in d_status (0 = served, 1 = store refused the shard's columns); the host must check
 * them before using the outputs. The queried shards must hold packing stores. */
int ig_respond_seeded_batch_device(ig_ctx* ctx, uint64_t db, uint64_t store, uint64_t handle, uint32_t count,
                                   const uint32_t* shard_ids, const uint8_t* d_seeds, const uint64_t* d_bs,
                                   uint64_t mod_switch_target, uint64_t* d_a_out, uint64_t* d_b_out,
                                   uint32_t* d_status);

/* Queries of several databases, parameter sets (record widths, exact or approximate gadget),
 * seats and mod-switch targets answered in one scan and one respond launch: a fused form of
 * one respond_seeded_batch call (respond.rs:1189-1202) per (key, database) group. Query i
 * reads shard shard_ids[i] of database dbs[i] under seat handles[i] of session store
 * stores[i], with seeds[32 i..] and bs[ring_dim i..], switched to ms_targets[i] (0: none;
 * ms_targets may be NULL for no switch at all); its response is a_out[ring_dim i..] and
 * b_out[ring_dim i..], the bytes ig_respond_seeded_batch gives for the same query. Every
 * database must share one ring_dim, and every queried shard must hold a packing store. The
 * launch runs the queries with the longest recursion (largest gamma) first. All or nothing,
 * refused whole on the first error. */
int ig_respond_mixed_batch(ig_ctx* ctx, uint32_t count, const uint64_t* dbs, const uint64_t* stores,
                           const uint64_t* handles, const uint32_t* shard_ids, const uint8_t* seeds, const uint64_t* bs,
                           const uint64_t* ms_targets, uint64_t* a_out, uint64_t* b_out);
/* Same with the seeds, b, a, b and status words in device memory (shard_ids, dbs, stores,
 * handles and ms_targets stay host arrays); enqueues on the context's lanes like
 * ig_respond_seeded_batch_device and returns, status words in d_status[i] (0 = served,
 * 1 = the shard's store refused its columns). */
int ig_respond_mixed_batch_device(ig_ctx* ctx, uint32_t count, const uint64_t* dbs, const uint64_t* stores,
                                  const uint64_t* handles, const uint32_t* shard_ids, const uint8_t* d_seeds,
                                  const uint64_t* d_bs, const uint64_t* ms_targets, uint64_t* d_a_out,
                                  uint64_t* d_b_out, uint32_t* d_status);

/* Allocation-free form of ig_respond_seeded_batch_device, with no counterpart in the
 * reference. For callers that must not have the library allocate device memory while
 * serving: servers that size every device buffer at start-up and refuse growth later,
 * and processes sharing a GPU under a memory cap, where an allocation on the request path
 * can fail or evict a neighbour. The call's scratch (fold of b, query descriptors, status
 * words) lives in one fixed device array of 528,640 bytes that every GPU loading the
 * library holds until the process exits; the call makes no cudaMalloc/cudaFree and no
 * other allocating call. Limits: at most 64 queries per call, gamma at most 1024, a
 * registered seat (handle) and packing stores on the queried shards; larger batches are
 * refused with IG_ERR_ARG before any work. The first call on a device resolves the
 * array's device address (cudaGetSymbolAddress). All calls share the array, and it keeps the last call's contents: calls that
 * overlap on the GPU (from different contexts of one device) race and must be serialised
 * by the caller. Inputs and outputs are device pointers as in
 * ig_respond_seeded_batch_device. The call blocks: it synchronises the context stream,
 * reads the batch's status words back and returns after the batch completes, with a
 * refused batch reported as in ig_respond_seeded_batch. */
int ig_respond_seeded_batch_noalloc(ig_ctx* ctx, uint64_t db, uint64_t store, uint64_t handle, uint32_t count,
                                    const uint32_t* shard_ids, const uint8_t* d_seeds, const uint64_t* d_bs,
                                    uint64_t mod_switch_target, uint64_t* d_a_out, uint64_t* d_b_out);

/* ---- special_modulus ------------------------------------------------------------------
 * The two-prime packed variant of src/special_modulus/ (mod.rs, server.rs): ciphertext
 * prime q < 2^29, special prime p < 2^31, 4-bit signed nibbles, all words 32-bit.
 *
 * Server::new / with_kernel (server.rs:145-164) over Params (mod.rs:62-159); the GPU path
 * serves ring_dim 2048 (Params::ring2048_cell256: gamma 512, q 536813569,
 * p 2147389441, 256-byte cells, 246-byte records, key-mask version 2). */
int ig_sm_server_create(ig_ctx* ctx, uint32_t ring_dim, uint32_t gamma, uint64_t q, uint64_t special_prime,
                        uint32_t cell_bytes, uint32_t record_bytes, uint32_t key_mask_version, uint64_t* server_out);
int ig_sm_server_destroy(ig_ctx* ctx, uint64_t server);
/* Server::seat (server.rs:177-203): the decoded PackingKey (mask seed, q limb, p limb, each
 * limb ring_dim residues) -> a 32,768-byte device seat (both limbs and the key's own mask,
 * NTT, Montgomery form). Refuses non-residues. */
int ig_sm_seat(ig_ctx* ctx, uint64_t server, const uint8_t mask_seed[32], const uint32_t* key_q,
               const uint32_t* key_p, uint64_t* seat_out);
int ig_sm_seat_destroy(ig_ctx* ctx, uint64_t seat);
/* Server::table (server.rs:211-249) -> ShardTable: at most ring_dim cells of cell_bytes,
 * bytes past each record zero; the step-1 table (4 MiB) and the nibbles (1 MiB) in HBM. */
int ig_sm_table(ig_ctx* ctx, uint64_t server, const uint8_t* cells, size_t nbytes, uint64_t* table_out);
int ig_sm_table_destroy(ig_ctx* ctx, uint64_t table);
/* Test hook: the table's step-1 words (gamma x ring_dim, Montgomery form, as the reference
 * holds them) copied to host memory. */
int ig_sm_table_step1(ig_ctx* ctx, uint64_t table, uint32_t* out);
/* Server::respond (server.rs:252-279) for `count` queries: query i reads tables[i] under
 * seats[i], its Query = seeds[32 i..] and bodies[ring_dim i..]; the Response is
 * mask_out[ring_dim i..] and body_out[2 record_bytes i..]. All or nothing. */
int ig_sm_respond_batch(ig_ctx* ctx, uint64_t server, uint32_t count, const uint64_t* tables, const uint64_t* seats,
                        const uint8_t* seeds, const uint32_t* bodies, uint32_t* mask_out, uint32_t* body_out);
/* Same with device-resident inputs and outputs; enqueues and returns, status words in
 * d_status (0 = served). */
int ig_sm_respond_batch_device(ig_ctx* ctx, uint64_t server, uint32_t count, const uint64_t* tables,
                               const uint64_t* seats, const uint8_t* d_seeds, const uint32_t* d_bodies,
                               uint32_t* d_mask_out, uint32_t* d_body_out, uint32_t* d_status);

/* Response::to_bytes (special_modulus/wire.rs:120-125): mask (n words) then body (nb
 * words), each packed at q's bit width; 9,208 bytes at the served set. */
int ig_sm_response_encode(const uint32_t* mask, uint32_t n, const uint32_t* body, uint32_t nb, uint64_t q,
                          uint8_t* out, size_t cap, size_t* len_out);

/* ---- serving loop (continuous batching) ----------------------------------------------------
 * No single counterpart in the reference, whose server answers one respond_seeded_batch call
 * at a time (respond.rs:1189-1202); this loop batches individually arriving queries instead.
 * Each request is one seeded query under a seat registered in `store`, on a shard whose
 * packing store was built. A dispatcher thread forms batches from the oldest waiting requests
 * on one ring: databases, parameter sets (record widths, exact or approximate gadget),
 * shards, seats and mod-switch targets may differ within a batch. Each batch runs on one of
 * `slots` streams, so batches overlap on the device.
 *
 * Admission is by memory: hbm_budget_bytes (0: room for every slot full of max_batch of the
 * largest requests) is allocated once at create as a device ring (with a pinned host
 * mirror), and a request joins a batch only while the bytes of its buffers (descriptor,
 * seed, b, b fold, a, b, status, wire) and of its key (its seat, counted once while any
 * request on it is in flight) fit what the batches in flight leave free; the others wait in
 * arrival order, and a request that could not fit even alone is refused (IG_ERR_NOMEM).
 * create refuses (IG_ERR_NOMEM) when the budget cannot be allocated. A request's result
 * equals ig_respond_seeded_batch's for the same query. Databases, shards and seats named by a
 * request must stay alive until the request's ticket is finished.
 *
 * ig_serve_submit copies seed (32 B) and b (ring_dim words) and returns a ticket; a_out and
 * b_out (ring_dim words each) are written before the ticket finishes. Submission is refused
 * (IG_ERR_NOMEM) while 8 x slots x max_batch requests are waiting.
 * ig_serve_wait blocks up to timeout_ms (< 0: no limit) and returns the request's status
 * (IG_ERR_PENDING on timeout, the ticket stays valid); err receives the refusal message.
 * ig_serve_stats reports counts, latency percentiles from submit to result and the memory
 * admitted; reset != 0 clears them. ig_serve_destroy finishes every submitted request, then
 * frees the loop. */
typedef struct ig_serve ig_serve;
typedef struct ig_serve_stats_t {
  uint64_t served, refused, batches, waiting, device_bytes;
  double mean_batch, p50_us, p99_us, max_us;
  /* Memory admission: the budget, the bytes (keys and buffers) of the requests in flight
   * now, and their peak since create or the last reset. */
  uint64_t budget_bytes, inflight_bytes, peak_inflight_bytes;
  /* Where a served request's time went: from submission to its batch's launch, and from the
   * launch to its result in the caller's buffer (percentiles in microseconds). */
  double queue_p50_us, queue_p99_us, exec_p50_us, exec_p99_us;
} ig_serve_stats_t;
int ig_serve_create(ig_ctx* ctx, uint32_t slots, uint32_t max_batch, uint64_t hbm_budget_bytes, ig_serve** out);
int ig_serve_submit(ig_serve* s, uint64_t db, uint64_t store, uint64_t handle, uint32_t shard_id,
                    const uint8_t* seed, const uint64_t* b, uint32_t ring_dim, uint64_t mod_switch_target,
                    uint64_t* a_out, uint64_t* b_out, uint64_t* ticket_out);
/* The same request answered as ServerResponse bytes (respond.rs:111-176) built on the GPU
 * next to the batch's responses: wire_out receives *wire_len bytes (at most wire_cap;
 * 10,446 at the 36-bit switch with gamma 256) when the ticket finishes. */
int ig_serve_submit_wire(ig_serve* s, uint64_t db, uint64_t store, uint64_t handle, uint32_t shard_id,
                         const uint8_t* seed, const uint64_t* b, uint32_t ring_dim, uint64_t mod_switch_target,
                         uint8_t* wire_out, size_t wire_cap, size_t* wire_len, uint64_t* ticket_out);
int ig_serve_wait(ig_serve* s, uint64_t ticket, int64_t timeout_ms, uint64_t* latency_ns, char* err, size_t err_len);
int ig_serve_stats(ig_serve* s, ig_serve_stats_t* out, int reset);
/* Native load driver for the loop: submits a trace of `count` requests (request i reads
 * shard_ids[i] under seat handles[i] with seed seeds[32 i..] and b bs[ring_dim i..]) from
 * the calling thread, each at t0 + arrival_ns[i] when arrival_ns is given (open loop), and
 * with at most `window` requests outstanding when window != 0 (closed loop). Returns when
 * every request has finished; a_out/b_out receive the responses (ring_dim words each),
 * latency_ns (optional) each request's submit-to-result time, elapsed_s the trace's
 * duration. The status is the first request's failure, IG_OK when all were served. */
int ig_serve_replay(ig_serve* s, uint64_t db, uint64_t store, uint32_t count, const uint32_t* shard_ids,
                    const uint64_t* handles, const uint8_t* seeds, const uint64_t* bs, uint32_t ring_dim,
                    uint64_t mod_switch_target, const uint64_t* arrival_ns, uint32_t window, uint64_t* a_out,
                    uint64_t* b_out, uint64_t* latency_ns, double* elapsed_s);
int ig_serve_destroy(ig_serve* s);

/* ---- NoPacking respond -------------------------------------------------------------------
 * respond / respond_seeded (respond.rs:614-643, 1229-1237), the unpacked variant: per query,
 * one RLWE ciphertext (a h_j, b h_j) per column j of its shard (plaintext_multiply_columns,
 * respond.rs:585-599) and their sum. Query i: shard_ids[i], a from seeds[32 i..] (seeded) or
 * as[ring_dim i..] (pass seeds null), b from bs[ring_dim i..]. out receives count x
 * (gamma + 1) ciphertexts of (a, b), ring_dim words each in coefficient form, the sum first.
 * No store or seat is needed. All or nothing. */
int ig_respond_nopacking_batch(ig_ctx* ctx, uint64_t db, uint32_t count, const uint32_t* shard_ids,
                               const uint8_t* seeds, const uint64_t* as, const uint64_t* bs, uint64_t* out);
/* The unpacked ServerResponse bytes (respond.rs:111-176): Full(ciphertext), the column
 * ciphertexts, packing_mode None. cts: `count` ciphertexts of (a, b), the response
 * ciphertext first. */
int ig_response_encode_full(const uint64_t* cts, uint32_t count, uint32_t ring_dim, uint64_t modulus, uint8_t* out,
                            size_t cap, size_t* len_out);

/* ---- OnePacking respond -------------------------------------------------------------------
 * respond_one_packing / respond_seeded_packed (respond.rs:696-729, 1241-1249): the column
 * products' coefficient-0 LWEs packed by the Galois-automorphism tree of
 * inspiring/automorph_pack.rs into one RLWE holding column k at coefficient k, scaled by d.
 * The CRS needs its Galois keys first: ig_crs_set_galois_keys takes ServerCrs::galois_keys,
 * `count` = log2(ring_dim) keys (key i for t = ring_dim / 2^i + 1) of `rows` = 3 rows (a, b),
 * ring_dim words each in coefficient form (keys[((i * rows + r) * 2 + {0 a, 1 b}) *
 * ring_dim + k]), refused as require_galois_keys refuses (setup.rs:195-226). A second call
 * replaces the keys. */
int ig_crs_set_galois_keys(ig_ctx* ctx, uint64_t crs, uint32_t count, uint32_t rows, const uint64_t* keys);
/* Query i: shard_ids[i], a from seeds[32 i..] (seeded) or as[ring_dim i..] (pass seeds null),
 * b from bs[ring_dim i..]. a_out, b_out receive count x ring_dim coefficient-form words over
 * q, or over mod_switch_target when nonzero; the response's packed_coefficients is gamma
 * and its packing_mode Tree. No store or seat is needed. All or nothing. */
int ig_respond_one_packing_batch(ig_ctx* ctx, uint64_t db, uint32_t count, const uint32_t* shard_ids,
                                 const uint8_t* seeds, const uint64_t* as, const uint64_t* bs,
                                 uint64_t mod_switch_target, uint64_t* a_out, uint64_t* b_out);

/* ---- client side (load generation and decoding) --------------------------------------
 * A ClientSession's query batch and record extraction on the GPU, for driving and checking
 * the server at saturation. ig_client_create takes the session's RLWE secret (ring_dim
 * words mod q, coefficient form) and its sampler's sigma. */
int ig_client_create(ig_ctx* ctx, uint64_t crs, const uint64_t* secret, double sigma, uint64_t* client_out);
int ig_client_destroy(ig_ctx* ctx, uint64_t client);
/* ClientSession::query_batch (session.rs:377-434): query i is the seeded RGSW row of index
 * indices[i] (SeededRgswCiphertext::encrypt_with_rng, rgsw/types.rs:345-388, one row of
 * power 1), its `a` seed seeds[32 i..] (the reference draws them from the caller's rng), its
 * error the next ring_dim samples of the session's Gaussian sampler (math/gaussian.rs:210-224)
 * in query order. The sampler is its ChaCha20 key sampler_key and its position
 * *sampler_word (32-bit keystream words consumed so far), advanced past the batch's draws.
 * Writes shard_ids_out[i] and b_out[ring_dim i..] (coefficient form); the queries' `a`
 * expand from the seeds on the server. */
int ig_client_query_batch(ig_ctx* ctx, uint64_t client, uint32_t count, const uint64_t* indices,
                          const uint8_t* seeds, const uint8_t* sampler_key, uint64_t* sampler_word,
                          uint32_t* shard_ids_out, uint64_t* b_out);
/* extract_inspiring / extract_packed / extract_inspiring_mod_switched (extract.rs:184-263,
 * mod_switch.rs:573-640) for `count` packed responses (a, b: count x ring_dim words over
 * `modulus`, 0 meaning q): decrypt, round by modulus / p, times d^-1 mod p when tree != 0,
 * then the record bytes (records_out: count x entry_size). A switched modulus m is served
 * when ring_dim * m * max|s| < q/2 (the 36-bit target is). */
int ig_client_extract_batch(ig_ctx* ctx, uint64_t client, uint32_t count, const uint64_t* a, const uint64_t* b,
                            uint64_t modulus, uint32_t entry_size, int tree, uint8_t* records_out);

/* ---- wire ------------------------------------------------------------------------------
 * ServerResponse bincode bytes of a packed response (respond.rs:111-176, tight codec
 * poly.rs:166-225): Packed{a, b_prefix (first `retained` b coefficients), retained}, no
 * column ciphertexts, Some(PackingMode::Inspiring). `modulus` is the ciphertext modulus
 * (the mod-switch target after a switch). Writes at most cap bytes; *len_out = size. */
int ig_response_encode(const uint64_t* a, const uint64_t* b, uint32_t ring_dim, uint32_t retained, uint64_t modulus,
                       uint8_t* out, size_t cap, size_t* len_out);
/* The same bytes with packing_mode Some(PackingMode::Tree) (a OnePacking response). */
int ig_response_encode_tree(const uint64_t* a, const uint64_t* b, uint32_t ring_dim, uint32_t retained,
                            uint64_t modulus, uint8_t* out, size_t cap, size_t* len_out);
/* The same bytes for `count` device-resident responses (d_a, d_b: count x ring_dim words)
 * into d_out (count x *len_out bytes, response r at r * *len_out), enqueued on the context
 * stream: the wire is built next to the responses, and only its bytes cross to the host
 * (10,446 B per query at the 36-bit switch instead of 32 KiB of words). d_status[r] gets
 * bit 1 when a coefficient is not below the modulus. With d_out null, only *len_out is
 * set. modulus must be at least 2^8. */
int ig_response_encode_device(ig_ctx* ctx, uint32_t count, const uint64_t* d_a, const uint64_t* d_b,
                              uint32_t ring_dim, uint32_t retained, uint64_t modulus, uint8_t* d_out,
                              size_t* len_out, uint32_t* d_status);

/* ---- RIMS codec ----------------------------------------------------------------------------
 * encode_response_packed / decode_response_packed (mod_switch.rs:254-521): the byte-aligned,
 * self-describing frame "RIMS", version 2, target modulus (u64 LE), ring_dim (u32 LE),
 * bytes per coefficient (ceil(bits(modulus - 1) / 8), at least 1), packing mode (0 none,
 * 1 InspiRING, 2 tree), shape (u32 LE: the column count unpacked, the retained b count
 * packed), then a, the retained b and each column ciphertext's a and b, every coefficient
 * in that many little-endian bytes.
 * packing_mode 0 takes retained == 0 (b is written whole) and `columns` ciphertexts of (a, b)
 * in cts (columns x 2 x ring_dim words); modes 1 and 2 take retained in 1..ring_dim and no
 * columns. A coefficient not below the modulus is refused (IG_ERR_SHAPE). */
int ig_response_encode_rims(const uint64_t* a, const uint64_t* b, uint32_t ring_dim, uint32_t retained,
                            uint32_t packing_mode, const uint64_t* cts, uint32_t columns, uint64_t modulus,
                            uint8_t* out, size_t cap, size_t* len_out);
/* Decodes a RIMS frame. With a, b and cts null it validates the whole frame and returns its
 * header (*modulus_out, *ring_dim_out, *packing_mode_out, *retained_out: 0 when unpacked,
 * *columns_out); with buffers (a: ring_dim words, b: ring_dim words, zero past the retained
 * prefix, cts: columns x 2 x ring_dim words) it also writes the coefficients. Refusals carry
 * the reference's message in err (when err_cap > 0): bad magic or truncated header,
 * unsupported version, zero modulus or ring_dim, a width that does not match the modulus,
 * an unknown packing mode, a retained count outside 1..ring_dim, a payload length
 * mismatch, a coefficient not below the modulus. */
int ig_response_decode_rims(const uint8_t* bytes, size_t len, uint64_t* modulus_out, uint32_t* ring_dim_out,
                            uint32_t* packing_mode_out, uint32_t* retained_out, uint32_t* columns_out, uint64_t* a,
                            uint64_t* b, uint64_t* cts, char* err, size_t err_cap);
/* The RIMS frames of `count` device-resident packed InspiRING responses (mode 1), built on
 * the context stream like ig_response_encode_device: d_out receives count x *len_out bytes,
 * d_status[r] gets bit 1 when a coefficient is not below the modulus; with d_out null only
 * *len_out is set. */
int ig_response_encode_rims_device(ig_ctx* ctx, uint32_t count, const uint64_t* d_a, const uint64_t* d_b,
                                   uint32_t ring_dim, uint32_t retained, uint64_t modulus, uint8_t* d_out,
                                   size_t* len_out, uint32_t* d_status);

/* ---- observability ------------------------------------------------------------------------
 * With RAVEN_PROFILE_RESPOND set in the environment (read once per process, as
 * respond.rs:1332-1345), every ig_respond_seeded_batch / ig_respond_batch call prints
 * "RAVEN_PROFILE num_cols=... queries=... column_check_us=... pack_us=..." to stderr, the
 * regions timed with CUDA events.
 * Per-region device timing of respond calls, the GPU form of the reference's
 * RAVEN_PROFILE_RESPOND regions (respond.rs:1295-1345): with profiling on, each kernel
 * launch is bracketed by CUDA events on the context stream. ig_profile_read synchronises,
 * writes the summed milliseconds and launch counts of regions 0..regions-1 (0 = shard scan,
 * 1 = recursion/respond, 2 = store fold) and, when reset != 0, clears the record. */
int ig_profile_enable(ig_ctx* ctx, int on);
int ig_profile_read(ig_ctx* ctx, double* ms, uint64_t* counts, int regions, int reset);
/* Integer roofline probe: runs blocks_per_sm x SMs CTAs of 256 threads, each thread iters
 * rounds of eight lazy butterflies (one Shoup product mod q each) on register-resident
 * words, and stores the measured butterflies per second. The respond kernels' transform
 * and product rates are reported against it. */
int ig_butterfly_peak(ig_ctx* ctx, int blocks_per_sm, int iters, double* per_s);
/* Kernel launches this context has made so far. */
uint64_t ig_launch_count(const ig_ctx* ctx);

/* ---- test hooks --------------------------------------------------------------------------
 * Forces the word-by-word `a` expansion the kernel otherwise takes only after a rejected
 * ChaCha word, so tests can check that path against the vectorised one. */
int ig_debug_force_serial_expand(ig_ctx* ctx, int on);
/* Host-side fault injection: the k-th device allocation of this context from now (1 = the
 * next) fails with IG_ERR_NOMEM, as a full GPU would make it; 0 disarms. The call that
 * made it is refused and leaves no half-built object; the context stays usable. */
int ig_debug_fail_alloc_at(ig_ctx* ctx, uint32_t k);
/* Copies a shard's store sums (gamma x ring_dim, NTT form times 2^64 mod q, the
 * reference's Montgomery layout) to host memory. */
int ig_debug_store_sums(ig_ctx* ctx, uint64_t db, uint32_t shard_id, uint64_t* out);

#ifdef __cplusplus
}
#endif
#endif
