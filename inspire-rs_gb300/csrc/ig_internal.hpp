// Internal (non-ABI) services of a context, for the runtime translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>

#include "ig_kernels.cuh"

struct ig_ctx;

namespace igint {
int fail(ig_ctx* c, int code, const char* fmt, ...);
cudaStream_t stream(ig_ctx* c);
int device(ig_ctx* c);
std::mutex& mutex(ig_ctx* c);
int dalloc(ig_ctx* c, void** p, size_t bytes);
void dfree(ig_ctx* c, void* p, size_t bytes);
int scratch(ig_ctx* c, const char* name, size_t bytes, void** out);
int stage_h2d(ig_ctx* c, void* dst, const void* src, size_t bytes);
void add_launches(ig_ctx* c, unsigned n);
// One extension slot per context for the special_modulus objects, freed at destroy.
void*& sm_slot(ig_ctx* c);
void set_sm_destructor(ig_ctx* c, void (*fn)(ig_ctx*, void*));

// One served request resolved against the context's objects (takes the context lock):
// the parameter set's device constants (the seat's own set when it shares the database's
// ring and width), the shard's device pointers, the seat's device words, and the shard's
// store state. Returns an IG_* status; on refusal `err` holds the
// reference's message.
struct RequestView {
  ig::CrsDev crs;
  const ig::CrsDev* crs_dev;  // device copy of crs, for launches that mix parameter sets
  ig::ShardDev shard;
  const uint64_t* seat;
  uint32_t seat_rows;         // key rows of the seat (its bytes: seat_rows x n x 8)
  uint64_t p;
  bool has_store;
  char err[512];
};
int resolve_request(ig_ctx* c, uint64_t db, uint64_t store, uint64_t handle, uint32_t shard, RequestView* out);
// CTAs per query (1, 2 or 4) for a respond launch of `count` queries of width `gamma` on
// ring n with `in_flight` queries expected on the device with it (its own included): the
// forced shape, else the shape the tuned table times fastest at that many queries, else the
// fixed rule: four CTAs while twice the queries fit the pair threshold, two while they fit
// it, else one.
int launch_ctas(ig_ctx* c, uint32_t n, uint32_t gamma, uint32_t count, uint32_t in_flight);
// The launch shape set by ig_ctx_set_launch_shape (0 when the context chooses).
int forced_ctas(ig_ctx* c);
// Device-path lanes (ig_ctx_set_lanes), for callers holding the context lock:
// lane_acquire picks the call's stream (the context stream when lanes == 1, lane -1) and
// orders the context stream after the lane's previous batch, so the lane's scratch can be
// rewritten; lane_enter, after the call's staging copies on the context stream, makes the
// lane wait for them; lane_release marks the lane's work for the next acquire and join.
int lanes(ig_ctx* c);
// A host-buffer call over lanes. begin (before the context lock) picks the call's lane and
// holds its mutex until the call ends; under the context lock, pinned() returns the lane's
// pinned landing buffer (grown to `bytes`), stream() the stream to launch on (after the
// call's staging copies: enter()), launched() marks the end of the call's device work; after
// the context lock is released, wait() blocks until that work is done. With one lane the
// call runs on the context stream.
struct HostCall {
  unsigned k = 0;
  std::unique_lock<std::mutex> lane_lock;
};
void host_call_begin(ig_ctx* c, HostCall& hc);
int host_call_pinned(ig_ctx* c, HostCall& hc, size_t bytes, void** pin);
cudaStream_t host_call_stream(ig_ctx* c, HostCall& hc);
int host_call_enter(ig_ctx* c, HostCall& hc);
int host_call_launched(ig_ctx* c, HostCall& hc);
int host_call_wait(ig_ctx* c, HostCall& hc);
int lane_acquire(ig_ctx* c, cudaStream_t* s, int* lane);
int lane_enter(ig_ctx* c, int lane);
int lane_release(ig_ctx* c, int lane);
int sm_count(ig_ctx* c);
}  // namespace igint
