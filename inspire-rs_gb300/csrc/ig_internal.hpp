// Internal (non-ABI) services of a context, for the runtime translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

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
}  // namespace igint
