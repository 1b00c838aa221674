// context_access.h — what the engine lends the other host translation units
// (division): the context's stream, carry-scan scratch, budgeted device
// allocation and the product dispatch of natural::_mul.
#pragma once

#include "../../include/natural_gb300.h"
#include "nn_internal.h"

namespace nn {
cudaStream_t ctx_stream(nn_context* c);
Scan& ctx_scan(nn_context* c);
nn_status ctx_alloc(nn_context* c, u64** p, u64 words);  // counted against the HBM budget
void ctx_free(nn_context* c, u64* p, u64 words);
nn_status ctx_mul(nn_context* c, u64* out, const u64* a, u64 na, const u64* b, u64 nb);  // natural.h:444-450
nn_status ctx_fail(nn_context* c, cudaError_t e, const char* what);
// A host table to device memory on the context's stream, through page-locked
// staging: the call returns once the copy is queued, and h_src may be reused.
cudaError_t ctx_upload(nn_context* c, void* d_dst, const void* h_src, u64 bytes);
void ctx_error(nn_context* c, const char* msg);
nn_status ctx_scratch(nn_context* c, int slot, u64 words, u64** p);  // grow-only staging, slots 0-2
}  // namespace nn
