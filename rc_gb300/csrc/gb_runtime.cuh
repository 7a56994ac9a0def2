// Internal runtime helpers shared by the translation units of librc_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace gb {

constexpr int kStageSlots = 6;
constexpr int kAuxEvents = 4;

// Per-host-thread stream and grow-only device buffers used by the synchronous
// reference-ABI entry points.
int stage_stream(cudaStream_t* out);
int stage_buffer(int slot, size_t bytes, void** out);
// A second stream and kAuxEvents events of the same thread, for overlapping a
// call's copies with its kernels.
int stage_aux(cudaStream_t* s2, cudaEvent_t** ev);

int sm_count();

// Every device allocation of the library goes through here: cudaMalloc, or
// GB_ERR_NOMEM when the allocation-failure hook (gb_debug_fail_allocs) says so.
int dev_alloc(void** p, size_t bytes, const char* what);

__global__ void k_zero_f32x2(float2* __restrict__ p, int64_t n);

}  // namespace gb
