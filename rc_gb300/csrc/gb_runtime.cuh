// Internal runtime helpers shared by the translation units of librc_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gb {

constexpr int kStageSlots = 9;
constexpr int kAuxEvents = 4;

// Per-host-thread stream and grow-only device buffers used by the synchronous
// reference-ABI entry points.
int stage_stream(cudaStream_t* out);
int stage_buffer(int slot, size_t bytes, void** out);
// A second stream and kAuxEvents events of the same thread, for overlapping a
// call's copies with its kernels.
int stage_aux(cudaStream_t* s2, cudaEvent_t** ev);

int sm_count();

// True when kernels on the current device may read and write this pageable
// host buffer directly (through the host's page tables, NVLink-C2C on Grace):
// the device reports pageable memory access using host page tables, the
// pointer is 16-byte aligned, the row pitch is an even number of doubles, and
// RC_GB300_HOST_DIRECT is not "0".
bool host_direct(const void* host, int64_t row_doubles);

// Every device allocation of the library goes through here: cudaMalloc, or
// GB_ERR_NOMEM when the allocation-failure hook (gb_debug_fail_allocs) says so.
int dev_alloc(void** p, size_t bytes, const char* what);

__global__ void k_zero_f32x2(float2* __restrict__ p, int64_t n);

}  // namespace gb
