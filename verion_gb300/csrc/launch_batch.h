// Host-side launcher of the batch kernel (kern_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include "batch.h"
#include "ctx.h"

namespace vgx {

// Resident batch CTAs per SM (occupancy of the batch kernel with its shared memory).
int batch_blocks_per_sm();
// Resource use of the batch kernel (registers, local and static shared bytes, first CUDA error).
int batch_kernel_info(int* regs, int* local_bytes, int* static_smem, int* error);
// Writes the start time to *t0, then runs `items` work items of `nreq` requests (sorted by item_begin).
cudaError_t launch_batch(int blocks, cudaStream_t s, const vgb::BatchReq* reqs, uint32_t nreq, uint32_t items,
                         uint32_t* next, vgb::BatchDone* done, uint32_t* err, unsigned long long* t0);

// The batch wavefront (kern_bwave.cu), launched inside stream capture: the start kernel; the loop
// body (two waves, and with `condition` the kernel that sets the WHILE node's condition `loop`);
// the tail kernel.
cudaError_t bwave_capture_start(cudaStream_t s, const vgb::WaveBatch& b, const vgk::Wave& w);
cudaError_t bwave_capture_body(cudaStream_t s, int trace_blocks, int shade_blocks, int sms, const vgb::WaveBatch& b,
                               const vgk::Wave& w, cudaGraphConditionalHandle loop, bool condition);
cudaError_t bwave_capture_tail(cudaStream_t s, const vgb::WaveBatch& b, const vgk::Wave& w);
// Resident 128-thread blocks per SM of the batch wavefront's traversal and shade stages.
void bwave_blocks_per_sm(int* trace, int* shade);

} // namespace vgx
