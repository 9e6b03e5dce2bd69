// Host runtime shared by the stencil and CG launchers: error reporting,
// device properties, a grow-only device workspace, launch counting.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include "../../include/perks.h"
#include "ptx.cuh"

namespace perks {

// Record a failure message for perks_last_error() and return `code`.
int fail(int code, const std::string& msg);
// Check a CUDA call; on error record it and return PERKS_ERR_CUDA (or OOM).
int cuda_fail(cudaError_t e, const char* what);
#define PERKS_CUDA(call)                                       \
  do {                                                         \
    cudaError_t perks_e_ = (call);                             \
    if (perks_e_ != cudaSuccess) return ::perks::cuda_fail(perks_e_, #call); \
  } while (0)

struct DeviceInfo {
  int device = -1;
  int sms = 0;
  size_t smem_optin = 0;  // max dynamic shared memory per block
  int coop = 0;
};
// Properties of the current device (cached per device). Returns nullptr and
// records an error when no device is usable.
const DeviceInfo* device_info();

// Grow-only per-device scratch buffers, keyed by slot. Not thread-safe (the
// reference API is single-threaded too). Returned memory is not cleared.
enum WorkSlot { kWsField0 = 0, kWsField1, kWsSync, kWsCgVec, kWsCgScalar, kWsCgMat, kWsCgSell, kWsSlots };
void* workspace(WorkSlot slot, size_t bytes, int* status);

void count_launch(int n = 1);

// Wait budget and grid-barrier test hook for the next launches (process-wide;
// set by perks_debug_set_wait_fault, default: kWaitBudget, no hook).
WaitCtl wait_ctl();

// rows x width bytes between pitched buffers; one linear copy when both
// pitches equal the width (a pitched copy of a dense field moves rows one
// by one, which is slower between host and device).
inline cudaError_t copy_rows(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t rows,
                             cudaMemcpyKind kind, cudaStream_t s) {
  if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * rows, kind, s);
  return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, s);
}

// Device status word + grid barrier words: 4 unsigned in kWsSync.
struct SyncWords {
  unsigned* bar;     // [2]
  unsigned* status;  // [1]
};
int sync_words(SyncWords* out, cudaStream_t s);
// Read the status word after a launch; maps device error bits to a status.
int check_status(const SyncWords& w, cudaStream_t s);

}  // namespace perks
