// perks_stencil2d_noalloc: the 2D stencil time loop for callers that cannot
// allocate device memory.
//
// Some host programs fix their whole device-memory footprint at start-up and
// must not allocate afterwards: a cudaMalloc in the middle of a run can
// synchronise the device, can fail once a memory pool owner has reserved the
// rest of the GPU, and some callers (a simulation driven from another
// framework's memory manager, a process under a hard memory budget) are not
// allowed to call it at all. perks_stencil2d grows a library-owned workspace
// with cudaMalloc on first use; this entry point instead takes every byte of
// scratch (the two internal ping-pong fields and the grid-barrier words) from
// one statically sized __device__ array that is part of the loaded library.
//
// Limits and behaviour:
//  * The scratch array holds kNoAllocScratchBytes (32 MiB). A call needs
//    2 * width_y * pitch * sizeof(REAL) + 256 bytes, where pitch is width_x
//    rounded up to the kernel's column-strip width; larger fields are
//    rejected with PERKS_ERR_INVALID_ARG and a message giving both sizes.
//    Every GPU that loads the library holds the array until the process exits.
//  * Every call looks up the array's device address on the current device
//    with cudaGetSymbolAddress (a lookup; it allocates nothing), so a device
//    reset between two calls, after which the library's device code is loaded
//    again and the array may sit elsewhere, cannot leave a stale address. The
//    first call on a device may load the library's device code: make that
//    first call before any stream capture.
//  * All calls share the one array and it keeps the last call's contents. The
//    barrier and status words are cleared at the start of every call; the
//    fields are fully rewritten from d_in. Calls whose GPU work overlaps (on
//    different streams or host threads) race on the array and must not be
//    issued.
//  * The call allocates nothing: no cudaMalloc, cudaFree, event creation or
//    allocating library routine. stats->ms is reported as 0 (no events).
//  * Reference evaluation order only (the bit-exact one); PERKS_ORDER_FAST is
//    rejected with PERKS_ERR_UNSUPPORTED.
#include <cuda_runtime.h>
#include <algorithm>
#include <string>
#include "runtime.cuh"
#include "stencil2d_host.cuh"

namespace perks {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device. In host code
// g_noalloc_scratch names a host-side stand-in, not device memory: only this
// looked-up address may be passed to copies and kernels.
static int noalloc_scratch(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
  *out = p;
  return PERKS_OK;
}

template <class T, int SHAPE, bool FAST>
static int noalloc2d(const perks_stencil_opts& o, const T* d_in, T* d_out, int wy, int wx, int steps,
                     perks_stencil_stats* st) {
  using Cf = Cfg2D<T, SHAPE, FAST>;
  constexpr int H = Cf::H;
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(o.stream);
  const bool persistent = o.kernel == PERKS_KERNEL_PERSISTENT;
  const int ctas = o.ctas > 0 ? std::min(o.ctas, dev->sms) : dev->sms;
  const long long warps = (long long)ctas * Cf::NW;
  const int ns = int((wx + Cf::SW - 1) / Cf::SW);
  if (ns > warps) return fail(PERKS_ERR_UNSUPPORTED, "width_x too large for the grid");
  const int nb = int(std::max<long long>(1, std::min<long long>(warps / ns, wy)));
  const int pitch = ns * Cf::SW;
  const int tymax = int((wy + nb - 1) / nb);
  const int grid = int(((long long)ns * nb + Cf::NW - 1) / Cf::NW);
  const size_t fbytes = ((size_t(wy) * pitch * sizeof(T)) + 255) & ~size_t(255);
  const size_t need = 2 * fbytes + 256;
  if (need > kNoAllocScratchBytes)
    return fail(PERKS_ERR_INVALID_ARG, "perks_stencil2d_noalloc: field needs " + std::to_string(need) +
                                           " bytes of scratch, the static array holds " +
                                           std::to_string(kNoAllocScratchBytes));
  int C = 0;
  if (steps > 1) C = std::max(0, std::min(max_cache_rows<Cf>(o, *dev), tymax - 2 * H));
  const size_t smem = Cf::ring_bytes + size_t(C) * Cf::res_row_bytes;
  if (smem > dev->smem_optin) return fail(PERKS_ERR_UNSUPPORTED, "shared memory budget exceeded");
  if (st) {
    *st = perks_stencil_stats{};
    st->grid_x = ns;
    st->grid_y = nb;
    st->grid_z = 1;
    st->tile_x = Cf::SW;
    st->tile_y = tymax;
    st->cached_rows = C;
  }
  if (steps == 0) {
    PERKS_CUDA(cudaMemcpyAsync(d_out, d_in, size_t(wy) * wx * sizeof(T), cudaMemcpyDeviceToDevice, s));
    PERKS_CUDA(cudaStreamSynchronize(s));
    return PERKS_OK;
  }
  void* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc != PERKS_OK) return rc;
  unsigned char* b = static_cast<unsigned char*>(base);
  T* f0 = reinterpret_cast<T*>(b);
  T* f1 = reinterpret_cast<T*>(b + fbytes);
  unsigned* words = reinterpret_cast<unsigned*>(b + 2 * fbytes);
  // barrier and status words must start at zero; the array keeps old contents
  PERKS_CUDA(cudaMemsetAsync(words, 0, 4 * sizeof(unsigned), s));
  PERKS_CUDA(copy_rows(f0, size_t(pitch) * sizeof(T), d_in, size_t(wx) * sizeof(T), size_t(wx) * sizeof(T),
                       wy, cudaMemcpyDeviceToDevice, s));
  Stencil2DParams p{};
  p.f[0] = f0;
  p.f[1] = f1;
  p.wy = wy;
  p.wx = wx;
  p.pitch = pitch;
  p.ns = ns;
  p.nb = nb;
  p.C = C;
  p.dirichlet = o.boundary == PERKS_BOUNDARY_DIRICHLET;
  p.alternate = persistent && o.l2_sweep;
  p.persistent = persistent;
  p.bar = words;
  p.status = words + 2;
  p.ctl = wait_ctl();
  auto kern = stencil2d_kernel<T, SHAPE, FAST, Cf>;
  PERKS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  if (persistent) {
    int per_sm = 0;
    PERKS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cf::NT, smem));
    if (per_sm * dev->sms < grid) return fail(PERKS_ERR_LAUNCH, "persistent grid does not fit");
    p.steps = steps;
    p.t0 = 0;
    void* args[] = {&p};
    PERKS_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(Cf::NT), args, smem, s));
    count_launch(1);
  } else {
    p.steps = 1;
    for (int t = 0; t < steps; t++) {
      p.t0 = t;
      kern<<<grid, Cf::NT, smem, s>>>(p);
    }
    PERKS_CUDA(cudaGetLastError());
    count_launch(steps);
  }
  PERKS_CUDA(copy_rows(d_out, size_t(wx) * sizeof(T), (steps & 1) ? f1 : f0, size_t(pitch) * sizeof(T),
                       size_t(wx) * sizeof(T), wy, cudaMemcpyDeviceToDevice, s));
  SyncWords sw{words, words + 2};
  rc = check_status(sw, s);
  if (rc != PERKS_OK) return rc;
  if (st) st->launches = persistent ? 1 : steps;
  return PERKS_OK;
}

template <class T, bool FAST>
static int noalloc_dispatch(const perks_stencil_opts& o, const void* in, void* out, int wy, int wx, int steps,
                            perks_stencil_stats* st) {
  const T* i = static_cast<const T*>(in);
  T* q = static_cast<T*>(out);
  switch (o.shape) {
    case PERKS_2D5PT: return noalloc2d<T, PERKS_2D5PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2DS9PT: return noalloc2d<T, PERKS_2DS9PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2D13PT: return noalloc2d<T, PERKS_2D13PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2D17PT: return noalloc2d<T, PERKS_2D17PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2D21PT: return noalloc2d<T, PERKS_2D21PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2DS25PT: return noalloc2d<T, PERKS_2DS25PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2D9PT: return noalloc2d<T, PERKS_2D9PT, FAST>(o, i, q, wy, wx, steps, st);
    case PERKS_2D25PT: return noalloc2d<T, PERKS_2D25PT, FAST>(o, i, q, wy, wx, steps, st);
    default: return fail(PERKS_ERR_INVALID_ARG, "not a 2D shape: " + std::to_string(o.shape));
  }
}

}  // namespace perks

using namespace perks;

extern "C" int perks_stencil2d_noalloc(const perks_stencil_opts* o, const void* d_in, void* d_out, int wy, int wx,
                                       int steps, perks_stencil_stats* st) {
  if (!o) return fail(PERKS_ERR_INVALID_ARG, "opts is NULL");
  if (o->shape < PERKS_2D5PT || o->shape > PERKS_2D25PT) return fail(PERKS_ERR_INVALID_ARG, "not a 2D shape");
  if (o->dtype != PERKS_FP32 && o->dtype != PERKS_FP64)
    return fail(PERKS_ERR_INVALID_ARG, "stencil dtype must be PERKS_FP32 or PERKS_FP64");
  if (o->boundary != PERKS_BOUNDARY_CLAMP && o->boundary != PERKS_BOUNDARY_DIRICHLET)
    return fail(PERKS_ERR_INVALID_ARG, "unknown boundary mode");
  if (o->order != PERKS_ORDER_REFERENCE && o->order != PERKS_ORDER_FAST)
    return fail(PERKS_ERR_INVALID_ARG, "unknown evaluation order");
  if (o->kernel != PERKS_KERNEL_PERSISTENT && o->kernel != PERKS_KERNEL_PER_STEP)
    return fail(PERKS_ERR_INVALID_ARG, "unknown kernel kind");
  if (o->tma) return fail(PERKS_ERR_UNSUPPORTED, "perks_stencil2d_noalloc runs the cp.async kernel only (tma = 0)");
  if (!d_in || !d_out) return fail(PERKS_ERR_INVALID_ARG, "null device pointer");
  if (wy <= 0 || wx <= 0 || steps < 0) return fail(PERKS_ERR_INVALID_ARG, "sizes must be positive, steps >= 0");
  if (o->order == PERKS_ORDER_FAST)
    return fail(PERKS_ERR_UNSUPPORTED, "perks_stencil2d_noalloc runs the reference evaluation order only");
  if (o->dtype == PERKS_FP32) return noalloc_dispatch<float, false>(*o, d_in, d_out, wy, wx, steps, st);
  return noalloc_dispatch<double, false>(*o, d_in, d_out, wy, wx, steps, st);
}
