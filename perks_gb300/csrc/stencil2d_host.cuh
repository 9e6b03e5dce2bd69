// Host launcher for the 2D stencil kernel: tile planning, shared-memory
// budget for resident rows, layout copies, cooperative or per-step launch.
#pragma once
#include <algorithm>
#include <string>
#include "runtime.cuh"
#include "stencil2d.cuh"

namespace perks {

int encode_tiled_2d(CUtensorMap* map, bool f64, void* base, int pitch, int rows, int box_x);

inline int ceil_div(long long a, long long b) { return int((a + b - 1) / b); }

// Rows per warp that the persistent kernel can keep in shared memory next to
// its prefetch ring (0 when caching is off or the kernel is not persistent).
template <class Cf>
int max_cache_rows(const perks_stencil_opts& o, const DeviceInfo& dev) {
  if (o.kernel != PERKS_KERNEL_PERSISTENT || o.cache_rows == 0) return 0;
  const long long avail = (long long)dev.smem_optin - (long long)Cf::ring_bytes - 256;
  int cmax = int(std::max<long long>(0, avail / (long long)Cf::res_row_bytes));
  if (o.cache_rows > 0) cmax = std::min(cmax, o.cache_rows);
  return cmax;
}

// Largest width_y at which every band keeps all its rows on chip except the
// H rows at each end, which go through the field as halo of the neighbouring
// bands (the reference's getMinWidthY, stencil/2dstencil/jacobi-2d.cu:79-136:
// cached rows per CTA x CTAs along y). 0 when nothing is cached.
template <class Cf>
int min_domain_rows(const perks_stencil_opts& o, int wx, int* wy) {
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  const int ctas = o.ctas > 0 ? std::min(o.ctas, dev->sms) : dev->sms;
  const long long warps = (long long)ctas * Cf::NW;
  const int ns = ceil_div(wx, Cf::SW);
  if (ns > warps)
    return fail(PERKS_ERR_UNSUPPORTED, "width_x " + std::to_string(wx) + " needs more than " +
                                           std::to_string(warps) + " column strips");
  const int cmax = max_cache_rows<Cf>(o, *dev);
  const long long rows = cmax > 0 ? (warps / ns) * (long long)(cmax + 2 * Cf::H) : 0;
  *wy = int(std::min<long long>(rows, 0x7fffffff));
  return PERKS_OK;
}

// d_in / d_out are device buffers, or host buffers when host_io is set: the
// field then goes straight between them and the internal pitched fields.
// TMA: rows reach the warps' rings by tensor copies instead of cp.async.
template <class T, int SHAPE, bool FAST, bool TMA = false>
int launch_stencil2d(const perks_stencil_opts& o, const T* d_in, T* d_out, int wy, int wx, int steps,
                     perks_stencil_stats* st, bool host_io = false) {
  using Cf = Cfg2D<T, SHAPE, FAST, TMA>;
  constexpr int H = Cf::H;
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(o.stream);
  const bool persistent = o.kernel == PERKS_KERNEL_PERSISTENT;
  const bool naive = o.kernel == PERKS_KERNEL_NAIVE;
  const int ctas = o.ctas > 0 ? std::min(o.ctas, dev->sms) : dev->sms;
  const long long warps = (long long)ctas * Cf::NW;
  const int ns = ceil_div(wx, Cf::SW);
  if (ns > warps)
    return fail(PERKS_ERR_UNSUPPORTED, "width_x " + std::to_string(wx) + " needs more than " +
                                           std::to_string(warps) + " column strips");
  const int nb = int(std::max<long long>(1, std::min<long long>(warps / ns, wy)));
  const int pitch = ns * Cf::SW;
  const int tymax = ceil_div(wy, nb);
  const int grid = ceil_div((long long)ns * nb, Cf::NW);

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
  const size_t elems = size_t(wy) * wx;
  if (steps == 0) {
    PERKS_CUDA(cudaMemcpyAsync(d_out, d_in, elems * sizeof(T), host_io ? cudaMemcpyHostToHost : cudaMemcpyDeviceToDevice,
                               s));
    PERKS_CUDA(cudaStreamSynchronize(s));
    return PERKS_OK;
  }

  int stt = PERKS_OK;
  const size_t fbytes = size_t(wy) * pitch * sizeof(T);
  T* f0 = static_cast<T*>(workspace(kWsField0, fbytes, &stt));
  if (!f0) return stt;
  T* f1 = static_cast<T*>(workspace(kWsField1, fbytes, &stt));
  if (!f1) return stt;
  SyncWords sw;
  if ((stt = sync_words(&sw, s)) != PERKS_OK) return stt;

  PERKS_CUDA(copy_rows(f0, size_t(pitch) * sizeof(T), d_in, size_t(wx) * sizeof(T), size_t(wx) * sizeof(T),
                       wy, host_io ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));

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
  p.bar = sw.bar;
  p.status = sw.status;
  p.ctl = wait_ctl();
  if constexpr (Cf::TMA) {
    for (int i = 0; i < 2; i++) {
      if ((stt = encode_tiled_2d(&p.map[i], sizeof(T) == 8, p.f[i], pitch, wy, Cf::HALF)) != PERKS_OK) return stt;
      if ((stt = encode_tiled_2d(&p.emap[i], sizeof(T) == 8, p.f[i], pitch, wy, Cf::EL)) != PERKS_OK) return stt;
    }
  }

  auto kern = stencil2d_kernel<T, SHAPE, FAST, Cf>;
  PERKS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  cudaEvent_t e0, e1;
  PERKS_CUDA(cudaEventCreate(&e0));
  PERKS_CUDA(cudaEventCreate(&e1));
  PERKS_CUDA(cudaEventRecord(e0, s));
  int launches = 0;
  if (naive) {
    const dim3 blk(32, 8), grd(unsigned(ceil_div(wx, 32)), unsigned(ceil_div(wy, 8)));
    for (int t = 0; t < steps; t++)
      stencil2d_naive<T, SHAPE, FAST, Cf::FIN><<<grd, blk, 0, s>>>((t & 1) ? f1 : f0, (t & 1) ? f0 : f1, wy, wx,
                                                                   pitch, p.dirichlet);
    launches = steps;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return cuda_fail(e, "stencil2d naive launch");
    }
  } else if (persistent) {
    int nb = 0;
    PERKS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, Cf::NT, smem));
    if (nb * dev->sms < grid) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail(PERKS_ERR_LAUNCH, "persistent grid of " + std::to_string(grid) + " CTAs does not fit (" +
                                        std::to_string(nb) + " per SM)");
    }
    p.steps = steps;
    p.t0 = 0;
    void* args[] = {&p};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(Cf::NT), args, smem, s);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return cuda_fail(e, "cudaLaunchCooperativeKernel(stencil2d)");
    }
    launches = 1;
  } else {
    p.steps = 1;
    for (int t = 0; t < steps; t++) {
      p.t0 = t;
      kern<<<grid, Cf::NT, smem, s>>>(p);
    }
    launches = steps;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return cuda_fail(e, "stencil2d per-step launch");
    }
  }
  PERKS_CUDA(cudaEventRecord(e1, s));
  count_launch(launches);
  PERKS_CUDA(copy_rows(d_out, size_t(wx) * sizeof(T), (steps & 1) ? f1 : f0, size_t(pitch) * sizeof(T),
                       size_t(wx) * sizeof(T), wy, host_io ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                       s));
  int rc = check_status(sw, s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != PERKS_OK) return rc;
  if (st) {
    st->ms = ms;
    st->gcells_per_s = double(elems) * steps / (double(ms) * 1e6);
    long long cached = 0;
    for (int b = 0; b < nb; b++) {
      int r0 = int((long long)b * wy / nb), r1 = int((long long)(b + 1) * wy / nb);
      cached += std::max(0, std::min(C, r1 - r0 - 2 * H));
    }
    st->cached_fraction = double(cached) / double(wy);
    st->launches = launches;
  }
  return PERKS_OK;
}

}  // namespace perks
