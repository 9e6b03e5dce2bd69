// Host launcher for the 3D stencil kernel: tensor maps, tile grid, per-CTA
// work ranges, cooperative (persistent) or one-launch-per-step execution.
#pragma once
#include <algorithm>
#include <string>
#include "runtime.cuh"
#include "stencil3d.cuh"

namespace perks {

int encode_tiled_3d(CUtensorMap* map, bool f64, void* base, int wx, int wy, int h, int px, int box_x, int box_y);

// Planes of CTA b's range that may stay resident: the segment (z-run of one
// tile) with the most planes no other CTA reads, capped at kr. The kernel
// makes the same choice.
inline int resident_planes_of(long long total, int h, int grid, int b, int H, int kr) {
  const long long c_lo = total * b / grid, c_hi = total * (b + 1) / grid;
  if (c_hi <= c_lo) return 0;
  const int nseg = int((c_hi - 1) / h - c_lo / h + 1);
  int best = 0;
  for (int k = 0; k < nseg; k++) {
    const long long tb = c_lo / h + k;
    const int zl = int(std::max(c_lo, tb * h) - tb * h), zh = int(std::min(c_hi, (tb + 1) * h) - tb * h);
    best = std::max(best, std::min(kr, (zh - H) - (zl + H)));
  }
  return best;
}

// Resident plane tiles per CTA that fit next to the ring (persistent
// launches that run more than one step), as opts.cache_rows asks: -1 as many
// as fit, 0 none, n at most n.
template <class Cf>
int max_resident_planes(const perks_stencil_opts& o, const DeviceInfo& dev) {
  if (o.kernel != PERKS_KERNEL_PERSISTENT || o.cache_rows == 0) return 0;
  const long long avail = (long long)dev.smem_optin - (long long)Cf::res_offset;
  int k = int(std::max<long long>(0, avail / (long long)Cf::res_plane_bytes));
  if (o.cache_rows > 0) k = std::min(k, o.cache_rows);
  return k;
}

// Largest height at which the persistent kernel keeps on chip every plane
// of every CTA's z-runs except the H at each end (the 3D counterpart of the
// reference's --small domain, stencil/3dstencil/j3d.driver.cpp:62-144). 0
// when no plane fits next to the ring.
template <class Cf>
int min_domain_planes(const perks_stencil_opts& o, int wy, int wx, int* h_out) {
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  *h_out = 0;
  perks_stencil_opts op = o;
  op.kernel = PERKS_KERNEL_PERSISTENT;
  const int kmax = max_resident_planes<Cf>(op, *dev);
  if (kmax == 0) return PERKS_OK;
  const int ctas = o.ctas > 0 ? std::min(o.ctas, dev->sms) : dev->sms;
  const long long tiles = (long long)((wx + Cf::SW - 1) / Cf::SW) * ((wy + Cf::TY - 1) / Cf::TY);
  const int H = Cf::H;
  auto fully_cached = [&](int h) {
    const long long total = tiles * h;
    const int grid = int(std::min<long long>(total, ctas));
    for (int b = 0; b < grid; b++) {
      const long long c_lo = total * b / grid, c_hi = total * (b + 1) / grid;
      const int nseg = int((c_hi - 1) / h - c_lo / h + 1);
      int eligible = 0;
      for (int k = 0; k < nseg; k++) {
        const long long tb = c_lo / h + k;
        const int zl = int(std::max(c_lo, tb * h) - tb * h), zh = int(std::min(c_hi, (tb + 1) * h) - tb * h);
        eligible += std::max(0, (zh - H) - (zl + H));
      }
      if (eligible > resident_planes_of(total, h, grid, b, H, kmax)) return false;
    }
    return true;
  };
  // beyond this height some CTA holds more than kmax + 2H planes of a run
  const long long top = ctas * (long long)(kmax + 2 * H) / tiles + 2;
  for (long long h = std::min<long long>(top, 1 << 20); h >= 1; h--) {
    if (fully_cached(int(h))) {
      *h_out = int(h);
      return PERKS_OK;
    }
  }
  return PERKS_OK;
}

// d_in / d_out are device buffers, or host buffers when host_io is set.
template <class T, int SHAPE, bool FAST>
int launch_stencil3d(const perks_stencil_opts& o, const T* d_in, T* d_out, int h, int wy, int wx, int steps,
                     perks_stencil_stats* st, bool host_io = false) {
  using Cf = Cfg3D<T, SHAPE, FAST>;
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(o.stream);
  const bool persistent = o.kernel == PERKS_KERNEL_PERSISTENT;
  const int ctas = o.ctas > 0 ? std::min(o.ctas, dev->sms) : dev->sms;
  const int gx = (wx + Cf::SW - 1) / Cf::SW;
  const int gy = (wy + Cf::TY - 1) / Cf::TY;
  const long long pairs = (long long)gx * gy * h;  // (tile, plane) pairs
  if (pairs > (1ll << 40)) return fail(PERKS_ERR_UNSUPPORTED, "3D domain too large");
  const int px = (wx + Cf::V16 - 1) / Cf::V16 * Cf::V16;
  if (Cf::smem_bytes > dev->smem_optin) return fail(PERKS_ERR_UNSUPPORTED, "shared memory budget exceeded");
  const int grid = int(std::min<long long>(pairs, ctas));
  // resident planes: no more than the longest eligible run needs
  int kr = 0;
  long long cached = 0;
  if (persistent && steps > 1) {
    const int kmax = max_resident_planes<Cf>(o, *dev);
    for (int b = 0; b < grid && kmax > 0; b++) {
      const int n = resident_planes_of(pairs, h, grid, b, Cf::H, kmax);
      kr = std::max(kr, n);
      cached += n;
    }
  }
  const size_t smem = kr > 0 ? Cf::res_offset + size_t(kr) * Cf::res_plane_bytes : Cf::smem_bytes;
  if (st) {
    *st = perks_stencil_stats{};
    st->grid_x = gx;
    st->grid_y = gy;
    st->grid_z = int((pairs + grid - 1) / grid);  // planes per CTA and step
    st->tile_x = Cf::SW;
    st->tile_y = Cf::TY;
    st->cached_rows = kr;  // planes per CTA
  }
  const size_t elems = size_t(h) * wy * wx;
  if (steps == 0) {
    PERKS_CUDA(cudaMemcpyAsync(d_out, d_in, elems * sizeof(T), host_io ? cudaMemcpyHostToHost : cudaMemcpyDeviceToDevice,
                               s));
    PERKS_CUDA(cudaStreamSynchronize(s));
    return PERKS_OK;
  }
  int stt = PERKS_OK;
  const size_t fbytes = size_t(h) * wy * px * sizeof(T);
  T* f0 = static_cast<T*>(workspace(kWsField0, fbytes, &stt));
  if (!f0) return stt;
  T* f1 = static_cast<T*>(workspace(kWsField1, fbytes, &stt));
  if (!f1) return stt;
  SyncWords sw;
  if ((stt = sync_words(&sw, s)) != PERKS_OK) return stt;
  PERKS_CUDA(copy_rows(f0, size_t(px) * sizeof(T), d_in, size_t(wx) * sizeof(T), size_t(wx) * sizeof(T),
                       size_t(h) * wy, host_io ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));

  Stencil3DParams p{};
  for (int i = 0; i < 2; i++) {
    void* base = i ? static_cast<void*>(f1) : static_cast<void*>(f0);
    if ((stt = encode_tiled_3d(&p.map[i], sizeof(T) == 8, base, wx, wy, h, px, Cf::SW, Cf::SR)) != PERKS_OK)
      return stt;
    if ((stt = encode_tiled_3d(&p.pmap[i], sizeof(T) == 8, base, wx, wy, h, px, Cf::HP, Cf::SR)) != PERKS_OK)
      return stt;
    if (kr > 0 && (stt = encode_tiled_3d(&p.hmap[i], sizeof(T) == 8, base, wx, wy, h, px, Cf::SW, Cf::H)) != PERKS_OK)
      return stt;
  }
  p.kr = kr;
  p.f[0] = f0;
  p.f[1] = f1;
  p.h = h;
  p.wy = wy;
  p.wx = wx;
  p.px = px;
  p.gx = gx;
  p.gy = gy;
  p.dirichlet = o.boundary == PERKS_BOUNDARY_DIRICHLET;
  p.alternate = persistent && o.l2_sweep;
  p.persistent = persistent;
  p.bar = sw.bar;
  p.status = sw.status;
  p.ctl = wait_ctl();

  // the kernel built with resident planes only where one is kept
  auto kern = kr > 0 ? stencil3d_kernel<T, SHAPE, FAST, Cfg3D<T, SHAPE, FAST, true>> : stencil3d_kernel<T, SHAPE, FAST, Cf>;
  PERKS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  cudaEvent_t e0, e1;
  PERKS_CUDA(cudaEventCreate(&e0));
  PERKS_CUDA(cudaEventCreate(&e1));
  PERKS_CUDA(cudaEventRecord(e0, s));
  int launches = 0;
  if (persistent) {
    int nb = 0;
    PERKS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, Cf::NT, smem));
    if ((long long)nb * dev->sms < grid) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail(PERKS_ERR_LAUNCH, "persistent 3D grid of " + std::to_string(grid) + " CTAs does not fit");
    }
    p.steps = steps;
    p.t0 = 0;
    void* args[] = {&p};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(Cf::NT), args, smem, s);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return cuda_fail(e, "cudaLaunchCooperativeKernel(stencil3d)");
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
      return cuda_fail(e, "stencil3d per-step launch");
    }
  }
  PERKS_CUDA(cudaEventRecord(e1, s));
  count_launch(launches);
  PERKS_CUDA(copy_rows(d_out, size_t(wx) * sizeof(T), (steps & 1) ? f1 : f0, size_t(px) * sizeof(T),
                       size_t(wx) * sizeof(T), size_t(h) * wy,
                       host_io ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  int rc = check_status(sw, s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != PERKS_OK) return rc;
  if (st) {
    st->ms = ms;
    st->gcells_per_s = double(elems) * steps / (double(ms) * 1e6);
    st->cached_fraction = double(cached) / double(pairs);
    st->launches = launches;
  }
  return PERKS_OK;
}

}  // namespace perks
