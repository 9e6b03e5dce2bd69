// Host launcher for the 3D stencil kernel: tensor maps, tile grid and z-slab
// split, resident-plane budget, cooperative or per-step launch.
#pragma once
#include <cudaTypedefs.h>
#include <algorithm>
#include <string>
#include "runtime.cuh"
#include "stencil3d.cuh"

namespace perks {

int encode_tiled_3d(CUtensorMap* map, bool f64, void* base, int wx, int wy, int h, int px, int box_x, int box_y);

template <class T, int SHAPE, bool FAST>
int launch_stencil3d(const perks_stencil_opts& o, const T* d_in, T* d_out, int h, int wy, int wx, int steps,
                     perks_stencil_stats* st) {
  using Cf = Cfg3D<T, SHAPE>;
  constexpr int H = Cf::H, R = Cf::R;
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(o.stream);
  const bool persistent = o.kernel == PERKS_KERNEL_PERSISTENT;
  const int ctas = o.ctas > 0 ? std::min(o.ctas, dev->sms) : dev->sms;
  const int gx = (wx + Cf::TX - 1) / Cf::TX;
  const int gy = (wy + Cf::TY - 1) / Cf::TY;
  const long long gxy = (long long)gx * gy;
  // z-slabs: use the remaining CTAs, keep at least 2H+1 planes per slab. When
  // the x-y tiles alone outnumber the CTAs, each CTA sweeps several tiles.
  int gz = persistent ? int(std::max<long long>(1, std::min<long long>(ctas / gxy, h / (2 * H + 1))))
                      : std::max(1, h / 64);
  gz = std::max(1, std::min(gz, h));
  const long long ntiles = gxy * gz;
  if (ntiles > (1ll << 30)) return fail(PERKS_ERR_UNSUPPORTED, "tile grid too large");
  const int px = (wx + Cf::V - 1) / Cf::V * Cf::V;
  const int znmax = (h + gz - 1) / gz;

  size_t fixed = Cf::ring_bytes + Cf::bar_bytes;
  int C = 0, M = 0;
  if (persistent && o.cache_rows != 0 && steps > 1 && ntiles <= ctas) {
    const size_t per = Cf::slot_bytes + size_t(Cf::SIDE) * sizeof(T);
    long long avail = (long long)dev->smem_optin - (long long)fixed - 256 - (long long)(R + H) * Cf::slot_bytes;
    int cmax = avail > 0 ? int(avail / (long long)per) : 0;
    if (o.cache_rows > 0) cmax = std::min(cmax, o.cache_rows);
    C = std::min(cmax, znmax - 2 * H);
    if (C <= 0) C = 0;
    M = C > 0 ? C + R + H : 0;
  }
  const size_t smem = fixed + size_t(M) * Cf::slot_bytes + size_t(C) * Cf::SIDE * sizeof(T);
  if (smem > dev->smem_optin) return fail(PERKS_ERR_UNSUPPORTED, "shared memory budget exceeded");
  if (st) {
    *st = perks_stencil_stats{};
    st->grid_x = gx;
    st->grid_y = gy;
    st->grid_z = gz;
    st->tile_x = Cf::TX;
    st->tile_y = Cf::TY;
    st->cached_rows = C;
  }
  const size_t elems = size_t(h) * wy * wx;
  if (steps == 0) {
    PERKS_CUDA(cudaMemcpyAsync(d_out, d_in, elems * sizeof(T), cudaMemcpyDeviceToDevice, s));
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
  PERKS_CUDA(cudaMemcpy2DAsync(f0, size_t(px) * sizeof(T), d_in, size_t(wx) * sizeof(T), size_t(wx) * sizeof(T),
                               size_t(h) * wy, cudaMemcpyDeviceToDevice, s));

  Stencil3DParams p{};
  const bool f64 = sizeof(T) == 8;
  for (int i = 0; i < 2; i++) {
    void* base = i ? (void*)f1 : (void*)f0;
    if ((stt = encode_tiled_3d(&p.map[i], f64, base, wx, wy, h, px, Cf::RWX, Cf::SR)) != PERKS_OK) return stt;
    if ((stt = encode_tiled_3d(&p.mapNS[i], f64, base, wx, wy, h, px, Cf::RWX, H)) != PERKS_OK) return stt;
    if ((stt = encode_tiled_3d(&p.mapWE[i], f64, base, wx, wy, h, px, Cf::HP, Cf::TY)) != PERKS_OK) return stt;
  }
  p.f[0] = f0;
  p.f[1] = f1;
  p.h = h;
  p.wy = wy;
  p.wx = wx;
  p.px = px;
  p.gx = gx;
  p.gy = gy;
  p.gz = gz;
  p.C = C;
  p.M = M;
  p.dirichlet = o.boundary == PERKS_BOUNDARY_DIRICHLET;
  p.alternate = persistent && o.l2_sweep;
  p.persistent = persistent;
  p.bar = sw.bar;
  p.status = sw.status;

  auto kern = stencil3d_kernel<T, SHAPE, FAST>;
  PERKS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const int grid = persistent ? int(std::min<long long>(ntiles, ctas)) : int(ntiles);
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
  PERKS_CUDA(cudaMemcpy2DAsync(d_out, size_t(wx) * sizeof(T), (steps & 1) ? f1 : f0, size_t(px) * sizeof(T),
                               size_t(wx) * sizeof(T), size_t(h) * wy, cudaMemcpyDeviceToDevice, s));
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
    for (int k = 0; k < gz; k++) {
      int z0 = int((long long)k * h / gz), z1 = int((long long)(k + 1) * h / gz);
      cached += std::max(0, std::min(C, z1 - z0 - 2 * H));
    }
    st->cached_fraction = double(cached) / double(h);
    st->launches = launches;
  }
  return PERKS_OK;
}

}  // namespace perks
