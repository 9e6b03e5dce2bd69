// 3D Jacobi time loop for sm_103a: z-streaming persistent cooperative kernel
// with a TMA (cp.async.bulk.tensor) plane pipeline.
//
// Work decomposition:
//   The internal field is [height][width_y][pitch_x] (pitch_x = width_x
//   rounded up to 16 bytes). CTA (tz, ty, tx) owns an x-y tile of TX x TY
//   cells and a z-slab [z0, z1). Each step it sweeps the slab plane by plane
//   in groups of R output planes. Input planes (tile plus H halo rows and HP
//   halo columns on each side) arrive in a ring of NR shared-memory slots, one
//   3D tiled TMA copy per plane; coordinates outside the field are zero-filled
//   by the TMA unit and then overwritten with clamped values in shared memory.
//   Each thread owns V consecutive columns of RY consecutive rows and keeps a
//   rolling register window of 2H+1 planes.
//   PERKS caching: planes [z0+H, z0+H+C) of the slab stay in shared memory for
//   the whole launch with the same skewed in-place update as the 2D kernel;
//   their tile-boundary rows and columns are stored to the field each step so
//   that neighbouring tiles can load them, and their halo ring is reloaded
//   from the field with four small TMA copies per plane per step.
//   Steps are separated by a bounded grid barrier.
#pragma once
#include <cuda.h>
#include <cstdint>
#include "ptx.cuh"
#include "shapes.cuh"

namespace perks {

struct Stencil3DParams {
  CUtensorMap map[2];     // plane box {TX+2HP, TY+2H, 1} over field 0 / 1
  CUtensorMap mapNS[2];   // box {TX+2HP, H, 1}: north/south halo strips of resident planes
  CUtensorMap mapWE[2];   // box {HP, TY, 1}: west/east halo strips of resident planes
  void* f[2];
  int h, wy, wx, px;      // domain and x pitch (elements)
  int gx, gy, gz;         // tile grid
  int steps, t0;
  int C, M;               // resident planes per slab (upper bound) and slots
  int dirichlet, alternate, persistent;
  unsigned* bar;
  unsigned* status;
};

template <class T, int SHAPE>
struct Cfg3D {
  static constexpr int H = ShapeInfo<SHAPE>::H;
  static constexpr bool BOX = ShapeInfo<SHAPE>::box;
  static constexpr int V = 16 / sizeof(T);
  static constexpr int NTX = (sizeof(T) == 4) ? 16 : 32;  // threads across x
  static constexpr int NTY = 256 / NTX;                   // threads across y
  static constexpr int NT = NTX * NTY;
  static constexpr int RY = 2;                            // rows per thread
  static constexpr int TX = NTX * V;                      // 64
  static constexpr int TY = NTY * RY;                     // 32 (f32) / 16 (f64)
  static constexpr int HP = ((H + V - 1) / V) * V;
  static constexpr int RWX = TX + 2 * HP;                 // slot row width
  static constexpr int SR = TY + 2 * H;                   // slot rows
  static constexpr int PLANE = SR * RWX;                  // elements per plane tile
  static constexpr int AL = 128 / sizeof(T);              // TMA destinations are 128-byte aligned
  static constexpr int SLOT = ((PLANE + AL - 1) / AL) * AL;  // slot stride (elements)
  static constexpr int SNS = ((H * RWX + AL - 1) / AL) * AL; // side-buffer strip strides
  static constexpr int SWE = ((HP * TY + AL - 1) / AL) * AL;
  static constexpr int SIDE = 2 * SNS + 2 * SWE;            // side buffer per resident plane
  static constexpr int R = 4;                             // output planes per group
  static constexpr int NR = 2 * R + 2 * H + 2;            // ring slots
  static_assert(NR <= 64, "phase mask");
  static constexpr size_t slot_bytes = size_t(SLOT) * sizeof(T);
  static constexpr size_t box_bytes = size_t(PLANE) * sizeof(T);   // bytes one plane copy delivers
  static constexpr size_t ring_bytes = size_t(NR) * slot_bytes;
  static constexpr size_t bar_bytes = (NR + 2) * sizeof(uint64_t);
};

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cta.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3, %4}], [%5], %6;" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

template <class T, int SHAPE, bool FAST>
__global__ void __launch_bounds__(Cfg3D<T, SHAPE>::NT, 1)
    stencil3d_kernel(const __grid_constant__ Stencil3DParams p) {
  using Cf = Cfg3D<T, SHAPE>;
  using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  constexpr int H = Cf::H, V = Cf::V, TX = Cf::TX, TY = Cf::TY, HP = Cf::HP, RWX = Cf::RWX, SR = Cf::SR;
  constexpr int PLANE = Cf::SLOT, R = Cf::R, NR = Cf::NR, RY = Cf::RY, NT = Cf::NT, NTX = Cf::NTX;
  constexpr int NW = 2 * H + 1;     // planes in the rolling window
  constexpr int WR = RY + 2 * H;    // window rows
  constexpr int WC = V + 2 * H;     // window columns

  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* ring = reinterpret_cast<T*>(smem_raw);
  T* res = ring + size_t(NR) * PLANE;
  T* side = res + size_t(p.M) * PLANE;  // halo strips of resident planes, [C][N,S,W,E]
  uint64_t* bars = reinterpret_cast<uint64_t*>(side + size_t(p.M > 0 ? p.C : 0) * Cf::SIDE);
  uint64_t* bar_res = bars + NR;

  const int tid = threadIdx.x;
  const int txi = tid % NTX, tyi = tid / NTX;
  const int h = p.h, wy = p.wy, wx = p.wx, px = p.px;
  const int ntiles = p.gx * p.gy * p.gz;
  // Geometry of the tile being swept (a CTA owns several tiles when the tile
  // grid is larger than the launch; resident planes then stay off).
  int x0 = 0, y0 = 0, z0 = 0, z1 = 0, ZN = 0, lw = 0, lwy = 0;
  bool fix_l = false, fix_r = false, fix_t = false, fix_b = false, any_fix = false;
  auto set_tile = [&](int b) {
    const int tj = b % p.gx;
    b /= p.gx;
    const int ti = b % p.gy;
    const int tk = b / p.gy;
    x0 = tj * TX;
    y0 = ti * TY;
    z0 = int((long long)tk * h / p.gz);
    z1 = int((long long)(tk + 1) * h / p.gz);
    ZN = z1 - z0;
    fix_l = !p.dirichlet && x0 == 0;
    fix_r = !p.dirichlet && x0 + TX + HP > wx;
    fix_t = !p.dirichlet && y0 == 0;
    fix_b = !p.dirichlet && y0 + TY + H > wy;
    any_fix = fix_l || fix_r || fix_t || fix_b;
    lw = wx - 1 - x0;   // tile-local last column
    lwy = wy - 1 - y0;  // tile-local last row
  };
  set_tile(blockIdx.x);
  const int C = (p.M > 0 && ntiles == int(gridDim.x)) ? max(0, min(p.C, ZN - 2 * H)) : 0;
  const int zres0 = z0 + H;
  const int M = p.M;
  const int cx = txi * V;      // thread's first column (tile-local)
  const int cy = tyi * RY;     // thread's first row (tile-local)

  GridBarrier gbar{p.bar, p.status, gridDim.x};
  const uint64_t pol = policy_evict_normal();
  const uint64_t pol_first = policy_evict_first();

  if (tid == 0) {
    for (int i = 0; i < NR + 1; i++) mbar_init(&bars[i], 1);
    fence_mbar_init();
  }
  __syncthreads();

  uint64_t phase = 0ull;
  uint32_t res_phase = 0u;
  int off = 0;
  bool ok = true;
  int issued = 0, waited = 0;
  bool fwd = true;

  auto slot_of_res = [&](int z) -> T* {
    int s = (z - zres0 + off) % M;
    if (s < 0) s += M;
    return res + size_t(s) * PLANE;
  };
  // Replace values outside the domain by clamped ones (columns first, then rows).
  auto fixup_plane = [&](T* slot) {
    if (fix_l || fix_r) {
      for (int r = tid; r < SR; r += NT) {
        T* row = slot + r * RWX;
        if (fix_l) {
          const T v = row[HP];
          for (int k = 1; k <= H; k++) row[HP - k] = v;
        }
        if (fix_r && lw < TX + HP - 1) {
          const T v = row[HP + lw];
          for (int k = 1; k <= H && HP + lw + k < RWX; k++) row[HP + lw + k] = v;
        }
      }
    }
    if (fix_t || fix_b) {
      __syncthreads();
      for (int c = tid; c < RWX; c += NT) {
        if (fix_t) {
          const T v = slot[H * RWX + c];
          for (int k = 1; k <= H; k++) slot[(H - k) * RWX + c] = v;
        }
        if (fix_b && lwy < TY + H - 1) {
          const T v = slot[(H + lwy) * RWX + c];
          for (int k = 1; k <= H && H + lwy + k < SR; k++) slot[(H + lwy + k) * RWX + c] = v;
        }
      }
    }
  };

  int tmx = x0 - HP, tmy = y0 - H;  // TMA box origin

  // ---------------------------------------------------------------- prologue
  if (C > 0) {
    const CUtensorMap* mp = &p.map[p.t0 & 1];
    if (tid == 0) {
      mbar_arrive_expect_tx(bar_res, unsigned(Cf::box_bytes) * unsigned(C));
      for (int z = zres0; z < zres0 + C; z++) tma_load_3d(slot_of_res(z), mp, tmx, tmy, z, bar_res, pol);
    }
    if (!mbar_wait(bar_res, res_phase & 1u)) {
      atomicOr(p.status, kErrCopyTimeout);
      ok = false;
    }
    res_phase ^= 1u;
    ok = __syncthreads_and(ok);
    if (ok && any_fix) {
      for (int k = 0; k < C; k++) fixup_plane(slot_of_res(zres0 + k));
    }
  }

  for (int it = 0; it < p.steps && ok; it++) {
    const int t = p.t0 + it;
    const CUtensorMap* mp = &p.map[t & 1];
    T* fout = static_cast<T*>(p.f[(t + 1) & 1]);
    fwd = !p.alternate || ((t & 1) == 0);
    auto plane_of = [&](int s) { return fwd ? z0 + s : z1 - 1 - s; };
    auto is_res = [&](int z) { return C > 0 && z >= zres0 && z < zres0 + C; };
    auto loaded = [&](int s) {
      const int z = plane_of(s);
      return z >= 0 && z < h && !is_res(z);
    };
    auto pos_of = [&](int z) { return fwd ? z - z0 : z1 - 1 - z; };
    auto slot_of = [&](int z) -> T* {
      z = min(max(z, 0), h - 1);
      if (is_res(z)) return slot_of_res(z);
      return ring + size_t((pos_of(z) + H) % NR) * PLANE;
    };
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    if (tile != int(blockIdx.x)) {
      set_tile(tile);
      tmx = x0 - HP;
      tmy = y0 - H;
    }
    __syncthreads();  // ring slots of the previous tile are no longer read
    issued = -H;
    auto produce = [&](int upto) {
      const int lim = min(upto, ZN + H);
      for (; issued < lim; issued++) {
        if (!loaded(issued)) continue;
        const int z = plane_of(issued);
        const int q = (issued + H) % NR;
        mbar_arrive_expect_tx(&bars[q], unsigned(Cf::box_bytes));
        const bool interior = z >= z0 + H && z < z1 - H;
        tma_load_3d(ring + size_t(q) * PLANE, mp, tmx, tmy, z, &bars[q], (p.alternate && interior) ? pol_first : pol);
      }
    };
    if (tid == 0) {
      fence_proxy_async_global();
      produce(NR - H);
      if (C > 0 && it > 0) {
        // reload the halo ring of every resident plane into the side buffer
        // (dense strips N, S, W, E); it is scattered into the slots below.
        const unsigned bns = unsigned(H * RWX * sizeof(T)), bwe = unsigned(HP * TY * sizeof(T));
        mbar_arrive_expect_tx(bar_res, (2 * bns + 2 * bwe) * unsigned(C));
        for (int k = 0; k < C; k++) {
          const int z = zres0 + k;
          T* sd = side + size_t(k) * Cf::SIDE;
          tma_load_3d(sd, &p.mapNS[t & 1], tmx, y0 - H, z, bar_res, pol);
          tma_load_3d(sd + Cf::SNS, &p.mapNS[t & 1], tmx, y0 + TY, z, bar_res, pol);
          tma_load_3d(sd + 2 * Cf::SNS, &p.mapWE[t & 1], x0 - HP, y0, z, bar_res, pol);
          tma_load_3d(sd + 2 * Cf::SNS + Cf::SWE, &p.mapWE[t & 1], x0 + TX, y0, z, bar_res, pol);
        }
      }
    }
    if (C > 0 && it > 0) {
      if (!mbar_wait(bar_res, res_phase & 1u)) {
        atomicOr(p.status, kErrCopyTimeout);
        ok = false;
      }
      res_phase ^= 1u;
      ok = __syncthreads_and(ok);
      if (!ok) break;
      // N/S strips: H rows of RWX; W/E strips: TY rows of HP.
      for (int i = tid; i < C * (2 * H * RWX + 2 * TY * HP); i += NT) {
        const int per = 2 * H * RWX + 2 * TY * HP;
        const int k = i / per;
        int j = i % per;
        T* sl = slot_of_res(zres0 + k);
        const T* sd = side + size_t(k) * Cf::SIDE;
        if (j < 2 * H * RWX) {
          const int sdn = j / (H * RWX);  // 0 = north, 1 = south
          const int e = j % (H * RWX);
          sl[(sdn ? H + TY : 0) * RWX + e] = sd[sdn * Cf::SNS + e];
        } else {
          j -= 2 * H * RWX;
          const int sde = j / (TY * HP);  // 0 = west, 1 = east
          const int e = j % (TY * HP);
          const int r = e / HP, c = e % HP;
          sl[(H + r) * RWX + (sde ? HP + TX : 0) + c] = sd[2 * Cf::SNS + sde * Cf::SWE + e];
        }
      }
      if (any_fix) {
        __syncthreads();
        for (int k = 0; k < C; k++) fixup_plane(slot_of_res(zres0 + k));
      }
    }

    waited = -H;
    for (int lo = 0; lo < ZN && ok; lo += R) {
      const int hi = min(lo + R, ZN);
      const int need_hi = hi + H;
      const int first_new = waited;
      for (; waited < need_hi; waited++) {
        if (!loaded(waited)) continue;
        const int q = (waited + H) % NR;
        if (!mbar_wait(&bars[q], unsigned(phase >> q) & 1u)) {
          atomicOr(p.status, kErrCopyTimeout);
          ok = false;
          break;
        }
        phase ^= (1ull << q);
      }
      ok = __syncthreads_and(ok);
      if (!ok) break;
      if (any_fix) {
        for (int s2 = first_new; s2 < need_hi; s2++)
          if (loaded(s2)) fixup_plane(ring + size_t((s2 + H) % NR) * PLANE);
        __syncthreads();
      }
      if (tid == 0) produce(lo - H + NR);

      const int za = fwd ? z0 + lo : z1 - hi;
      const int nz = hi - lo;
      // Rolling window over planes za-H .. za+nz-1+H.
      constexpr int WCOL = Cf::BOX ? WC : V;
      constexpr int WROW = Cf::BOX ? WR : RY;
      T win[NW][WROW][WCOL];
      auto load_plane = [&](T (&dst)[WROW][WCOL], int z) {
        const T* sl = slot_of(z);
#pragma unroll
        for (int r = 0; r < WROW; r++) {
          const T* row = sl + (cy + r + (Cf::BOX ? 0 : H)) * RWX + HP + cx;
          VT v = *reinterpret_cast<const VT*>(row);
          const T* ve = reinterpret_cast<const T*>(&v);
          if constexpr (Cf::BOX) {
#pragma unroll
            for (int e = 0; e < V; e++) dst[r][H + e] = ve[e];
#pragma unroll
            for (int k = 1; k <= H; k++) {
              dst[r][H - k] = row[-k];
              dst[r][H + V - 1 + k] = row[V - 1 + k];
            }
          } else {
#pragma unroll
            for (int e = 0; e < V; e++) dst[r][e] = ve[e];
          }
        }
      };
#pragma unroll
      for (int j = 0; j < 2 * H; j++) load_plane(win[j], za - H + j);
#pragma unroll
      for (int k = 0; k < R; k++) {
        if (k < nz) {
          const int z = za + k;
          load_plane(win[(k + 2 * H) % NW], z + H);
          // star shapes: cross window of the centre plane
          T cr[Cf::BOX ? 1 : WR][Cf::BOX ? 1 : WC];
          if constexpr (!Cf::BOX) {
            const T* sl = slot_of(z);
#pragma unroll
            for (int r = 0; r < WR; r++) {
              const T* row = sl + (cy + r) * RWX + HP + cx;
              if (r >= H && r < H + RY) {
                VT v = *reinterpret_cast<const VT*>(row);
                const T* ve = reinterpret_cast<const T*>(&v);
#pragma unroll
                for (int e = 0; e < V; e++) cr[r][H + e] = ve[e];
#pragma unroll
                for (int kk = 1; kk <= H; kk++) {
                  cr[r][H - kk] = row[-kk];
                  cr[r][H + V - 1 + kk] = row[V - 1 + kk];
                }
              } else {
                VT v = *reinterpret_cast<const VT*>(row);
                const T* ve = reinterpret_cast<const T*>(&v);
#pragma unroll
                for (int e = 0; e < V; e++) cr[r][H + e] = ve[e];
              }
            }
          }
#pragma unroll
          for (int ry = 0; ry < RY; ry++) {
            const int y = y0 + cy + ry;
            T o[V];
#pragma unroll
            for (int e = 0; e < V; e++) {
              auto u = [&](int dz, int dy, int dx) -> T {
                if constexpr (Cf::BOX) {
                  return win[(k + H + dz) % NW][ry + H + dy][H + e + dx];
                } else {
                  if (dz == 0) return cr[ry + H + dy][H + e + dx];
                  return win[(k + H + dz) % NW][ry][e];
                }
              };
              o[e] = stencil_point<T, SHAPE, FAST>(u);
            }
            if (p.dirichlet) {
              const bool fixed = z < H || z >= h - H || y < H || y >= wy - H;
#pragma unroll
              for (int e = 0; e < V; e++) {
                const int x = x0 + cx + e;
                const T old = Cf::BOX ? win[(k + H) % NW][ry + H][H + e] : win[(k + H) % NW][ry][e];
                if (fixed || x < H || x >= wx - H) o[e] = old;
              }
            }
            VT ov;
            T* oe = reinterpret_cast<T*>(&ov);
#pragma unroll
            for (int e = 0; e < V; e++) oe[e] = o[e];
            const bool inside = (y < wy) && (x0 + cx < px);
            if (is_res(z)) {
              const int tz = fwd ? z - (R + H) : z + (R + H);
              int s = (tz - zres0 + off) % M;
              if (s < 0) s += M;
              *reinterpret_cast<VT*>(res + size_t(s) * PLANE + (H + cy + ry) * RWX + HP + cx) = ov;
              const bool edge = (cy + ry < H) || (cy + ry >= TY - H) || (cx < HP) || (cx >= TX - HP);
              if (inside && edge) *reinterpret_cast<VT*>(fout + (size_t(z) * wy + y) * px + x0 + cx) = ov;
            } else if (inside) {
              *reinterpret_cast<VT*>(fout + (size_t(z) * wy + y) * px + x0 + cx) = ov;
            }
          }
        }
      }
    }
    }  // tile loop
    if (ok && ntiles > int(gridDim.x)) {
      set_tile(blockIdx.x);
      tmx = x0 - HP;
      tmy = y0 - H;
    }
    if (!ok) break;
    if (M > 0) {
      off = fwd ? off - (R + H) : off + (R + H);
      off %= M;
      if (off < 0) off += M;
    }
    if (it + 1 < p.steps) {
      fence_proxy_async_global();
      if (p.persistent) {
        if (!gbar.sync()) { ok = false; break; }
      }
    }
  }
  if (ok && C > 0) {
    __syncthreads();
    T* fnew = static_cast<T*>(p.f[(p.t0 + p.steps) & 1]);
    for (int k = 0; k < C; k++) {
      const int z = zres0 + k;
      const T* sl = slot_of_res(z);
#pragma unroll
      for (int ry = 0; ry < RY; ry++) {
        const int y = y0 + cy + ry;
        if (y < wy && x0 + cx < px)
          *reinterpret_cast<VT*>(fnew + (size_t(z) * wy + y) * px + x0 + cx) =
              *reinterpret_cast<const VT*>(sl + (H + cy + ry) * RWX + HP + cx);
      }
    }
  }
  if (!ok) {
    __syncthreads();
    if (tid == 0) {
      uint64_t ph = phase;
      for (int s = waited; s < issued; s++) {
        const int z = fwd ? z0 + s : z1 - 1 - s;
        if (z < 0 || z >= h || (C > 0 && z >= zres0 && z < zres0 + C)) continue;
        const int q = (s + H) % NR;
        long long tw = clock64();
        while (!mbar_try_wait(&bars[q], unsigned(ph >> q) & 1u)) {
          if (clock64() - tw > (1ll << 28)) break;
        }
        ph ^= (1ull << q);
      }
    }
  }
}

}  // namespace perks
