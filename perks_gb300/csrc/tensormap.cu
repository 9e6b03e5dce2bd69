// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include "runtime.cuh"

namespace perks {

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

// 3D tensor map over a [h][wy][px] field with logical x extent wx; box
// {box_x, box_y, 1}; out-of-range elements read as zero.
int encode_tiled_3d(CUtensorMap* map, bool f64, void* base, int wx, int wy, int h, int px, int box_x, int box_y) {
  auto enc = get_encode();
  if (!enc) return fail(PERKS_ERR_NO_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  const size_t es = f64 ? 8 : 4;
  cuuint64_t dims[3] = {cuuint64_t(wx), cuuint64_t(wy), cuuint64_t(h)};
  cuuint64_t strides[2] = {cuuint64_t(px) * es, cuuint64_t(px) * es * cuuint64_t(wy)};
  cuuint32_t box[3] = {cuuint32_t(box_x), cuuint32_t(box_y), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims,
                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(PERKS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ") for box " +
                                    std::to_string(box_x) + "x" + std::to_string(box_y));
  return PERKS_OK;
}

// 2D tensor map over a row-major [rows][pitch] field; box {box_x, 1};
// out-of-range elements read as zero.
int encode_tiled_2d(CUtensorMap* map, bool f64, void* base, int pitch, int rows, int box_x) {
  auto enc = get_encode();
  if (!enc) return fail(PERKS_ERR_NO_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  const size_t es = f64 ? 8 : 4;
  cuuint64_t dims[2] = {cuuint64_t(pitch), cuuint64_t(rows)};
  cuuint64_t strides[1] = {cuuint64_t(pitch) * es};
  cuuint32_t box[2] = {cuuint32_t(box_x), 1};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims,
                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(PERKS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ") for a 2D box of " +
                                    std::to_string(box_x));
  return PERKS_OK;
}

}  // namespace perks
