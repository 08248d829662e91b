// Host-side construction of the TMA tensor maps of the fused step kernel.
// cuTensorMapEncodeTiled is taken from the driver through the runtime's
// entry-point query, so the library needs no link against libcuda.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>

#include "engine_internal.h"
#include "tma.cuh"

namespace fdtd {

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                 CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

// One 3-D map over a padded array for the tile loads: dims {kPadX + Ni + 2,
// Nj + 2 kPadY, Nk} (the left margin, the grid and the two right ghost
// columns, the last column a two-step tile reads; every ghost row), box
// {box_w, box rows, 1}.  Box columns past the second ghost column are outside
// the map: the copy engine fills them with zeros instead of reading memory (a
// tile narrower than 32 columns reads only what it uses).
bool encode(CUtensorMap* m, CUtensorMapDataType dt, size_t es, void* base, const PLayout& L, int box_w,
            int box_rows) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)(kPadX + L.Ni + 2), (cuuint64_t)(L.Nj + 2 * kPadY), (cuuint64_t)L.Nk};
  const cuuint64_t strides[2] = {(cuuint64_t)(L.pitch * es), (cuuint64_t)(L.pplane * es)};
  const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(m, dt, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Columns of the right margin a store map covers: the ghost column and the
// rest of the 16-byte unit that holds it for 2-byte words.
constexpr int kRightMargin = 8;

// One 3-D map over the grid rows of a padded array with their x margins
// (ghost rows excluded): dims {kPadX + Ni + kRightMargin, Nj, Nk} from padded
// column 0, box {32, tile_y, 1}.  x coordinate kPadX + x is cell x; a store
// at 0 fills the left margin (cells -32 .. -1), one at kPadX + Ni the first
// kRightMargin columns of the right margin (the copy engine clips the rest).
// Rows outside the grid are not written.
bool encode_store(CUtensorMap* m, CUtensorMapDataType dt, size_t es, void* base, const PLayout& L,
                  int tile_y) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  void* origin = static_cast<unsigned char*>(base) + L.at(-kPadX, 0, 0) * es;
  const cuuint64_t dims[3] = {(cuuint64_t)(L.Ni + kPadX + kRightMargin), (cuuint64_t)L.Nj, (cuuint64_t)L.Nk};
  const cuuint64_t strides[2] = {(cuuint64_t)(L.pitch * es), (cuuint64_t)(L.pplane * es)};
  const cuuint32_t box[3] = {32, (cuuint32_t)tile_y, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(m, dt, 3, origin, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t build_tma_store_maps(void* maps, const PLayout& L, HiType ht, void* const hi[6], LoT* const lo[6],
                                 int tile_y) {
  TmaMaps* m = static_cast<TmaMaps*>(maps);
  std::memset(m, 0, sizeof(TmaMaps));
  const CUtensorMapDataType dt = ht == HiType::F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  const size_t es = ht == HiType::F32 ? 4 : 2;
  for (int c = 0; c < 6; ++c) {
    if (!encode_store(&m->hi[c], dt, es, hi[c], L, tile_y)) return cudaErrorInvalidValue;
    if (lo && lo[c] && !encode_store(&m->lo[c], CU_TENSOR_MAP_DATA_TYPE_UINT16, sizeof(LoT), lo[c], L, tile_y))
      return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

cudaError_t build_tma_maps(void* maps, const PLayout& L, HiType ht, void* const hi[6], LoT* const lo[6],
                           const int box_w[6], const int lo_box_w[6], int tile_y, BoxTrim trim) {
  TmaMaps* m = static_cast<TmaMaps*>(maps);
  std::memset(m, 0, sizeof(TmaMaps));
  const CUtensorMapDataType dt = ht == HiType::F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  const size_t es = ht == HiType::F32 ? 4 : 2;
  for (int c = 0; c < 6; ++c) {
    // B-first sweeps: only Ex and Ez (0, 2) carry a second halo row (the
    // row above the tile); every other box is one row shorter.
    const bool tall = trim == BoxTrim::None || c == 0 || c == 2;
    const int rows = tall ? tile_y + 2 : tile_y + 1;
    if (!encode(&m->hi[c], dt, es, hi[c], L, box_w[c], rows)) return cudaErrorInvalidValue;
    if (lo && lo[c] && !encode(&m->lo[c], CU_TENSOR_MAP_DATA_TYPE_UINT16, sizeof(LoT), lo[c], L, lo_box_w[c], rows))
      return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

}  // namespace fdtd
