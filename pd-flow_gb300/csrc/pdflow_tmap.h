// Host-side tensor maps of plane groups for the register-resident tile kernels.
//
// The arena carves a pair's planes of one level size back to back at a fixed
// stride (each plane rounded up to 256 bytes), so a run of consecutive planes
// is one 4D tensor (rows, columns, planes, arena slots).  One TMA tensor copy
// of a box (32 rows, 32 columns, all planes of the run, 1 slot) then moves a
// tile's region of every plane of the run, where one copy per plane would
// cost an instruction issue per plane on the critical path of the tile.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace pdflow {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry-point query (the
// library links no driver library); null: not available.
inline EncodeTiledFn tensor_map_encoder()
{
    static const EncodeTiledFn fn = [] {
        void* q = nullptr;
        cudaDriverEntryPointQueryResult qr = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &q, 12000, cudaEnableDefault, &qr) !=
                cudaSuccess ||
            qr != cudaDriverEntryPointSuccess)
            q = nullptr;
        return reinterpret_cast<EncodeTiledFn>(q);
    }();
    return fn;
}

// Whether planes[0..n) lie at one fixed stride (returned in *stride, bytes).
inline bool equally_spaced(const float* const* planes, int n, size_t* stride)
{
    if (n < 2) return false;
    const intptr_t d = reinterpret_cast<intptr_t>(planes[1]) - reinterpret_cast<intptr_t>(planes[0]);
    if (d <= 0 || (d % 16) != 0) return false;
    for (int k = 2; k < n; ++k)
        if (reinterpret_cast<intptr_t>(planes[k]) - reinterpret_cast<intptr_t>(planes[k - 1]) != d) return false;
    *stride = size_t(d);
    return true;
}

// 4D map (rows, columns, planes, slots) of n planes of R x C floats starting
// at `first`, `plane_stride` bytes apart, pair slots `pstride` bytes apart;
// box (box_r, box_c, n, 1).  False if the encoder is missing or refuses.
inline bool encode_plane_group(CUtensorMap* m, const float* first, unsigned n, size_t plane_stride, unsigned R,
                               unsigned C, unsigned slots, size_t pstride, unsigned box_r, unsigned box_c)
{
    const EncodeTiledFn encode = tensor_map_encoder();
    if (!encode) return false;
    const cuuint64_t dims[4] = {R, C, n, slots};
    const cuuint64_t strides[3] = {cuuint64_t(R) * 4u, plane_stride, pstride};
    const cuuint32_t box[4] = {box_r, box_c, n, 1}, estr[4] = {1, 1, 1, 1};
    return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(first), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace pdflow
