// Tensor maps of the generic kernel (host side).
//
// The kernel moves 16 KB tiles as boxes of 128 rows x 128 bytes through the
// tensor-memory accelerator with the 128-byte swizzle, so that each thread's
// 128-byte row lands in shared memory with its eight 16-byte chunks rotated
// by (row & 7): bank-conflict-free for the thread that reads its own row,
// in logical order, with compile-time register indices.
#include <cudaTypedefs.h>

#include <mutex>

#include "gps_internal.h"

namespace gps {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

cudaError_t encode_one(CUtensorMap* map, const void* base, uint64_t n, uint32_t elem_size) {
    auto fn = encode_fn();
    if (fn == nullptr) return cudaErrorNotSupported;
    // 16-byte struct elements travel as four 32-bit words each.
    if (elem_size == 16) {
        n *= 4;
        elem_size = 4;
    }
    const uint64_t row_elems = 128 / elem_size;
    // Row coordinates are 32-bit signed in the copy instructions.
    if (n / row_elems > 0x7FFFFF00ull) return cudaErrorInvalidValue;
    // Full rows only; a buffer shorter than one row still gets a valid map
    // (one row) that the kernel never uses.
    const uint64_t rows = n / row_elems > 0 ? n / row_elems : 1;
    const cuuint64_t dims[2] = {row_elems, rows};
    const cuuint64_t strides[1] = {128};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(row_elems), 128};
    const cuuint32_t estrides[2] = {1, 1};
    const CUtensorMapDataType dt =
        elem_size == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
    const CUresult r = fn(map, dt, 2, const_cast<void*>(base), dims, strides, box, estrides,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

cudaError_t encode_row_maps(const void* in, void* out, uint64_t n, uint32_t elem_size, RowMaps* maps) {
    cudaError_t err = encode_one(&maps->in, in, n, elem_size);
    if (err == cudaSuccess) err = encode_one(&maps->out, out, n, elem_size);
    return err;
}

}  // namespace gps
