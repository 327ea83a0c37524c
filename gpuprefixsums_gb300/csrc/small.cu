// Scans of small inputs in one CTA (n <= kSmallMaxBytes / sizeof(T)).
//
// The persistent two-pass kernels pay a fixed cost of a few microseconds
// per launch for their pipeline (unit claim, reduce pass, lookback hand-off,
// reload, store, last-CTA-out bookkeeping) that dominates below ~2^16
// elements. Here one block of 1024 threads walks the input in chunks of 32
// bytes per thread (8 u32 or 4 u64): load (16-byte vectors when both buffers allow),
// tile scan of the chunk with the library's block primitives
// (include/gps_device.cuh), add the running carry, store. The next chunk's
// loads are issued before the current chunk is scanned.
#include "gps_device.cuh"
#include "gps_internal.h"

namespace gps {
namespace {

constexpr int kSmallThreads = 1024;
template <typename T>
constexpr int kSmallItems = 32 / static_cast<int>(sizeof(T));

template <typename T, bool VEC>
__device__ __forceinline__ void load_chunk(const T* in, uint64_t n, uint64_t base, T (&v)[kSmallItems<T>]) {
    const uint64_t i0 = base + static_cast<uint64_t>(threadIdx.x) * kSmallItems<T>;
    if (VEC && i0 + kSmallItems<T> <= n) {
        constexpr int EPV = 16 / sizeof(T);
#pragma unroll
        for (int j = 0; j < kSmallItems<T> / EPV; ++j) {
            const uint4 q = *reinterpret_cast<const uint4*>(in + i0 + j * EPV);
            const T* qt = reinterpret_cast<const T*>(&q);
#pragma unroll
            for (int e = 0; e < EPV; ++e) v[j * EPV + e] = qt[e];
        }
    } else {
#pragma unroll
        for (int e = 0; e < kSmallItems<T>; ++e) v[e] = i0 + e < n ? in[i0 + e] : T(0);
    }
}

template <typename T, bool INCL, bool VEC>
__global__ void __launch_bounds__(kSmallThreads, 1)
    small_scan_kernel(const T* in, T* out, uint64_t n, const T* carry_in, T* carry_out) {
    constexpr int ITEMS = kSmallItems<T>;
    constexpr int CHUNK = kSmallThreads * ITEMS;
    __shared__ gps_device::BlockScanStorage<kSmallThreads, T> st;
    T carry = carry_in != nullptr ? *carry_in : T(0);
    T v[ITEMS], nxt[ITEMS];
    load_chunk<T, VEC>(in, n, 0, v);
    for (uint64_t base = 0; base < n; base += CHUNK) {
        const bool more = base + CHUNK < n;
        if (more) load_chunk<T, VEC>(in, n, base + CHUNK, nxt);
        // The scan's barriers also order every thread's loads of this chunk
        // before any store to it (in-place scans).
        const T total = gps_device::tile_scan<kSmallThreads, ITEMS, INCL>(v, st);
        const uint64_t i0 = base + static_cast<uint64_t>(threadIdx.x) * ITEMS;
        if (VEC && i0 + ITEMS <= n) {
            constexpr int EPV = 16 / sizeof(T);
#pragma unroll
            for (int j = 0; j < ITEMS / EPV; ++j) {
                uint4 q;
                T* qt = reinterpret_cast<T*>(&q);
#pragma unroll
                for (int e = 0; e < EPV; ++e) qt[e] = carry + v[j * EPV + e];
                *reinterpret_cast<uint4*>(out + i0 + j * EPV) = q;
            }
        } else {
#pragma unroll
            for (int e = 0; e < ITEMS; ++e)
                if (i0 + e < n) out[i0 + e] = carry + v[e];
        }
        carry += total;
        if (more) {
#pragma unroll
            for (int e = 0; e < ITEMS; ++e) v[e] = nxt[e];
        }
    }
    if (carry_out != nullptr && threadIdx.x == 0) *carry_out = carry;
}

template <typename T, bool INCL>
cudaError_t launch_small_t(const ScanArgs& a, cudaStream_t stream, LaunchInfo* info) {
    const bool vec = ((reinterpret_cast<uintptr_t>(a.in) | reinterpret_cast<uintptr_t>(a.out)) & 15u) == 0;
    const T* in = static_cast<const T*>(a.in);
    T* out = static_cast<T*>(a.out);
    const T* cin = static_cast<const T*>(a.carry_in);
    T* cout = static_cast<T*>(a.carry_out);
    if (info) *info = LaunchInfo{1, kSmallThreads, 0};
    if (vec)
        small_scan_kernel<T, INCL, true><<<1, kSmallThreads, 0, stream>>>(in, out, a.n, cin, cout);
    else
        small_scan_kernel<T, INCL, false><<<1, kSmallThreads, 0, stream>>>(in, out, a.n, cin, cout);
    return cudaGetLastError();
}

}  // namespace

uint64_t small_scan_max_elems(gps_dtype dtype) { return kSmallMaxBytes / dtype_size(dtype); }

cudaError_t launch_small(gps_dtype dtype, bool inclusive, const ScanArgs& a, cudaStream_t stream, LaunchInfo* info) {
    if (dtype == GPS_DTYPE_U64)
        return inclusive ? launch_small_t<uint64_t, true>(a, stream, info) : launch_small_t<uint64_t, false>(a, stream, info);
    return inclusive ? launch_small_t<uint32_t, true>(a, stream, info) : launch_small_t<uint32_t, false>(a, stream, info);
}

}  // namespace gps
