// Scan operations for the generic single-pass kernel (scan_seg.cuh).
//
// Each operation fixes
//   T  element type in memory,
//   S  running state inside a CTA (the element type, or a double-float pair
//      for the compensated FP32 scan),
//   C  value carried between lookback units in the tile descriptors (the
//      element type, or FP64 for the compensated FP32 scan),
// and the associative combine of S and of C. Integer scans wrap mod 2^w.
#pragma once
#include <cstdint>

namespace gps {

template <typename S>
__device__ __forceinline__ S shfl_any(S s, uint32_t src);
template <typename S>
__device__ __forceinline__ S shfl_up_any(S s, uint32_t d);

template <>
__device__ __forceinline__ uint32_t shfl_any(uint32_t s, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, s, src); }
template <>
__device__ __forceinline__ uint64_t shfl_any(uint64_t s, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, s, src); }
template <>
__device__ __forceinline__ float shfl_any(float s, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, s, src); }
template <>
__device__ __forceinline__ double shfl_any(double s, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, s, src); }
template <>
__device__ __forceinline__ uint32_t shfl_up_any(uint32_t s, uint32_t d) { return __shfl_up_sync(0xFFFFFFFFu, s, d); }
template <>
__device__ __forceinline__ uint64_t shfl_up_any(uint64_t s, uint32_t d) { return __shfl_up_sync(0xFFFFFFFFu, s, d); }
template <>
__device__ __forceinline__ float shfl_up_any(float s, uint32_t d) { return __shfl_up_sync(0xFFFFFFFFu, s, d); }

// ------------------------------------------------------------- integers
template <typename U>
struct OpInt {
    using T = U;
    using S = U;
    using C = U;
    static constexpr bool kPackedRowSum = false;
    __device__ static S zero() { return 0; }
    __device__ static S lift(T x) { return x; }
    __device__ static S add(S a, S b) { return a + b; }
    __device__ static S acc(S a, T x) { return a + x; }
    __device__ static S combine(S a, S b) { return a + b; }
    __device__ static S norm(S a) { return a; }
    __device__ static T out(S s) { return s; }
    __device__ static C to_chain(S s) { return s; }
    __device__ static S from_chain(C c) { return c; }
    __device__ static C chain_zero() { return 0; }
    __device__ static C chain_add(C a, C b) { return a + b; }
    __device__ static uint64_t chain_bits(C c) { return static_cast<uint64_t>(c); }
    __device__ static C chain_from_bits(uint64_t b) { return static_cast<C>(b); }
    static constexpr int kDescWords = 1;
    __device__ static uint64_t chain_word(C c, int) { return chain_bits(c); }
    __device__ static C chain_from_words(const uint64_t* w) { return chain_from_bits(w[0]); }
    __device__ static S shfl(S s, uint32_t src) { return shfl_any(s, src); }
    __device__ static S shfl_up(S s, uint32_t d) { return shfl_up_any(s, d); }
    __device__ static C chain_shfl_xor(C c, uint32_t m) { return __shfl_xor_sync(0xFFFFFFFFu, c, m); }
};
using OpU32 = OpInt<uint32_t>;
using OpU64 = OpInt<uint64_t>;

// ------------------------------------------------------------ plain FP32
// Left-to-right float additions inside a thread, float shuffle and block
// trees, float carried between units: the uncompensated baseline.
struct OpF32 {
    using T = float;
    using S = float;
    using C = float;
    static constexpr bool kPackedRowSum = false;
    __device__ static S zero() { return 0.0f; }
    __device__ static S lift(T x) { return x; }
    __device__ static S add(S a, S b) { return a + b; }
    __device__ static S acc(S a, T x) { return a + x; }
    __device__ static S combine(S a, S b) { return a + b; }
    __device__ static S norm(S a) { return a; }
    __device__ static T out(S s) { return s; }
    __device__ static C to_chain(S s) { return s; }
    __device__ static S from_chain(C c) { return c; }
    __device__ static C chain_zero() { return 0.0f; }
    __device__ static C chain_add(C a, C b) { return a + b; }
    __device__ static uint64_t chain_bits(C c) { return __float_as_uint(c); }
    __device__ static C chain_from_bits(uint64_t b) { return __uint_as_float(static_cast<uint32_t>(b)); }
    static constexpr int kDescWords = 1;
    __device__ static uint64_t chain_word(C c, int) { return chain_bits(c); }
    __device__ static C chain_from_words(const uint64_t* w) { return chain_from_bits(w[0]); }
    __device__ static S shfl(S s, uint32_t src) { return shfl_any(s, src); }
    __device__ static S shfl_up(S s, uint32_t d) { return shfl_up_any(s, d); }
    __device__ static C chain_shfl_xor(C c, uint32_t m) { return __shfl_xor_sync(0xFFFFFFFFu, c, m); }
};

// ------------------------------------------------------ compensated FP32
// Double-float state: hi carries the rounded sum, lo the rounding error of
// everything added so far. Combining two states is Knuth's TwoSum on the high
// parts (exact for operands of any magnitude order), the low parts are added
// to the error, and Fast2Sum renormalises the pair (Dekker 1971; Knuth, TAOCP
// vol. 2, 4.2.2). Adding one input to a state (acc) is TwoSum without the
// renormalisation: the only dependency from one item to the next is then a
// single FP32 add on hi and one on lo, and norm() renormalises with TwoSum
// once per thread. combine() merges two states the same lazy way (used by
// the warp, block and chunk scans, whose chains are then one FP32 add deep per
// step); lo stays within a few units in the last place of hi, and hi + lo is
// exact in FP64 and rounds once to the FP32 output. Bulk arithmetic stays in
// FP32; only the value carried from one lookback unit to the next is FP64.
struct F2 {
    float hi, lo;
};

// Two FP32 lanes in one 64-bit register for the packed add.rn.f32x2 /
// sub.rn.f32x2 instructions (two IEEE round-to-nearest operations each).
__device__ __forceinline__ uint64_t f2_pack(float a, float b) {
    uint64_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ void f2_unpack(uint64_t d, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(d));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

struct OpF32C {
    using T = float;
    using S = F2;
    using C = double;
    // The reduce pass sums a row as two half-chains (even and odd items) in
    // packed FP32x2 TwoSums: half the instructions of one chain.
    static constexpr bool kPackedRowSum = true;
    __device__ static S zero() { return F2{0.0f, 0.0f}; }
    __device__ static S lift(T x) { return F2{x, 0.0f}; }
    __device__ static S add(S a, S b) {
        const float s = a.hi + b.hi;
        const float bb = s - a.hi;
        float e = (a.hi - (s - bb)) + (b.hi - bb);
        e += a.lo + b.lo;
        const float hi = s + e;
        const float lo = e - (hi - s);
        return F2{hi, lo};
    }
    __device__ static S acc(S a, T x) {
        const float s = a.hi + x;
        const float bb = s - a.hi;
        const float e = (a.hi - (s - bb)) + (x - bb);
        return F2{s, a.lo + e};
    }
    __device__ static S combine(S a, S b) {
        const float s = a.hi + b.hi;
        const float bb = s - a.hi;
        const float e = (a.hi - (s - bb)) + (b.hi - bb);
        return F2{s, a.lo + (b.lo + e)};
    }
    __device__ static S norm(S a) {
        const float s = a.hi + a.lo;
        const float bb = s - a.hi;
        return F2{s, (a.hi - (s - bb)) + (a.lo - bb)};
    }
    __device__ static T out(S s) { return s.hi + s.lo; }
    // Aggregate of N items (N even) without segment heads: TwoSum on the
    // pairs (even item, odd item) of two independent chains at once, the
    // errors of each chain summed lazily, then the two chains combined.
    template <int N>
    __device__ static S row_sum(const float (&v)[N]) {
        static_assert(N % 2 == 0, "pairs of items");
        uint64_t hi = f2_pack(0.0f, 0.0f), lo = hi;
#pragma unroll
        for (int m = 0; m < N / 2; ++m) {
            const uint64_t x = f2_pack(v[2 * m], v[2 * m + 1]);
            const uint64_t s = f2_add(hi, x);
            const uint64_t bb = f2_sub(s, hi);
            const uint64_t e = f2_add(f2_sub(hi, f2_sub(s, bb)), f2_sub(x, bb));
            lo = f2_add(lo, e);
            hi = s;
        }
        F2 a, b;
        f2_unpack(hi, a.hi, b.hi);
        f2_unpack(lo, a.lo, b.lo);
        return norm(combine(a, b));
    }
    __device__ static C to_chain(S s) { return static_cast<double>(s.hi) + static_cast<double>(s.lo); }
    __device__ static S from_chain(C c) {
        const float hi = static_cast<float>(c);
        const float lo = static_cast<float>(c - static_cast<double>(hi));
        return F2{hi, lo};
    }
    __device__ static C chain_zero() { return 0.0; }
    __device__ static C chain_add(C a, C b) { return a + b; }
    __device__ static uint64_t chain_bits(C c) { return static_cast<uint64_t>(__double_as_longlong(c)); }
    __device__ static C chain_from_bits(uint64_t b) { return __longlong_as_double(static_cast<long long>(b)); }
    static constexpr int kDescWords = 1;
    __device__ static uint64_t chain_word(C c, int) { return chain_bits(c); }
    __device__ static C chain_from_words(const uint64_t* w) { return chain_from_bits(w[0]); }
    __device__ static S shfl(S s, uint32_t src) {
        return F2{__shfl_sync(0xFFFFFFFFu, s.hi, src), __shfl_sync(0xFFFFFFFFu, s.lo, src)};
    }
    __device__ static S shfl_up(S s, uint32_t d) {
        return F2{__shfl_up_sync(0xFFFFFFFFu, s.hi, d), __shfl_up_sync(0xFFFFFFFFu, s.lo, d)};
    }
    __device__ static C chain_shfl_xor(C c, uint32_t m) { return __shfl_xor_sync(0xFFFFFFFFu, c, m); }
};

// ------------------------------------------------ four u32 members (struct)
// Elements of four independent u32 members, each scanned on its own (wrapping
// mod 2^32): a struct scan of vec4<u32>, as the reference's WebGPU struct
// variant scans four members with per-member descriptors
// (GPUPrefixSumsWebGPUapis/SharedShaders/csdldf_struct.wgsl:19,144-300). The
// 128-bit chain value takes two descriptor words.
struct OpU32x4 {
    using T = uint4;
    using S = uint4;
    using C = uint4;
    static constexpr bool kPackedRowSum = false;
    static constexpr int kDescWords = 2;
    __device__ static S zero() { return make_uint4(0u, 0u, 0u, 0u); }
    __device__ static S lift(T x) { return x; }
    __device__ static S add(S a, S b) { return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
    __device__ static S acc(S a, T x) { return add(a, x); }
    __device__ static S combine(S a, S b) { return add(a, b); }
    __device__ static S norm(S a) { return a; }
    __device__ static T out(S s) { return s; }
    __device__ static C to_chain(S s) { return s; }
    __device__ static S from_chain(C c) { return c; }
    __device__ static C chain_zero() { return zero(); }
    __device__ static C chain_add(C a, C b) { return add(a, b); }
    __device__ static uint64_t chain_word(C c, int w) {
        return w == 0 ? (static_cast<uint64_t>(c.y) << 32) | c.x : (static_cast<uint64_t>(c.w) << 32) | c.z;
    }
    __device__ static C chain_from_words(const uint64_t* w) {
        return make_uint4(static_cast<uint32_t>(w[0]), static_cast<uint32_t>(w[0] >> 32), static_cast<uint32_t>(w[1]),
                          static_cast<uint32_t>(w[1] >> 32));
    }
    __device__ static S shfl(S s, uint32_t src) {
        return make_uint4(__shfl_sync(0xFFFFFFFFu, s.x, src), __shfl_sync(0xFFFFFFFFu, s.y, src),
                          __shfl_sync(0xFFFFFFFFu, s.z, src), __shfl_sync(0xFFFFFFFFu, s.w, src));
    }
    __device__ static S shfl_up(S s, uint32_t d) {
        return make_uint4(__shfl_up_sync(0xFFFFFFFFu, s.x, d), __shfl_up_sync(0xFFFFFFFFu, s.y, d),
                          __shfl_up_sync(0xFFFFFFFFu, s.z, d), __shfl_up_sync(0xFFFFFFFFu, s.w, d));
    }
    __device__ static C chain_shfl_xor(C c, uint32_t m) {
        return make_uint4(__shfl_xor_sync(0xFFFFFFFFu, c.x, m), __shfl_xor_sync(0xFFFFFFFFu, c.y, m),
                          __shfl_xor_sync(0xFFFFFFFFu, c.z, m), __shfl_xor_sync(0xFFFFFFFFu, c.w, m));
    }
};

}  // namespace gps
