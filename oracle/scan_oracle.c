/*
 * scan_oracle.c -- CPU oracle for the GB300 prefix-scan library.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: the tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it; the library never
 * does. It restates, in plain C, what the reference computes:
 *
 *   - the serial validation scan, GPUPrefixSumsD3D12/Shaders/Utility.hlsl:99-125
 *     (ValidateRandomInclusive / ValidateRandomExclusive): one running sum over
 *     the input, compared after (inclusive) or before (exclusive) adding
 *     element i, with uint wraparound;
 *   - the known-answer checks of the CUDA harness,
 *     GPUPrefixSumsCUDA/UtilityKernels.cuh:15-38 (InitOne, ValidateInclusive
 *     expects i + 1, ValidateExclusive expects i);
 *   - the seeded input generator of the D3D12 harness,
 *     GPUPrefixSumsD3D12/Shaders/Utility.hlsl:37-66 (InitRandom, a hybrid
 *     Tausworthe generator after GPU Gems 3 ch. 37, values & 1023).
 *
 * It adds what the reference does not have but the tests need: a u64 scan, a
 * segmented scan over CSR offsets, a multi-threaded three-phase CPU scan (the
 * timed CPU baseline; same results as the serial loop), and an exact FP32
 * prefix sum rounded once to double (a fixed-point superaccumulator), used as
 * the FP64 oracle for error measurement.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ----------------------------------------------------------- serial scans */

/* Utility.hlsl:99-125 restated: sum += x[i] with the compare placed after
 * (inclusive) or before (exclusive) the add. */
void oracle_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, int inclusive) {
    uint32_t sum = 0;
    if (inclusive) {
        for (uint64_t i = 0; i < n; ++i) {
            sum += in[i];
            out[i] = sum;
        }
    } else {
        for (uint64_t i = 0; i < n; ++i) {
            const uint32_t x = in[i];
            out[i] = sum;
            sum += x;
        }
    }
}

void oracle_scan_u64(const uint64_t* in, uint64_t* out, uint64_t n, int inclusive) {
    uint64_t sum = 0;
    if (inclusive) {
        for (uint64_t i = 0; i < n; ++i) {
            sum += in[i];
            out[i] = sum;
        }
    } else {
        for (uint64_t i = 0; i < n; ++i) {
            const uint64_t x = in[i];
            out[i] = sum;
            sum += x;
        }
    }
}

/* Mismatch count between `scan` and the serial scan of `in`, exactly as the
 * reference's serial validator counts errors (Utility.hlsl:101-125). */
uint64_t oracle_validate_u32(const uint32_t* in, const uint32_t* scan, uint64_t n, int inclusive) {
    uint32_t sum = 0;
    uint64_t errors = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (inclusive) {
            sum += in[i];
            errors += scan[i] != sum;
        } else {
            errors += scan[i] != sum;
            sum += in[i];
        }
    }
    return errors;
}

uint64_t oracle_validate_u64(const uint64_t* in, const uint64_t* scan, uint64_t n, int inclusive) {
    uint64_t sum = 0;
    uint64_t errors = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (inclusive) {
            sum += in[i];
            errors += scan[i] != sum;
        } else {
            errors += scan[i] != sum;
            sum += in[i];
        }
    }
    return errors;
}

/* Known-answer check of UtilityKernels.cuh:22-38 for all-ones input:
 * inclusive expects i + 1, exclusive expects i (mod 2^32). */
uint64_t oracle_validate_ones_u32(const uint32_t* scan, uint64_t n, int inclusive) {
    uint64_t errors = 0;
    for (uint64_t i = 0; i < n; ++i) errors += scan[i] != (uint32_t)(inclusive ? i + 1 : i);
    return errors;
}

/* InitOne, UtilityKernels.cuh:15-20. */
void oracle_init_one_u32(uint32_t* out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) out[i] = 1;
}

/* InitRandom of the D3D12 harness, Utility.hlsl:37-66: each of the 65536
 * generator threads (256 groups x 256 threads) seeds four states from its id
 * and the seed, takes one Tausworthe/LCG step, and writes the same value
 * (combined states & 1023) to every index it strides over. */
void oracle_init_random_taus(uint32_t* out, uint64_t n, uint32_t seed) {
    const uint64_t stride = 256u * 256u;
    for (uint64_t id = 0; id < stride && id < n; ++id) {
        uint32_t z1 = (uint32_t)(id << 2) * seed;
        uint32_t z2 = ((uint32_t)(id << 2) + 1u) * seed;
        uint32_t z3 = ((uint32_t)(id << 2) + 2u) * seed;
        uint32_t z4 = ((uint32_t)(id << 2) + 3u) * seed;
        z1 = ((z1 & 4294967294u) << 12) ^ (((z1 << 13) ^ z1) >> 19);
        z2 = ((z2 & 4294967288u) << 4) ^ (((z2 << 2) ^ z2) >> 25);
        z3 = ((z3 & 4294967280u) << 17) ^ (((z3 << 3) ^ z3) >> 11);
        z4 = z4 * 1664525u + 1013904223u;
        const uint32_t t = (z1 ^ z2 ^ z3 ^ z4) & 1023u;
        for (uint64_t i = id; i < n; i += stride) out[i] = t;
    }
}

/* ------------------------------------------------------- segmented scans */

/* Independent scans of the segments [offsets[s], offsets[s+1]). */
void oracle_segscan_u32(const uint32_t* in, uint32_t* out, const uint64_t* offsets, uint64_t num_segments,
                        int inclusive) {
    for (uint64_t s = 0; s < num_segments; ++s) {
        const uint64_t b = offsets[s], e = offsets[s + 1];
        oracle_scan_u32(in + b, out + b, e - b, inclusive);
    }
}

void oracle_segscan_u64(const uint64_t* in, uint64_t* out, const uint64_t* offsets, uint64_t num_segments,
                        int inclusive) {
    for (uint64_t s = 0; s < num_segments; ++s) {
        const uint64_t b = offsets[s], e = offsets[s + 1];
        oracle_scan_u64(in + b, out + b, e - b, inclusive);
    }
}

/* ------------------------------------------- multi-threaded CPU baseline */

typedef struct {
    const uint32_t* in;
    uint32_t* out;
    uint64_t begin, end;
    uint32_t sum;
    uint32_t offset;
    int inclusive;
    int phase;
} mt_job;

static void* mt_worker(void* arg) {
    mt_job* j = (mt_job*)arg;
    if (j->phase == 0) {
        uint32_t s = 0;
        for (uint64_t i = j->begin; i < j->end; ++i) s += j->in[i];
        j->sum = s;
    } else {
        uint32_t sum = j->offset;
        if (j->inclusive) {
            for (uint64_t i = j->begin; i < j->end; ++i) {
                sum += j->in[i];
                j->out[i] = sum;
            }
        } else {
            for (uint64_t i = j->begin; i < j->end; ++i) {
                const uint32_t x = j->in[i];
                j->out[i] = sum;
                sum += x;
            }
        }
    }
    return NULL;
}

/* Reduce-then-scan on host threads: per-thread chunk sums, a serial scan of
 * those sums, then per-thread scans with their offsets. Same result as
 * oracle_scan_u32. Returns 0 on success. */
int oracle_scan_u32_mt(const uint32_t* in, uint32_t* out, uint64_t n, int inclusive, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if ((uint64_t)threads > n) threads = n ? (int)n : 1;
    mt_job jobs[256];
    pthread_t tids[256];
    const uint64_t per = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        jobs[t].in = in;
        jobs[t].out = out;
        jobs[t].begin = (uint64_t)t * per < n ? (uint64_t)t * per : n;
        jobs[t].end = (uint64_t)(t + 1) * per < n ? (uint64_t)(t + 1) * per : n;
        jobs[t].inclusive = inclusive;
        jobs[t].phase = 0;
    }
    for (int phase = 0; phase < 2; ++phase) {
        for (int t = 0; t < threads; ++t) {
            jobs[t].phase = phase;
            if (pthread_create(&tids[t], NULL, mt_worker, &jobs[t]) != 0) return -1;
        }
        for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
        if (phase == 0) {
            uint32_t run = 0;
            for (int t = 0; t < threads; ++t) {
                jobs[t].offset = run;
                run += jobs[t].sum;
            }
        }
    }
    return 0;
}

/* ------------------------------------------ exact FP32 prefix -> double */

/* Fixed point with the least significant bit at 2^-149 (the smallest FP32
 * subnormal), 384-bit two's complement: every FP32 value and every sum of up
 * to 2^100 of them is exact. */
#define ACC_LIMBS 6
typedef struct {
    uint64_t w[ACC_LIMBS];
} superacc;

static void acc_add_shifted(superacc* a, uint32_t m, int shift, int negative) {
    const int idx = shift >> 6, bit = shift & 63;
    const unsigned __int128 v = (unsigned __int128)m << bit;
    uint64_t part[2] = {(uint64_t)v, (uint64_t)(v >> 64)};
    if (!negative) {
        unsigned __int128 carry = 0;
        for (int k = idx; k < ACC_LIMBS; ++k) {
            const uint64_t add = (k - idx) < 2 ? part[k - idx] : 0;
            const unsigned __int128 s = (unsigned __int128)a->w[k] + add + carry;
            a->w[k] = (uint64_t)s;
            carry = s >> 64;
            if (k - idx >= 1 && carry == 0) break;
        }
    } else {
        uint64_t borrow = 0;
        for (int k = idx; k < ACC_LIMBS; ++k) {
            const uint64_t sub = (k - idx) < 2 ? part[k - idx] : 0;
            const uint64_t x = a->w[k];
            const uint64_t d1 = x - sub;
            const uint64_t b1 = x < sub;
            const uint64_t d2 = d1 - borrow;
            const uint64_t b2 = d1 < borrow;
            a->w[k] = d2;
            borrow = b1 | b2;
            if (k - idx >= 1 && borrow == 0) break;
        }
    }
}

static void acc_add_float(superacc* a, float f) {
    uint32_t bits;
    memcpy(&bits, &f, sizeof(bits));
    const int negative = (int)(bits >> 31);
    const uint32_t exp = (bits >> 23) & 0xFFu;
    const uint32_t frac = bits & 0x7FFFFFu;
    if (exp == 0xFFu) return; /* inf / nan are not generated by the tests */
    const uint32_t m = exp ? (frac | 0x800000u) : frac;
    if (m == 0) return;
    const int shift = exp ? (int)exp - 1 : 0;
    acc_add_shifted(a, m, shift, negative);
}

/* Round-to-nearest-even conversion of the accumulator to double. */
static double acc_to_double(const superacc* a) {
    superacc m = *a;
    const int negative = (int)(m.w[ACC_LIMBS - 1] >> 63);
    if (negative) { /* two's complement magnitude: invert and add one */
        uint64_t carry = 1;
        for (int k = 0; k < ACC_LIMBS; ++k) {
            const uint64_t x = ~m.w[k];
            const uint64_t s = x + carry;
            carry = s < x;
            m.w[k] = s;
        }
    }
    int top = -1;
    for (int k = ACC_LIMBS - 1; k >= 0; --k) {
        if (m.w[k]) {
            top = k * 64 + 63 - __builtin_clzll(m.w[k]);
            break;
        }
    }
    if (top < 0) return 0.0;
    /* The 64 bits ending at bit `top`, and a sticky bit for all bits below. */
    uint64_t hi64;
    int sticky = 0;
    const int lo_pos = top - 63;
    if (lo_pos <= 0) {
        hi64 = m.w[0] << (-lo_pos);
    } else {
        const int limb = lo_pos >> 6, sh = lo_pos & 63;
        hi64 = m.w[limb] >> sh;
        if (sh && limb + 1 < ACC_LIMBS) hi64 |= m.w[limb + 1] << (64 - sh);
        if (sh && (m.w[limb] & ((1ull << sh) - 1u))) sticky = 1;
        for (int k = 0; k < limb && !sticky; ++k) sticky = m.w[k] != 0;
    }
    uint64_t mant = hi64 >> 11; /* 53 bits, leading one at bit 52 */
    const uint64_t round_bit = (hi64 >> 10) & 1u;
    const int rest = (hi64 & 0x3FFu) != 0 || sticky;
    int e = top;
    if (round_bit && (rest || (mant & 1u))) {
        ++mant;
        if (mant >> 53) {
            mant >>= 1;
            ++e;
        }
    }
    const double r = ldexp((double)mant, e - 52 - 149);
    return negative ? -r : r;
}

/* out[i] = exact in[0] + ... + in[i], rounded once to double. */
void oracle_scan_f32_exact(const float* in, double* out, uint64_t n, int inclusive) {
    superacc a;
    memset(&a, 0, sizeof(a));
    for (uint64_t i = 0; i < n; ++i) {
        if (inclusive) {
            acc_add_float(&a, in[i]);
            out[i] = acc_to_double(&a);
        } else {
            out[i] = acc_to_double(&a);
            acc_add_float(&a, in[i]);
        }
    }
}

/* Plain serial FP32 scan (left-to-right float adds), for reference. */
void oracle_scan_f32_serial(const float* in, float* out, uint64_t n, int inclusive) {
    float sum = 0.0f;
    for (uint64_t i = 0; i < n; ++i) {
        if (inclusive) {
            sum += in[i];
            out[i] = sum;
        } else {
            out[i] = sum;
            sum += in[i];
        }
    }
}

/* Stream compaction: out[j] = the j-th in[i] with flags[i] != 0, by an
 * exclusive scan of the flags done inline (the output index of a selected
 * element is the number of selected elements before it). Returns the count.
 * Element size 4 or 8 bytes. */
uint64_t oracle_select(const void* in, const uint8_t* flags, void* out, uint64_t n, int elem_size) {
    uint64_t j = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (flags[i] != 0) {
            memcpy((uint8_t*)out + j * (uint64_t)elem_size, (const uint8_t*)in + i * (uint64_t)elem_size,
                   (size_t)elem_size);
            ++j;
        }
    }
    return j;
}

int oracle_version(void) { return 1; }
