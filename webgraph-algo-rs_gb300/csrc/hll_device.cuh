// Device-side HyperLogLog arithmetic for sm_103a.
//
// Counter layout is the reference's (src/utils/slice_counter_array.rs:166-169
// with hyper_log_log_logic.rs:72-115): counter i occupies bytes
// [i*B, (i+1)*B), B = 2^log2m * 5 / 8, 5-bit registers packed LSB-first into
// little-endian words. Register width is always 5: register_size(n) =
// max(5, ceil(ln(log2(n)/ln 2))) exceeds 5 only for log2(n) > 102.
//
// GPU restructuring: a counter is split into register-aligned chunks of at
// most 64 registers (320 bits = 40 bytes). The reference's broadword max
// (hyper_log_log_logic.rs:469-576) never carries, borrows or shifts across a
// register boundary, and 320 is a multiple of both 5 and 32, so each chunk is
// merged independently by one lane, on ten 32-bit words, with the very same
// formula:
//     z    = ((((y | H) - (x & ~H)) | (y ^ x)) ^ (y | ~x)) & H
//     mask = ((((z >> 4) | H) - L) | H) ^ z
//     x    = x ^ ((x ^ y) & mask)
// (H / L: highest / lowest bit of every register), the multi-word
// subtractions running as one PTX borrow chain.
//
// count() (hyper_log_log_logic.rs:169-186) is computed exactly: the harmonic
// sum of 2^-v over <= 2^12 registers is a multiple of 2^-31 below 2^13, so it
// is accumulated as the integer sum of 2^(31-v) and scaled by 2^-31 without
// rounding; Rust's `(1 << 31) as f64` on an i32 literal gives -2^31, so a
// register holding 31 contributes -1 instead of +1 (the "i32 quirk").
// alpha*m^2 / hm is one IEEE division; m*ln(m/z) comes from a host table
// evaluated with the platform libm as Rust's f64::ln does.
#pragma once

#include <cstdint>

namespace hbd {

template <int LOG2M>
struct Geo {
    static constexpr int M = 1 << LOG2M;
    static constexpr int CHUNK_REGS = M < 64 ? M : 64;
    static constexpr int CHUNKS = M / CHUNK_REGS;               // chunks per counter
    static constexpr int NW = (CHUNK_REGS * 5 + 31) / 32;       // 32-bit words per chunk
    static constexpr int COUNTER_BYTES = M * 5 / 8;
    static constexpr int CHUNK_BYTES = CHUNK_REGS * 5 / 8;      // 10, 20 or 40
};

// Word i of the mask with bit `bit` of each of `regs` 5-bit registers set.
__host__ __device__ constexpr uint32_t mask_word(int regs, int i, int bit) {
    uint32_t w = 0;
    for (int k = 0; k < regs; k++) {
        int p = 5 * k + bit;
        if (p >= 32 * i && p < 32 * i + 32) w |= 1u << (p - 32 * i);
    }
    return w;
}

// ---------------------------------------------------------------------------
// multi-word subtraction r = a - b (little-endian words) as one borrow chain
// ---------------------------------------------------------------------------
template <int NW>
struct SubChain;

template <>
struct SubChain<3> {
    static __device__ __forceinline__ void run(uint32_t (&r)[3], const uint32_t (&a)[3],
                                               const uint32_t (&b)[3]) {
        asm("sub.cc.u32 %0, %3, %6;\n\t"
            "subc.cc.u32 %1, %4, %7;\n\t"
            "subc.u32 %2, %5, %8;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(b[0]), "r"(b[1]), "r"(b[2]));
    }
};

template <>
struct SubChain<5> {
    static __device__ __forceinline__ void run(uint32_t (&r)[5], const uint32_t (&a)[5],
                                               const uint32_t (&b)[5]) {
        asm("sub.cc.u32 %0, %5, %10;\n\t"
            "subc.cc.u32 %1, %6, %11;\n\t"
            "subc.cc.u32 %2, %7, %12;\n\t"
            "subc.cc.u32 %3, %8, %13;\n\t"
            "subc.u32 %4, %9, %14;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(b[0]), "r"(b[1]),
              "r"(b[2]), "r"(b[3]), "r"(b[4]));
    }
};

template <>
struct SubChain<10> {
    static __device__ __forceinline__ void run(uint32_t (&r)[10], const uint32_t (&a)[10],
                                               const uint32_t (&b)[10]) {
        asm("sub.cc.u32 %0, %10, %20;\n\t"
            "subc.cc.u32 %1, %11, %21;\n\t"
            "subc.cc.u32 %2, %12, %22;\n\t"
            "subc.cc.u32 %3, %13, %23;\n\t"
            "subc.cc.u32 %4, %14, %24;\n\t"
            "subc.cc.u32 %5, %15, %25;\n\t"
            "subc.cc.u32 %6, %16, %26;\n\t"
            "subc.cc.u32 %7, %17, %27;\n\t"
            "subc.cc.u32 %8, %18, %28;\n\t"
            "subc.u32 %9, %19, %29;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]),
              "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]),
              "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]));
    }
};

// x = register-wise max(x, y) over one chunk of REGS registers; ORs into
// `grew` the bits of x that took y's value and changed.
template <int REGS>
__device__ __forceinline__ void merge_chunk(uint32_t (&x)[(REGS * 5 + 31) / 32],
                                            const uint32_t (&y)[(REGS * 5 + 31) / 32],
                                            uint32_t& grew) {
    constexpr int NW = (REGS * 5 + 31) / 32;
    uint32_t a[NW], b[NW], z[NW];
#pragma unroll
    for (int i = 0; i < NW; i++) {
        const uint32_t H = mask_word(REGS, i, 4);
        a[i] = y[i] | H;
        b[i] = x[i] & ~H;
    }
    SubChain<NW>::run(z, a, b);
#pragma unroll
    for (int i = 0; i < NW; i++) {
        const uint32_t H = mask_word(REGS, i, 4);
        z[i] = ((z[i] | (y[i] ^ x[i])) ^ (y[i] | ~x[i])) & H;
    }
    uint32_t t[NW], l[NW], mk[NW];
#pragma unroll
    for (int i = 0; i < NW; i++) {
        const uint32_t H = mask_word(REGS, i, 4);
        const uint32_t sh = (i + 1 < NW) ? __funnelshift_r(z[i], z[i + 1 < NW ? i + 1 : i], 4)
                                         : (z[i] >> 4);
        t[i] = sh | H;
        l[i] = mask_word(REGS, i, 0);
    }
    SubChain<NW>::run(mk, t, l);
#pragma unroll
    for (int i = 0; i < NW; i++) {
        const uint32_t H = mask_word(REGS, i, 4);
        const uint32_t m = (mk[i] | H) ^ z[i];
        const uint32_t d = (x[i] ^ y[i]) & m;
        grew |= d;
        x[i] = x[i] ^ d;
    }
}

template <int REGS>
__device__ __forceinline__ void merge_chunk(uint32_t (&x)[(REGS * 5 + 31) / 32],
                                            const uint32_t (&y)[(REGS * 5 + 31) / 32]) {
    uint32_t unused = 0;
    merge_chunk<REGS>(x, y, unused);
}

template <int NW>
struct AddChain;
template <>
struct AddChain<3> {
    static __device__ __forceinline__ void run(uint32_t (&r)[3], const uint32_t (&a)[3],
                                               const uint32_t (&b)[3]) {
        asm("add.cc.u32 %0, %3, %6;\n\t"
            "addc.cc.u32 %1, %4, %7;\n\t"
            "addc.u32 %2, %5, %8;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(b[0]), "r"(b[1]), "r"(b[2]));
    }
};
template <>
struct AddChain<5> {
    static __device__ __forceinline__ void run(uint32_t (&r)[5], const uint32_t (&a)[5],
                                               const uint32_t (&b)[5]) {
        asm("add.cc.u32 %0, %5, %10;\n\t"
            "addc.cc.u32 %1, %6, %11;\n\t"
            "addc.cc.u32 %2, %7, %12;\n\t"
            "addc.cc.u32 %3, %8, %13;\n\t"
            "addc.u32 %4, %9, %14;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(b[0]), "r"(b[1]),
              "r"(b[2]), "r"(b[3]), "r"(b[4]));
    }
};
template <>
struct AddChain<10> {
    static __device__ __forceinline__ void run(uint32_t (&r)[10], const uint32_t (&a)[10],
                                               const uint32_t (&b)[10]) {
        asm("add.cc.u32 %0, %10, %20;\n\t"
            "addc.cc.u32 %1, %11, %21;\n\t"
            "addc.cc.u32 %2, %12, %22;\n\t"
            "addc.cc.u32 %3, %13, %23;\n\t"
            "addc.cc.u32 %4, %14, %24;\n\t"
            "addc.cc.u32 %5, %15, %25;\n\t"
            "addc.cc.u32 %6, %16, %26;\n\t"
            "addc.cc.u32 %7, %17, %27;\n\t"
            "addc.cc.u32 %8, %18, %28;\n\t"
            "addc.u32 %9, %19, %29;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]),
              "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]),
              "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]));
    }
};

// Partial count of one chunk: hsum += sum over registers of 2^(31-v),
// zeroes += #(v == 0), and, only when `with31`, c31 += #(v == 31).
//  * 2^(31-v): funnel-shifting 0x80000000 right by the raw extracted field
//    uses the shift amount mod 32, so the unmasked field gives the term in
//    one instruction.
//  * zero registers, broadword: ((x & ~H) + low4) | x has bit 4 of a
//    register set iff the register is non-zero (low4 = bits 0-3 of every
//    register; the add never carries out of a register).
template <int REGS>
__device__ __forceinline__ void count_chunk(const uint32_t (&w)[(REGS * 5 + 31) / 32],
                                            uint64_t& hsum, uint32_t& zeroes, uint32_t& c31,
                                            bool with31) {
    constexpr int NW = (REGS * 5 + 31) / 32;
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int k = 0; k < REGS; k++) {
        const int p = 5 * k;
        const int i = p / 32, s = p % 32;
        const uint32_t raw =
            (s + 5 <= 32) ? (w[i] >> s) : __funnelshift_r(w[i], w[(i + 1) < NW ? i + 1 : i], s);
        const uint32_t term = __funnelshift_r(0x80000000u, 0u, raw);
        asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, 0;" : "+r"(lo), "+r"(hi) : "r"(term));
    }
    hsum += ((uint64_t)hi << 32) | lo;
    uint32_t t[NW], low4[NW], sum[NW];
#pragma unroll
    for (int i = 0; i < NW; i++) {
        const uint32_t H = mask_word(REGS, i, 4);
        low4[i] = mask_word(REGS, i, 0) | mask_word(REGS, i, 1) | mask_word(REGS, i, 2) |
                  mask_word(REGS, i, 3);
        t[i] = w[i] & ~H;
    }
    AddChain<NW>::run(sum, t, low4);
    uint32_t nz = 0;
#pragma unroll
    for (int i = 0; i < NW; i++) nz += __popc((sum[i] | w[i]) & mask_word(REGS, i, 4));
    zeroes += (uint32_t)REGS - nz;
    if (with31) {
#pragma unroll
        for (int k = 0; k < REGS; k++) {
            const int p = 5 * k;
            const int i = p / 32, s = p % 32;
            const uint32_t raw = (s + 5 <= 32) ? (w[i] >> s)
                                               : __funnelshift_r(w[i], w[(i + 1) < NW ? i + 1 : i], s);
            c31 += ((raw & 31u) == 31u);
        }
    }
}

// HLL:181-185 from the exact integer harmonic sum (reference arithmetic, f64
// pipe). Used where counts are rare (init, weighted init).
__device__ __forceinline__ double estimate(int64_t hsum, uint32_t zeroes, double alpha_m_m,
                                           double m, const double* __restrict__ ln_table) {
    const double hm = (double)hsum * 0x1p-31;
    double e = __ddiv_rn(alpha_m_m, hm);
    if (zeroes != 0u && e < 2.5 * m) e = __ldg(ln_table + zeroes);
    return e;
}

// |x| < 2^53 converted to double by bit assembly (exact; no f64 instruction).
__device__ __forceinline__ double exact_u64_to_double(uint64_t u) {
    if (u == 0) return 0.0;
    const int lz = __clzll((long long)u);
    const uint64_t e = (uint64_t)(63 - lz + 1023);
    const uint64_t mant = (u << lz) >> 11;  // 53 bits, leading one at bit 52
    return __longlong_as_double((long long)((e << 52) | (mant & ((1ull << 52) - 1))));
}

// The same estimate with one f64 instruction (the division) on the hot path:
//   alpha*m^2 / (H * 2^-31) == (alpha*m^2*2^31) / H exactly (power-of-two
//   scaling), so a_scaled = alpha*m^2*2^31 is precomputed; H > 0 converts
//   exactly; `e < 2.5m` between positive finite doubles is an integer compare
//   of their bit patterns. H <= 0 (only reachable through the i32 quirk)
//   takes the reference arithmetic.
__device__ __forceinline__ double estimate_fast(int64_t hsum, uint32_t zeroes, double alpha_m_m,
                                                double a_scaled, long long small_bits, double m,
                                                const double* __restrict__ ln_table) {
    if (hsum <= 0) return estimate(hsum, zeroes, alpha_m_m, m, ln_table);
    const double e = __ddiv_rn(a_scaled, exact_u64_to_double((uint64_t)hsum));
    if (zeroes != 0u && __double_as_longlong(e) < small_bits) return __ldg(ln_table + zeroes);
    return e;
}

// delta / d correctly rounded, for a positive integer-valued d with
// rd = RN(1/d): q0 = RN(delta*rd), r = delta - d*q0 (exact by fma),
// q1 = RN(q0 + r*rd). Markstein's correction step (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990); checked against true division in the tests.
__device__ __forceinline__ double div_by_small_int(double delta, double d, double rd) {
    const double q0 = __dmul_rn(delta, rd);
    const double r = __fma_rn(-q0, d, delta);
    return __fma_rn(r, rd, q0);
}

__device__ __forceinline__ int64_t signed_hsum(uint64_t hsum, uint32_t c31, int quirk) {
    return quirk ? (int64_t)hsum - 2 * (int64_t)c31 : (int64_t)hsum;
}

// ---------------------------------------------------------------------------
// chunk load / store
// ---------------------------------------------------------------------------
template <int LOG2M>
__device__ __forceinline__ void load_chunk(const uint8_t* __restrict__ base, uint64_t node, int c,
                                           uint32_t (&w)[Geo<LOG2M>::NW]) {
    using G = Geo<LOG2M>;
    const uint8_t* p = base + node * (uint64_t)G::COUNTER_BYTES + (uint64_t)c * G::CHUNK_BYTES;
    if constexpr (G::CHUNK_BYTES == 40) {
        const uint2* q = reinterpret_cast<const uint2*>(p);
#pragma unroll
        for (int i = 0; i < 5; i++) {
            const uint2 t = __ldg(q + i);
            w[2 * i] = t.x;
            w[2 * i + 1] = t.y;
        }
    } else if constexpr (G::CHUNK_BYTES == 20) {
        const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
        for (int i = 0; i < 5; i++) w[i] = __ldg(q + i);
    } else {
        const uint16_t* q = reinterpret_cast<const uint16_t*>(p);
        const uint32_t h0 = __ldg(q), h1 = __ldg(q + 1), h2 = __ldg(q + 2), h3 = __ldg(q + 3),
                       h4 = __ldg(q + 4);
        w[0] = h0 | (h1 << 16);
        w[1] = h2 | (h3 << 16);
        w[2] = h4;
    }
}

template <int LOG2M>
__device__ __forceinline__ void store_chunk(uint8_t* __restrict__ base, uint64_t node, int c,
                                            const uint32_t (&w)[Geo<LOG2M>::NW]) {
    using G = Geo<LOG2M>;
    uint8_t* p = base + node * (uint64_t)G::COUNTER_BYTES + (uint64_t)c * G::CHUNK_BYTES;
    if constexpr (G::CHUNK_BYTES == 40) {
        uint2* q = reinterpret_cast<uint2*>(p);
#pragma unroll
        for (int i = 0; i < 5; i++) q[i] = make_uint2(w[2 * i], w[2 * i + 1]);
    } else if constexpr (G::CHUNK_BYTES == 20) {
        uint32_t* q = reinterpret_cast<uint32_t*>(p);
#pragma unroll
        for (int i = 0; i < 5; i++) q[i] = w[i];
    } else {
        uint16_t* q = reinterpret_cast<uint16_t*>(p);
        q[0] = (uint16_t)w[0];
        q[1] = (uint16_t)(w[0] >> 16);
        q[2] = (uint16_t)w[1];
        q[3] = (uint16_t)(w[1] >> 16);
        q[4] = (uint16_t)w[2];
    }
}

// ---------------------------------------------------------------------------
// node hashers (see the oracle for the parity status of each)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t rotl64(uint64_t x, int b) { return (x << b) | (x >> (64 - b)); }

__device__ __forceinline__ void sip_round(uint64_t& v0, uint64_t& v1, uint64_t& v2, uint64_t& v3) {
    v0 += v1; v1 = rotl64(v1, 13); v1 ^= v0; v0 = rotl64(v0, 32);
    v2 += v3; v3 = rotl64(v3, 16); v3 ^= v2;
    v0 += v3; v3 = rotl64(v3, 21); v3 ^= v0;
    v2 += v1; v1 = rotl64(v1, 17); v1 ^= v2; v2 = rotl64(v2, 32);
}

// SipHash-1-3, keys (0,0), over the 8 little-endian bytes of x.
__device__ __forceinline__ uint64_t hash_sip13(uint64_t x) {
    uint64_t v0 = 0x736f6d6570736575ull, v1 = 0x646f72616e646f6dull;
    uint64_t v2 = 0x6c7967656e657261ull, v3 = 0x7465646279746573ull;
    v3 ^= x;
    sip_round(v0, v1, v2, v3);
    v0 ^= x;
    const uint64_t b = 8ull << 56;
    v3 ^= b;
    sip_round(v0, v1, v2, v3);
    v0 ^= b;
    v2 ^= 0xff;
    sip_round(v0, v1, v2, v3);
    sip_round(v0, v1, v2, v3);
    sip_round(v0, v1, v2, v3);
    return v0 ^ v1 ^ v2 ^ v3;
}

__device__ __forceinline__ uint64_t hash_jenkins(uint64_t x, uint64_t seed) {
    uint64_t a = seed, b = seed, c = 0x9e3779b97f4a7c13ull;
    a += x;
    a -= b; a -= c; a ^= (c >> 43);
    b -= c; b -= a; b ^= (a << 9);
    c -= a; c -= b; c ^= (b >> 8);
    a -= b; a -= c; a ^= (c >> 38);
    b -= c; b -= a; b ^= (a << 23);
    c -= a; c -= b; c ^= (b >> 5);
    a -= b; a -= c; a ^= (c >> 35);
    b -= c; b -= a; b ^= (a << 49);
    c -= a; c -= b; c ^= (b >> 11);
    a -= b; a -= c; a ^= (c >> 12);
    b -= c; b -= a; b ^= (a << 18);
    c -= a; c -= b; c ^= (b >> 22);
    return c;
}

__device__ __forceinline__ bool test_bit(const uint32_t* __restrict__ bits, uint64_t i) {
    return (__ldg(bits + (i >> 5)) >> (i & 31)) & 1u;
}

}  // namespace hbd
