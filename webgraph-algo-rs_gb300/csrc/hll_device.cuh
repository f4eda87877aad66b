// Device-side HyperLogLog arithmetic for sm_103a.
//
// The reference keeps counter i in bytes [i*B, (i+1)*B), B = 2^log2m * 5 / 8,
// with 5-bit registers packed LSB-first into little-endian words
// (src/utils/slice_counter_array.rs:166-169, hyper_log_log_logic.rs:72-115).
// Register width is always 5: register_size(n) = max(5, ceil(ln(log2(n)/ln 2)))
// exceeds 5 only for log2(n) > 102. That packed form is the interchange
// format (hb_get_registers packs on the device, k_pack_counters).
//
// In HBM a counter holds one register per byte: counter i occupies bytes
// [i*m, (i+1)*m), register j is byte j. A register never exceeds 31
// (trailing zeros of a value with bit 30 set, plus one), so bits 5-7 of every
// byte are zero, and the register-wise max of the reference's broadword merge
// (hyper_log_log_logic.rs:469-576) becomes, per 32-bit word of four registers,
//     t    = x + 0x80808080 - y        bit 7 of a byte set iff x >= y there;
//                                      no borrow leaves a byte (x+128-y > 0)
//     keep = prmt(t, sign-replicate)   0xff where x >= y, else 0x00
//     x    = y ^ ((x ^ y) & keep)
// three integer instructions per four registers, against about fourteen per
// word of the packed broadword form. Counters of 2^log2m bytes are also
// 16-byte aligned (128-bit loads and stores) and, at log2m >= 6, never cross a
// 64-byte boundary, so a counter gather moves exactly its own sectors.
//
// A counter is processed in chunks of at most 64 registers (64 bytes, 16
// words, four 128-bit accesses), one lane per chunk: at log2m <= 6 a whole
// counter is one lane's, so per-arc work (successor id, address, loop) is not
// repeated across lanes.
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
    static constexpr int CHUNKS = M / CHUNK_REGS;            // chunks per counter
    static constexpr int NW = CHUNK_REGS / 4;                // 32-bit words per chunk
    static constexpr int COUNTER_BYTES = M;                  // device stride, one byte per register
    static constexpr int CHUNK_BYTES = CHUNK_REGS;           // 16, 32 or 64
    static constexpr int PACKED_BYTES = M * 5 / 8;           // the reference's counter size
};

// Replicates bit 7 of every byte of t over its byte (PTX prmt, sign mode).
__device__ __forceinline__ uint32_t byte_signs(uint32_t t) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(t), "r"(0u), "r"(0xBA98u));
    return r;
}

// x = register-wise max(x, y) over one chunk of REGS byte registers; ORs into
// `grew` the bits of x that changed.
template <int REGS>
__device__ __forceinline__ void merge_chunk(uint32_t (&x)[REGS / 4], const uint32_t (&y)[REGS / 4],
                                            uint32_t& grew) {
#pragma unroll
    for (int i = 0; i < REGS / 4; i++) {
        // x + 0x80808080 - y == (x | 0x80808080) - y: bit 7 of every byte of x is 0
        const uint32_t keep = byte_signs(x[i] + 0x80808080u - y[i]);
        const uint32_t r = y[i] ^ ((x[i] ^ y[i]) & keep);
        grew |= r ^ x[i];
        x[i] = r;
    }
}

// the same without the change mask: three instructions per word (one
// three-input add, one byte permute, one three-input logic op)
template <int REGS>
__device__ __forceinline__ void merge_chunk(uint32_t (&x)[REGS / 4], const uint32_t (&y)[REGS / 4]) {
#pragma unroll
    for (int i = 0; i < REGS / 4; i++) {
        const uint32_t keep = byte_signs(x[i] + 0x80808080u - y[i]);
        x[i] = y[i] ^ ((x[i] ^ y[i]) & keep);
    }
}

// Number of zero bytes of w (all bytes below 0x80): ((b | 0x80) - 1) keeps
// bit 7 iff b != 0, and never borrows across bytes.
__device__ __forceinline__ uint32_t zero_bytes(uint32_t w) {
    return 4u - __popc(((w | 0x80808080u) - 0x01010101u) & 0x80808080u);
}

// Partial count of one chunk: hsum += sum over registers of 2^(31-v),
// zeroes += #(v == 0), and, only when `with31`, c31 += #(v == 31).
// 2^(31-v): funnel-shifting 0x80000000 right uses the shift amount mod 32, so
// the word shifted right by 8k gives register k's term without masking.
template <int REGS>
__device__ __forceinline__ void count_chunk(const uint32_t (&w)[REGS / 4], uint64_t& hsum,
                                            uint32_t& zeroes, uint32_t& c31, bool with31) {
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int i = 0; i < REGS / 4; i++) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t term = __funnelshift_r(0x80000000u, 0u, w[i] >> (8 * k));
            asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, 0;" : "+r"(lo), "+r"(hi) : "r"(term));
        }
        zeroes += zero_bytes(w[i]);
        if (with31) c31 += zero_bytes(w[i] ^ 0x1f1f1f1fu);
    }
    hsum += ((uint64_t)hi << 32) | lo;
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
//   takes the reference arithmetic. (An all-integer correctly rounded
//   division measured no faster inside the union kernel, whose f64 pipe is
//   about 17% busy.)
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
// 32-byte pieces move as one 256-bit access (sm_100 and later): half the
// load instructions and L1 wavefronts of 128-bit accesses for a divergent
// gather. Chunks of 32 or 64 bytes are 32-byte aligned.
__device__ __forceinline__ void ld_nc_256(const void* p, uint32_t* w) {
    asm("ld.global.nc.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]),
          "=r"(w[7])
        : "l"(p));
}

__device__ __forceinline__ void st_256(void* p, const uint32_t* w) {
    asm volatile("st.global.v8.u32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :
                 : "l"(p), "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]),
                   "r"(w[6]), "r"(w[7])
                 : "memory");
}

template <int LOG2M>
__device__ __forceinline__ void load_chunk(const uint8_t* __restrict__ base, uint64_t node, int c,
                                           uint32_t (&w)[Geo<LOG2M>::NW]) {
    using G = Geo<LOG2M>;
    const uint8_t* p = base + node * (uint64_t)G::COUNTER_BYTES + (uint64_t)c * G::CHUNK_BYTES;
    if constexpr (G::NW >= 8) {
#pragma unroll
        for (int i = 0; i < G::NW / 8; i++) ld_nc_256(p + 32 * i, w + 8 * i);
    } else {
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(p));
        w[0] = t.x;
        w[1] = t.y;
        w[2] = t.z;
        w[3] = t.w;
    }
}

// Requests chunk c of counter `node` into L2 (level 1) or L1 (level 2)
// without waiting for it: the sectors of a later load_chunk are then on chip.
template <int LOG2M>
__device__ __forceinline__ void prefetch_chunk(const uint8_t* __restrict__ base, uint64_t node, int c,
                                               uint32_t level) {
    using G = Geo<LOG2M>;
    const uint8_t* p = base + node * (uint64_t)G::COUNTER_BYTES + (uint64_t)c * G::CHUNK_BYTES;
    if (level == 2) {
#pragma unroll
        for (int i = 0; i < G::CHUNK_BYTES; i += 32) asm volatile("prefetch.global.L1 [%0];" ::"l"(p + i));
    } else {
#pragma unroll
        for (int i = 0; i < G::CHUNK_BYTES; i += 32) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + i));
    }
}

template <int LOG2M>
__device__ __forceinline__ void store_chunk(uint8_t* __restrict__ base, uint64_t node, int c,
                                            const uint32_t (&w)[Geo<LOG2M>::NW]) {
    using G = Geo<LOG2M>;
    uint8_t* p = base + node * (uint64_t)G::COUNTER_BYTES + (uint64_t)c * G::CHUNK_BYTES;
    if constexpr (G::NW >= 8) {
#pragma unroll
        for (int i = 0; i < G::NW / 8; i++) st_256(p + 32 * i, w + 8 * i);
    } else {
        *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
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
