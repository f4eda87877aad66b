// CPU oracle — test infrastructure only.
//
// This header restates, in plain C++17, the HyperLogLog counter logic of the
// reference crate webgraph-algo 0.1.0 (src/utils/hyper_log_log/hyper_log_log_logic.rs,
// cited below as "HLL:<line>") together with the two node hashers HyperBall uses:
//   * Rust std DefaultHasher = SipHash-1-3 with zero keys over the 8-byte
//     little-endian usize (third-party behaviour of Rust std, not vendored in the
//     reference; restated from the SipHash paper, Aumasson & Bernstein 2012);
//   * the Jenkins 64-bit mix of tests/test_hyperball.rs:25-172.
//
// It is linked only by the oracle library (oracle/hyperball_oracle.cpp), which
// the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load as the
// checker. Nothing in the product path includes this file.
//
// Parity status: the HLL arithmetic and the Jenkins hasher are pinned by the
// reference's Java-produced cnr-2000 goldens (tests/hyperball_results/*). No
// reference test fixes a DefaultHasher output; the SipHash round function is
// pinned by the SipHash-2-4 test vector of the paper, and the SipHash-1-3 node
// hash by an independent SipHash-1-3: CPython's bytes hash, whose key is zero
// under PYTHONHASHSEED=0 as Rust's DefaultHasher::new() key is (1,012 values,
// tests/test_oracle.py). What stays assumed is Rust std's DefaultHasher itself
// (SipHash-1-3, zero keys, a usize written as its 8 little-endian bytes).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace hbo {

// std::f64::consts::LN_2
constexpr double LN_2 = 0.693147180559945309417232121458176568;

enum HashKind : int { HASH_SIP13 = 0, HASH_JENKINS = 1 };

// Rust `f as usize` saturates: NaN and negatives map to 0.
inline uint64_t rust_f64_to_u64(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)x;
}

// HLL:301-303  register_size(n) = max(5, ceil(ln(ln(n)/LN_2/LN_2)))
inline int register_size(uint64_t n) {
    double v = std::log((std::log((double)n) / LN_2) / LN_2);
    uint64_t c = rust_f64_to_u64(std::ceil(v));
    return (int)std::max<uint64_t>(5, c);
}

// HLL:285-294
inline double rel_std(int log2m) {
    double tmp;
    switch (log2m) {
        case 4: tmp = 1.106; break;
        case 5: tmp = 1.070; break;
        case 6: tmp = 1.054; break;
        case 7: tmp = 1.046; break;
        default: tmp = 1.04; break;
    }
    return tmp / std::sqrt((double)(1ull << log2m));
}

inline uint64_t rotl64(uint64_t x, int b) { return (x << b) | (x >> (64 - b)); }

// One SipRound (SipHash paper, Fig. 2.1).
inline void sip_round(uint64_t& v0, uint64_t& v1, uint64_t& v2, uint64_t& v3) {
    v0 += v1; v1 = rotl64(v1, 13); v1 ^= v0; v0 = rotl64(v0, 32);
    v2 += v3; v3 = rotl64(v3, 16); v3 ^= v2;
    v0 += v3; v3 = rotl64(v3, 21); v3 ^= v0;
    v2 += v1; v1 = rotl64(v1, 17); v1 ^= v2; v2 = rotl64(v2, 32);
}

// Generic SipHash-c-d over a byte string (used to check the round function
// against the paper's SipHash-2-4 vector).
inline uint64_t siphash(int c_rounds, int d_rounds, uint64_t k0, uint64_t k1,
                        const uint8_t* msg, size_t len) {
    uint64_t v0 = k0 ^ 0x736f6d6570736575ull;
    uint64_t v1 = k1 ^ 0x646f72616e646f6dull;
    uint64_t v2 = k0 ^ 0x6c7967656e657261ull;
    uint64_t v3 = k1 ^ 0x7465646279746573ull;
    size_t full = len / 8;
    for (size_t i = 0; i < full; i++) {
        uint64_t mi = 0;
        for (int b = 0; b < 8; b++) mi |= (uint64_t)msg[8 * i + b] << (8 * b);
        v3 ^= mi;
        for (int r = 0; r < c_rounds; r++) sip_round(v0, v1, v2, v3);
        v0 ^= mi;
    }
    uint64_t last = (uint64_t)(len & 0xff) << 56;
    for (size_t b = 0; b < len % 8; b++) last |= (uint64_t)msg[8 * full + b] << (8 * b);
    v3 ^= last;
    for (int r = 0; r < c_rounds; r++) sip_round(v0, v1, v2, v3);
    v0 ^= last;
    v2 ^= 0xff;
    for (int r = 0; r < d_rounds; r++) sip_round(v0, v1, v2, v3);
    return v0 ^ v1 ^ v2 ^ v3;
}

// Rust std DefaultHasher::hash_one(x as usize): SipHash-1-3, keys (0, 0), over
// the 8 little-endian bytes of x (usize::hash -> write_usize -> write(to_ne_bytes)).
inline uint64_t hash_sip13_u64(uint64_t x) {
    uint8_t b[8];
    for (int i = 0; i < 8; i++) b[i] = (uint8_t)(x >> (8 * i));
    return siphash(1, 3, 0, 0, b, 8);
}

// tests/test_hyperball.rs:33-153: a = b = seed, c = 0x9e3779b97f4a7c13, one
// 8-byte word digested, finish() returns c.
inline uint64_t hash_jenkins_u64(uint64_t x, uint64_t seed) {
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

inline uint64_t hash_node(int kind, uint64_t seed, uint64_t x) {
    return kind == HASH_JENKINS ? hash_jenkins_u64(x, seed) : hash_sip13_u64(x);
}

// HLL:451-467 multiple-precision subtraction x -= y.
template <class W>
inline void subtract(W* x, const W* y, size_t len) {
    bool borrow = false;
    for (size_t i = 0; i < len; i++) {
        W xw = x[i];
        W yw = y[i];
        if (!borrow) {
            borrow = xw < yw;
        } else if (xw != 0) {
            xw = (W)(xw - 1);
            borrow = xw < yw;
        } else {
            xw = (W)(xw - 1);
        }
        x[i] = (W)(xw - yw);
    }
}

// The HyperLogLog logic of HLL:35-47, built as in HLL:374-428.
template <class W>
struct HllLogic {
    static constexpr int WBITS = (int)(8 * sizeof(W));
    int log2m = 0;
    uint64_t num_registers = 0;
    uint64_t num_registers_minus_1 = 0;
    int rsize = 0;
    uint64_t sentinel_mask = 0;
    size_t words_per_counter = 0;
    double alpha_m_m = 0.0;
    std::vector<W> msb, lsb;
    int hash_kind = HASH_SIP13;
    uint64_t seed = 0;
    // HLL:178 `1.0 / (1 << value) as f64` shifts an i32 literal: a register
    // value of 31 yields i32::MIN, i.e. a term of -2^-31. true = Rust semantics.
    bool i32_shift_quirk = true;

    HllLogic() = default;
    HllLogic(int log2m_, uint64_t num_elements, int hash_kind_, uint64_t seed_, bool quirk = true) {
        if (log2m_ < 4)
            throw std::invalid_argument(
                "the logarithm of the number of registers per counter should be at least 4; got " +
                std::to_string(log2m_));
        log2m = log2m_;
        num_registers = 1ull << log2m;
        rsize = register_size(num_elements);
        sentinel_mask = 1ull << ((1 << rsize) - 2);
        double alpha;
        switch (log2m) {
            case 4: alpha = 0.673; break;
            case 5: alpha = 0.697; break;
            case 6: alpha = 0.709; break;
            default: alpha = 0.7213 / (1.0 + 1.079 / (double)num_registers); break;
        }
        num_registers_minus_1 = num_registers - 1;
        uint64_t bits = num_registers * (uint64_t)rsize;
        if (bits % WBITS != 0)
            throw std::invalid_argument("W should allow counter backends to be aligned");
        words_per_counter = bits / WBITS;
        msb.assign(words_per_counter, 0);
        lsb.assign(words_per_counter, 0);
        for (uint64_t i = 0; i < num_registers; i++) {
            set_register(msb.data(), i, (W)((W)1 << (rsize - 1)));
            set_register(lsb.data(), i, (W)1);
        }
        double mf = (double)num_registers;
        alpha_m_m = alpha * (mf * mf);
        hash_kind = hash_kind_;
        seed = seed_;
        i32_shift_quirk = quirk;
    }

    // W::MAX >> (W::BITS - register_size), computed without integer promotion
    // (for u16, ~(W)0 would promote to int -1 and shift arithmetically).
    W reg_mask() const { return (W)((((uint64_t)1) << rsize) - 1); }

    // HLL:72-87
    W get_register(const W* backend, uint64_t index) const {
        const W mask = reg_mask();
        uint64_t pos = index * (uint64_t)rsize;
        size_t wi = pos / WBITS;
        int bi = (int)(pos % WBITS);
        if (bi + rsize <= WBITS) return (W)((backend[wi] >> bi) & mask);
        return (W)(((backend[wi] >> bi) | (W)(backend[wi + 1] << (WBITS - bi))) & mask);
    }

    // HLL:91-115
    void set_register(W* backend, uint64_t index, W value) const {
        const W mask = reg_mask();
        uint64_t pos = index * (uint64_t)rsize;
        size_t wi = pos / WBITS;
        int bi = (int)(pos % WBITS);
        if (bi + rsize <= WBITS) {
            W w = backend[wi];
            w &= (W)~(W)(mask << bi);
            w |= (W)(value << bi);
            backend[wi] = w;
        } else {
            W w = backend[wi];
            w &= (W)(((W)1 << bi) - 1);
            w |= (W)(value << bi);
            backend[wi] = w;
            W w2 = backend[wi + 1];
            w2 &= (W)~(W)(mask >> (WBITS - bi));
            w2 |= (W)(value >> (WBITS - bi));
            backend[wi + 1] = w2;
        }
    }

    // HLL:151-167, with the element hashed by the selected hasher.
    void add(W* backend, uint64_t element) const {
        uint64_t x = hash_node(hash_kind, seed, element);
        add_hash(backend, x);
    }

    void add_hash(W* backend, uint64_t x) const {
        uint64_t j = x & num_registers_minus_1;
        uint64_t y = (x >> log2m) | sentinel_mask;
        uint64_t r = (uint64_t)__builtin_ctzll(y);
        W cur = get_register(backend, j);
        W cand = (W)(r + 1);
        W nv = std::max(cur, cand);
        if (cur != nv) set_register(backend, j, nv);
    }

    // HLL:169-186
    double count(const W* backend, const double* ln_table = nullptr) const {
        double harmonic_mean = 0.0;
        uint64_t zeroes = 0;
        for (uint64_t i = 0; i < num_registers; i++) {
            uint64_t value = (uint64_t)get_register(backend, i);
            if (value == 0) zeroes++;
            double denom;
            if (i32_shift_quirk) {
                // (1i32 << value) as f64, with the shift amount taken mod 32
                // exactly as Rust's release-mode wrapping shift.
                int32_t s = (int32_t)((uint32_t)1u << (value & 31));
                denom = (double)s;
            } else {
                denom = std::ldexp(1.0, (int)value);
            }
            harmonic_mean += 1.0 / denom;
        }
        double estimate = alpha_m_m / harmonic_mean;
        double mf = (double)num_registers;
        if (zeroes != 0 && estimate < 2.5 * mf) {
            estimate = ln_table ? ln_table[zeroes] : mf * std::log(mf / (double)zeroes);
        }
        return estimate;
    }

    // HLL:469-576, acc and mask are the helper's scratch vectors.
    void merge(W* x, const W* y, std::vector<W>& acc, std::vector<W>& mask) const {
        const size_t nw = words_per_counter;
        const int rm1 = rsize - 1;
        const int shift_rm1 = WBITS - rm1;
        acc.resize(nw);
        mask.resize(nw);
        for (size_t i = 0; i < nw; i++) acc[i] = (W)(y[i] | msb[i]);
        for (size_t i = 0; i < nw; i++) mask[i] = (W)(x[i] & (W)~msb[i]);
        subtract(acc.data(), mask.data(), nw);
        for (size_t i = 0; i < nw; i++)
            acc[i] = (W)(((W)(acc[i] | (W)(y[i] ^ x[i])) ^ (W)(y[i] | (W)~x[i])) & msb[i]);
        for (size_t i = nw - 1; i-- > 0;)
            mask[i] = (W)((W)(acc[i] >> rm1) | (W)(acc[i + 1] << shift_rm1) | msb[i]);
        mask[nw - 1] = (W)((W)(acc[nw - 1] >> rm1) | msb[nw - 1]);
        subtract(mask.data(), lsb.data(), nw);
        for (size_t i = 0; i < nw; i++) mask[i] = (W)((W)(mask[i] | msb[i]) ^ acc[i]);
        for (size_t i = 0; i < nw; i++) x[i] = (W)(x[i] ^ (W)((W)(x[i] ^ y[i]) & mask[i]));
    }
};

// m * ln(m / z) for z = 0..m (entry 0 unused), the small-range correction of
// HLL:182-184, evaluated with the platform libm exactly as Rust's f64::ln.
inline std::vector<double> ln_table(uint64_t m) {
    std::vector<double> t(m + 1, 0.0);
    double mf = (double)m;
    for (uint64_t z = 1; z <= m; z++) t[z] = mf * std::log(mf / (double)z);
    return t;
}

}  // namespace hbo
