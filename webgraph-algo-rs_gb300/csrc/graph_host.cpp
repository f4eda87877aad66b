// Host-side graph layer: the BVGraph decoder (the CSR container, the host
// transpose and the synthetic generators are in graph_gen.cpp).
//
// CSR layout (the device layout too): offsets[n+1] as u64, successors[m] as
// u32, every successor list sorted ascending without duplicates.
//
// BVGraph: the reference loads graphs with webgraph 0.2.0 (third party, not
// vendored; src/main.rs:56-58 and tests/test_hyperball.rs:226-227 call
// `BvGraph::with_basename(..).load()`). This decoder is written from the
// published BVGraph format (Boldi & Vigna, "The WebGraph Framework I:
// Compression Techniques", WWW 2004, and the BVGraph format documentation):
// per node an outdegree, a reference with copy blocks, intervals and
// zeta-coded residual gaps, read MSB-first from the .graph bit stream.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "hb_internal.h"

namespace hbg {

// ---------------------------------------------------------------------------
// BVGraph decoder
// ---------------------------------------------------------------------------
enum Code { C_UNARY, C_GAMMA, C_DELTA, C_ZETA, C_NIBBLE };

struct BitReader {
    const uint8_t* p;
    uint64_t nbits;
    uint64_t pos = 0;
    bool overflow = false;
    BitReader(const uint8_t* data, uint64_t nbytes) : p(data), nbits(nbytes * 8) {}
    inline uint64_t bit() {
        if (pos >= nbits) {
            overflow = true;
            return 0;
        }
        uint64_t b = (p[pos >> 3] >> (7 - (pos & 7))) & 1;
        pos++;
        return b;
    }
    inline uint64_t bits(int len) {
        uint64_t x = 0;
        for (int i = 0; i < len; i++) x = (x << 1) | bit();
        return x;
    }
    inline uint64_t unary() {
        uint64_t x = 0;
        while (bit() == 0) {
            x++;
            if (overflow) return 0;
        }
        return x;
    }
    inline uint64_t gamma() {
        uint64_t msb = unary();
        if (msb > 63) {
            overflow = true;
            return 0;
        }
        return ((1ull << msb) | bits((int)msb)) - 1;
    }
    inline uint64_t delta() {
        uint64_t msb = gamma();
        if (msb > 63) {
            overflow = true;
            return 0;
        }
        return ((1ull << msb) | bits((int)msb)) - 1;
    }
    inline uint64_t zeta(int k) {
        uint64_t h = unary();
        if ((h + 1) * (uint64_t)k > 63) {
            overflow = true;
            return 0;
        }
        uint64_t left = 1ull << (h * k);
        uint64_t m = bits((int)(h * k + k - 1));
        if (m < left) return m + left - 1;
        return (m << 1) + bit() - 1;
    }
    inline uint64_t nibble() {
        uint64_t x = 0;
        for (;;) {
            uint64_t nb = bits(4);
            x = (x << 3) | (nb & 7);
            if (nb & 8) break;
            if (overflow) return 0;
        }
        return x;
    }
    inline uint64_t read(Code c, int k) {
        switch (c) {
            case C_UNARY: return unary();
            case C_GAMMA: return gamma();
            case C_DELTA: return delta();
            case C_ZETA: return zeta(k);
            case C_NIBBLE: return nibble();
        }
        return 0;
    }
};

static inline int64_t nat2int(uint64_t x) { return (int64_t)(x >> 1) ^ -(int64_t)(x & 1); }

static bool read_file(const std::string& path, std::vector<uint8_t>& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    f.seekg(0, std::ios::end);
    std::streamoff sz = f.tellg();
    f.seekg(0);
    out.resize((size_t)sz);
    if (sz > 0) f.read((char*)out.data(), sz);
    return (bool)f;
}

static std::map<std::string, std::string> read_properties(const std::string& path) {
    std::map<std::string, std::string> m;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string k = line.substr(0, eq), v = line.substr(eq + 1);
        while (!v.empty() && (v.back() == '\r' || v.back() == ' ')) v.pop_back();
        m[k] = v;
    }
    return m;
}

int load_bvgraph(const std::string& basename, Csr& g, std::string& err, uint64_t* bits_checked) {
    auto props = read_properties(basename + ".properties");
    if (props.empty()) {
        err = "cannot read " + basename + ".properties";
        return HB_ERR_IO;
    }
    auto geti = [&](const char* k, int64_t def) -> int64_t {
        auto it = props.find(k);
        return it == props.end() ? def : std::atoll(it->second.c_str());
    };
    const uint64_t n = (uint64_t)geti("nodes", -1);
    const uint64_t m = (uint64_t)geti("arcs", -1);
    const int window = (int)geti("windowsize", 7);
    const int min_interval = (int)geti("minintervallength", 4);
    const int zk = (int)geti("zetak", 3);
    if (props.count("version") && geti("version", 0) != 0) {
        err = "unsupported BVGraph version";
        return HB_ERR_INVALID;
    }
    if (props.count("endianness") && props["endianness"] != "big") {
        err = "only big-endian (Java) BVGraph bit streams are supported";
        return HB_ERR_INVALID;
    }
    Code c_outdeg = C_GAMMA, c_block = C_GAMMA, c_resid = C_ZETA, c_ref = C_UNARY,
         c_blockcount = C_GAMMA;
    {
        std::string flags = props.count("compressionflags") ? props["compressionflags"] : "";
        std::stringstream ss(flags);
        std::string tok;
        while (std::getline(ss, tok, '|')) {
            while (!tok.empty() && tok[0] == ' ') tok.erase(0, 1);
            while (!tok.empty() && tok.back() == ' ') tok.pop_back();
            if (tok.empty()) continue;
            size_t us = tok.rfind('_');
            std::string what = tok.substr(0, us), code = tok.substr(us + 1);
            Code c;
            if (code == "GAMMA") c = C_GAMMA;
            else if (code == "DELTA") c = C_DELTA;
            else if (code == "ZETA") c = C_ZETA;
            else if (code == "NIBBLE") c = C_NIBBLE;
            else if (code == "UNARY") c = C_UNARY;
            else {
                err = "unknown code in compressionflags: " + tok;
                return HB_ERR_INVALID;
            }
            if (what == "OUTDEGREES") c_outdeg = c;
            else if (what == "BLOCKS") c_block = c;
            else if (what == "RESIDUALS") c_resid = c;
            else if (what == "REFERENCES") c_ref = c;
            else if (what == "BLOCK_COUNT") c_blockcount = c;
            else if (what == "OFFSETS") {
            } else {
                err = "unknown compression flag: " + tok;
                return HB_ERR_INVALID;
            }
        }
    }
    std::vector<uint8_t> data;
    if (!read_file(basename + ".graph", data)) {
        err = "cannot read " + basename + ".graph";
        return HB_ERR_IO;
    }
    BitReader br(data.data(), data.size());
    g.n = n;
    g.offsets.assign(n + 1, 0);
    g.successors.clear();
    g.successors.reserve(m);
    std::vector<uint64_t> node_bitpos(n + 1, 0);
    std::vector<uint32_t> extra;
    std::vector<uint64_t> blocks;
    for (uint64_t x = 0; x < n; x++) {
        node_bitpos[x] = br.pos;
        const uint64_t d = br.read(c_outdeg, zk);
        const uint64_t row_start = g.successors.size();
        if (d > 0) {
            uint64_t ref = 0;
            if (window > 0) ref = br.read(c_ref, zk);
            if (ref > x || ref > (uint64_t)window) {
                err = "corrupt BVGraph: bad reference at node " + std::to_string(x);
                return HB_ERR_INVALID;
            }
            std::vector<uint32_t> copied;
            if (ref > 0) {
                const uint64_t bc = br.read(c_blockcount, zk);
                blocks.resize(bc);
                for (uint64_t i = 0; i < bc; i++) blocks[i] = br.read(c_block, zk) + (i == 0 ? 0 : 1);
                const uint64_t rs = g.offsets[x - ref], re = g.offsets[x - ref + 1];
                uint64_t idx = rs;
                for (uint64_t i = 0; i < bc; i++) {
                    if (idx + blocks[i] > re) {
                        err = "corrupt BVGraph: copy block overflow at node " + std::to_string(x);
                        return HB_ERR_INVALID;
                    }
                    if (i % 2 == 0)
                        for (uint64_t j = 0; j < blocks[i]; j++) copied.push_back(g.successors[idx + j]);
                    idx += blocks[i];
                }
                if (bc % 2 == 0)
                    for (; idx < re; idx++) copied.push_back(g.successors[idx]);
            }
            if (copied.size() > d) {
                err = "corrupt BVGraph: too many copied arcs at node " + std::to_string(x);
                return HB_ERR_INVALID;
            }
            const uint64_t extra_count = d - copied.size();
            extra.clear();
            if (extra_count > 0) {
                uint64_t interval_total = 0;
                if (min_interval > 0) {
                    const uint64_t ic = br.gamma();
                    if (ic > 0) {
                        int64_t left = (int64_t)x + nat2int(br.gamma());
                        uint64_t len = br.gamma() + (uint64_t)min_interval;
                        for (uint64_t j = 0; j < len; j++) extra.push_back((uint32_t)(left + (int64_t)j));
                        int64_t prev = left + (int64_t)len;
                        interval_total += len;
                        for (uint64_t i = 1; i < ic; i++) {
                            left = prev + (int64_t)br.gamma() + 1;
                            len = br.gamma() + (uint64_t)min_interval;
                            for (uint64_t j = 0; j < len; j++) extra.push_back((uint32_t)(left + (int64_t)j));
                            prev = left + (int64_t)len;
                            interval_total += len;
                        }
                    }
                }
                if (interval_total > extra_count) {
                    err = "corrupt BVGraph: interval overflow at node " + std::to_string(x);
                    return HB_ERR_INVALID;
                }
                const uint64_t residuals = extra_count - interval_total;
                if (residuals > 0) {
                    int64_t prev = (int64_t)x + nat2int(br.read(c_resid, zk));
                    extra.push_back((uint32_t)prev);
                    for (uint64_t i = 1; i < residuals; i++) {
                        prev = prev + (int64_t)br.read(c_resid, zk) + 1;
                        extra.push_back((uint32_t)prev);
                    }
                }
            }
            // merge copied + intervals + residuals (all disjoint) into sorted order
            g.successors.insert(g.successors.end(), copied.begin(), copied.end());
            g.successors.insert(g.successors.end(), extra.begin(), extra.end());
            std::sort(g.successors.begin() + (int64_t)row_start, g.successors.end());
            for (uint64_t a = row_start; a < g.successors.size(); a++) {
                if (g.successors[a] >= n) {
                    err = "corrupt BVGraph: successor out of range at node " + std::to_string(x);
                    return HB_ERR_INVALID;
                }
            }
        }
        if (br.overflow) {
            err = "corrupt BVGraph: bit stream ended early at node " + std::to_string(x);
            return HB_ERR_INVALID;
        }
        g.offsets[x + 1] = g.successors.size();
    }
    node_bitpos[n] = br.pos;
    g.m = g.successors.size();
    if (m != (uint64_t)-1 && g.m != m) {
        err = "BVGraph arc count " + std::to_string(g.m) + " != properties " + std::to_string(m);
        return HB_ERR_INVALID;
    }
    // Cross-check against the .offsets file (gamma-coded bit-offset gaps) when present.
    if (bits_checked) *bits_checked = 0;
    std::vector<uint8_t> od;
    if (read_file(basename + ".offsets", od)) {
        BitReader ob(od.data(), od.size());
        uint64_t pos = 0, checked = 0;
        for (uint64_t x = 0; x <= n; x++) {
            uint64_t gap = ob.gamma();
            if (ob.overflow) break;
            pos += gap;
            if (pos != node_bitpos[x]) {
                err = "BVGraph .offsets disagree with decoded stream at node " + std::to_string(x);
                return HB_ERR_INVALID;
            }
            checked++;
        }
        if (bits_checked) *bits_checked = checked;
    }
    return HB_OK;
}

}  // namespace hbg
