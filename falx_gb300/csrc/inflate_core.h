// DEFLATE (RFC 1951) decoding of one bgzf block, shared by the GPU kernel
// (one warp per block, every lane holding the same decoder state) and a host
// build of the same code used by the tests. The reference inflates bgzf
// blocks with flate2 / libdeflate on CPU threads (bgzf.rs:146-160,
// :180-191) and, in its GPU pipeline example, with one thread per block
// (examples/gpu_pipeline.rs:1-8).
//
// The decoder is warp-uniform: every lane runs the same bit reader, table
// lookups and bounds checks on the same values, so the warp never diverges
// while it decodes; the work that is parallel goes to the lanes through the
// Sink: a literal is stored by one lane, a match's bytes are copied by all
// lanes at once (byte k of a match
// at distance d comes from position pos - d + k mod d, which is already
// written, so the copy has no dependencies inside it), and the fast decode
// tables are filled one entry per lane.
//
// Every read is bounded by the block's compressed bytes and every write by
// its declared uncompressed size (ISIZE); each loop iteration consumes input
// bits or produces output, so a corrupt block ends with an error status.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GZ_HD __host__ __device__ __forceinline__
#else
#define GZ_HD inline
#endif

namespace falx {
namespace gz {

constexpr int kLitFast = 10;   // bits resolved by one lookup: literal / length codes
constexpr int kDistFast = 8;   // distance codes

// One member of the bgzf stream: compressed payload and its place in the
// inflated output (host scan of the gzip headers, bgzf.rs:61-108).
struct Block {
    uint64_t in_off;   // raw DEFLATE payload in the compressed stream
    uint64_t out_off;  // first byte in the inflated output
    uint32_t in_len;
    uint32_t out_len;  // ISIZE
};

enum Status : int32_t {
    OK = 0,
    ERR_TRUNCATED = 1,   // the payload ended inside a code or a header
    ERR_BLOCK_TYPE = 2,  // BTYPE 3
    ERR_STORED_LEN = 3,  // LEN != ~NLEN
    ERR_CODES = 4,       // a code-length set that is over-subscribed or has no end-of-block code
    ERR_SYMBOL = 5,      // a bit pattern that is no code, or a reserved symbol
    ERR_DISTANCE = 6,    // a match reaching before the block's first byte
    ERR_OVERFLOW = 7,    // more output than ISIZE
    ERR_SIZE = 8,        // less output than ISIZE
    ERR_BOUNDS = 9,      // the block's ranges lie outside the buffers
};

// Length and distance bases / extra bits (RFC 1951 section 3.2.5).
struct Consts {
    uint16_t len_base[29];
    uint8_t len_extra[29];
    uint16_t dist_base[30];
    uint8_t dist_extra[30];
};

// Decode tables of the current DEFLATE block (a warp's slice of shared
// memory on the GPU).
struct Tables {
    uint16_t lcount[16], dcount[16];  // codes per length
    uint16_t lsym[288], dsym[32];     // symbols ordered by (length, value)
    uint16_t lfast[1 << kLitFast];    // (length << 9) | symbol, 0: longer code
    uint16_t dfast[1 << kDistFast];
    uint8_t lens[320];                // code lengths being read
};

// LSB-first bit reader over p[0, n).
struct Bits {
    const uint8_t *p;
    uint32_t n;    // payload bytes
    uint32_t pos;  // next byte to load
    uint64_t buf;  // loaded bits, first bit in bit 0
    int32_t cnt;   // bits in buf that came from the payload
    bool bad;      // a read went past the payload

    // Keeps at least 33 bits buffered while input remains. Away from the
    // payload's ends, 4 bytes at any alignment come from the two aligned
    // words that hold them (both inside the payload: pos >= 4 and
    // pos + 8 <= n); near the ends, one byte at a time.
    GZ_HD void refill() {
        if (cnt > 32) return;
        if (pos >= 4 && pos + 8 <= n) {
            const uintptr_t a = (uintptr_t)(p + pos);
            const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
            const uint32_t sh = 8u * (uint32_t)(a & 3u);
            const uint32_t v = sh ? (w[0] >> sh) | (w[1] << (32u - sh)) : w[0];
            buf |= (uint64_t)v << cnt;
            pos += 4;
            cnt += 32;
            return;
        }
        while (cnt <= 56 && pos < n) {
            buf |= (uint64_t)p[pos++] << cnt;
            cnt += 8;
        }
    }
    GZ_HD uint32_t peek(int k) const { return (uint32_t)(buf & ((1ull << k) - 1ull)); }
    GZ_HD void drop(int k) {
        if (k > cnt) {
            bad = true;
            buf = 0;
            cnt = 0;
        } else {
            buf >>= k;
            cnt -= k;
        }
    }
    GZ_HD uint32_t get(int k) {
        refill();
        const uint32_t v = peek(k);
        drop(k);
        return v;
    }
    // To the next byte boundary; bytes loaded but not used go back.
    GZ_HD void align() {
        drop(cnt & 7);
        pos -= (uint32_t)(cnt >> 3);
        buf = 0;
        cnt = 0;
    }
};

// Counts per length and symbols in canonical order; false when the lengths
// over-subscribe the code space. Incomplete codes are accepted: an unused
// pattern decodes as an error.
GZ_HD bool build_sorted(const uint8_t *len, int n, uint16_t *count, uint16_t *sym) {
    uint16_t c[16], offs[16];
    for (int i = 0; i < 16; i++) c[i] = 0;
    for (int s = 0; s < n; s++) c[len[s]]++;
    int left = 1;
    for (int l = 1; l < 16; l++) {
        left = (left << 1) - c[l];
        if (left < 0) return false;
    }
    offs[1] = 0;
    for (int l = 1; l < 15; l++) offs[l + 1] = (uint16_t)(offs[l] + c[l]);
    for (int s = 0; s < n; s++)
        if (len[s]) sym[offs[len[s]]++] = (uint16_t)s;
    for (int i = 0; i < 16; i++) count[i] = c[i];
    return true;
}

// Table entry for the F-bit pattern i (first code bit in bit 0): the code
// it starts with when that code is at most F bits long, else 0.
GZ_HD uint16_t fast_entry(uint32_t i, int F, const uint16_t *count, const uint16_t *sym) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l <= F; l++) {
        code |= (int)((i >> (l - 1)) & 1u);
        const int c = count[l];
        if (code - first < c) return (uint16_t)((l << 9) | sym[index + code - first]);
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return 0;
}

// One symbol: a table lookup, or the canonical walk bit by bit for codes
// longer than the table. 511 (no symbol of either alphabet) when the bits
// are no code.
GZ_HD int decode(Bits &b, const uint16_t *fast, int F, const uint16_t *count, const uint16_t *sym) {
    b.refill();
    if (fast) {
        const uint16_t e = fast[b.peek(F)];
        if (e) {
            b.drop(e >> 9);
            return e & 511;
        }
    }
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; l++) {
        code |= (int)((b.buf >> (l - 1)) & 1u);
        const int c = count[l];
        if (code - first < c) {
            b.drop(l);
            return sym[index + code - first];
        }
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    b.drop(15);
    return 511;
}

// Code lengths of a dynamic block (RFC 1951 section 3.2.7) into T.lens and
// the two code tables. The sink fills the fast tables.
template <class Sink>
GZ_HD int read_dynamic(Bits &b, Tables &T, Sink &out, uint32_t &nlen) {
    // order of the code-length code lengths (RFC 1951 section 3.2.7)
    const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    nlen = b.get(5) + 257;
    const uint32_t ndist = b.get(5) + 1;
    const uint32_t ncode = b.get(4) + 4;
    if (b.bad) return ERR_TRUNCATED;
    if (nlen > 286 || ndist > 30) return ERR_CODES;
    out.sync();
    for (int i = 0; i < 19; i++) T.lens[order[i]] = (uint8_t)((uint32_t)i < ncode ? b.get(3) : 0u);
    if (b.bad) return ERR_TRUNCATED;
    out.sync();
    // the code-length code: symbols 0-18, up to 7 bits, decoded bit by bit
    if (!build_sorted(T.lens, 19, T.dcount, T.dsym)) return ERR_CODES;
    out.sync();
    const uint32_t total = nlen + ndist;
    uint32_t idx = 0;
    while (idx < total) {
        const int s = decode(b, nullptr, 0, T.dcount, T.dsym);
        if (b.bad) return ERR_TRUNCATED;
        if (s > 18) return ERR_SYMBOL;
        if (s < 16) {
            T.lens[idx++] = (uint8_t)s;
            continue;
        }
        uint32_t rep, v = 0;
        if (s == 16) {
            if (idx == 0) return ERR_CODES;
            v = T.lens[idx - 1];
            rep = 3 + b.get(2);
        } else if (s == 17) {
            rep = 3 + b.get(3);
        } else {
            rep = 11 + b.get(7);
        }
        if (b.bad) return ERR_TRUNCATED;
        if (idx + rep > total) return ERR_CODES;
        for (uint32_t k = 0; k < rep; k++) T.lens[idx++] = (uint8_t)v;
    }
    if (T.lens[256] == 0) return ERR_CODES;  // no end-of-block code
    out.sync();
    if (!build_sorted(T.lens, (int)nlen, T.lcount, T.lsym)) return ERR_CODES;
    if (!build_sorted(T.lens + nlen, (int)ndist, T.dcount, T.dsym)) return ERR_CODES;
    out.sync();
    out.fill_fast(T.lfast, kLitFast, T.lcount, T.lsym);
    out.fill_fast(T.dfast, kDistFast, T.dcount, T.dsym);
    return OK;
}

// The fixed codes (RFC 1951 section 3.2.6); distance codes 30 and 31 take
// part in the code but are rejected when decoded.
template <class Sink>
GZ_HD void read_fixed(Tables &T, Sink &out) {
    out.sync();
    for (int s = 0; s < 288; s++) T.lens[s] = (uint8_t)(s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8);
    out.sync();
    build_sorted(T.lens, 288, T.lcount, T.lsym);
    out.sync();
    for (int s = 0; s < 32; s++) T.lens[s] = 5;
    out.sync();
    build_sorted(T.lens, 32, T.dcount, T.dsym);
    out.sync();
    out.fill_fast(T.lfast, kLitFast, T.lcount, T.lsym);
    out.fill_fast(T.dfast, kDistFast, T.dcount, T.dsym);
}

// Inflate one raw DEFLATE stream of exactly out_len bytes through `out`.
template <class Sink>
GZ_HD int inflate_stream(Bits &b, Tables &T, const Consts &K, Sink &out, uint32_t out_len) {
    uint32_t pos = 0;
    for (;;) {
        const uint32_t hdr = b.get(3);
        if (b.bad) return ERR_TRUNCATED;
        const uint32_t type = hdr >> 1;
        if (type == 0) {
            b.align();
            if (b.bad) return ERR_TRUNCATED;
            if (b.n - b.pos < 4) return ERR_TRUNCATED;
            const uint32_t len = (uint32_t)b.p[b.pos] | ((uint32_t)b.p[b.pos + 1] << 8);
            const uint32_t nl = (uint32_t)b.p[b.pos + 2] | ((uint32_t)b.p[b.pos + 3] << 8);
            if (len != (~nl & 0xFFFFu)) return ERR_STORED_LEN;
            b.pos += 4;
            if (b.n - b.pos < len) return ERR_TRUNCATED;
            if (out_len - pos < len) return ERR_OVERFLOW;
            out.stored(b.p + b.pos, pos, len);
            b.pos += len;
            pos += len;
        } else if (type == 1 || type == 2) {
            uint32_t nlen = 288;
            if (type == 1) {
                read_fixed(T, out);
            } else {
                const int rc = read_dynamic(b, T, out, nlen);
                if (rc) return rc;
            }
            // Symbols: a read past the payload sets b.bad and yields zero
            // bits from then on; every iteration writes output (bounded by
            // out_len) or leaves the loop, and b.bad is checked when it does.
            for (;;) {
                int s = decode(b, T.lfast, kLitFast, T.lcount, T.lsym);
                if (s < 256) {
                    if (pos >= out_len) return b.bad ? ERR_TRUNCATED : ERR_OVERFLOW;
                    out.literal(pos, (uint32_t)s);
                    pos++;
                    continue;
                }
                if (s == 256) break;
                s -= 257;
                if (s >= 29) return b.bad ? ERR_TRUNCATED : ERR_SYMBOL;
                const uint32_t len = K.len_base[s] + b.get(K.len_extra[s]);
                const int ds = decode(b, T.dfast, kDistFast, T.dcount, T.dsym);
                if (ds >= 30) return b.bad ? ERR_TRUNCATED : ERR_SYMBOL;
                const uint32_t dist = K.dist_base[ds] + b.get(K.dist_extra[ds]);
                if (dist > pos) return b.bad ? ERR_TRUNCATED : ERR_DISTANCE;
                if (out_len - pos < len) return b.bad ? ERR_TRUNCATED : ERR_OVERFLOW;
                out.match(pos, dist, len);
                pos += len;
            }
            if (b.bad) return ERR_TRUNCATED;
        } else {
            return ERR_BLOCK_TYPE;
        }
        if (hdr & 1u) break;
    }
    out.flush();
    return pos == out_len ? OK : ERR_SIZE;
}

// RFC 1951 section 3.2.5 tables, computed from their definition: lengths
// 3-10 then runs of four codes per extra bit up to 5 (258 alone);
// distances 1-4 then pairs of codes per extra bit up to 13.
GZ_HD void make_consts(Consts &K) {
    uint32_t base = 3;
    for (int i = 0; i < 28; i++) {
        const int extra = i < 8 ? 0 : (i - 4) / 4;
        K.len_base[i] = (uint16_t)base;
        K.len_extra[i] = (uint8_t)extra;
        base += 1u << extra;
    }
    K.len_base[28] = 258;
    K.len_extra[28] = 0;
    base = 1;
    for (int i = 0; i < 30; i++) {
        const int extra = i < 4 ? 0 : (i - 2) / 2;
        K.dist_base[i] = (uint16_t)base;
        K.dist_extra[i] = (uint8_t)extra;
        base += 1u << extra;
    }
}

}  // namespace gz
}  // namespace falx
