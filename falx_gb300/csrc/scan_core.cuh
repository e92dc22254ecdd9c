// Device building blocks of the single-pass structural scan: byte-class
// masks from 4-byte SWAR words, per-dialect region automata as packed
// transfer functions, block scans, and the bounded decoupled look-back.
#pragma once
#include <cstdint>

namespace falx {

constexpr int kThreads = 256;          // threads per CTA
constexpr int kThreadBytes = 64;       // bytes per thread: one 64-bit mask word
constexpr int kTile = kThreads * kThreadBytes;  // 16 KiB per tile
constexpr int kPre = 16;               // bytes kept before the tile (previous-byte lookups)
constexpr int kWarps = kThreads / 32;

// Dialect numbering matches include/falx_gpu.h.
enum : int { D_CSV = 0, D_CSV_HASH = 1, D_TSV = 2, D_LOGFMT = 3, D_NDJSON = 4 };

// ---------------------------------------------------------------------------
// Byte classes. Every test is exact per byte (no borrow between bytes): the
// flag of byte k lands in bit 8k+7.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t zero_flags(uint32_t x) {
    uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
    return ~(t | x) & 0x80808080u;
}
__device__ __forceinline__ uint32_t eq_flags(uint32_t w, uint32_t c) {
    return zero_flags(w ^ (c * 0x01010101u));
}

// Two words of byte flags (bits 7,15,23,31) -> 8 linear mask bits in bits
// 24..31 of the result: word `lo` bytes 0-3 -> bits 24-27, word `hi` bytes
// 0-3 -> bits 28-31. One multiply moves all eight flags; every partial
// product lands on a distinct bit, so no carries disturb the top byte.
__device__ __forceinline__ uint32_t gather8(uint32_t lo, uint32_t hi) {
    return (hi | (lo >> 4)) * 0x00204081u;
}
// Four word flags of one 16-byte chunk -> 16 linear bits.
__device__ __forceinline__ uint32_t gather16(uint32_t f0, uint32_t f1, uint32_t f2, uint32_t f3) {
    return __byte_perm(gather8(f0, f1), gather8(f2, f3), 0x0073) & 0xFFFFu;
}

// Four 16-bit chunk masks loaded in rotated slot order (slot k holds chunk
// (k + r) & 3) -> the linear 64-bit mask.
__device__ __forceinline__ uint64_t assemble64(uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3,
                                               int r) {
    uint32_t lo = m0 | (m1 << 16), hi = m2 | (m3 << 16);
    if (r & 2) { uint32_t t = lo; lo = hi; hi = t; }
    if (r & 1) {
        uint32_t nlo = __funnelshift_l(hi, lo, 16);
        uint32_t nhi = __funnelshift_l(lo, hi, 16);
        lo = nlo; hi = nhi;
    }
    return (uint64_t)lo | ((uint64_t)hi << 32);
}

// Bit i of the result = XOR of bits 0..=i.
__device__ __forceinline__ uint64_t prefix_xor64(uint64_t x) {
    x ^= x << 1; x ^= x << 2; x ^= x << 4; x ^= x << 8; x ^= x << 16; x ^= x << 32;
    return x;
}

__device__ __forceinline__ uint64_t range_mask(unsigned from, unsigned to) {
    uint64_t hi = to >= 64 ? ~0ull : ((1ull << to) - 1);
    return hi & ~((1ull << from) - 1);
}

// ---------------------------------------------------------------------------
// Region automata as transfer functions: f maps entry state s (0..3) to exit
// state, packed two bits per state. compose(a, b) applies a, then b.
// ---------------------------------------------------------------------------
constexpr uint32_t kIdentity = 0xE4u;  // 0 -> 0, 1 -> 1, 2 -> 2, 3 -> 3

__device__ __forceinline__ uint32_t fapply(uint32_t f, uint32_t s) { return (f >> (2 * s)) & 3u; }

__device__ __forceinline__ uint32_t fcompose(uint32_t a, uint32_t b) {
    uint32_t r = 0;
#pragma unroll
    for (int s = 0; s < 4; s++) r |= fapply(b, fapply(a, s)) << (2 * s);
    return r;
}

// csv_hash states.
constexpr uint32_t R_N = 0, R_Q = 1, R_C = 2;

// Three-state NORMAL/QUOTE/COMMENT walk over the event bits of one 64-byte
// word (the interp.rs:93-133 resolver). Returns the inert mask; updates s.
__device__ __forceinline__ uint64_t resolve_regions(uint64_t q, uint64_t h, uint64_t nl, uint32_t &s) {
    uint64_t inert = 0, ev = q | h | nl;
    unsigned run = 0;
    while (ev) {
        unsigned p = __ffsll((long long)ev) - 1;
        uint64_t bit = 1ull << p;
        if (s == R_Q) {
            if (q & bit) { inert |= range_mask(run, p); s = R_N; }
        } else if (s == R_C) {
            if (nl & bit) { inert |= range_mask(run, p); s = R_N; }
        } else {
            if (q & bit) { s = R_Q; run = p; }
            else if (h & bit) { s = R_C; run = p; }
        }
        ev &= ev - 1;
    }
    if (s != R_N) inert |= range_mask(run, 64);
    return inert;
}

// Backslash escapes (formats.rs:334-343 form): returns the not-escaped mask
// for carry-in e and sets e to the carry-out.
__device__ __forceinline__ uint64_t not_escaped64(uint64_t bs, uint32_t &e) {
    const uint64_t EVEN = 0x5555555555555555ull;
    uint64_t v2 = EVEN ^ bs;
    uint64_t partial = EVEN + v2;
    uint32_t c1 = partial < EVEN;
    uint64_t sum = partial + e;
    uint32_t c2 = sum < partial;
    e = c1 | c2;
    return EVEN ^ sum;
}

// ---------------------------------------------------------------------------
// Per-thread classification of 64 bytes held in 16 words (rotated chunk
// order r). Output masks are linear in position.
// ---------------------------------------------------------------------------
struct Masks {
    uint64_t s;    // structural candidates (separators | '\n')
    uint64_t nl;   // '\n'
    uint64_t q;    // quote (0 unless `special`)
    uint64_t x;    // csv_hash: '#'; logfmt/ndjson: '\\' (0 unless `special`)
    bool special;  // any quote / '#' / backslash in the 64 bytes
};

template <int D>
__device__ __forceinline__ Masks classify(const uint32_t (&w)[16], int r) {
    Masks m;
    uint32_t sm[4], nm[4];
    uint32_t spacc = 0;
    uint32_t sf[16];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t fs[4], fn[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            uint32_t v = w[4 * k + j];
            uint32_t n = eq_flags(v, '\n');
            uint32_t s;
            if (D == D_TSV) s = n | eq_flags(v, '\t');
            else if (D == D_LOGFMT) s = n | eq_flags(v, ' ') | eq_flags(v, '=');
            else if (D == D_NDJSON) s = n;
            else s = n | eq_flags(v, ',');
            uint32_t sp = 0;
            if (D == D_CSV) sp = eq_flags(v, '"');
            else if (D == D_CSV_HASH) sp = zero_flags((v | 0x01010101u) ^ 0x23232323u);  // '"' or '#'
            else if (D == D_LOGFMT || D == D_NDJSON) sp = eq_flags(v, '"') | eq_flags(v, '\\');
            fs[j] = s; fn[j] = n; sf[4 * k + j] = sp; spacc |= sp;
        }
        sm[k] = gather16(fs[0], fs[1], fs[2], fs[3]);
        nm[k] = gather16(fn[0], fn[1], fn[2], fn[3]);
    }
    m.s = assemble64(sm[0], sm[1], sm[2], sm[3], r);
    m.nl = assemble64(nm[0], nm[1], nm[2], nm[3], r);
    m.special = spacc != 0;
    m.q = 0; m.x = 0;
    if (D != D_TSV && m.special) {
        uint32_t qm[4], xm[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t fq[4], fx[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint32_t v = w[4 * k + j];
                if (D == D_CSV) { fq[j] = sf[4 * k + j]; fx[j] = 0; }
                else if (D == D_CSV_HASH) {
                    uint32_t odd = (v << 7) & 0x80808080u;  // bit 0 of each byte: '#' is odd, '"' even
                    fq[j] = sf[4 * k + j] & ~odd;
                    fx[j] = sf[4 * k + j] & odd;
                } else {
                    fq[j] = eq_flags(v, '"');
                    fx[j] = eq_flags(v, '\\');
                }
            }
            qm[k] = gather16(fq[0], fq[1], fq[2], fq[3]);
            xm[k] = gather16(fx[0], fx[1], fx[2], fx[3]);
        }
        m.q = assemble64(qm[0], qm[1], qm[2], qm[3], r);
        m.x = assemble64(xm[0], xm[1], xm[2], xm[3], r);
    }
    return m;
}

// Transfer function of one thread's 64 bytes.
//  CSV: state = inside quotes (0/1).  CSV_HASH: N/Q/C.  TSV: stateless.
//  LOGFMT/NDJSON: state = escape carry | quote parity << 1.
// `ls_in`: the byte before is '\n' (or the word holds file position 0).
template <int D>
__device__ __forceinline__ uint32_t thread_function(const Masks &m, uint64_t ls_bits) {
    if (D == D_TSV) return kIdentity;
    if (D == D_CSV) {
        uint32_t par = __popcll(m.q) & 1;
        return par ? 0xE1u : kIdentity;  // swap 0 <-> 1
    }
    if (D == D_CSV_HASH) {
        if (!m.special) {
            uint32_t fc = m.nl ? R_N : R_C;
            return R_N | (R_Q << 2) | (fc << 4) | (3u << 6);
        }
        uint64_t h = m.x & ls_bits;
        uint32_t fn, fq, fc;
        if (h == 0) {
            uint32_t par = __popcll(m.q) & 1;
            fn = par ? R_Q : R_N;
            fq = par ? R_N : R_Q;
            if (m.nl == 0) {
                fc = R_C;
            } else {
                unsigned k = __ffsll((long long)m.nl) - 1;
                uint64_t rest = k == 63 ? 0 : (m.q >> (k + 1));
                fc = (__popcll(rest) & 1) ? R_Q : R_N;
            }
        } else {
            fn = R_N; resolve_regions(m.q, h, m.nl, fn);
            fq = R_Q; resolve_regions(m.q, h, m.nl, fq);
            fc = R_C; resolve_regions(m.q, h, m.nl, fc);
        }
        return fn | (fq << 2) | (fc << 4) | (3u << 6);
    }
    // LOGFMT / NDJSON
    if (!m.special) return (0u) | (0u << 2) | (2u << 4) | (2u << 6);  // escape carry cleared
    uint32_t r = 0;
#pragma unroll
    for (uint32_t e = 0; e < 2; e++) {
        uint32_t eo = e;
        uint64_t ne = not_escaped64(m.x, eo);
        uint32_t par = __popcll(m.q & ne) & 1;
#pragma unroll
        for (uint32_t p = 0; p < 2; p++) {
            uint32_t s = e | (p << 1);
            r |= (eo | ((p ^ par) << 1)) << (2 * s);
        }
    }
    return r;
}

// Structural mask of one thread's 64 bytes given its entry state.
template <int D>
__device__ __forceinline__ uint64_t structural_mask(const Masks &m, uint64_t ls_bits, uint32_t state) {
    if (D == D_TSV) return m.s;
    if (D == D_CSV) {
        if (!m.special) return state ? 0 : m.s;
        uint64_t inq = prefix_xor64(m.q) ^ (state ? ~0ull : 0ull);
        return m.s & ~inq;
    }
    if (D == D_CSV_HASH) {
        if (!m.special) {
            if (state == R_N) return m.s;
            if (state == R_Q) return 0;
            if (m.nl == 0) return 0;
            return m.s & ~((1ull << (__ffsll((long long)m.nl) - 1)) - 1);
        }
        uint64_t h = m.x & ls_bits;
        if (h == 0) {
            const uint64_t inq = prefix_xor64(m.q);
            if (state != R_C) return m.s & ~(inq ^ (state == R_Q ? ~0ull : 0ull));
            // a comment runs to the first newline; from there the state is
            // NORMAL and quote parity restarts: inside quotes where the prefix
            // XOR differs from its value just before the newline
            if (m.nl == 0) return 0;
            const uint64_t from = ~0ull << (__ffsll((long long)m.nl) - 1);
            const uint64_t before = (uint64_t)(__popcll(m.q & ~from) & 1);
            return m.s & from & ~(inq ^ (0ull - before));
        }
        uint32_t s = state;
        uint64_t inert = resolve_regions(m.q, h, m.nl, s);
        return m.s & ~inert;
    }
    // LOGFMT / NDJSON
    uint32_t p = state >> 1;
    if (!m.special) return p ? 0 : m.s;
    uint32_t e = state & 1;
    uint64_t ne = not_escaped64(m.x, e);
    uint64_t inq = prefix_xor64(m.q & ne) ^ (p ? ~0ull : 0ull);
    return m.s & ~inq;
}

// "Outside any region" test for a state (record boundaries are structural
// newlines, after which the automaton is outside).
template <int D>
__device__ __forceinline__ bool state_outside(uint32_t s) {
    if (D == D_TSV) return true;
    if (D == D_CSV) return s == 0;
    if (D == D_CSV_HASH) return s == R_N;
    return (s >> 1) == 0;
}

// ---------------------------------------------------------------------------
// Memory-ordering helpers for the look-back status words.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// ---------------------------------------------------------------------------
// TMA bulk copy (cp.async.bulk) into shared memory with an mbarrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait on an mbarrier phase. Returns false if the wait gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t max_ns) {
    uint32_t addr = smem_u32(bar);
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t i = 0;; i++) {
        if ((i & 63) == 63 && globaltimer_ns() - t0 > max_ns) return false;
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
}

}  // namespace falx
