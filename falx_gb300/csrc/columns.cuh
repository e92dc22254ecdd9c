// Record-parallel materialisation from the tape.
//
// The index kernel leaves the tape in HBM: separator offsets `seps` and per
// terminated record `(separators before << 32) | terminator offset` in
// `ends` (csv_geo.rs:1838-1849 push_tape). A record's fields are then a
// contiguous run of `seps`, so every record can be decoded independently.
// Record block b holds the 512 records [512 b, 512 b + 512). Its CTA stages
// their tape entries and bytes, counts its rows (csv_hash comment records
// are not rows, csv_hash.rs:1381) and the cleaned bytes of its string
// cells, publishes those sums, and finds the sums of the blocks before it
// with a decoupled look-back (one warp, bounded waits); then it decodes its
// cells (ColumnSink semantics, csv_geo.rs:952-1101; decoders
// csv_geo.rs:1313-1486, csv_hash.rs:1688-1791), writes values, validity,
// string offsets and bytes, and adds its field-byte and count/sum totals
// (csv_hash.rs:1095-1230, csv_geo.rs:1605-1770).
#pragma once

#include <cstdint>

#include "decimal.cuh"
#include "swar.cuh"
#include "rows.cuh"
#include "scan_core.cuh"
#include "tile.cuh"

namespace falx {

constexpr int kRecPerThread = 2;
constexpr int kRecBlock = kThreads * kRecPerThread;  // records per CTA
constexpr int kRecWords = kRecBlock / 64 + 1;        // validity words a block's rows can touch
constexpr int kSepWin = 3072;                        // separators staged per CTA
constexpr int kDataWin = 32768;                      // bytes staged per CTA

// Look-back record of one record block, tagged with the call's epoch:
// flag = epoch * 4 + 1 once the block's own sums are published, + 2 once
// the sums up to and including it are.
struct BlkStatus {
    uint32_t flag;
    uint32_t rows;
    uint32_t arena[kMaxStr];
    uint32_t incl_rows;
    uint32_t pad;
    unsigned long long incl_arena[kMaxStr];
};

struct ColParams {
    const uint8_t *data;
    const uint8_t *abase;  // data rounded down to 16 bytes
    uint32_t shift;        // data - abase
    uint64_t len;
    const uint32_t *seps;
    uint64_t seps_cap;
    const uint64_t *ends;
    uint64_t ends_cap;
    BlkStatus *status;  // per record block
    uint32_t epoch;
    uint32_t blk0;     // first record block of the launch (ticket k runs block blk0 + k)
    uint64_t wait_ns;  // look-back wait limit
    DevHeader *hdr;
    // Launches over consecutive chunks of one input (pipelined host-buffer
    // calls): the tape counts through this chunk come from seed_hi (the
    // header after the chunk's index pass) instead of the header; the launch
    // takes the record blocks that end before the chunk's last terminator
    // (all the rest when `last`), from its own ticket, and its last block
    // writes the rows and arena bytes through it to chunk_out[0..4]
    // (chunk_out[5] = 1 once written).
    const SeedRec *seed_lo;  // the previous chunk's seed record, NULL for the first chunk
    const SeedRec *seed_hi;
    uint32_t *ticket;
    unsigned long long *chunk_out;
    uint32_t last;
    RowSpec rows;
};

// Shared memory of one record block. The tape entries of its records, their
// separators and the bytes they span are staged with coalesced loads; what
// does not fit the windows is read from global memory.
// Record counts of the tape, read on the device from the index pass's
// header (the host does not wait between the two launches).
struct TapeCounts {
    uint64_t n_seps, n_ends;
    uint64_t n_recs;    // n_ends, plus one for a trailing record without terminator
    uint32_t n_blocks;  // record blocks: this launch takes [blk_lo, n_blocks)
    uint32_t blk_lo;
};

struct ColSmem {
    alignas(16) uint64_t ends[kRecBlock + 2];  // ends[R0 - 2 + i]: 16-byte copies of even pairs
    alignas(16) uint32_t seps[kSepWin + 4];    // seps[sep_lo + i], sep_lo a multiple of 4
    uint32_t warp_rows[kWarps];
    uint32_t warp_len[kWarps][kMaxStr];
    uint32_t row_base;
    uint32_t arena_base[kMaxStr];
    uint64_t vbits[kMaxCols][kRecWords];
    uint32_t blk;
    uint32_t fb_next;  // the next chunk of 32 records for the field-byte / count-sum totals
    unsigned long long red[kWarps][14];
    alignas(16) uint8_t data[kDataWin + 16];  // 16 bytes of slack for word reads near the window end
};

// Asynchronous global -> shared copies (all of a CTA's copies in flight at
// once; completed by cp_async_wait_all + a barrier).
template <int N>
__device__ __forceinline__ void cp_async_ca(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "n"(N)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// File positions and separator ordinals fit 32 bits (inputs are shorter
// than 4 GiB), so the per-cell arithmetic is 32-bit.
struct Rec {
    uint32_t start, end;  // [start, end): the record without its terminator
    uint32_t end2;        // end of its last field: `end` less a trailing '\r' (csv_geo.rs:1055-1060)
    uint32_t sb;          // index of its first separator in `seps`
    uint32_t nf;          // fields
    bool row;             // a row (inside the file and not a comment)
};

// The block's staged windows with their bounds in registers (the cells
// loop stores through generic pointers, after which shared-memory fields
// would be read again).
struct Win {
    const uint32_t *sseps;
    const uint8_t *sdata;
    const uint32_t *gseps;
    const uint8_t *gdata;
    uint32_t sep_lo, sep_n;
    uint32_t dlo, dn;  // staged bytes: file positions [dlo, dlo + dn), dlo taken mod 2^32
    __device__ __forceinline__ uint32_t sep(uint32_t i) const {
        const uint32_t j = i - sep_lo;
        return j < sep_n ? sseps[j] : gseps[i];
    }
    // [a, a + n) is staged, at offset o (a before the window wraps to an
    // offset above dn)
    __device__ __forceinline__ bool staged(uint32_t a, uint32_t n, uint32_t &o) const {
        o = a - dlo;
        return o <= dn && n <= dn - o;
    }
    __device__ __forceinline__ const uint8_t *ptr(uint32_t a, uint32_t n) const {
        uint32_t o;
        return staged(a, n, o) ? sdata + o : gdata + a;
    }
    __device__ __forceinline__ uint8_t byte(uint32_t a) const { return *ptr(a, 1); }
    // field f of record r: [from, to)
    __device__ __forceinline__ bool field(const Rec &r, uint32_t f, uint32_t &from, uint32_t &to) const {
        if (f >= r.nf) return false;
        from = f == 0 ? r.start : sep(r.sb + f - 1) + 1;
        to = f + 1 < r.nf ? sep(r.sb + f) : r.end2;
        return true;
    }
};

// ---- word-at-a-time (SWAR) cell decoding from the staged bytes.
// Shared-memory words at any byte offset: two aligned loads and a funnel
// shift per 32-bit word (little-endian: the first byte is the low byte).
__device__ __forceinline__ uint32_t lds_u32(const uint8_t *base, uint32_t o) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(base + (o & ~3u));
    return __funnelshift_r(w[0], w[1], 8u * (o & 3u));
}
__device__ __forceinline__ uint64_t lds_u64(const uint8_t *base, uint32_t o) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(base + (o & ~3u));
    const uint32_t sh = 8u * (o & 3u), a = w[0], b = w[1], c = w[2];
    return (uint64_t)__funnelshift_r(a, b, sh) | ((uint64_t)__funnelshift_r(b, c, sh) << 32);
}

// 1-10 plain digits at shared offset o (swar.cuh).
__device__ __forceinline__ bool swar_u32(const uint8_t *sd, uint32_t o, uint32_t n, uint32_t &v) {
    if (n - 1u <= 7u) return swar::u32_word(lds_u64(sd, o), n, v);
    if (n - 9u <= 1u) return swar::u32_word10(lds_u32(sd, o), lds_u64(sd, o + n - 8u), n, v);
    return false;
}

// [+-]?d{1,3}.d{6} at shared offset o (swar.cuh): mantissa m, sign and the
// f64 bits of m / 1e6.
__device__ __forceinline__ bool swar_fixed6(const uint8_t *sd, uint32_t o, uint32_t n, uint64_t &bits, uint32_t &m,
                                            bool &neg) {
    if (n - 8u > 3u) return false;  // n in [8, 11]
    const uint32_t c0 = sd[o];
    const uint32_t sg = (c0 == '-' || c0 == '+') ? 1u : 0u;
    const uint32_t k = n - 7u - sg;  // integer digits
    if (k - 1u > 2u) return false;
    return swar::fixed6_words(c0, k, lds_u64(sd, o + n - 8u), lds_u32(sd, o + sg), bits, m, neg);
}

// An unquoted staged cell copied to dst (any alignment): bytes up to a
// 4-byte boundary of dst, then aligned word stores, then the tail.
__device__ __forceinline__ void copy_staged(const uint8_t *sd, uint32_t o, uint32_t n, uint8_t *dst) {
    uint32_t i = (uint32_t)((4u - ((uintptr_t)dst & 3u)) & 3u);
    if (i > n) i = n;
    for (uint32_t k = 0; k < i; k++) dst[k] = sd[o + k];
    for (; i + 4 <= n; i += 4) *reinterpret_cast<uint32_t *>(dst + i) = lds_u32(sd, o + i);
    for (; i < n; i++) dst[i] = sd[o + i];
}

// A string cell outside the staged window, cleaned into the arena (out of
// line: rare, and the cell loop is instruction-fetch bound).
__device__ __noinline__ void copy_unstaged(const uint8_t *src, uint32_t n, uint8_t *arena, uint32_t pos,
                                           uint64_t cap) {
    copy_clean(src, n, arena, pos, cap);
}

// Select from a small per-thread array by a warp-uniform slot without
// dynamic register indexing (which would move the array to local memory).
template <typename T, int N>
__device__ __forceinline__ T pick(const T (&a)[N], int k) {
    T x = a[0];
#pragma unroll
    for (int j = 1; j < N; j++) x = k == j ? a[j] : x;
    return x;
}

// Cells the word-at-a-time paths do not take (other shapes, quoted
// numbers, cells outside the staged window) go to the general decoders,
// kept out of line so the per-cell loop stays small. A fast path that
// accepts a cell gives exactly the general decoder's value.
// The out-of-line decoders return by value: a local whose address reached
// a call would live in local memory on the fast path too.
struct Slow64 {
    uint64_t v;
    bool ok;
};
__device__ __noinline__ Slow64 slow_u32(const uint8_t *s, uint32_t n) {
    uint32_t v = 0;
    const bool ok = dec::numeric_view(s, n) && dec::parse_u32(s, n, v);
    return {v, ok};
}
__device__ __noinline__ Slow64 slow_f64(const uint8_t *s, uint32_t n) {
    double v = 0;
    const bool ok = dec::numeric_view(s, n) && dec::parse_f64(s, n, v);
    return {dec::d2u(v), ok};
}
// An i64 cell: 1-8 plain digits word at a time when staged, else the full
// decoder.
__device__ __noinline__ Slow64 i64_cell(const uint8_t *sd, bool staged, uint32_t o, const uint8_t *s, uint32_t n) {
    uint32_t u;
    if (staged && swar_u32(sd, o, n, u)) return {u, true};
    int64_t v = 0;
    const bool ok = dec::numeric_view(s, n) && dec::parse_i64(s, n, v);
    return {(uint64_t)v, ok};
}
// One count / sum cell: whether it is a value, its bits, and its exact
// x1e6 value when it has one.
struct StatCell {
    uint64_t bits;
    int64_t e6;
    bool value, exact;
};
__device__ __noinline__ StatCell stat_slow(const uint8_t *s, uint32_t n) {
    StatCell r = {0, 0, false, false};
    double v;
    if (!dec::numeric_view(s, n) || !dec::parse_f64(s, n, v)) return r;
    r.value = true;
    r.bits = dec::d2u(v);
    r.exact = dec::exact_e6(s, n, r.e6);
    return r;
}
// Count / sum of one f64 cell (csv_geo.rs:1735-1750): values, bit checksum,
// exact x1e6 sum. The fixed shape is exact in micro-units: +-m.
__device__ __forceinline__ void stat_value(StatAcc &a, int k, const Win &W, uint32_t from, uint32_t to) {
    const uint32_t n = to - from;
    uint64_t bits;
    uint32_t m, o;
    bool neg;
    if (W.staged(from, n, o) && swar_fixed6(W.sdata, o, n, bits, m, neg)) {
        a.values[k]++;
        a.checksum[k] += bits;
        a.sum_e6[k] += neg ? 0ull - (unsigned long long)m : (unsigned long long)m;
        return;
    }
    const StatCell r = stat_slow(W.ptr(from, n), n);
    if (!r.value) return;
    a.values[k]++;
    a.checksum[k] += r.bits;
    if (r.exact) a.sum_e6[k] += (unsigned long long)r.e6;
    else a.inexact[k]++;
}

// A quoted cell s[0, n) (n >= 2, s[0] and s[n-1] are '"') cleaned by the
// whole warp (csv_hash.rs:1749-1782 append_clean): the inner bytes in
// chunks of 32, one per lane. Within a run of consecutive quotes the second
// of each pair is dropped, so a quote is dropped when its position in its
// run is odd; a run that goes on past a chunk carries its parity. Kept
// bytes go to dst[at + ...] below cap when dst is given. Returns the
// cleaned length; `sum`, when given, gets the sum of the kept byte values
// added. Called by all 32 lanes with the same arguments.
__device__ uint32_t warp_clean(const uint8_t *s, uint32_t n, uint8_t *dst, uint32_t at, uint64_t cap, int lane,
                               uint64_t *sum = nullptr) {
    const uint8_t *in = s + 1;
    const uint32_t il = n - 2;
    const uint32_t below = (1u << lane) - 1u;
    uint32_t out = 0, carry = 0;  // cleaned bytes so far; parity of the quote run reaching this chunk
    for (uint32_t base = 0; base < il; base += 32) {
        const uint32_t j = base + (uint32_t)lane;
        const bool inb = j < il;
        const uint8_t c = inb ? in[j] : (uint8_t)0;
        const bool isq = inb && c == '"';
        const uint32_t q = __ballot_sync(0xffffffffu, isq);
        const uint32_t valid = il - base >= 32 ? 0xffffffffu : (1u << (il - base)) - 1u;
        const uint32_t nq = ~q & below;  // non-quotes before me in the chunk
        const uint32_t pos = nq ? (uint32_t)lane - (32u - __clz(nq)) : carry + (uint32_t)lane;
        const bool drop = isq && (pos & 1u);
        const uint32_t dm = __ballot_sync(0xffffffffu, drop);
        const uint32_t keep = valid & ~dm;
        if (dst && inb && !drop) {
            const uint64_t o = (uint64_t)at + out + __popc(keep & below);
            if (o < cap) dst[o] = c;
        }
        out += __popc(keep);
        if (sum) *sum += __reduce_add_sync(0xffffffffu, inb && !drop ? (uint32_t)c : 0u);
        // the run at the end of the chunk: its parity carries into the next
        const uint32_t last = 31u - __clz(valid);
        const uint32_t lastpos = __shfl_sync(0xffffffffu, pos, (int)last);
        carry = (q >> last) & 1u ? (lastpos + 1u) & 1u : 0u;
    }
    return out;
}

// Sum of the byte values of p[0, n) (any alignment; shared or global).
__device__ __forceinline__ uint32_t byte_sum(const uint8_t *p, uint32_t n) {
    uint32_t s = 0, i = 0;
    while (i < n && ((uintptr_t)(p + i) & 3u)) s += p[i++];
    for (; i + 4 <= n; i += 4) s = __dp4a(*reinterpret_cast<const uint32_t *>(p + i), 0x01010101u, s);
    while (i < n) s += p[i++];
    return s;
}

// City text lane of the warp's records (csv_geo_text.rs:1845-1937): per row
// whose city field is present, one value, its cleaned length and the sum of
// its cleaned byte values; quoted cells are cleaned by the whole warp. All
// 32 lanes call it.
__device__ __forceinline__ void warp_text_cell(const Win &W, const Rec &x, uint32_t f, int lane, uint64_t &values,
                                               uint64_t &bytes, uint64_t &checksum) {
    uint32_t a = 0, b = 0;
    const bool present = x.row && W.field(x, f, a, b);
    const uint32_t n = b - a;
    const uint8_t *src = present ? W.ptr(a, n) : nullptr;
    const bool quoted = present && n >= 2 && src[0] == '"' && src[n - 1] == '"';
    if (present) values++;
    if (present && !quoted) {
        bytes += n;
        checksum += byte_sum(src, n);
    }
    for (uint32_t need = __ballot_sync(0xffffffffu, quoted); need; need &= need - 1) {
        const int sl = __ffs(need) - 1;
        const uint8_t *ps = reinterpret_cast<const uint8_t *>(
            __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(src), sl));
        uint64_t sum = 0;
        const uint32_t cl = warp_clean(ps, __shfl_sync(0xffffffffu, n, sl), nullptr, 0, 0, lane, &sum);
        if (lane == sl) {
            bytes += cl;
            checksum += sum;
        }
    }
}

// Cleaned bytes of all fields of the warp's records (csv_hash.rs:1207-1230):
// every byte but the separators and a trailing '\r', less what cleaning
// removes from quoted fields. Each thread cleans its own short quoted
// fields; quoted fields longer than kLongCell are cleaned by the whole warp
// afterwards, so one long field does not hold up a lane. All 32 lanes call
// it (rows or not).
constexpr uint32_t kLongCell = 64;

__device__ __forceinline__ uint32_t warp_field_bytes(const Win &W, const Rec &x, int lane) {
    uint32_t tot = x.row ? (x.end2 - x.start) - (x.nf - 1) : 0u;
    const uint32_t nr = x.row ? x.nf : 0u;
    bool longq = false;
    uint32_t from = x.start;
    for (uint32_t f = 0; f < nr; f++) {
        const uint32_t to = f + 1 < nr ? W.sep(x.sb + f) : x.end2;
        const uint32_t n = to - from;
        if (n >= 2 && W.byte(from) == '"') {
            if (n <= kLongCell) tot -= n - cleaned_len(W.ptr(from, n), n);
            else longq = true;
        }
        from = to + 1;
    }
    if (__ballot_sync(0xffffffffu, longq) == 0) return tot;
    // the long quoted fields, one warp-wide cleaning each
    const uint32_t nf = longq ? x.nf : 0u;
    uint32_t mx = nf;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    from = x.start;
    for (uint32_t f = 0; f < mx; f++) {
        bool quoted = false;
        const uint8_t *src = nullptr;
        uint32_t n = 0;
        if (f < nf) {
            const uint32_t to = f + 1 < nf ? W.sep(x.sb + f) : x.end2;
            n = to - from;
            if (n > kLongCell) {
                src = W.ptr(from, n);
                quoted = src[0] == '"' && src[n - 1] == '"';
            }
            from = to + 1;
        }
        for (uint32_t need = __ballot_sync(0xffffffffu, quoted); need; need &= need - 1) {
            const int sl = __ffs(need) - 1;
            const uint8_t *ps = reinterpret_cast<const uint8_t *>(
                __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(src), sl));
            const uint32_t ns = __shfl_sync(0xffffffffu, n, sl);
            const uint32_t cl = warp_clean(ps, ns, nullptr, 0, 0, lane);
            if (lane == sl) tot -= ns - cl;
        }
    }
    return tot;
}

// Record li of the block starting at record R0 (E[li] = ends[R0 + li - 1]).
template <int D>
__device__ __forceinline__ Rec make_rec(const ColParams &p, const TapeCounts &tc, const Win &W, const uint64_t *E,
                                        uint64_t R0, int li) {
    Rec x;
    x.row = false;
    x.nf = 0;
    x.start = x.end = x.end2 = x.sb = 0;
    const uint64_t r = R0 + (uint64_t)li;
    if (r >= tc.n_recs) return x;
    const uint64_t pe = r == 0 ? 0ull : E[li];
    x.start = r == 0 ? 0u : (uint32_t)pe + 1;
    x.sb = r == 0 ? 0u : (uint32_t)(pe >> 32);
    // after the last terminator there is a record only if bytes remain
    // (csv_geo.rs:1094-1100)
    if (r >= tc.n_ends && (uint64_t)x.start >= p.len) return x;
    uint32_t se;
    if (r < tc.n_ends) {
        const uint64_t e = E[li + 1];
        x.end = (uint32_t)e;
        se = (uint32_t)(e >> 32);
    } else {
        x.end = (uint32_t)p.len;
        se = (uint32_t)tc.n_seps;
    }
    x.nf = se - x.sb + 1;
    x.row = !(D == D_CSV_HASH && x.start < x.end && W.byte(x.start) == '#');
    x.end2 = x.end;
    if (x.row && x.end > x.start && W.byte(x.end - 1) == '\r') x.end2 = x.end - 1;
    return x;
}

// STATS: the count / sum sink is requested (its code is compiled only
// into the kernels that need it: a smaller kernel fetches faster).
template <int D, bool STATS>
__device__ __forceinline__ void columns_block(const ColParams &p, const TapeCounts &tc, ColSmem &S, uint32_t blk) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const RowSpec &rs = p.rows;
    const uint64_t R0 = (uint64_t)blk * kRecBlock;
    for (int i = tid; i < rs.ncols * kRecWords; i += kThreads) S.vbits[i / kRecWords][i % kRecWords] = 0;
    if (tid == 0) S.fb_next = 0;

    // ---- windows: from the block's first record to its last, computed by
    // every thread from the two tape entries that bound them
    const uint64_t last = (R0 + kRecBlock < tc.n_recs ? R0 + kRecBlock : tc.n_recs) - 1;
    const uint64_t e_first = R0 == 0 ? 0ull : __ldcg(reinterpret_cast<const unsigned long long *>(p.ends) + R0 - 1);
    const uint64_t e_last = last < tc.n_ends ? __ldcg(reinterpret_cast<const unsigned long long *>(p.ends) + last) : 0ull;
    const bool al16 = ((uintptr_t)p.ends & 15) == 0 && ((uintptr_t)p.seps & 15) == 0;
    const uint64_t sb = R0 == 0 ? 0 : e_first >> 32;
    const uint64_t se = last < tc.n_ends ? e_last >> 32 : tc.n_seps;
    const uint64_t sep_lo = al16 ? sb & ~3ull : sb;  // 16-byte aligned start
    const uint32_t sep_n = (uint32_t)(sb - sep_lo) + (uint32_t)(se - sb < (uint64_t)kSepWin ? se - sb : (uint64_t)kSepWin);
    int64_t data_lo;
    uint32_t data_n;
    {
        const int64_t lo = R0 == 0 ? 0 : (int64_t)(uint32_t)e_first + 1;
        const int64_t hi = last < tc.n_ends ? (int64_t)(uint32_t)e_last : (int64_t)p.len;
        const int64_t q0 = (lo + p.shift) & ~15ll;  // 16-byte aligned address offset
        const int64_t qend = (int64_t)((p.shift + p.len + 15) & ~15ull);
        int64_t qn = ((hi + p.shift + 15) & ~15ll) - q0;
        if (qn > qend - q0) qn = qend - q0;
        if (qn > kDataWin) qn = kDataWin;
        if (qn < 0) qn = 0;
        data_lo = q0 - p.shift;
        data_n = (uint32_t)qn;
    }
    // ---- stage the block's tape entries (ends[R0 - 1 .. R0 + kRecBlock - 1]
    // in 16-byte pairs from the even index R0 - 2), separators and bytes
    for (int j = tid; j < (kRecBlock + 2) / 2; j += kThreads) {
        const int64_t e0 = (int64_t)R0 - 2 + 2 * j;
        if (al16 && e0 >= 0 && (uint64_t)e0 + 1 < tc.n_ends) {
            cp_async_ca<16>(&S.ends[2 * j], p.ends + e0);
        } else {
            if (e0 >= 0 && (uint64_t)e0 < tc.n_ends) cp_async_ca<8>(&S.ends[2 * j], p.ends + e0);
            if (e0 + 1 >= 0 && (uint64_t)(e0 + 1) < tc.n_ends) cp_async_ca<8>(&S.ends[2 * j + 1], p.ends + e0 + 1);
        }
    }
    if (al16) {
        for (uint32_t j = tid; 4 * j < sep_n; j += kThreads) {
            const uint64_t i0 = sep_lo + 4 * j;
            if (i0 + 3 < tc.n_seps) {
                cp_async_ca<16>(&S.seps[4 * j], p.seps + i0);
            } else {
                for (uint32_t q = 0; q < 4 && i0 + q < tc.n_seps; q++) cp_async_ca<4>(&S.seps[4 * j + q], p.seps + i0 + q);
            }
        }
    } else {
        for (uint32_t i = tid; i < sep_n; i += kThreads) cp_async_ca<4>(&S.seps[i], p.seps + sep_lo + i);
    }
    {
        const uint8_t *src = p.abase + (data_lo + p.shift);
        for (uint32_t i = tid; i < data_n / 16; i += kThreads) cp_async_ca<16>(S.data + 16 * i, src + 16 * i);
    }
    cp_async_wait_all();
    __syncthreads();
    const uint64_t *E = S.ends + 1;  // E[i] = ends[R0 - 1 + i]
    const Win W{S.seps, S.data, p.seps, p.data, (uint32_t)sep_lo, sep_n, (uint32_t)data_lo, data_n};

    // ---- this thread's records: warp w owns records [64 w, 64 w + 64) of
    // the block and lane L takes records L and L + 32 of them, so a warp's
    // loads, value stores and validity ballots each cover 32 consecutive
    // records
    Rec rec[kRecPerThread];
#pragma unroll
    for (int i = 0; i < kRecPerThread; i++) rec[i] = make_rec<D>(p, tc, W, E, R0, warp * 64 + i * 32 + lane);

    // ---- per record: row (0/1) and cleaned bytes of each string slot
    const int nv = 1 + rs.nstr;  // values scanned: rows, then string slots
    uint32_t v[kRecPerThread][1 + kMaxStr];
#pragma unroll
    for (int i = 0; i < kRecPerThread; i++) {
        v[i][0] = rec[i].row;
#pragma unroll
        for (int k = 1; k < 1 + kMaxStr; k++) v[i][k] = 0;
    }
    for (int c = 0; c < rs.ncols; c++) {
        if (rs.type[c] != 3) continue;
        const int k = rs.str_slot[c];
        const uint32_t f = rs.field[c];
#pragma unroll
        for (int i = 0; i < kRecPerThread; i++) {
            uint32_t a, b, l = 0;
            bool quoted = false;
            const uint8_t *src = nullptr;
            if (rec[i].row && W.field(rec[i], f, a, b)) {
                l = b - a;
                src = W.ptr(a, l);
                quoted = l >= 2 && src[0] == '"' && src[l - 1] == '"';
            }
            // quoted cells: cleaned length by the whole warp, one cell at a time
            for (uint32_t need = __ballot_sync(0xffffffffu, quoted); need; need &= need - 1) {
                const int sl = __ffs(need) - 1;
                const uint8_t *ps = reinterpret_cast<const uint8_t *>(
                    __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(src), sl));
                const uint32_t cl = warp_clean(ps, __shfl_sync(0xffffffffu, l, sl), nullptr, 0, 0, lane);
                if (lane == sl) l = cl;
            }
#pragma unroll
            for (int j = 0; j < kMaxStr; j++) v[i][1 + j] += j == k ? l : 0u;
        }
    }

    // ---- exclusive prefixes in record order: a warp's records 0-31 (i = 0)
    // come before 32-63 (i = 1); then warps in order
    uint32_t ex[kRecPerThread][1 + kMaxStr];
#pragma unroll
    for (int k = 0; k < 1 + kMaxStr; k++) {
        if (k >= nv) break;
        uint32_t x0 = v[0][k], x1 = v[1][k];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o0 = __shfl_up_sync(0xffffffffu, x0, d);
            const uint32_t o1 = __shfl_up_sync(0xffffffffu, x1, d);
            if (lane >= d) {
                x0 += o0;
                x1 += o1;
            }
        }
        const uint32_t t0 = __shfl_sync(0xffffffffu, x0, 31);
        ex[0][k] = x0 - v[0][k];
        ex[1][k] = t0 + x1 - v[1][k];
        if (lane == 31) {
            if (k == 0) S.warp_rows[warp] = t0 + x1;
            else S.warp_len[warp][k - 1] = t0 + x1;
        }
    }
    __syncthreads();
    if (warp == 0) {
        // warp prefixes and block totals
        uint32_t tot[1 + kMaxStr] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 1 + kMaxStr; k++) {
            if (k >= nv) break;
            const uint32_t w = lane < kWarps ? (k == 0 ? S.warp_rows[lane] : S.warp_len[lane][k - 1]) : 0u;
            uint32_t x = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += o;
            }
            if (lane < kWarps) {
                if (k == 0) S.warp_rows[lane] = x - w;
                else S.warp_len[lane][k - 1] = x - w;
            }
            tot[k] = __shfl_sync(0xffffffffu, x, 31);
        }
        // publish the block's sums, then add up those of the blocks before it
        BlkStatus *me = p.status + blk;
        if (lane == 0) {
            me->rows = tot[0];
#pragma unroll
            for (int k = 0; k < kMaxStr; k++) me->arena[k] = tot[1 + k];
            st_release(&me->flag, p.epoch * 4 + 1);
        }
        unsigned long long pre[1 + kMaxStr] = {0, 0, 0, 0, 0};
        const uint64_t t0 = globaltimer_ns();
        for (int64_t hi = (int64_t)blk - 1; hi >= 0; hi -= 32) {
            // lane l watches block hi - l: wait until no block nearer than
            // the nearest inclusive prefix is still unpublished
            const int64_t j = hi - lane;
            uint32_t fi;
            for (uint32_t it = 0;; it++) {
                const uint32_t flag = j >= 0 ? ld_acquire(&p.status[j].flag) : 0u;
                const bool cur = (flag >> 2) == p.epoch;
                const uint32_t bi = __ballot_sync(0xffffffffu, j >= 0 && cur && (flag & 3) >= 2);
                const uint32_t bm = __ballot_sync(0xffffffffu, j >= 0 && !(cur && (flag & 3) >= 1));
                fi = bi ? __ffs(bi) - 1 : 32u;
                const uint32_t fm = bm ? __ffs(bm) - 1 : 32u;
                if (fm > fi || bm == 0) break;
                if ((it & 15) == 15) {
                    const bool stop = lane == 0 && (aborted(p.hdr) || globaltimer_ns() - t0 > p.wait_ns);
                    if (__any_sync(0xffffffffu, stop)) {
                        if (lane == 0) fail(p.hdr, ERR_TIMEOUT);
                        fi = 0;
                        hi = -1;
                        break;
                    }
                }
                __nanosleep(64);
            }
            if (hi < 0) break;
            unsigned long long v[1 + kMaxStr] = {0, 0, 0, 0, 0};
            if ((uint32_t)lane < fi && j >= 0) {
                v[0] = p.status[j].rows;
#pragma unroll
                for (int k = 0; k < kMaxStr; k++) v[1 + k] = p.status[j].arena[k];
            } else if ((uint32_t)lane == fi) {
                v[0] = p.status[j].incl_rows;
#pragma unroll
                for (int k = 0; k < kMaxStr; k++) v[1 + k] = p.status[j].incl_arena[k];
            }
#pragma unroll
            for (int k = 0; k < 1 + kMaxStr; k++) {
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], d);
                pre[k] += v[k];
            }
            if (fi < 32) break;
        }
        if (lane == 0) {
            me->incl_rows = (uint32_t)(pre[0] + tot[0]);
#pragma unroll
            for (int k = 0; k < kMaxStr; k++) me->incl_arena[k] = pre[1 + k] + tot[1 + k];
            st_release(&me->flag, p.epoch * 4 + 2);
            S.row_base = (uint32_t)pre[0];
#pragma unroll
            for (int k = 0; k < kMaxStr; k++) S.arena_base[k] = (uint32_t)pre[1 + k];  // i32 offsets: checked on the host
            if (blk == tc.n_blocks - 1) {
                p.hdr->n_rows = pre[0] + tot[0];
#pragma unroll
                for (int k = 0; k < kMaxStr; k++) p.hdr->arena[k] = pre[1 + k] + tot[1 + k];
                if (p.chunk_out) {
                    p.chunk_out[0] = pre[0] + tot[0];
#pragma unroll
                    for (int k = 0; k < kMaxStr; k++) p.chunk_out[1 + k] = pre[1 + k] + tot[1 + k];
                    p.chunk_out[5] = 1;
                }
            }
        }
    }
    {
        // ---- field-byte and count / sum totals of all the block's records
        // (they need no prefix): warps 1-7 take their own two chunks of 32
        // records (already in registers), then warp 0's two chunks from a
        // shared counter, which warp 0 joins after its look-back (a fixed
        // split of all 16 chunks left two warps a third chunk while the rest
        // waited at the barrier); warp sums into shared memory for the
        // block totals at the end
        StatAcc acc = {};
        uint32_t fb_fields = 0, fb_bytes = 0;  // below 2^32: the input is shorter than 4 GiB
        uint64_t tx_values = 0, tx_bytes = 0, tx_sum = 0;
        if (rs.want_fb || STATS) {
            // (the loop is warp-uniform: a warp's lanes take consecutive
            // records of one chunk, so the field-byte cleaning can use the
            // whole warp)
            for (int it = warp == 0 ? kRecPerThread : 0;; it++) {
                Rec x;
                if (it < kRecPerThread) {
                    x = it ? rec[1] : rec[0];
                } else {
                    uint32_t ch = 0;
                    if (lane == 0) ch = atomicAdd(&S.fb_next, 1u);
                    ch = __shfl_sync(0xffffffffu, ch, 0);
                    if (ch >= (uint32_t)kRecPerThread) break;  // warp 0's chunks
                    x = make_rec<D>(p, tc, W, E, R0, (int)ch * 32 + lane);
                }
                if (STATS && x.row) {
                    acc.records++;
#pragma unroll
                    for (int k = 0; k < 2; k++) {
                        uint32_t a, b;
                        if (W.field(x, rs.stats_field[k], a, b)) stat_value(acc, k, W, a, b);
                    }
                }
                if (rs.want_fb) {
                    if (x.row) fb_fields += x.nf;
                    fb_bytes += warp_field_bytes(W, x, lane);
                }
                if (STATS && rs.want_text) warp_text_cell(W, x, rs.text_field, lane, tx_values, tx_bytes, tx_sum);
            }
        }
        unsigned long long r[14] = {fb_fields,      fb_bytes,       acc.records,    acc.values[0], acc.values[1],
                                    acc.checksum[0], acc.checksum[1], acc.sum_e6[0],  acc.sum_e6[1], acc.inexact[0],
                                    acc.inexact[1],  tx_values,       tx_bytes,       tx_sum};
        if (!STATS) {
            uint32_t f = fb_fields, by = fb_bytes;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                f += __shfl_down_sync(0xffffffffu, f, d);
                by += __shfl_down_sync(0xffffffffu, by, d);
            }
            r[0] = f;
            r[1] = by;
        } else {
#pragma unroll
            for (int k = 0; k < 14; k++) {
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) r[k] += __shfl_down_sync(0xffffffffu, r[k], d);
            }
        }
        if (lane == 0)
            for (int k = 0; k < 14; k++) S.red[warp][k] = r[k];
    }
    __syncthreads();
    const int nred = STATS ? 14 : rs.want_fb ? 2 : 0;  // block totals: st_records .. st_text[2] follow fb

    // ---- cells, column by column
    const uint32_t row_base = S.row_base;
    const uint32_t wrow = S.warp_rows[warp];  // the warp's first row, block-relative
    uint32_t grow[kRecPerThread];             // file row of each record
#pragma unroll
    for (int i = 0; i < kRecPerThread; i++) grow[i] = row_base + wrow + ex[i][0];
    if (rs.rows_cap && blk == 0 && tid == 0)  // string offsets start at 0, rows or not
        for (int c = 0; c < rs.ncols; c++)
            if (rs.type[c] == 3) static_cast<int32_t *>(rs.values[c])[0] = 0;
    uint32_t okm[kRecPerThread] = {0, 0};  // per record: valid columns
    // Records outer, columns inner: a record's fields are picked once, not
    // once per column (1.95 -> 1.88 ms per GiB); one copy of the cell code
    // for both records (a smaller loop body measured faster than the
    // unrolled pair: instruction fetch).
#pragma unroll 1
    for (int i = 0; i < kRecPerThread; i++) {
        const Rec x = i ? rec[1] : rec[0];
        const uint32_t g = i ? grow[1] : grow[0];
        uint32_t okb = 0;  // the record's valid columns
        for (int c = 0; c < rs.ncols; c++) {
            const uint32_t f = rs.field[c], ty = rs.type[c];
            const int k = rs.str_slot[c];
            const uint32_t abase = ty == 3 ? S.arena_base[k] + S.warp_len[warp][k] : 0u;
            if (ty == 3) {
                // strings: every lane takes part (quoted cells are cleaned by
                // the whole warp after the plain copies)
                const uint32_t pos = abase + (i ? pick(ex[1], 1 + k) : pick(ex[0], 1 + k));
                uint32_t a = 0, b = 0, o;
                const bool present = x.row && W.field(x, f, a, b);
                const uint32_t n = b - a;
                uint8_t *arena = rs.str_data[c];
                uint32_t len = 0;
                bool quoted = false;
                const uint8_t *src = nullptr;
                if (present) {
                    src = W.ptr(a, n);
                    quoted = n >= 2 && src[0] == '"' && src[n - 1] == '"';
                    if (!quoted) {
                        if (W.staged(a, n, o) && (uint64_t)pos + n <= rs.str_cap[c]) copy_staged(W.sdata, o, n, arena + pos);
                        else copy_unstaged(src, n, arena, pos, rs.str_cap[c]);
                        len = n;
                    }
                }
                for (uint32_t need = __ballot_sync(0xffffffffu, quoted); need; need &= need - 1) {
                    const int sl = __ffs(need) - 1;
                    const uint8_t *ps = reinterpret_cast<const uint8_t *>(
                        __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(src), sl));
                    const uint32_t cl = warp_clean(ps, __shfl_sync(0xffffffffu, n, sl), arena,
                                                   __shfl_sync(0xffffffffu, pos, sl), rs.str_cap[c], lane);
                    if (lane == sl) len = cl;
                }
                if (x.row && g < rs.rows_cap) static_cast<int32_t *>(rs.values[c])[(uint64_t)g + 1] = (int32_t)(pos + len);
                okb |= (uint32_t)present << c;
                continue;
            }
            if (!x.row) continue;
            uint32_t a = 0, b = 0, o;
            const bool present = W.field(x, f, a, b);
            const uint32_t n = b - a;
            const bool st = present && W.staged(a, n, o);
            const bool store = g < rs.rows_cap;
            bool ok = present;
            if (ty == 1) {
                uint32_t v = 0;
                if (present && !(st && swar_u32(W.sdata, o, n, v))) {
                    const Slow64 r = slow_u32(W.ptr(a, n), n);
                    v = (uint32_t)r.v;
                    ok = r.ok;
                }
                if (store) static_cast<uint32_t *>(rs.values[c])[g] = ok ? v : 0u;
            } else if (ty == 2) {
                uint64_t bits = 0;
                uint32_t m;
                bool neg;
                if (present && !(st && swar_fixed6(W.sdata, o, n, bits, m, neg))) {
                    const Slow64 r = slow_f64(W.ptr(a, n), n);
                    bits = r.v;
                    ok = r.ok;
                }
                if (store) static_cast<uint64_t *>(rs.values[c])[g] = ok ? bits : 0ull;
            } else if (ty == 0) {
                // out of line: the cell loop is instruction-fetch bound, and
                // i64 columns are rarer than u32 / f64 / str
                const Slow64 r = present ? i64_cell(W.sdata, st, o, W.ptr(a, n), n) : Slow64{0, false};
                ok = r.ok;
                if (store) static_cast<int64_t *>(rs.values[c])[g] = ok ? (int64_t)r.v : 0;
            } else {
                ok = present && n > 0;
                if (store) {
                    uint32_t *sp = static_cast<uint32_t *>(rs.values[c]);
                    sp[2 * (uint64_t)g] = ok ? a : 0u;
                    sp[2 * (uint64_t)g + 1] = ok ? b : 0u;
                }
            }
            okb |= (uint32_t)ok << c;
        }
        if (i) okm[1] = okb;
        else okm[0] = okb;
    }
    // ---- validity: the warp's rows are consecutive, at most 64 of them;
    // one 64-bit word per column and warp. With every record a row, record
    // L + 32 i of the warp is its row L + 32 i and the word is two ballots;
    // otherwise rows are ranked within the warp and the bits OR-reduced.
    {
        const uint32_t rm0 = __ballot_sync(0xffffffffu, rec[0].row), rm1 = __ballot_sync(0xffffffffu, rec[1].row);
        const bool dense = (rm0 & rm1) == 0xffffffffu;
        const uint32_t lt = (1u << lane) - 1u;
        const uint32_t r0 = __popc(rm0 & lt), r1 = __popc(rm0) + __popc(rm1 & lt);  // row ranks
        const uint32_t lb = (row_base & 63) + wrow;
        for (int c = 0; c < rs.ncols; c++) {
            uint64_t word;
            if (dense) {
                word = (uint64_t)__ballot_sync(0xffffffffu, (okm[0] >> c) & 1u) |
                       ((uint64_t)__ballot_sync(0xffffffffu, (okm[1] >> c) & 1u) << 32);
            } else {
                uint64_t mine = 0;
                if (rec[0].row) mine |= (uint64_t)((okm[0] >> c) & 1u) << r0;
                if (rec[1].row) mine |= (uint64_t)((okm[1] >> c) & 1u) << r1;
                word = (uint64_t)__reduce_or_sync(0xffffffffu, (uint32_t)mine) |
                       ((uint64_t)__reduce_or_sync(0xffffffffu, (uint32_t)(mine >> 32)) << 32);
            }
            if (lane == 0 && word) {
                atomicOr((unsigned long long *)&S.vbits[c][lb >> 6], (unsigned long long)(word << (lb & 63)));
                if (lb & 63) atomicOr((unsigned long long *)&S.vbits[c][(lb >> 6) + 1],
                                      (unsigned long long)(word >> (64 - (lb & 63))));
            }
        }
    }
    __syncthreads();

    // ---- validity words of the block's rows
    {
        const uint64_t w0 = (uint64_t)row_base >> 6;
        const uint64_t maxw = (rs.rows_cap + 63) / 64;
        for (int i = tid; i < rs.ncols * kRecWords; i += kThreads) {
            const int c = i / kRecWords, wi = i % kRecWords;
            const uint64_t vb = S.vbits[c][wi];
            if (vb && w0 + wi < maxw) atomicOr((unsigned long long *)&rs.valid[c][w0 + wi], (unsigned long long)vb);
        }
    }

    // ---- block totals
    if (tid < nred) {
        unsigned long long t = 0;
        for (int w = 0; w < kWarps; w++) t += S.red[w][tid];
        if (t) {
            if (tid < 2) atomicAdd(tid == 0 ? &p.hdr->fb_fields : &p.hdr->fb_bytes, t);
            else atomicAdd(&p.hdr->st_records + (tid - 2), t);
        }
    }
}

// Persistent launch: CTAs take record blocks from an atomic ticket in the
// header, so every block before the one a CTA holds has been taken by a
// running CTA and its look-back always progresses. The record counts come
// from the index pass's header; a tape larger than the buffers it was
// written to (the index pass bounds its writes) flags ERR_TAPE and the host
// runs both passes again with buffers of the exact size.
template <int D, bool STATS>
__global__ void __launch_bounds__(kThreads, 3) columns_kernel(const __grid_constant__ ColParams p) {
    extern __shared__ __align__(16) uint8_t col_smem_raw[];
    ColSmem &S = *reinterpret_cast<ColSmem *>(col_smem_raw);
    const int tid = threadIdx.x;
    TapeCounts tc;
    if (p.seed_hi) {
        tc.n_ends = p.seed_hi->n_terms;
        tc.n_seps = p.seed_hi->n_struct - p.seed_hi->n_terms;
    } else {
        tc.n_ends = *(volatile const unsigned long long *)&p.hdr->n_terms;
        tc.n_seps = *(volatile const unsigned long long *)&p.hdr->n_struct - tc.n_ends;
    }
    tc.n_recs = tc.n_ends + 1;
    tc.n_blocks = (uint32_t)((tc.n_recs + kRecBlock - 1) / kRecBlock);
    tc.blk_lo = 0;
    if (p.seed_hi && !p.last) tc.n_blocks = (uint32_t)(tc.n_ends / kRecBlock);  // blocks whose records all end here
    if (p.seed_lo) tc.blk_lo = (uint32_t)(p.seed_lo->n_terms / kRecBlock);  // the previous chunk's launch took the blocks before
    if (tc.n_seps > p.seps_cap || tc.n_ends > p.ends_cap) {
        if (tid == 0 && blockIdx.x == 0) atomicOr(&p.hdr->error, ERR_TAPE);
        return;
    }
    unsigned int *ticket = p.ticket ? p.ticket : &p.hdr->col_ticket;
    for (;;) {
        if (tid == 0) S.blk = tc.blk_lo + p.blk0 + atomicAdd(ticket, 1u);
        __syncthreads();  // also: the previous block is done with shared memory
        const uint32_t blk = S.blk;
        if (blk >= tc.n_blocks) break;
        columns_block<D, STATS>(p, tc, S, blk);
    }
}

}  // namespace falx

