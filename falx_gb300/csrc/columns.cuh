// Record-parallel materialisation from the tape.
//
// The index kernel leaves the tape in HBM: separator offsets `seps` and per
// terminated record `(separators before << 32) | terminator offset` in
// `ends` (csv_geo.rs:1838-1849 push_tape). A record's fields are then a
// contiguous run of `seps`, so every record can be decoded independently.
// Three launches, none of which waits on another CTA:
//  1. count: one CTA per 512 consecutive records (two per thread) counts
//     its rows (csv_hash comment records are not rows, csv_hash.rs:1381) and
//     the cleaned bytes of its string cells;
//  2. scan: one CTA turns those per-block sums into exclusive prefixes;
//  3. cells: the same blocks again, now knowing the rows and arena bytes
//     before them, decode their cells (ColumnSink semantics,
//     csv_geo.rs:952-1101; decoders csv_geo.rs:1313-1486,
//     csv_hash.rs:1688-1791), write values, validity, string offsets and
//     bytes, and add their field-byte and count/sum totals
//     (csv_hash.rs:1095-1230, csv_geo.rs:1605-1770).
#pragma once

#include <cstdint>

#include "decimal.cuh"
#include "rows.cuh"
#include "scan_core.cuh"
#include "tile.cuh"

namespace falx {

constexpr int kRecPerThread = 2;
constexpr int kRecBlock = kThreads * kRecPerThread;  // records per CTA
constexpr int kRecWords = kRecBlock / 64 + 1;        // validity words a block's rows can touch
constexpr int kSepWin = 3072;                        // separators staged per CTA
constexpr int kDataWin = 32768;                      // bytes staged per CTA (cells pass)

struct RecSums {  // one per record block: rows and string-arena bytes
    uint32_t rows;
    uint32_t arena[kMaxStr];
    uint32_t pad[3];
};

struct ColParams {
    const uint8_t *data;
    const uint8_t *abase;  // data rounded down to 16 bytes
    uint32_t shift;        // data - abase
    uint64_t len;
    const uint32_t *seps;
    uint64_t n_seps;
    const uint64_t *ends;
    uint64_t n_ends;
    uint64_t n_recs;  // n_ends, plus one for a trailing record without terminator
    RecSums *sums;    // per block: its sums (count), then the sums before it (cells)
    DevHeader *hdr;
    RowSpec rows;
};

// Shared memory of one record block. The tape entries of its records and
// (cells pass) the bytes they span are staged with coalesced loads; what
// does not fit the windows is read from global memory.
struct ColSmem {
    uint64_t ends[kRecBlock + 1];  // ends[r0 - 1 + i]
    uint32_t seps[kSepWin];
    uint32_t warp_rows[kWarps];
    uint32_t warp_len[kWarps][kMaxStr];
    uint32_t row_base;
    uint32_t arena_base[kMaxStr];
    uint64_t sep_lo;
    uint32_t sep_n;
    int64_t data_lo;  // file position of data[0]
    uint32_t data_n;
    uint64_t vbits[kMaxCols][kRecWords];
    unsigned long long red[kWarps][12];
    alignas(16) uint8_t data[kDataWin];  // last: the count pass launches without it
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

struct Rec {
    int64_t start, end;  // [start, end): the record without its terminator
    uint64_t sb;         // index of its first separator in `seps`
    uint32_t nf;         // fields
    bool row;            // a row (inside the file and not a comment)
};

struct ColView {
    const ColParams &p;
    const ColSmem &S;
    __device__ __forceinline__ uint32_t sep(uint64_t i) const {
        const uint64_t j = i - S.sep_lo;
        return j < S.sep_n ? S.seps[j] : p.seps[i];
    }
    __device__ __forceinline__ const uint8_t *bytes(int64_t a, int64_t b) const {
        return (a >= S.data_lo && b <= S.data_lo + (int64_t)S.data_n) ? S.data + (a - S.data_lo) : p.data + a;
    }
    // Field f of a record: [from, to), the last field without a '\r' before
    // the record end (csv_geo.rs:1055-1060).
    __device__ __forceinline__ bool field(const Rec &r, uint32_t f, int64_t &from, int64_t &to) const {
        if (f >= r.nf) return false;
        from = f == 0 ? r.start : (int64_t)sep(r.sb + f - 1) + 1;
        if (f + 1 < r.nf) {
            to = (int64_t)sep(r.sb + f);
        } else {
            to = r.end;
            if (to > r.start && bytes(to - 1, to)[0] == '\r') to--;
        }
        return true;
    }
};

// Common cell shapes, decoded inline; anything else goes to the general
// decoders (kept out of line so the per-cell loop stays small). A fast path
// that accepts a cell gives exactly the general decoder's value.

// 1-9 plain digits.
__device__ __forceinline__ bool fast_u32(const uint8_t *s, uint32_t n, uint32_t &v) {
    if (n == 0 || n > 9) return false;
    uint32_t x = 0;
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t d = (uint32_t)s[k] - '0';
        if (d > 9) return false;
        x = x * 10 + d;
    }
    v = x;
    return true;
}

// [+-]?d{1,3}.d{6}: m / 1e6 correctly rounded (csv_geo.rs:1414-1475).
__device__ __forceinline__ bool fast_fixed6(const uint8_t *s, uint32_t n, uint64_t &bits) {
    if (n < 8 || n > 11) return false;
    const uint8_t c0 = s[0];
    const uint32_t i = (c0 == '-' || c0 == '+') ? 1u : 0u;
    if (n - i < 8 || n - i > 10 || s[n - 7] != '.') return false;
    uint32_t frac = 0, ip = 0;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const uint32_t d = (uint32_t)s[n - 6 + k] - '0';
        if (d > 9) return false;
        frac = frac * 10 + d;
    }
    for (uint32_t k = i; k + 7 < n; k++) {
        const uint32_t d = (uint32_t)s[k] - '0';
        if (d > 9) return false;
        ip = ip * 10 + d;
    }
    bits = dec::eisel_lemire((uint64_t)ip * 1000000u + frac, -6) | ((uint64_t)(c0 == '-') << 63);
    return true;
}

__device__ __noinline__ bool slow_i64(const uint8_t *s, uint32_t n, int64_t &v) {
    return dec::numeric_view(s, n) && dec::parse_i64(s, n, v);
}
__device__ __noinline__ bool slow_u32(const uint8_t *s, uint32_t n, uint32_t &v) {
    return dec::numeric_view(s, n) && dec::parse_u32(s, n, v);
}
__device__ __noinline__ bool slow_f64(const uint8_t *s, uint32_t n, uint64_t &bits) {
    double v;
    if (!(dec::numeric_view(s, n) && dec::parse_f64(s, n, v))) return false;
    bits = dec::d2u(v);
    return true;
}

// Count / sum of one f64 cell (csv_geo.rs:1735-1750): values, bit checksum,
// exact x1e6 sum. The fixed shape needs no general decoder.
__device__ __noinline__ void stat_slow(StatAcc &a, int k, const uint8_t *s, uint32_t n) { stat_cell(a, k, s, n); }
__device__ __forceinline__ void stat_value(StatAcc &a, int k, const uint8_t *s, uint32_t n) {
    uint64_t bits;
    if (fast_fixed6(s, n, bits)) {
        // d{1,3}.d{6} is exact in micro-units: +-(ip * 1e6 + frac)
        const uint32_t i = (s[0] == '-' || s[0] == '+') ? 1u : 0u;
        int64_t e6 = 0;
        for (uint32_t q = i; q < n; q++)
            if (s[q] != '.') e6 = e6 * 10 + (s[q] - '0');
        a.values[k]++;
        a.checksum[k] += bits;
        a.sum_e6[k] += (unsigned long long)(s[0] == '-' ? -e6 : e6);
        return;
    }
    stat_slow(a, k, s, n);
}

// A string cell's cleaned bytes into the arena at `at` (bounded by cap);
// returns the cleaned length. Unquoted cells are copied with byte stores up
// to a 4-byte boundary of the destination and word stores after it.
__device__ __forceinline__ uint32_t copy_cell(const uint8_t *s, uint32_t n, uint8_t *arena, uint64_t at,
                                              uint64_t cap) {
    if ((n >= 2 && s[0] == '"' && s[n - 1] == '"') || at + n > cap) return copy_clean(s, n, arena, at, cap);
    uint8_t *dst = arena + at;
    uint32_t i = 0;
    const uint32_t head = (uint32_t)((4 - ((uintptr_t)dst & 3)) & 3);
    for (; i < head && i < n; i++) dst[i] = s[i];
    for (; i + 4 <= n; i += 4)
        *reinterpret_cast<uint32_t *>(dst + i) = (uint32_t)s[i] | ((uint32_t)s[i + 1] << 8) |
                                                 ((uint32_t)s[i + 2] << 16) | ((uint32_t)s[i + 3] << 24);
    for (; i < n; i++) dst[i] = s[i];
    return n;
}

// A non-string cell (I64, U32, F64, BYTES) of row g: stores the value (a
// zero placeholder when invalid) and returns its validity.
__device__ __forceinline__ bool decode_value(const RowSpec &rs, int c, uint64_t g, const uint8_t *s, uint32_t n,
                                             bool present, int64_t from, int64_t to) {
    const uint32_t ty = rs.type[c];
    const bool store = g < rs.rows_cap;
    bool ok = false;
    if (ty == 0) {
        int64_t v = 0;
        if (present) ok = slow_i64(s, n, v);
        if (store) static_cast<int64_t *>(rs.values[c])[g] = ok ? v : 0;
    } else if (ty == 1) {
        uint32_t v = 0;
        if (present) ok = fast_u32(s, n, v) || slow_u32(s, n, v);
        if (store) static_cast<uint32_t *>(rs.values[c])[g] = ok ? v : 0u;
    } else if (ty == 2) {
        uint64_t bits = 0;
        if (present) ok = fast_fixed6(s, n, bits) || slow_f64(s, n, bits);
        if (store) static_cast<uint64_t *>(rs.values[c])[g] = ok ? bits : 0ull;
    } else {
        ok = present && n > 0;
        if (store) {
            uint32_t *sp = static_cast<uint32_t *>(rs.values[c]);
            sp[2 * g] = ok ? (uint32_t)from : 0u;
            sp[2 * g + 1] = ok ? (uint32_t)to : 0u;
        }
    }
    return ok;
}

template <int D, bool COUNT>
__global__ void __launch_bounds__(kThreads) columns_kernel(const __grid_constant__ ColParams p) {
    extern __shared__ __align__(16) uint8_t col_smem_raw[];
    ColSmem &S = *reinterpret_cast<ColSmem *>(col_smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const RowSpec &rs = p.rows;
    const uint32_t blk = blockIdx.x;
    const uint64_t R0 = (uint64_t)blk * kRecBlock;
    if (!COUNT)
        for (int i = tid; i < rs.ncols * kRecWords; i += kThreads) S.vbits[i / kRecWords][i % kRecWords] = 0;

    // ---- stage the tape entries of the block's records
    for (int i = tid; i <= kRecBlock; i += kThreads) {
        const int64_t e = (int64_t)R0 - 1 + i;
        if (e >= 0 && (uint64_t)e < p.n_ends) cp_async_ca<8>(&S.ends[i], p.ends + e);
    }
    cp_async_wait_all();
    __syncthreads();
    if (tid == 0) {
        // separator and byte windows: from the block's first record to its last
        const uint64_t last = (R0 + kRecBlock < p.n_recs ? R0 + kRecBlock : p.n_recs) - 1;
        const uint64_t sb = R0 == 0 ? 0 : S.ends[0] >> 32;
        const uint64_t se = last < p.n_ends ? S.ends[last - R0 + 1] >> 32 : p.n_seps;
        S.sep_lo = sb;
        S.sep_n = (uint32_t)(se - sb < (uint64_t)kSepWin ? se - sb : (uint64_t)kSepWin);
        const int64_t lo = R0 == 0 ? 0 : (int64_t)(uint32_t)S.ends[0] + 1;
        const int64_t hi = last < p.n_ends ? (int64_t)(uint32_t)S.ends[last - R0 + 1] : (int64_t)p.len;
        const int64_t q0 = (lo + p.shift) & ~15ll;  // 16-byte aligned address offset
        const int64_t qend = (int64_t)((p.shift + p.len + 15) & ~15ull);
        int64_t qn = ((hi + p.shift + 15) & ~15ll) - q0;
        if (qn > qend - q0) qn = qend - q0;
        if (qn > kDataWin) qn = kDataWin;
        if (qn < 0) qn = 0;
        S.data_lo = q0 - p.shift;
        S.data_n = COUNT ? 0u : (uint32_t)qn;  // the count pass reads its few bytes in place
    }
    __syncthreads();
    for (uint32_t i = tid; i < S.sep_n; i += kThreads) cp_async_ca<4>(&S.seps[i], p.seps + S.sep_lo + i);
    if (!COUNT) {
        const uint8_t *src = p.abase + (S.data_lo + p.shift);
        for (uint32_t i = tid; i < S.data_n / 16; i += kThreads) cp_async_ca<16>(S.data + 16 * i, src + 16 * i);
    }
    cp_async_wait_all();
    __syncthreads();
    const ColView V{p, S};

    // ---- this thread's records
    Rec rec[kRecPerThread];
    uint32_t my_rows = 0;
#pragma unroll
    for (int i = 0; i < kRecPerThread; i++) {
        const uint64_t r = R0 + (uint64_t)tid * kRecPerThread + i;
        const int li = tid * kRecPerThread + i;  // S.ends[li] = ends[r - 1]
        Rec &x = rec[i];
        x.row = false;
        x.nf = 0;
        if (r >= p.n_recs) continue;
        const uint64_t pe = r == 0 ? 0ull : S.ends[li];
        x.start = r == 0 ? 0 : (int64_t)(uint32_t)pe + 1;
        x.sb = r == 0 ? 0 : pe >> 32;
        // after the last terminator there is a record only if bytes remain
        // (csv_geo.rs:1094-1100)
        if (r >= p.n_ends && x.start >= (int64_t)p.len) continue;
        uint64_t se;
        if (r < p.n_ends) {
            const uint64_t e = S.ends[li + 1];
            x.end = (int64_t)(uint32_t)e;
            se = e >> 32;
        } else {
            x.end = (int64_t)p.len;
            se = p.n_seps;
        }
        x.nf = (uint32_t)(se - x.sb) + 1;
        x.row = !(D == D_CSV_HASH && x.start < x.end && V.bytes(x.start, x.start + 1)[0] == '#');
        my_rows += x.row;
    }

    // ---- string cell lengths
    uint32_t slen[kMaxStr] = {0, 0, 0, 0};
    for (int c = 0; c < rs.ncols; c++) {
        if (rs.type[c] != 3) continue;
        const int k = rs.str_slot[c];
#pragma unroll
        for (int i = 0; i < kRecPerThread; i++) {
            int64_t a, b;
            if (rec[i].row && V.field(rec[i], rs.field[c], a, b)) slen[k] += cleaned_len(V.bytes(a, b), (uint32_t)(b - a));
        }
    }

    // ---- block scan of (rows, string bytes)
    uint32_t v[1 + kMaxStr] = {my_rows, slen[0], slen[1], slen[2], slen[3]};
    uint32_t ex[1 + kMaxStr];
#pragma unroll
    for (int k = 0; k < 1 + kMaxStr; k++) {
        uint32_t x = v[k];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += o;
        }
        ex[k] = x - v[k];
        if (lane == 31) {
            if (k == 0) S.warp_rows[warp] = x;
            else S.warp_len[warp][k - 1] = x;
        }
    }
    __syncthreads();
    if (warp == 0) {
        // warp prefixes and block totals
#pragma unroll
        for (int k = 0; k < 1 + kMaxStr; k++) {
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
            if (COUNT && lane == 31) {
                if (k == 0) p.sums[blk].rows = x;
                else p.sums[blk].arena[k - 1] = x;
            }
        }
        if (!COUNT && lane == 0) {
            S.row_base = p.sums[blk].rows;
#pragma unroll
            for (int k = 0; k < kMaxStr; k++) S.arena_base[k] = p.sums[blk].arena[k];
        }
    }
    if (COUNT) return;
    __syncthreads();

    // ---- cells of this thread's rows
    const uint32_t row_base = S.row_base;
    const uint32_t vshift = row_base & 63;
    uint32_t lrow = S.warp_rows[warp] + ex[0];  // row of the block's rows, block-relative
    uint64_t at[kMaxStr];
#pragma unroll
    for (int k = 0; k < kMaxStr; k++) at[k] = (uint64_t)S.arena_base[k] + S.warp_len[warp][k] + ex[1 + k];
    StatAcc acc = {};
    if (rs.rows_cap && blk == 0 && tid == 0)  // string offsets start at 0, rows or not
        for (int c = 0; c < rs.ncols; c++)
            if (rs.type[c] == 3) static_cast<int32_t *>(rs.values[c])[0] = 0;
    const uint32_t lrow0 = lrow;
    uint32_t okm[kRecPerThread] = {0, 0};  // per record: valid columns
#pragma unroll
    for (int i = 0; i < kRecPerThread; i++) {
        const Rec &x = rec[i];
        if (!x.row) continue;
        const uint64_t g = (uint64_t)row_base + lrow;
        for (int c = 0; c < rs.ncols; c++) {
            int64_t a = 0, b = 0;
            const bool present = V.field(x, rs.field[c], a, b);
            const uint32_t n = (uint32_t)(b - a);
            bool ok;
            if (rs.type[c] == 3) {
                const int k = rs.str_slot[c];
                ok = present;
                if (present) at[k] += copy_cell(V.bytes(a, b), n, rs.str_data[c], at[k], rs.str_cap[c]);
                if (g < rs.rows_cap) static_cast<int32_t *>(rs.values[c])[g + 1] = (int32_t)at[k];
            } else {
                ok = decode_value(rs, c, g, present ? V.bytes(a, b) : nullptr, n, present, a, b);
            }
            okm[i] |= (uint32_t)ok << c;
        }
        if (rs.want_stats) {
            acc.records++;
            for (int k = 0; k < 2; k++) {
                int64_t a, b;
                if (V.field(x, rs.stats_field[k], a, b)) stat_value(acc, k, V.bytes(a, b), (uint32_t)(b - a));
            }
        }
        if (rs.want_fb) {
            for (uint32_t f = 0; f < x.nf; f++) {
                int64_t a, b;
                V.field(x, f, a, b);
                acc.fields++;
                acc.bytes += cleaned_len(V.bytes(a, b), (uint32_t)(b - a));
            }
        }
        lrow++;
    }
    // validity: the warp's rows are consecutive, at most 64 of them; one
    // 64-bit word per column per warp, OR-reduced across the lanes
    {
        const uint32_t wr = S.warp_rows[warp];  // the warp's first row, block-relative
        const uint32_t ro = lrow0 - wr;         // this lane's first row within the warp
        for (int c = 0; c < rs.ncols; c++) {
            uint64_t mine = 0;
            uint32_t k = 0;
#pragma unroll
            for (int i = 0; i < kRecPerThread; i++) {
                if (!rec[i].row) continue;
                mine |= (uint64_t)((okm[i] >> c) & 1u) << (ro + k);
                k++;
            }
            const uint32_t lo = __reduce_or_sync(0xffffffffu, (uint32_t)mine);
            const uint32_t hi = __reduce_or_sync(0xffffffffu, (uint32_t)(mine >> 32));
            if (lane == 0 && (lo | hi)) {
                const uint64_t word = (uint64_t)lo | ((uint64_t)hi << 32);
                const uint32_t lb = vshift + wr;
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

    // ---- field bytes and count / sum totals
    if (rs.want_fb || rs.want_stats) {
        unsigned long long r[11] = {acc.fields, acc.bytes, acc.records, acc.values[0], acc.values[1],
                                    acc.checksum[0], acc.checksum[1], acc.sum_e6[0], acc.sum_e6[1],
                                    acc.inexact[0], acc.inexact[1]};
#pragma unroll
        for (int k = 0; k < 11; k++) {
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) r[k] += __shfl_down_sync(0xffffffffu, r[k], d);
            if (lane == 0) S.red[warp][k] = r[k];
        }
        __syncthreads();
        if (tid < 11) {
            unsigned long long t = 0;
            for (int w = 0; w < kWarps; w++) t += S.red[w][tid];
            if (t) {
                if (tid < 2) atomicAdd(tid == 0 ? &p.hdr->fb_fields : &p.hdr->fb_bytes, t);
                else atomicAdd(&p.hdr->st_records + (tid - 2), t);
            }
        }
    }
}

}  // namespace falx

namespace falx {

// Exclusive prefixes of the per-block sums, and the totals. One CTA of
// 1024 threads; warp w owns a contiguous run of blocks and reads it 32
// entries at a time (coalesced): first its total, then, after a scan of the
// 32 totals, the prefixes.
__global__ void __launch_bounds__(1024) columns_scan(RecSums *sums, uint32_t n, DevHeader *hdr) {
    __shared__ unsigned long long wsum[32][1 + kMaxStr];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t per = (n + 31) / 32, lo = min(n, warp * per), hi = min(n, lo + per);
    unsigned long long tot[1 + kMaxStr] = {0, 0, 0, 0, 0};
    for (uint32_t i = lo + lane; i < hi; i += 32) {
        const RecSums v = sums[i];
        tot[0] += v.rows;
#pragma unroll
        for (int k = 0; k < kMaxStr; k++) tot[1 + k] += v.arena[k];
    }
#pragma unroll
    for (int k = 0; k < 1 + kMaxStr; k++) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) tot[k] += __shfl_xor_sync(0xffffffffu, tot[k], d);
        if (lane == 0) wsum[warp][k] = tot[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < 1 + kMaxStr; k++) {
            const unsigned long long w = wsum[lane][k];
            unsigned long long x = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long o = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += o;
            }
            wsum[lane][k] = x - w;
            if (lane == 31) {
                if (k == 0) hdr->n_rows = x;
                else hdr->arena[k - 1] = x;
            }
        }
    }
    __syncthreads();
    unsigned long long carry[1 + kMaxStr];
#pragma unroll
    for (int k = 0; k < 1 + kMaxStr; k++) carry[k] = wsum[warp][k];
    for (uint32_t i0 = lo; i0 < hi; i0 += 32) {
        const uint32_t i = i0 + lane;
        RecSums v = {};
        if (i < hi) v = sums[i];
        uint32_t val[1 + kMaxStr] = {v.rows, v.arena[0], v.arena[1], v.arena[2], v.arena[3]};
#pragma unroll
        for (int k = 0; k < 1 + kMaxStr; k++) {
            unsigned long long x = val[k];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long o = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += o;
            }
            const unsigned long long ex = carry[k] + x - val[k];
            carry[k] += __shfl_sync(0xffffffffu, x, 31);
            if (i < hi) {
                if (k == 0) sums[i].rows = (uint32_t)ex;
                else sums[i].arena[k - 1] = (uint32_t)ex;
            }
        }
    }
}

}  // namespace falx
