// Row phase of the tile scan: record walking, typed column decode, field-byte
// and count/sum sinks, string arenas.
//
// Record ownership: a tile owns the records that START inside it (record
// starts are file position 0 and the byte after every structural newline;
// csv_hash records whose first byte is '#' are comments and are skipped,
// csv_hash.rs:1381). The record crossing the tile end continues into a halo
// staged with the tile; a record longer than the halo continues through a
// byte-serial walk of global memory from the halo's exit state. This gives
// each record exactly one owner, like the reference's terminator-ownership
// rule for its chunked drivers (csv_geo.rs:952-1000), and the rows come out
// in file order.
#pragma once
#include "decimal.cuh"
#include "scan_core.cuh"

namespace falx {

constexpr int kMaxStr = 4;          // string columns with an arena per call
constexpr int kHaloBytes = 1024;    // bytes staged after each tile
constexpr int kMaxCols = 32;
constexpr int kLocalRows = 1024;    // rows per tile with shared-memory validity staging
constexpr int kVWords = kLocalRows / 64 + 2;
constexpr int kRowCap = kLocalRows; // rows per tile on the data-parallel path
constexpr int kTermCap = 2048;      // terminators per tile (+ halo) on the data-parallel path
constexpr int kStageCap = 4096;     // staged structurals of the tile itself (the halo adds up to kHaloBytes)

struct RowSpec {
    int ncols;
    int nstr;
    uint32_t max_field;  // 1 + largest declared field index (0 = none)
    uint64_t rows_cap;
    uint32_t field[kMaxCols];
    uint32_t type[kMaxCols];
    int32_t str_slot[kMaxCols];
    void *values[kMaxCols];
    uint64_t *valid[kMaxCols];
    uint8_t *str_data[kMaxCols];
    uint64_t str_cap[kMaxCols];
    int want_fb;
    int want_stats;
    uint32_t stats_field[2];
    int want_text;        // City text lane (with want_stats): values, cleaned bytes, byte checksum
    uint32_t text_field;
};

template <bool ROWS>
struct RowShared {};

template <>
struct RowShared<true> {
    uint64_t vbits[kMaxCols][kVWords];
    uint32_t colmask[64];      // declared columns per field ordinal (< 64)
    uint32_t high_fields;      // a declared field ordinal is >= 64
    uint32_t n_halo;
    uint32_t halo_kind;        // 0 terminated inside the halo, 1 ends at EOF, 2 continues past it
    uint32_t halo_exit;
    unsigned long long red[kWarps][12];
    uint32_t warp_len[kWarps][kMaxStr];
    uint32_t arena_base[kMaxStr];
    uint32_t tile_len[kMaxStr];
    // data-parallel path: per row its start (tile-relative), its first
    // structural and its terminator ordinal; per terminator its structural
    uint16_t row_pos[kRowCap];
    uint16_t row_k[kRowCap];
    uint16_t row_t[kRowCap];
    uint16_t term_k[kTermCap];
    uint32_t fast;
};

struct RowCtx {
    int64_t vs;          // file position of the tile's first byte
    int64_t len;
    uint8_t *buf;        // buf[kPre] holds position vs
    int64_t buf_end;     // file position one past the staged bytes
    uint32_t n_tile;     // staged structurals that belong to the tile
    uint32_t row_base;   // global index of the tile's first row
    uint32_t exit_state; // region state at the tile end
    uint32_t tile;
    uint32_t epoch;
    const uint8_t *data;
    void *astatus;
    unsigned long long *hdr_arena;
    unsigned long long *hdr_fb;  // fields, bytes
    unsigned long long *hdr_st;  // records, values[2], checksum[2], sum_e6[2], inexact[2]
    uint32_t *hdr_error;
    uint32_t *hdr_abort;
    bool last_tile;
};

struct ArenaStatusView {
    uint32_t flag;
    uint32_t pad[3];
    uint32_t agg[kMaxStr];
    uint32_t incl[kMaxStr];
};

// Byte-serial automaton used past the halo (scalar.rs:23-59 semantics).
template <int D>
__device__ __forceinline__ bool serial_step(uint8_t c, uint32_t &s, bool &ls) {
    bool st = false;
    if (D == D_TSV) {
        st = c == '\t' || c == '\n';
    } else if (D == D_CSV) {
        if (c == '"') s ^= 1;
        else if (!s && (c == ',' || c == '\n')) st = true;
    } else if (D == D_CSV_HASH) {
        if (s == R_C) {
            if (c == '\n') { s = R_N; st = true; }
        } else if (c == '"') {
            s = s == R_Q ? R_N : R_Q;
        } else if (s == R_N && c == '#' && ls) {
            s = R_C;
        } else if (s == R_N && (c == ',' || c == '\n')) {
            st = true;
        }
        ls = c == '\n';
    } else {
        uint32_t e = s & 1, p = s >> 1;
        if (c == '"' && !e) p ^= 1;
        else if (!p && (c == '\n' || (D == D_LOGFMT && (c == ' ' || c == '=')))) st = true;
        e = (c == '\\') ? (e ^ 1) : 0;
        s = e | (p << 1);
    }
    return st;
}

// Cleaned length of a raw field (csv_hash.rs:1207-1230).
__device__ __forceinline__ uint32_t cleaned_len(const uint8_t *s, uint32_t len) {
    if (len >= 2 && s[0] == '"' && s[len - 1] == '"') {
        uint32_t il = len - 2, o = 0, i = 0;
        const uint8_t *in = s + 1;
        while (i < il) {
            o++;
            i += (in[i] == '"' && i + 1 < il && in[i + 1] == '"') ? 2 : 1;
        }
        return o;
    }
    return len;
}

// Append the cleaned field to `dst` (csv_hash.rs:1749-1782); `cap` bounds it.
// Copies the cleaned bytes of a raw field to dst[at..] (bounded by cap)
// and returns the cleaned length.
__device__ __forceinline__ uint32_t copy_clean(const uint8_t *s, uint32_t len, uint8_t *dst, uint64_t at,
                                               uint64_t cap) {
    if (len >= 2 && s[0] == '"' && s[len - 1] == '"') {
        uint32_t il = len - 2, i = 0, o = 0;
        const uint8_t *in = s + 1;
        while (i < il) {
            if (at + o < cap) dst[at + o] = in[i];
            o++;
            i += (in[i] == '"' && i + 1 < il && in[i + 1] == '"') ? 2 : 1;
        }
        return o;
    }
    for (uint32_t i = 0; i < len; i++)
        if (at + i < cap) dst[at + i] = s[i];
    return len;
}

struct StatAcc {
    unsigned long long fields, bytes, records, values[2], checksum[2], sum_e6[2], inexact[2];
};

// Walks one record: yields fields as (ordinal, from, to) spans.
template <int D>
struct Walker {
    const uint16_t *stage;
    uint32_t k, n_total;
    int64_t vs, len;
    uint32_t halo_kind, halo_exit;
    int64_t halo_end;
    const uint8_t *data;
    bool serial = false;
    int64_t sp;      // serial position
    uint32_t ss;     // serial state
    bool sls;        // serial line-start

    // Next structural of the record: returns false at EOF (no terminator).
    __device__ __forceinline__ bool next(int64_t &pos, bool &is_term) {
        if (!serial) {
            if (k < n_total) {
                uint16_t e = stage[k++];
                pos = vs + (e & 0x7FFF);
                is_term = e >> 15;
                return true;
            }
            if (halo_kind != 2) return false;
            serial = true;
            sp = halo_end;
            ss = halo_exit;
            sls = data[halo_end - 1] == '\n';
        }
        while (sp < len) {
            uint8_t c = data[sp];
            bool st = serial_step<D>(c, ss, sls);
            int64_t p = sp++;
            if (st) {
                pos = p;
                is_term = c == '\n';
                return true;
            }
        }
        return false;
    }
};

__device__ __forceinline__ const uint8_t *cell_ptr(const RowCtx &rc, int64_t a, int64_t b) {
    const int64_t lo = rc.vs - kPre;
    if (a >= lo && b <= rc.buf_end) return rc.buf + (a - lo);
    return rc.data + a;
}

// Decode one present or missing column cell of row g.
__device__ __forceinline__ bool decode_cell(const RowSpec &rs, int c, uint64_t g, const uint8_t *s, uint32_t n,
                                            bool present, int64_t from, int64_t to, uint32_t (&slen)[kMaxStr]) {
    const uint32_t ty = rs.type[c];
    bool ok = false;
    const bool store = g < rs.rows_cap;
    if (ty == 0) {  // I64
        int64_t v = 0;
        if (present) {
            const uint8_t *p = s;
            uint32_t l = n;
            ok = dec::numeric_view(p, l) && dec::parse_i64(p, l, v);
        }
        if (store) static_cast<int64_t *>(rs.values[c])[g] = ok ? v : 0;
    } else if (ty == 1) {  // U32
        uint32_t v = 0;
        if (present) {
            const uint8_t *p = s;
            uint32_t l = n;
            ok = dec::numeric_view(p, l) && dec::parse_u32(p, l, v);
        }
        if (store) static_cast<uint32_t *>(rs.values[c])[g] = ok ? v : 0u;
    } else if (ty == 2) {  // F64
        double v = 0.0;
        if (present) {
            const uint8_t *p = s;
            uint32_t l = n;
            ok = dec::numeric_view(p, l) && dec::parse_f64(p, l, v);
        }
        if (store) static_cast<double *>(rs.values[c])[g] = ok ? v : 0.0;
    } else if (ty == 3) {  // STR: length now, bytes in the arena pass
        ok = present;
        if (present) slen[rs.str_slot[c]] += cleaned_len(s, n);
    } else {  // BYTES
        ok = present && n > 0;
        if (store) {
            uint32_t *sp = static_cast<uint32_t *>(rs.values[c]);
            sp[2 * g] = ok ? (uint32_t)from : 0u;
            sp[2 * g + 1] = ok ? (uint32_t)to : 0u;
        }
    }
    return ok;
}

__device__ __forceinline__ void stat_cell(StatAcc &a, int k, const uint8_t *s, uint32_t n) {
    const uint8_t *p = s;
    uint32_t l = n;
    double v;
    if (!dec::numeric_view(p, l) || !dec::parse_f64(p, l, v)) return;
    a.values[k]++;
    a.checksum[k] += dec::d2u(v);
    int64_t e6;
    if (dec::exact_e6(p, l, e6)) a.sum_e6[k] += (unsigned long long)e6;
    else a.inexact[k]++;
}

// String-arena look-back (one warp): returns, for each string column slot,
// the arena bytes of the file before this tile; publishes the tile's totals.
__device__ inline void arena_lookback(const RowCtx &rc, const uint32_t (&tot)[kMaxStr], int lane,
                               unsigned long long (&pre)[kMaxStr]) {
    ArenaStatusView *as = static_cast<ArenaStatusView *>(rc.astatus);
    ArenaStatusView *me = &as[rc.tile];
    if (lane == 0) {
        for (int k = 0; k < kMaxStr; k++) me->agg[k] = tot[k];
        st_release(&me->flag, rc.epoch * 4 + 1);
    }
    __syncwarp();
    for (int k = 0; k < kMaxStr; k++) pre[k] = 0;
    const uint64_t t0 = globaltimer_ns();
    for (int64_t hi = (int64_t)rc.tile - 1; hi >= 0; hi -= 32) {
        const int64_t j = hi - lane;
        const bool in = j >= 0;
        uint32_t flag = 0, ball_incl = 0;
        bool gave_up = false;
        for (uint32_t it = 0;; it++) {
            if (in) flag = ld_acquire(&as[j].flag);
            const bool cur = (flag >> 2) == rc.epoch;
            const uint32_t not_ready = __ballot_sync(0xffffffffu, in && !(cur && (flag & 3) >= 1));
            ball_incl = __ballot_sync(0xffffffffu, in && cur && (flag & 3) == 2);
            const int first_incl = ball_incl ? __ffs(ball_incl) - 1 : 32;
            const int first_wait = not_ready ? __ffs(not_ready) - 1 : 32;
            if (first_wait > first_incl || not_ready == 0) break;
            if ((it & 63) == 63) {
                const bool stop = lane == 0 && (*(volatile uint32_t *)rc.hdr_abort ||
                                                globaltimer_ns() - t0 > 4000000000ull);
                if (__any_sync(0xffffffffu, stop)) {
                    gave_up = true;
                    break;
                }
            }
            __nanosleep(32);
        }
        if (gave_up) {
            if (lane == 0) {
                atomicOr(rc.hdr_error, 1u);
                atomicExch(rc.hdr_abort, 1u);
            }
            break;
        }
        const int sidx = ball_incl ? __ffs(ball_incl) - 1 : 32;
        for (int k = 0; k < kMaxStr; k++) {
            uint32_t v = 0;
            if (in && lane < sidx) v = ld_relaxed(&as[j].agg[k]);
            else if (in && lane == sidx) v = ld_relaxed(&as[j].incl[k]);
            unsigned long long vv = v;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) vv += __shfl_xor_sync(0xffffffffu, vv, d);
            pre[k] += vv;
        }
        if (ball_incl) break;
    }
    if (lane == 0) {
        bool over = false;
        for (int k = 0; k < kMaxStr; k++) {
            const unsigned long long inc = pre[k] + tot[k];
            if (inc > 0x7FFFFFFFull) over = true;
            me->incl[k] = (uint32_t)inc;
        }
        st_release(&me->flag, rc.epoch * 4 + 2);
        if (over) atomicOr(rc.hdr_error, 2u);
        if (rc.last_tile)
            for (int k = 0; k < kMaxStr; k++) rc.hdr_arena[k] = pre[k] + tot[k];
    }
}

// Block reduction of the sink accumulators into the call totals.
__device__ inline void reduce_sinks(const RowSpec &rs, const RowCtx &rc, RowShared<true> &sh, const StatAcc &acc, int tid) {
    const int lane = tid & 31, warp = tid >> 5;
    unsigned long long v[11] = {acc.fields, acc.bytes, acc.records, acc.values[0], acc.values[1],
                                acc.checksum[0], acc.checksum[1], acc.sum_e6[0], acc.sum_e6[1],
                                acc.inexact[0], acc.inexact[1]};
#pragma unroll
    for (int k = 0; k < 11; k++) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], d);
        if (lane == 0) sh.red[warp][k] = v[k];
    }
    __syncthreads();
    if (tid < 11) {
        unsigned long long t = 0;
        for (int w = 0; w < kWarps; w++) t += sh.red[w][tid];
        if (t) {
            if (tid < 2) atomicAdd(&rc.hdr_fb[tid], t);
            else atomicAdd(&rc.hdr_st[tid - 2], t);
        }
    }
}

// Span of field `f` of row `r` on the data-parallel path.
struct Cell {
    int64_t from, to;
    bool present;
};

__device__ __forceinline__ Cell cell_span(const RowCtx &rc, const RowShared<true> &sh, const uint16_t *stage,
                                          uint32_t n_total, uint32_t n_term_all, uint32_t r, uint32_t f) {
    Cell c;
    const uint32_t k0 = sh.row_k[r];
    const uint32_t t = sh.row_t[r];
    const bool closed = t < n_term_all;
    const uint32_t kt = closed ? sh.term_k[t] : n_total;  // EOF rows: all remaining entries are separators
    const uint32_t nf = kt - k0 + (closed ? 1 : 1);
    const int64_t row0 = rc.vs + sh.row_pos[r];
    c.present = f < nf;
    if (!c.present) {
        c.from = c.to = 0;
        return c;
    }
    c.from = f == 0 ? row0 : rc.vs + (stage[k0 + f - 1] & 0x7FFF) + 1;
    if (f + 1 == nf) {
        int64_t to = closed ? rc.vs + (stage[kt] & 0x7FFF) : rc.len;
        if (to > c.from && cell_ptr(rc, to - 1, to)[0] == '\r') to--;
        c.to = to;
    } else {
        c.to = rc.vs + (stage[k0 + f] & 0x7FFF);
    }
    return c;
}

// Data-parallel row phase for ordinary tiles: the work is spread over
// (row, column) cells and structural entries instead of per-thread walks.
template <int D>
__device__ void rows_fast(const RowSpec &rs, const RowCtx &rc, RowShared<true> &sh, const uint16_t *stage,
                          uint32_t nrows, uint32_t nterm_tile, bool tile_rec0, int tid) {
    const int lane = tid & 31, warp = tid >> 5;
    const uint32_t n_total = rc.n_tile + sh.n_halo;
    const bool last_open = nrows > 0 && sh.row_t[nrows - 1] == nterm_tile;
    const uint32_t n_term_all = nterm_tile + (last_open && sh.halo_kind == 0 ? 1u : 0u);
    const uint32_t vshift = rc.row_base & 63;
    StatAcc acc = {};

    // ---- string lengths: thread t owns rows [t*chunk, (t+1)*chunk)
    const uint32_t chunk = (nrows + kThreads - 1) / kThreads;
    const uint32_t r0 = min(nrows, tid * chunk), r1 = min(nrows, r0 + chunk);
    uint32_t slen[kMaxStr] = {0, 0, 0, 0};
    if (rs.nstr > 0) {
        for (int c = 0; c < rs.ncols; c++) {
            if (rs.type[c] != 3) continue;
            const int k = rs.str_slot[c];
            for (uint32_t r = r0; r < r1; r++) {
                const Cell cl = cell_span(rc, sh, stage, n_total, n_term_all, r, rs.field[c]);
                if (cl.present) slen[k] += cleaned_len(cell_ptr(rc, cl.from, cl.to), (uint32_t)(cl.to - cl.from));
            }
        }
        for (int k = 0; k < kMaxStr; k++) {
            uint32_t x = slen[k], xi = x;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t o = __shfl_up_sync(0xffffffffu, xi, d);
                if (lane >= d) xi += o;
            }
            if (lane == 31) sh.warp_len[warp][k] = xi;
            slen[k] = xi - x;  // exclusive within the warp
        }
        __syncthreads();
        if (tid == 0) {
            for (int k = 0; k < kMaxStr; k++) {
                uint32_t run = 0;
                for (int w = 0; w < kWarps; w++) {
                    uint32_t t = sh.warp_len[w][k];
                    sh.warp_len[w][k] = run;
                    run += t;
                }
                sh.tile_len[k] = run;
            }
        }
        __syncthreads();
    }

    // ---- numeric / bytes / validity: warps take 32 consecutive rows of one
    // column; with string columns warp 0 runs the arena look-back meanwhile
    const uint32_t rpad = (nrows + 31) & ~31u;
    const uint32_t ncell = rpad * (uint32_t)rs.ncols;
    const uint32_t w0 = rs.nstr > 0 ? 32u : 0u;
    for (uint32_t i = (uint32_t)tid - w0; (uint32_t)tid >= w0 && i < ncell; i += kThreads - w0) {
        const int c = (int)(i / rpad);
        const uint32_t r = i % rpad;
        bool ok = false;
        if (r < nrows) {
            const uint64_t g = (uint64_t)rc.row_base + r;
            const Cell cl = cell_span(rc, sh, stage, n_total, n_term_all, r, rs.field[c]);
            if (rs.type[c] == 3) {
                ok = cl.present;  // lengths and bytes are handled by the arena pass
            } else {
                uint32_t dummy[kMaxStr] = {0, 0, 0, 0};
                const uint32_t n = (uint32_t)(cl.to - cl.from);
                ok = decode_cell(rs, c, g, cl.present ? cell_ptr(rc, cl.from, cl.to) : nullptr, n, cl.present,
                                 cl.from, cl.to, dummy);
            }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, ok);
        if (lane == 0 && bal) {
            const uint32_t bo = vshift + (r - lane);
            const uint32_t w = bo >> 6, sh6 = bo & 63;
            atomicOr((unsigned long long *)&sh.vbits[c][w], (unsigned long long)bal << sh6);
            if (sh6 > 32) atomicOr((unsigned long long *)&sh.vbits[c][w + 1], (unsigned long long)bal >> (64 - sh6));
        }
    }

    // ---- string arenas: the tile's arena offsets (warp 0, overlapping the cells)
    if (rs.nstr > 0 && warp == 0) {
        uint32_t tot[kMaxStr];
        for (int k = 0; k < kMaxStr; k++) tot[k] = sh.tile_len[k];
        unsigned long long pre[kMaxStr];
        arena_lookback(rc, tot, lane, pre);
        if (lane == 0)
            for (int k = 0; k < kMaxStr; k++) sh.arena_base[k] = (uint32_t)pre[k];
    }

    // ---- count / sum sink over two fields
    if (rs.want_stats) {
        for (uint32_t i = tid; i < 2 * nrows; i += kThreads) {
            const int k = i >= nrows ? 1 : 0;
            const uint32_t r = i - k * nrows;
            const Cell cl = cell_span(rc, sh, stage, n_total, n_term_all, r, rs.stats_field[k]);
            if (cl.present) stat_cell(acc, k, cell_ptr(rc, cl.from, cl.to), (uint32_t)(cl.to - cl.from));
        }
        if (tid == 0) acc.records += nrows;
    }

    // ---- field bytes: one structural entry per field
    if (rs.want_fb) {
        uint32_t first = 0;
        if (!tile_rec0) first = nterm_tile > 0 ? (uint32_t)sh.term_k[0] + 1 : n_total;
        const uint32_t last = last_open ? n_total : (nterm_tile > 0 ? (uint32_t)sh.term_k[nterm_tile - 1] + 1 : 0);
        const int64_t rec0 = rc.vs > 0 ? rc.vs : 0;
        for (uint32_t i = first + tid; i < last; i += kThreads) {
            const uint16_t e = stage[i];
            const int64_t pos = rc.vs + (e & 0x7FFF);
            const bool starts_rec = i == 0 || (stage[i - 1] >> 15);
            const int64_t from = i == 0 ? rec0 : rc.vs + (stage[i - 1] & 0x7FFF) + 1;
            int64_t to = pos;
            if (e >> 15) {
                if (D == D_CSV_HASH && starts_rec && to > from && cell_ptr(rc, from, from + 1)[0] == '#') continue;
                if (to > from && cell_ptr(rc, to - 1, to)[0] == '\r') to--;
            }
            acc.fields++;
            acc.bytes += cleaned_len(cell_ptr(rc, from, to), (uint32_t)(to - from));
        }
        // a last row without terminator ends its last field at end of file
        if (tid == 0 && last_open && n_term_all == nterm_tile) {
            const uint32_t k0 = sh.row_k[nrows - 1];
            const int64_t from = n_total > k0 ? rc.vs + (stage[n_total - 1] & 0x7FFF) + 1 : rc.vs + sh.row_pos[nrows - 1];
            int64_t to = rc.len;
            if (to > from && cell_ptr(rc, to - 1, to)[0] == '\r') to--;
            acc.fields++;
            acc.bytes += cleaned_len(cell_ptr(rc, from, to), (uint32_t)(to - from));
        }
    }

    __syncthreads();

    // validity words (row bits staged relative to the tile's first row)
    {
        const uint64_t w0 = (uint64_t)rc.row_base >> 6;
        const uint64_t maxw = (rs.rows_cap + 63) / 64;
        for (int i = tid; i < rs.ncols * kVWords; i += kThreads) {
            const int c = i / kVWords, wi = i % kVWords;
            const uint64_t v = sh.vbits[c][wi];
            if (v && w0 + wi < maxw) atomicOr((unsigned long long *)&rs.valid[c][w0 + wi], (unsigned long long)v);
        }
    }
    if (rs.want_fb || rs.want_stats) reduce_sinks(rs, rc, sh, acc, tid);

    if (rs.nstr > 0) {
        if (rc.tile == 0 && tid == 0)
            for (int c = 0; c < rs.ncols; c++)
                if (rs.type[c] == 3) static_cast<int32_t *>(rs.values[c])[0] = 0;
        for (int c = 0; c < rs.ncols; c++) {
            if (rs.type[c] != 3) continue;
            const int k = rs.str_slot[c];
            uint64_t at = (uint64_t)sh.arena_base[k] + sh.warp_len[warp][k] + slen[k];
            for (uint32_t r = r0; r < r1; r++) {
                const uint64_t g = (uint64_t)rc.row_base + r;
                const Cell cl = cell_span(rc, sh, stage, n_total, n_term_all, r, rs.field[c]);
                if (cl.present) {
                    const uint32_t n = (uint32_t)(cl.to - cl.from);
                    const uint8_t *src = cell_ptr(rc, cl.from, cl.to);
                    at += copy_clean(src, n, rs.str_data[c], at, rs.str_cap[c]);
                }
                if (g < rs.rows_cap) static_cast<int32_t *>(rs.values[c])[g + 1] = (int32_t)at;
            }
        }
    }
}

template <int D>
__device__ void rows_phase(const RowSpec &rs, const RowCtx &rc, RowShared<true> &sh, uint16_t *stage,
                           uint64_t rows_m, uint64_t stm, uint64_t term, uint32_t excl_struct, uint32_t excl_term,
                           uint32_t excl_rows, uint32_t nterm_tile, uint32_t nrows_tile, bool tile_rec0,
                           bool overflow, int64_t base_t, int tid) {
    const int lane = tid & 31, warp = tid >> 5;
    const int64_t ve = rc.vs + kTile;

    // ---- setup: column lookup by field ordinal, zeroed validity staging
    if (tid < 64) {
        uint32_t mk = 0;
        for (int c = 0; c < rs.ncols; c++)
            if (rs.field[c] == (uint32_t)tid) mk |= 1u << c;
        sh.colmask[tid] = mk;
    }
    if (tid == 0) {
        uint32_t hf = 0;
        for (int c = 0; c < rs.ncols; c++) hf |= rs.field[c] >= 64;
        sh.high_fields = hf;
    }
    for (int i = tid; i < rs.ncols * kVWords; i += kThreads) sh.vbits[i / kVWords][i % kVWords] = 0;

    // ---- row and terminator tables for the data-parallel path
    const bool tables = !overflow && nrows_tile <= (uint32_t)kRowCap && nterm_tile < (uint32_t)kTermCap;
    if (tables) {
        uint64_t mm = rows_m;
        uint32_t r = excl_rows;
        while (mm) {
            const unsigned b = __ffsll((long long)mm) - 1;
            mm &= mm - 1;
            const uint64_t below = (1ull << b) - 1;
            sh.row_pos[r] = (uint16_t)(base_t - rc.vs + b);
            sh.row_k[r] = (uint16_t)(excl_struct + __popcll(stm & below));
            sh.row_t[r] = (uint16_t)(excl_term + __popcll(term & below));
            r++;
        }
        uint64_t tm = term;
        while (tm) {
            const unsigned b = __ffsll((long long)tm) - 1;
            sh.term_k[excl_term + __popcll(term & ((1ull << b) - 1))] =
                (uint16_t)(excl_struct + __popcll(stm & ((1ull << b) - 1)));
            tm &= tm - 1;
        }
    }

    // ---- halo: structurals after the tile up to the first terminator
    if (warp == 0) {
        uint32_t n_halo = 0, kind = 1, hexit = rc.exit_state;
        if (ve < rc.len && !overflow) {
            Masks m;
            m.s = m.nl = m.q = m.x = 0;
            m.special = false;
            uint32_t f = kIdentity;
            uint64_t ls = 0;
            constexpr int kHaloLanes = kHaloBytes / kThreadBytes;
            if (lane < kHaloLanes) {
                const int r = (lane >> 1) & 3;
                uint32_t w[16];
                const uint4 *src = reinterpret_cast<const uint4 *>(rc.buf + kPre + kTile + lane * kThreadBytes);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    uint4 v = src[(k + r) & 3];
                    w[4 * k] = v.x; w[4 * k + 1] = v.y; w[4 * k + 2] = v.z; w[4 * k + 3] = v.w;
                }
                m = classify<D>(w, r);
                bool pnl = rc.buf[kPre + kTile + lane * kThreadBytes - 1] == '\n';
                ls = (m.nl << 1) | (uint64_t)pnl;
                f = thread_function<D>(m, ls);
            }
            uint32_t incl = f;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl = fcompose(o, incl);
            }
            uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
            if (lane == 0) excl = kIdentity;
            uint32_t s_in = fapply(excl, rc.exit_state);
            uint64_t hs = lane < kHaloLanes ? structural_mask<D>(m, ls, s_in) : 0;
            uint64_t ht = hs & m.nl;
            uint32_t ball = __ballot_sync(0xffffffffu, ht != 0);
            uint64_t keep = hs;
            if (ball) {
                int fl = __ffs(ball) - 1;
                if (lane > fl) keep = 0;
                else if (lane == fl) {
                    unsigned b = __ffsll((long long)ht) - 1;
                    keep = hs & (b == 63 ? ~0ull : ((2ull << b) - 1));
                }
                kind = 0;
            } else {
                kind = (ve + kHaloBytes >= rc.len) ? 1 : 2;
            }
            uint32_t cnt = __popcll(keep);
            uint32_t ci = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t o = __shfl_up_sync(0xffffffffu, ci, d);
                if (lane >= d) ci += o;
            }
            uint32_t at = rc.n_tile + ci - cnt;
            while (keep) {
                unsigned b = __ffsll((long long)keep) - 1;
                stage[at++] = (uint16_t)((kTile + lane * kThreadBytes + b) | (((ht >> b) & 1) << 15));
                keep &= keep - 1;
            }
            n_halo = __shfl_sync(0xffffffffu, ci, 31);
            hexit = fapply(__shfl_sync(0xffffffffu, incl, 31), rc.exit_state);
        }
        if (lane == 0) {
            sh.n_halo = n_halo;
            sh.halo_kind = kind;
            sh.halo_exit = hexit;
            if (tables && kind == 0 && n_halo > 0) sh.term_k[nterm_tile] = (uint16_t)(rc.n_tile + n_halo - 1);
            const bool last_open = nrows_tile > 0 && tables && sh.row_t[nrows_tile - 1] == nterm_tile;
            sh.fast = tables && !(last_open && kind == 2);
        }
    }
    __syncthreads();
    if (sh.fast) {
        rows_fast<D>(rs, rc, sh, stage, nrows_tile, nterm_tile, tile_rec0, tid);
        return;
    }

    // ---- per-thread rows
    StatAcc acc = {};
    uint32_t slen[kMaxStr] = {0, 0, 0, 0};
    Walker<D> wk;
    wk.stage = stage;
    wk.n_total = rc.n_tile + sh.n_halo;
    wk.vs = rc.vs;
    wk.len = rc.len;
    wk.halo_kind = sh.halo_kind;
    wk.halo_exit = sh.halo_exit;
    wk.halo_end = ve + kHaloBytes;
    wk.data = rc.data;
    const uint32_t vshift = rc.row_base & 63;
    const bool need_walk_all = rs.want_fb != 0;
    uint64_t mm = rows_m;
    uint32_t lr = excl_rows;
    while (mm) {
        const unsigned b = __ffsll((long long)mm) - 1;
        mm &= mm - 1;
        const int64_t r0 = base_t + b;
        const uint64_t g = (uint64_t)rc.row_base + lr;
        wk.k = excl_struct + __popcll(stm & ((1ull << b) - 1));
        wk.serial = overflow;  // tiles too dense to stage walk their records byte by byte
        wk.sp = r0;
        wk.ss = 0;
        wk.sls = true;
        uint32_t done = 0;  // columns written
        int64_t fs = r0;
        uint32_t ord = 0;
        for (;;) {
            int64_t pos;
            bool is_term;
            bool got = wk.next(pos, is_term);
            const bool last = !got || is_term;
            if (!got) pos = rc.len;
            int64_t fend = pos;
            if (last && fend > r0 && (cell_ptr(rc, fend - 1, fend))[0] == '\r') fend--;
            const uint32_t n = (uint32_t)(fend - fs);
            const uint8_t *s = cell_ptr(rc, fs, fend);
            if (rs.want_fb) {
                acc.fields++;
                acc.bytes += cleaned_len(s, n);
            }
            if (ord < rs.max_field) {
                uint32_t cm = ord < 64 ? sh.colmask[ord] : 0;
                if (ord >= 64 && sh.high_fields)
                    for (int c = 0; c < rs.ncols; c++)
                        if (rs.field[c] == ord) cm |= 1u << c;
                while (cm) {
                    int c = __ffs(cm) - 1;
                    cm &= cm - 1;
                    bool ok = decode_cell(rs, c, g, s, n, true, fs, fend, slen);
                    done |= 1u << c;
                    if (ok) {
                        const uint32_t lb = vshift + lr;
                        if (lb < 64 * kVWords) atomicOr((unsigned long long *)&sh.vbits[c][lb >> 6], 1ull << (lb & 63));
                        else if (g < rs.rows_cap) atomicOr((unsigned long long *)&rs.valid[c][g >> 6], 1ull << (g & 63));
                    }
                }
                if (rs.want_stats) {
                    if (ord == rs.stats_field[0]) stat_cell(acc, 0, s, n);
                    if (ord == rs.stats_field[1]) stat_cell(acc, 1, s, n);
                }
            }
            ord++;
            if (last) break;
            fs = pos + 1;
            if (!need_walk_all && ord >= rs.max_field) break;
        }
        // missing fields: zero placeholders, invalid
        uint32_t rest = (rs.ncols >= 32 ? 0xFFFFFFFFu : ((1u << rs.ncols) - 1)) & ~done;
        while (rest) {
            int c = __ffs(rest) - 1;
            rest &= rest - 1;
            decode_cell(rs, c, g, nullptr, 0, false, 0, 0, slen);
        }
        if (rs.want_stats) acc.records++;
        lr++;
    }
    __syncthreads();

    // ---- validity words (row bits staged relative to the tile's first row)
    {
        const uint64_t w0 = (uint64_t)rc.row_base >> 6;
        const uint64_t maxw = (rs.rows_cap + 63) / 64;
        for (int i = tid; i < rs.ncols * kVWords; i += kThreads) {
            int c = i / kVWords, wi = i % kVWords;
            uint64_t v = sh.vbits[c][wi];
            if (v && w0 + wi < maxw) atomicOr((unsigned long long *)&rs.valid[c][w0 + wi], (unsigned long long)v);
        }
    }

    // ---- reductions for the sinks
    if (rs.want_fb || rs.want_stats) {
        unsigned long long v[12] = {acc.fields, acc.bytes, acc.records, acc.values[0], acc.values[1],
                                    acc.checksum[0], acc.checksum[1], acc.sum_e6[0], acc.sum_e6[1],
                                    acc.inexact[0], acc.inexact[1], 0};
#pragma unroll
        for (int k = 0; k < 11; k++) {
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], d);
            if (lane == 0) sh.red[warp][k] = v[k];
        }
        __syncthreads();
        if (tid < 11) {
            unsigned long long t = 0;
            for (int w = 0; w < kWarps; w++) t += sh.red[w][tid];
            if (t) {
                if (tid < 2) atomicAdd(&rc.hdr_fb[tid], t);
                else atomicAdd(&rc.hdr_st[tid - 2], t);
            }
        }
    }

    // ---- string arenas: block scan of lengths, look-back, copy
    if (rs.nstr > 0) {
        uint32_t excl_len[kMaxStr];
        for (int k = 0; k < kMaxStr; k++) {
            uint32_t x = slen[k];
            uint32_t xi = x;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t o = __shfl_up_sync(0xffffffffu, xi, d);
                if (lane >= d) xi += o;
            }
            if (lane == 31) sh.warp_len[warp][k] = xi;
            excl_len[k] = xi - x;
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t tot[kMaxStr];
            for (int k = 0; k < kMaxStr; k++) {
                uint32_t run = 0;
                for (int w = 0; w < kWarps; w++) run += sh.warp_len[w][k];
                tot[k] = run;
            }
            __syncwarp();
            if (lane == 0) {
                for (int k = 0; k < kMaxStr; k++) {
                    uint32_t run = 0;
                    for (int w = 0; w < kWarps; w++) {
                        uint32_t t = sh.warp_len[w][k];
                        sh.warp_len[w][k] = run;
                        run += t;
                    }
                    sh.tile_len[k] = run;
                }
            }
            ArenaStatusView *as = static_cast<ArenaStatusView *>(rc.astatus);
            ArenaStatusView *me = &as[rc.tile];
            if (lane == 0) {
                for (int k = 0; k < kMaxStr; k++) me->agg[k] = tot[k];
                st_release(&me->flag, rc.epoch * 4 + 1);
            }
            __syncwarp();
            unsigned long long pre[kMaxStr] = {0, 0, 0, 0};
            for (int64_t hi = (int64_t)rc.tile - 1; hi >= 0; hi -= 32) {
                const int64_t j = hi - lane;
                const bool in = j >= 0;
                uint32_t flag = 0;
                bool gave_up = false;
                const uint64_t t0 = globaltimer_ns();
                for (uint32_t it = 0;; it++) {
                    if (in) flag = ld_acquire(&as[j].flag);
                    bool ready = !in || ((flag >> 2) == rc.epoch && (flag & 3) >= 1);
                    if (__all_sync(0xffffffffu, ready)) break;
                    if ((it & 63) == 63) {
                        bool stop = lane == 0 && (*(volatile uint32_t *)rc.hdr_abort ||
                                                  globaltimer_ns() - t0 > 4000000000ull);
                        if (__any_sync(0xffffffffu, stop)) {
                            gave_up = true;
                            break;
                        }
                    }
                    __nanosleep(32);
                }
                if (gave_up) {
                    if (lane == 0) {
                        atomicOr(rc.hdr_error, 1u);
                        atomicExch(rc.hdr_abort, 1u);
                    }
                    break;
                }
                const uint32_t ball = __ballot_sync(0xffffffffu, in && (flag & 3) == 2);
                const int sidx = ball ? __ffs(ball) - 1 : 32;
                for (int k = 0; k < kMaxStr; k++) {
                    uint32_t v = 0;
                    if (in && lane < sidx) v = ld_relaxed(&as[j].agg[k]);
                    else if (in && lane == sidx) v = ld_relaxed(&as[j].incl[k]);
                    unsigned long long vv = v;
#pragma unroll
                    for (int d = 16; d > 0; d >>= 1) vv += __shfl_xor_sync(0xffffffffu, vv, d);
                    pre[k] += vv;
                }
                if (ball) break;
            }
            if (lane == 0) {
                bool over = false;
                for (int k = 0; k < kMaxStr; k++) {
                    unsigned long long inc = pre[k] + tot[k];
                    if (inc > 0x7FFFFFFFull) over = true;
                    me->incl[k] = (uint32_t)inc;
                    sh.arena_base[k] = (uint32_t)pre[k];
                }
                st_release(&me->flag, rc.epoch * 4 + 2);
                if (over) atomicOr(rc.hdr_error, 2u);
                if (rc.last_tile)
                    for (int k = 0; k < kMaxStr; k++) rc.hdr_arena[k] = pre[k] + tot[k];
            }
        }
        __syncthreads();
        uint64_t at[kMaxStr];
        for (int k = 0; k < kMaxStr; k++) at[k] = (uint64_t)sh.arena_base[k] + sh.warp_len[warp][k] + excl_len[k];
        if (rc.tile == 0 && tid == 0)
            for (int c = 0; c < rs.ncols; c++)
                if (rs.type[c] == 3) static_cast<int32_t *>(rs.values[c])[0] = 0;
        // Second walk: copy cleaned bytes, write offsets.
        mm = rows_m;
        lr = excl_rows;
        while (mm) {
            const unsigned b = __ffsll((long long)mm) - 1;
            mm &= mm - 1;
            const int64_t r0 = base_t + b;
            const uint64_t g = (uint64_t)rc.row_base + lr;
            wk.k = excl_struct + __popcll(stm & ((1ull << b) - 1));
            wk.serial = overflow;
            wk.sp = r0;
            wk.ss = 0;
            wk.sls = true;
            int64_t fs = r0;
            uint32_t ord = 0;
            for (;;) {
                int64_t pos;
                bool is_term;
                bool got = wk.next(pos, is_term);
                bool last = !got || is_term;
                if (!got) pos = rc.len;
                int64_t fend = pos;
                if (last && fend > r0 && (cell_ptr(rc, fend - 1, fend))[0] == '\r') fend--;
                if (ord < rs.max_field) {
                    uint32_t cm = ord < 64 ? sh.colmask[ord] : 0;
                    if (ord >= 64 && sh.high_fields)
                        for (int c = 0; c < rs.ncols; c++)
                            if (rs.field[c] == ord) cm |= 1u << c;
                    while (cm) {
                        int c = __ffs(cm) - 1;
                        cm &= cm - 1;
                        if (rs.type[c] != 3) continue;
                        int k = rs.str_slot[c];
                        const uint32_t n = (uint32_t)(fend - fs);
                        const uint8_t *s = cell_ptr(rc, fs, fend);
                        copy_clean(s, n, rs.str_data[c], at[k], rs.str_cap[c]);
                        at[k] += cleaned_len(s, n);
                    }
                }
                ord++;
                if (last || ord >= rs.max_field) break;
                fs = pos + 1;
            }
            if (g < rs.rows_cap)
                for (int c = 0; c < rs.ncols; c++)
                    if (rs.type[c] == 3) static_cast<int32_t *>(rs.values[c])[g + 1] = (int32_t)at[rs.str_slot[c]];
            lr++;
        }
    }
}

}  // namespace falx
