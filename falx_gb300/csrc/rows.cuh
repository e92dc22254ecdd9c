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
constexpr int kLocalRows = 2048;    // rows per tile with shared-memory validity staging
constexpr int kVWords = kLocalRows / 64 + 2;

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
__device__ __forceinline__ void copy_clean(const uint8_t *s, uint32_t len, uint8_t *dst, uint64_t at, uint64_t cap) {
    if (len >= 2 && s[0] == '"' && s[len - 1] == '"') {
        uint32_t il = len - 2, i = 0;
        const uint8_t *in = s + 1;
        while (i < il) {
            if (at < cap) dst[at] = in[i];
            at++;
            i += (in[i] == '"' && i + 1 < il && in[i + 1] == '"') ? 2 : 1;
        }
        return;
    }
    for (uint32_t i = 0; i < len; i++, at++)
        if (at < cap) dst[at] = s[i];
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

template <int D>
__device__ void rows_phase(const RowSpec &rs, const RowCtx &rc, RowShared<true> &sh, uint16_t *stage,
                           uint64_t rows_m, uint64_t stm, uint64_t term, uint32_t excl_struct, uint32_t excl_rows,
                           int64_t base_t, int tid) {
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

    // ---- halo: structurals after the tile up to the first terminator
    if (warp == 0) {
        uint32_t n_halo = 0, kind = 1, hexit = rc.exit_state;
        if (ve < rc.len) {
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
        }
    }
    __syncthreads();

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
        wk.serial = false;
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
        if (tid == 0) {
            uint32_t tot[kMaxStr];
            for (int k = 0; k < kMaxStr; k++) {
                uint32_t run = 0;
                for (int w = 0; w < kWarps; w++) {
                    uint32_t t = sh.warp_len[w][k];
                    sh.warp_len[w][k] = run;
                    run += t;
                }
                tot[k] = run;
                sh.tile_len[k] = run;
            }
            ArenaStatusView *as = static_cast<ArenaStatusView *>(rc.astatus);
            ArenaStatusView *me = &as[rc.tile];
            for (int k = 0; k < kMaxStr; k++) me->agg[k] = tot[k];
            st_release(&me->flag, rc.epoch * 4 + 1);
            unsigned long long pre[kMaxStr] = {0, 0, 0, 0};
            for (int64_t j = (int64_t)rc.tile - 1; j >= 0; j--) {
                uint32_t flag = 0, polls = 0;
                bool gave_up = false;
                const uint64_t t0 = globaltimer_ns();
                for (;;) {
                    flag = ld_acquire(&as[j].flag);
                    if ((flag >> 2) == rc.epoch && (flag & 3) >= 1) break;
                    if ((++polls & 255) == 0 &&
                        (*(volatile uint32_t *)rc.hdr_abort || globaltimer_ns() - t0 > 4000000000ull)) {
                        atomicOr(rc.hdr_error, 1u);
                        atomicExch(rc.hdr_abort, 1u);
                        gave_up = true;
                        break;
                    }
                    __nanosleep(64);
                }
                if (gave_up) break;
                if ((flag & 3) == 2) {
                    for (int k = 0; k < kMaxStr; k++) pre[k] += ld_relaxed(&as[j].incl[k]);
                    break;
                }
                for (int k = 0; k < kMaxStr; k++) pre[k] += ld_relaxed(&as[j].agg[k]);
            }
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
            wk.serial = false;
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
