/*
 * Multi-threaded port of the reference's `_par` drivers: the timed CPU
 * baseline. TEST INFRASTRUCTURE ONLY (see oracle.h): never linked by the
 * product.
 *
 * Structure follows the reference:
 *  - chunks of (len / threads) rounded up to 64 bytes (csv_geo.rs:96-103);
 *  - csv: speculative quote parity, odd-entry chunks re-indexed
 *    (csv_geo.rs:95-149);
 *  - csv_hash: phase 1 per-chunk region transfer functions (region_scan3),
 *    phase 2 serial composition, phase 3 seeded pass per chunk
 *    (csv_hash.rs:345-399, :984-1051, :1507-1601);
 *  - record ownership for the sinks: a chunk emits the records after its
 *    first terminator and finishes the record open at its end
 *    (csv_geo.rs:952-1000).
 * Block classification: on aarch64 NEON byte compares with pairwise-add
 * movemasks and the quote prefix XOR as one PMULL carry-less multiply (the
 * reference's NEON tier, csv_geo.rs:2696, which also requires the AES/PMULL
 * extension); elsewhere portable 64-bit SWAR. Cells: SWAR fast paths for
 * plain u32 and [-]d{1,3}.d{6} f64 ahead of the full parsers, as the
 * reference's parse_fixed_6_decimal_signed / parse_f64_cell do
 * (csv_geo.rs:1313-1475). orc_par_parse runs the index, field-byte, column
 * and count / sum sinks in one pass per chunk, as parse_columns_chunks_par
 * does for columns (csv_hash.rs:1507-1601). It is a reported baseline, not
 * a target.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#if defined(__aarch64__) && defined(__ARM_NEON) && defined(__ARM_FEATURE_AES)
#include <arm_neon.h>
#define ORC_NEON 1
#endif

/* ------------------------------------------------------------------------- */
/* SWAR block classification: bit i = (p[i] == c) for a 64-byte block.        */
/* ------------------------------------------------------------------------- */

static inline uint64_t load64(const uint8_t *p) {
    uint64_t v;
    memcpy(&v, p, 8);
    return v;
}

static inline uint64_t eq8(uint64_t w, uint8_t c) {
    uint64_t x = w ^ (0x0101010101010101ull * c);
    uint64_t t = (x & 0x7F7F7F7F7F7F7F7Full) + 0x7F7F7F7F7F7F7F7Full;
    return ~(t | x) & 0x8080808080808080ull;
}

static inline uint64_t movemask8(uint64_t f) { return ((f >> 7) * 0x0102040810204080ull) >> 56; }

typedef struct {
    uint64_t nl, sep, q, h, bs;
} bmask;

#ifdef ORC_NEON
/* 64 compare results (0xFF / 0 bytes) -> a 64-bit mask in byte order. */
static inline uint64_t nmask(uint8x16_t a, uint8x16_t b, uint8x16_t c, uint8x16_t d) {
    static const uint8_t wts[16] = {1, 2, 4, 8, 16, 32, 64, 128, 1, 2, 4, 8, 16, 32, 64, 128};
    const uint8x16_t w = vld1q_u8(wts);
    uint8x16_t s0 = vpaddq_u8(vandq_u8(a, w), vandq_u8(b, w));
    uint8x16_t s1 = vpaddq_u8(vandq_u8(c, w), vandq_u8(d, w));
    s0 = vpaddq_u8(s0, s1);
    s0 = vpaddq_u8(s0, s0);
    return vgetq_lane_u64(vreinterpretq_u64_u8(s0), 0);
}
#define NEQ(ch) nmask(vceqq_u8(v0, vdupq_n_u8(ch)), vceqq_u8(v1, vdupq_n_u8(ch)), vceqq_u8(v2, vdupq_n_u8(ch)), \
                      vceqq_u8(v3, vdupq_n_u8(ch)))
static inline void classify_block(int dialect, const uint8_t *p, bmask *m) {
    const uint8x16_t v0 = vld1q_u8(p), v1 = vld1q_u8(p + 16), v2 = vld1q_u8(p + 32), v3 = vld1q_u8(p + 48);
    m->nl = NEQ('\n');
    m->sep = dialect == ORC_TSV ? NEQ('\t') : dialect == ORC_LOGFMT ? (NEQ(' ') | NEQ('=')) :
             dialect == ORC_NDJSON ? 0 : NEQ(',');
    m->q = dialect == ORC_TSV ? 0 : NEQ('"');
    m->h = dialect == ORC_CSV_HASH ? NEQ('#') : 0;
    m->bs = (dialect == ORC_LOGFMT || dialect == ORC_NDJSON) ? NEQ('\\') : 0;
}
#undef NEQ
#else
static inline void classify_block(int dialect, const uint8_t *p, bmask *m) {
    uint64_t nl = 0, sep = 0, q = 0, h = 0, bs = 0;
    for (int k = 0; k < 8; k++) {
        uint64_t w = load64(p + 8 * k);
        nl |= movemask8(eq8(w, '\n')) << (8 * k);
        if (dialect == ORC_TSV) {
            sep |= movemask8(eq8(w, '\t')) << (8 * k);
        } else if (dialect == ORC_LOGFMT) {
            sep |= movemask8(eq8(w, ' ') | eq8(w, '=')) << (8 * k);
        } else if (dialect != ORC_NDJSON) {
            sep |= movemask8(eq8(w, ',')) << (8 * k);
        }
        if (dialect != ORC_TSV) q |= movemask8(eq8(w, '"')) << (8 * k);
        if (dialect == ORC_CSV_HASH) h |= movemask8(eq8(w, '#')) << (8 * k);
        if (dialect == ORC_LOGFMT || dialect == ORC_NDJSON) bs |= movemask8(eq8(w, '\\')) << (8 * k);
    }
    m->nl = nl;
    m->sep = sep;
    m->q = q;
    m->h = h;
    m->bs = bs;
}
#endif

static inline uint64_t pxor(uint64_t x) {
#ifdef ORC_NEON
    /* carry-less multiply by all ones: bit i = XOR of bits 0..i */
    return vgetq_lane_u64(vreinterpretq_u64_p128(vmull_p64((poly64_t)x, (poly64_t)~0ull)), 0);
#else
    x ^= x << 1; x ^= x << 2; x ^= x << 4; x ^= x << 8; x ^= x << 16; x ^= x << 32;
    return x;
#endif
}

static inline uint64_t rmask(unsigned from, unsigned to) {
    uint64_t hi = to >= 64 ? ~0ull : ((1ull << to) - 1);
    return hi & ~((1ull << from) - 1);
}

/* resolve_regions with the generated fast paths (csv_hash.rs:2151-2222) */
static inline uint64_t regions(uint64_t q, uint64_t s, uint64_t nl, uint64_t *state) {
    if (*state == 0 && (q | s) == 0) return 0;
    if (*state != 2 && s == 0) {
        uint64_t inert = pxor(q);
        if (*state == 1) inert = ~inert;
        *state = inert >> 63;
        return inert;
    }
    uint64_t inert = 0, ev = q | s | nl;
    unsigned run = 0;
    while (ev) {
        unsigned p = (unsigned)__builtin_ctzll(ev);
        uint64_t bit = 1ull << p;
        if (*state == 1) {
            if (q & bit) { inert |= rmask(run, p); *state = 0; }
        } else if (*state == 2) {
            if (nl & bit) { inert |= rmask(run, p); *state = 0; }
        } else {
            if (q & bit) { *state = 1; run = p; }
            else if (s & bit) { *state = 2; run = p; }
        }
        ev &= ev - 1;
    }
    if (*state != 0) inert |= rmask(run, 64);
    return inert;
}

/* One block step: carries c[0], c[1] as in the generated kernels. */
static inline void step(int dialect, const bmask *m, uint64_t c[2], uint64_t *st, uint64_t *term) {
    const uint64_t EVEN = 0x5555555555555555ull;
    uint64_t s;
    switch (dialect) {
    case ORC_CSV: {
        uint64_t par = pxor(m->q) ^ c[0];
        c[0] = (uint64_t)((int64_t)par >> 63);
        s = (m->nl | m->sep) & ~par;
        break;
    }
    case ORC_CSV_HASH: {
        uint64_t ls = (m->nl << 1) | c[0];
        c[0] = m->nl >> 63;
        uint64_t inert = regions(m->q, m->h & ls, m->nl, &c[1]);
        s = (m->nl | m->sep) & ~inert;
        break;
    }
    case ORC_TSV:
        s = m->nl | m->sep;
        break;
    default: {
        uint64_t v2 = EVEN ^ m->bs, partial = EVEN + v2;
        uint64_t c1 = partial < EVEN, sum = partial + c[0], c2 = sum < partial;
        c[0] = c1 | c2;
        uint64_t par = pxor(m->q & (EVEN ^ sum)) ^ c[1];
        c[1] = (uint64_t)((int64_t)par >> 63);
        s = (m->nl | m->sep) & ~par;
        break;
    }
    }
    *st = s;
    *term = s & m->nl;
}

/* Load a 64-byte block at `off` (zero padded past `n`). */
static inline const uint8_t *block_at(const uint8_t *d, uint64_t n, uint64_t off, uint8_t *tmp, uint64_t *live) {
    if (off + 64 <= n) {
        *live = ~0ull;
        return d + off;
    }
    uint64_t rem = n - off;
    memset(tmp, 0, 64);
    memcpy(tmp, d + off, rem);
    *live = (1ull << rem) - 1;
    return tmp;
}

/* ------------------------------------------------------------------------- */
/* Chunking and entry states.                                                */
/* ------------------------------------------------------------------------- */

typedef struct {
    int dialect;
    const uint8_t *d;
    uint64_t n;
    int threads;
    uint64_t bounds[257];
    uint64_t seed[256][2]; /* entry carries per chunk */
} plan_t;

typedef struct {
    plan_t *pl;
    int t;
    uint64_t states[4]; /* exit state per entry state */
} scan_job;

/* Phase 1: the chunk's exit region for every entry region (region_scan3). */
static void *scan3(void *arg) {
    scan_job *j = (scan_job *)arg;
    plan_t *pl = j->pl;
    uint64_t s = pl->bounds[j->t], e = pl->bounds[j->t + 1];
    uint64_t st[3] = {0, 1, 2};
    uint64_t ls = s == 0 ? 1 : (pl->d[s - 1] == '\n');
    uint8_t tmp[64];
    for (uint64_t off = s; off < e; off += 64) {
        uint64_t live;
        const uint8_t *p = block_at(pl->d, e, off, tmp, &live);
        bmask m;
        classify_block(ORC_CSV_HASH, p, &m);
        uint64_t l = (m.nl << 1) | ls;
        ls = m.nl >> 63;
        uint64_t h = m.h & l;
        for (int k = 0; k < 3; k++) regions(m.q, h, m.nl, &st[k]);
    }
    for (int k = 0; k < 3; k++) j->states[k] = st[k];
    return NULL;
}

/* Quote parity of a chunk (csv_geo.rs:1902-1919). */
static void *parity(void *arg) {
    scan_job *j = (scan_job *)arg;
    plan_t *pl = j->pl;
    uint64_t s = pl->bounds[j->t], e = pl->bounds[j->t + 1], par = 0;
    uint8_t tmp[64];
    for (uint64_t off = s; off < e; off += 64) {
        uint64_t live;
        const uint8_t *p = block_at(pl->d, e, off, tmp, &live);
        bmask m;
        classify_block(ORC_CSV, p, &m);
        par ^= (uint64_t)__builtin_popcountll(m.q & live) & 1;
    }
    j->states[0] = par;
    return NULL;
}

static void run_threads(int n, void *(*fn)(void *), void *jobs, size_t stride) {
    pthread_t th[256];
    for (int t = 0; t < n; t++) pthread_create(&th[t], NULL, fn, (char *)jobs + stride * (size_t)t);
    for (int t = 0; t < n; t++) pthread_join(th[t], NULL);
}

/* Plan chunks and resolve every chunk's entry carries. Dialects with
 * backslash escapes keep one chunk (the reference has no chunked driver for
 * their structural index). */
static void make_plan(plan_t *pl, int dialect, const uint8_t *d, uint64_t n, int threads) {
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > n / 64 + 1) threads = (int)(n / 64 + 1);
    if (threads > 256) threads = 256;
    if (dialect == ORC_LOGFMT || dialect == ORC_NDJSON) threads = 1;
    uint64_t chunk = (n / (uint64_t)threads + 63) & ~63ull;
    if (chunk == 0) threads = 1;
    pl->dialect = dialect;
    pl->d = d;
    pl->n = n;
    pl->threads = threads;
    for (int t = 0; t <= threads; t++) {
        uint64_t b = t == threads ? n : (uint64_t)t * chunk;
        pl->bounds[t] = b < n ? b : n;
    }
    scan_job jobs[256];
    for (int t = 0; t < threads; t++) {
        jobs[t].pl = pl;
        jobs[t].t = t;
    }
    if (dialect == ORC_CSV_HASH && threads > 1) {
        run_threads(threads, scan3, jobs, sizeof(scan_job));
        uint64_t region = 0;
        for (int t = 0; t < threads; t++) {
            uint64_t b = pl->bounds[t];
            pl->seed[t][0] = b == 0 ? 1 : (d[b - 1] == '\n');
            pl->seed[t][1] = region;
            region = jobs[t].states[region];
        }
    } else if (dialect == ORC_CSV && threads > 1) {
        run_threads(threads, parity, jobs, sizeof(scan_job));
        uint64_t par = 0;
        for (int t = 0; t < threads; t++) {
            pl->seed[t][0] = par ? ~0ull : 0;
            pl->seed[t][1] = 0;
            par ^= jobs[t].states[0];
        }
    } else {
        for (int t = 0; t < threads; t++) {
            pl->seed[t][0] = dialect == ORC_CSV_HASH ? 1 : 0;
            pl->seed[t][1] = 0;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Parallel structural index.                                                */
/* ------------------------------------------------------------------------- */

typedef struct {
    plan_t *pl;
    int t;
    uint32_t *part;
    uint64_t cnt, cap;
    uint32_t *out;
    uint64_t at, out_cap;
} idx_job;

static void *idx_chunk(void *arg) {
    idx_job *j = (idx_job *)arg;
    plan_t *pl = j->pl;
    uint64_t s = pl->bounds[j->t], e = pl->bounds[j->t + 1];
    uint64_t c[2] = {pl->seed[j->t][0], pl->seed[j->t][1]};
    j->cap = (e - s) / 4 + 64;
    j->part = (uint32_t *)malloc(j->cap * 4);
    j->cnt = 0;
    uint8_t tmp[64];
    for (uint64_t off = s; off < e; off += 64) {
        uint64_t live;
        const uint8_t *p = block_at(pl->d, e, off, tmp, &live);
        bmask m;
        classify_block(pl->dialect, p, &m);
        uint64_t st, term;
        step(pl->dialect, &m, c, &st, &term);
        st &= live;
        if (j->cnt + 64 > j->cap) {
            j->cap = j->cap * 2 + 64;
            j->part = (uint32_t *)realloc(j->part, j->cap * 4);
        }
        while (st) {
            j->part[j->cnt++] = (uint32_t)(off + (uint64_t)__builtin_ctzll(st));
            st &= st - 1;
        }
    }
    return NULL;
}

static void *idx_copy(void *arg) {
    idx_job *j = (idx_job *)arg;
    uint64_t n = j->cnt;
    if (j->at < j->out_cap) memcpy(j->out + j->at, j->part, (j->at + n <= j->out_cap ? n : j->out_cap - j->at) * 4);
    free(j->part);
    return NULL;
}

uint64_t orc_par_index(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t *out, uint64_t cap) {
    plan_t *pl = (plan_t *)malloc(sizeof(plan_t));
    make_plan(pl, dialect, d, n, threads);
    idx_job jobs[256];
    for (int t = 0; t < pl->threads; t++) {
        jobs[t].pl = pl;
        jobs[t].t = t;
    }
    run_threads(pl->threads, idx_chunk, jobs, sizeof(idx_job));
    uint64_t total = 0;
    for (int t = 0; t < pl->threads; t++) {
        jobs[t].at = total;
        jobs[t].out = out;
        jobs[t].out_cap = cap;
        total += jobs[t].cnt;
    }
    run_threads(pl->threads, idx_copy, jobs, sizeof(idx_job));
    free(pl);
    return total;
}

/* ------------------------------------------------------------------------- */
/* Chunk record sinks with terminator ownership.                             */
/* ------------------------------------------------------------------------- */

/* Fixed [-]d{1,3}.d{6} and Clinger fast paths ahead of the full parser, as
 * the reference's parse_f64_cell does (csv_geo.rs:1313-1401). */
static int fast_f64(const uint8_t *s, uint64_t len, double *out) {
    static const double P10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                   1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    uint64_t i = 0;
    int neg = 0;
    if (len && (s[0] == '-' || s[0] == '+')) { neg = s[0] == '-'; i = 1; }
    uint64_t m = 0, nd = 0;
    int e10 = 0;
    while (i < len && (uint8_t)(s[i] - '0') < 10) { m = m * 10 + (s[i] - '0'); nd++; i++; }
    if (i < len && s[i] == '.') {
        i++;
        while (i < len && (uint8_t)(s[i] - '0') < 10) { m = m * 10 + (s[i] - '0'); nd++; e10--; i++; }
    }
    if (nd == 0 || nd > 15 || i != len || e10 < -22) return orc_parse_f64(s, len, out);
    double v = (double)m / P10[-e10];
    union { double f; uint64_t u; } b;
    b.f = v;
    b.u |= (uint64_t)neg << 63;
    *out = b.f;
    return 1;
}

/* Every byte of x is an ASCII digit: a byte above '9' reaches bit 7 when
 * 0x46 is added, one below '0' when 0x30 is subtracted (a carry or borrow
 * between bytes only comes from a byte that fails itself). */
static inline int all_digits8(uint64_t x) {
    return (((x + 0x4646464646464646ull) | (x - 0x3030303030303030ull)) & 0x8080808080808080ull) == 0;
}
/* Eight ASCII digits, the first in the low byte, as a number (pairwise
 * multiply-and-add: digit pairs, then fours, then eight). */
static inline uint32_t swar8(uint64_t x) {
    x -= 0x3030303030303030ull;
    x = (x * 10 + (x >> 8)) & 0x00FF00FF00FF00FFull;
    x = (x * 100 + (x >> 16)) & 0x0000FFFF0000FFFFull;
    return (uint32_t)((x * 10000 + (x >> 32)) & 0xFFFFFFFFull);
}
/* 1-8 plain digits. */
static inline int swar_u32(const uint8_t *s, uint64_t len, uint32_t *out) {
    if (len < 1 || len > 8) return 0;
    uint64_t v = 0;
    memcpy(&v, s, len);
    const uint64_t x = len == 8 ? v : (v << (8 * (8 - len))) | (0x3030303030303030ull >> (8 * len));
    if (!all_digits8(x)) return 0;
    *out = swar8(x);
    return 1;
}
/* [+-]?d{1,3}.d{6}: the integer mantissa over 1e6 in IEEE division, sign
 * OR'd into bit 63 (csv_geo.rs:1313-1322, :1414-1475). */
static inline int swar_fixed6(const uint8_t *s, uint64_t len, double *out) {
    if (len < 8 || len > 11) return 0;
    const uint64_t sg = s[0] == '-' || s[0] == '+';
    const uint64_t k = len - 7 - sg; /* integer digits */
    if (k < 1 || k > 3) return 0;
    uint64_t t;
    memcpy(&t, s + len - 8, 8); /* last integer digit, '.', six fraction digits */
    if (((t >> 8) & 0xFF) != '.') return 0;
    const uint64_t fr = (t & ~0xFFFFull) | 0x3030ull;
    if (!all_digits8(fr)) return 0;
    uint64_t ip = 0;
    for (uint64_t i = 0; i < k; i++) {
        const uint8_t c = s[sg + i];
        if ((uint8_t)(c - '0') > 9) return 0;
        ip = ip * 10 + (uint64_t)(c - '0');
    }
    union { double f; uint64_t u; } b;
    b.f = (double)(ip * 1000000 + swar8(fr)) / 1e6;
    b.u |= (uint64_t)(s[0] == '-') << 63;
    *out = b.f;
    return 1;
}

static uint64_t fb_len(const uint8_t *raw, uint64_t len) {
    if (len >= 2 && raw[0] == '"' && raw[len - 1] == '"') {
        uint64_t il = len - 2, o = 0, i = 0;
        const uint8_t *in = raw + 1;
        while (i < il) {
            o++;
            i += (in[i] == '"' && i + 1 < il && in[i + 1] == '"') ? 2 : 1;
        }
        return o;
    }
    return len;
}

typedef struct {
    uint32_t field, type;
    void *vals;      /* growable */
    uint64_t *valid; /* growable */
    int32_t *offs;   /* STR */
    uint8_t *arena;
    uint64_t alen, acap;
} pcol;

typedef struct {
    plan_t *pl;
    int t;
    int ncols;
    const orc_col *spec;
    pcol cols[32];
    uint64_t rows, rcap;
    uint64_t fields, bytes;
    int want_cols, want_fb, want_idx, want_stats;
    uint32_t sf[2];   /* count / sum fields */
    orc_geo_stats st; /* count / sum of the chunk */
    uint32_t *ipart;  /* structural index of the chunk's own bytes */
    uint64_t icnt, icap;
    /* concatenation */
    uint64_t row_at;
    uint64_t *arena_at;
    orc_col *out;
    uint64_t rows_cap;
} sink_job;

static void grow_rows(sink_job *j) {
    uint64_t nc = j->rcap * 2 + 1024;
    for (int k = 0; k < j->ncols; k++) {
        pcol *c = &j->cols[k];
        size_t es = c->type == ORC_U32 ? 4 : c->type == ORC_STR ? 0 : 8;
        if (es) c->vals = realloc(c->vals, nc * es);
        if (c->type == ORC_STR) c->offs = (int32_t *)realloc(c->offs, (nc + 1) * 4);
        c->valid = (uint64_t *)realloc(c->valid, ((nc + 63) / 64) * 8);
        memset(c->valid + (j->rcap + 63) / 64, 0, (((nc + 63) / 64) - (j->rcap + 63) / 64) * 8);
    }
    j->rcap = nc;
}

/* Fields beyond the span buffer are counted by the caller for field bytes
 * and read as missing for columns (declared fields stay below it). */
#define MAXF 512

static void emit_record(sink_job *j, const uint8_t *d, uint64_t rs, uint64_t end, const uint64_t *fs, const uint64_t *fe,
                        uint32_t nf) {
    if (j->pl->dialect == ORC_CSV_HASH && end > rs && d[rs] == '#') return;
    if (j->want_stats) {
        j->st.records++;
        for (int k = 0; k < 2; k++) {
            if (j->sf[k] >= nf) continue;
            const uint8_t *raw = d + fs[j->sf[k]];
            const uint64_t len = fe[j->sf[k]] - fs[j->sf[k]];
            double v;
            uint64_t bits;
            int64_t e6;
            int exact;
            if (swar_fixed6(raw, len, &v)) { /* exact in micro-units */
                union { double f; uint64_t u; } b;
                b.f = v;
                bits = b.u;
                const uint64_t sg = raw[0] == '-' || raw[0] == '+';
                int64_t mm = 0;
                for (uint64_t i = sg; i < len; i++)
                    if (raw[i] != '.') mm = mm * 10 + (raw[i] - '0');
                e6 = raw[0] == '-' ? -mm : mm;
                exact = 1;
            } else if (!orc_stats_cell(raw, len, &bits, &e6, &exact)) {
                continue;
            }
            union { double f; uint64_t u; } b;
            b.u = bits;
            j->st.values[k]++;
            j->st.checksum[k] += bits;
            j->st.fold[k] += b.f;
            if (exact) j->st.sum_e6[k] = (int64_t)((uint64_t)j->st.sum_e6[k] + (uint64_t)e6);
            else j->st.inexact[k]++;
        }
    }
    if (!j->want_cols) return;
    if (j->rows >= j->rcap) grow_rows(j);
    uint64_t r = j->rows++;
    uint8_t scratch[256];
    for (int k = 0; k < j->ncols; k++) {
        pcol *c = &j->cols[k];
        int present = c->field < nf;
        const uint8_t *raw = present ? d + fs[c->field] : NULL;
        uint64_t len = present ? fe[c->field] - fs[c->field] : 0;
        const uint8_t *v = raw;
        uint64_t vl = len;
        if (present && c->type != ORC_STR && c->type != ORC_BYTES && len && raw[0] == '"') {
            if (len >= 2 && raw[len - 1] == '"' && len - 2 <= sizeof scratch) {
                uint64_t o = 0, i = 1;
                while (i + 1 < len) {
                    scratch[o++] = raw[i];
                    i += (raw[i] == '"' && i + 2 < len && raw[i + 1] == '"') ? 2 : 1;
                }
                v = scratch;
                vl = o;
            }
        }
        int ok = 0;
        switch (c->type) {
        case ORC_I64: {
            int64_t x = 0;
            if (present) ok = orc_parse_i64(v, vl, &x);
            ((int64_t *)c->vals)[r] = ok ? x : 0;
            break;
        }
        case ORC_U32: {
            uint32_t x = 0;
            if (present) ok = swar_u32(v, vl, &x) || orc_parse_u32(v, vl, &x);
            ((uint32_t *)c->vals)[r] = ok ? x : 0;
            break;
        }
        case ORC_F64: {
            double x = 0;
            if (present) ok = swar_fixed6(v, vl, &x) || fast_f64(v, vl, &x);
            ((double *)c->vals)[r] = ok ? x : 0.0;
            break;
        }
        case ORC_STR: {
            if (present) {
                if (c->alen + len > c->acap) {
                    c->acap = (c->alen + len) * 2 + 4096;
                    c->arena = (uint8_t *)realloc(c->arena, c->acap);
                }
                if (len >= 2 && raw[0] == '"' && raw[len - 1] == '"') {
                    uint64_t i = 1;
                    while (i + 1 < len) {
                        c->arena[c->alen++] = raw[i];
                        i += (raw[i] == '"' && i + 2 < len && raw[i + 1] == '"') ? 2 : 1;
                    }
                } else {
                    memcpy(c->arena + c->alen, raw, len);
                    c->alen += len;
                }
                ok = 1;
            }
            c->offs[r + 1] = (int32_t)c->alen;
            break;
        }
        default: {
            ok = present && len > 0;
            ((uint32_t *)c->vals)[2 * r] = ok ? (uint32_t)fs[c->field] : 0;
            ((uint32_t *)c->vals)[2 * r + 1] = ok ? (uint32_t)fe[c->field] : 0;
            break;
        }
        }
        if (ok) c->valid[r >> 6] |= 1ull << (r & 63);
    }
}

static void *sink_chunk(void *arg) {
    sink_job *j = (sink_job *)arg;
    plan_t *pl = j->pl;
    const uint8_t *d = pl->d;
    const uint64_t n = pl->n, s = pl->bounds[j->t], e = pl->bounds[j->t + 1];
    uint64_t c[2] = {pl->seed[j->t][0], pl->seed[j->t][1]};
    int emitting = j->t == 0, done = 0;
    uint64_t rs = s, fsc = s;
    uint64_t fs[MAXF], fe[MAXF];
    uint32_t nf = 0;
    uint8_t tmp[64];
    j->rows = 0;
    j->rcap = 0;
    if (j->want_cols) grow_rows(j);
    for (int k = 0; k < j->ncols; k++)
        if (j->cols[k].type == ORC_STR) j->cols[k].offs[0] = 0;
    for (uint64_t off = s; off < n && !done; off += 64) {
        uint64_t live;
        const uint8_t *p = block_at(d, n, off, tmp, &live);
        bmask m;
        classify_block(pl->dialect, p, &m);
        uint64_t st, term;
        step(pl->dialect, &m, c, &st, &term);
        st &= live;
        if (j->want_idx && off < e) {
            uint64_t sti = e - off < 64 ? st & ((1ull << (e - off)) - 1) : st;
            if (j->icnt + 64 > j->icap) {
                j->icap = j->icap * 2 + 4096;
                j->ipart = (uint32_t *)realloc(j->ipart, j->icap * 4);
            }
            while (sti) {
                j->ipart[j->icnt++] = (uint32_t)(off + (uint64_t)__builtin_ctzll(sti));
                sti &= sti - 1;
            }
        }
        while (st) {
            uint64_t bit = st & (0 - st);
            uint64_t pos = off + (uint64_t)__builtin_ctzll(st);
            if (term & bit) {
                if (emitting) {
                    uint64_t to = (pos > rs && d[pos - 1] == '\r') ? pos - 1 : pos;
                    if (nf < MAXF) { fs[nf] = fsc; fe[nf] = to; nf++; }
                    if (j->want_fb && !(pl->dialect == ORC_CSV_HASH && pos > rs && d[rs] == '#')) {
                        j->fields++;
                        j->bytes += fb_len(d + fsc, to - fsc);
                    }
                    emit_record(j, d, rs, pos, fs, fe, nf);
                } else {
                    emitting = 1;
                }
                rs = fsc = pos + 1;
                nf = 0;
                if (pos >= e) { done = 1; break; }
            } else if (emitting) {
                if (nf < MAXF) { fs[nf] = fsc; fe[nf] = pos; nf++; }
                if (j->want_fb) {
                    j->fields++;
                    j->bytes += fb_len(d + fsc, pos - fsc);
                }
                fsc = pos + 1;
            }
            st &= st - 1;
        }
    }
    if (emitting && !done && rs < n) {
        uint64_t to = (n > rs && d[n - 1] == '\r') ? n - 1 : n;
        if (nf < MAXF) { fs[nf] = fsc; fe[nf] = to; nf++; }
        if (j->want_fb && !(pl->dialect == ORC_CSV_HASH && n > rs && d[rs] == '#')) {
            j->fields++;
            j->bytes += fb_len(d + fsc, to - fsc);
        }
        emit_record(j, d, rs, n, fs, fe, nf);
    }
    return NULL;
}

static void *sink_copy(void *arg) {
    sink_job *j = (sink_job *)arg;
    for (int k = 0; k < j->ncols; k++) {
        pcol *c = &j->cols[k];
        orc_col *o = &j->out[k];
        uint64_t r0 = j->row_at, nr = j->rows;
        if (r0 + nr > j->rows_cap) nr = r0 < j->rows_cap ? j->rows_cap - r0 : 0;
        size_t es = c->type == ORC_U32 ? 4 : c->type == ORC_BYTES ? 8 : 8;
        if (c->type == ORC_STR) {
            uint64_t a0 = j->arena_at[k];
            if (a0 + c->alen <= o->str_cap) memcpy(o->str_data + a0, c->arena, c->alen);
            for (uint64_t r = 0; r < nr; r++) ((int32_t *)o->values)[r0 + r + 1] = (int32_t)(a0 + c->offs[r + 1]);
        } else if (nr) {
            memcpy((uint8_t *)o->values + r0 * es, c->vals, nr * es);
        }
        /* chunks meet inside a bitmap word: OR atomically */
        for (uint64_t r = 0; r < nr; r++)
            if (c->valid[r >> 6] >> (r & 63) & 1)
                __atomic_fetch_or(&o->valid[(r0 + r) >> 6], 1ull << ((r0 + r) & 63), __ATOMIC_RELAXED);
    }
    return NULL;
}

static void free_job(sink_job *j) {
    free(j->ipart);
    for (int k = 0; k < j->ncols; k++) {
        free(j->cols[k].vals);
        free(j->cols[k].valid);
        free(j->cols[k].offs);
        free(j->cols[k].arena);
    }
}

int orc_par_columns(int dialect, const uint8_t *d, uint64_t n, int threads, orc_col *cols, int ncols,
                    uint64_t rows_cap, uint64_t *rows_out) {
    plan_t *pl = (plan_t *)malloc(sizeof(plan_t));
    make_plan(pl, dialect, d, n, threads);
    sink_job *jobs = (sink_job *)calloc((size_t)pl->threads, sizeof(sink_job));
    for (int t = 0; t < pl->threads; t++) {
        jobs[t].pl = pl;
        jobs[t].t = t;
        jobs[t].ncols = ncols;
        jobs[t].want_cols = 1;
        for (int k = 0; k < ncols; k++) {
            jobs[t].cols[k].field = cols[k].field;
            jobs[t].cols[k].type = cols[k].type;
        }
    }
    run_threads(pl->threads, sink_chunk, jobs, sizeof(sink_job));
    uint64_t rows = 0;
    uint64_t *arena_at = (uint64_t *)calloc((size_t)pl->threads * 32, 8);
    uint64_t alen[32] = {0};
    int over = 0;
    for (int k = 0; k < ncols; k++) {
        if (cols[k].valid) memset(cols[k].valid, 0, ((rows_cap + 63) / 64) * 8);
        if (cols[k].type == ORC_STR && cols[k].values) ((int32_t *)cols[k].values)[0] = 0;
    }
    for (int t = 0; t < pl->threads; t++) {
        jobs[t].row_at = rows;
        jobs[t].arena_at = arena_at + 32 * t;
        jobs[t].out = cols;
        jobs[t].rows_cap = rows_cap;
        for (int k = 0; k < ncols; k++) {
            jobs[t].arena_at[k] = alen[k];
            alen[k] += jobs[t].cols[k].alen;
        }
        rows += jobs[t].rows;
    }
    for (int k = 0; k < ncols; k++) {
        cols[k].str_len = alen[k];
        if (cols[k].type == ORC_STR && alen[k] > cols[k].str_cap) over = 1;
    }
    if (rows > rows_cap) over = 1;
    run_threads(pl->threads, sink_copy, jobs, sizeof(sink_job));
    for (int t = 0; t < pl->threads; t++) free_job(&jobs[t]);
    free(arena_at);
    free(jobs);
    free(pl);
    *rows_out = rows;
    return over ? -1 : 0;
}

void orc_par_field_bytes(int dialect, const uint8_t *d, uint64_t n, int threads, uint64_t *fields, uint64_t *bytes) {
    plan_t *pl = (plan_t *)malloc(sizeof(plan_t));
    make_plan(pl, dialect, d, n, threads);
    sink_job *jobs = (sink_job *)calloc((size_t)pl->threads, sizeof(sink_job));
    for (int t = 0; t < pl->threads; t++) {
        jobs[t].pl = pl;
        jobs[t].t = t;
        jobs[t].want_fb = 1;
    }
    run_threads(pl->threads, sink_chunk, jobs, sizeof(sink_job));
    uint64_t f = 0, b = 0;
    for (int t = 0; t < pl->threads; t++) {
        f += jobs[t].fields;
        b += jobs[t].bytes;
        free_job(&jobs[t]);
    }
    free(jobs);
    free(pl);
    *fields = f;
    *bytes = b;
}

/* ------------------------------------------------------------------------- */
/* One pass per chunk: structural index, field bytes, columns and count /    */
/* sum together.                                                             */
/* ------------------------------------------------------------------------- */

typedef struct {
    sink_job *j;
    uint32_t *out;
    uint64_t at, cap;
} icopy_job;

static void *icopy(void *arg) {
    icopy_job *c = (icopy_job *)arg;
    const uint64_t n = c->j->icnt;
    if (c->at < c->cap) memcpy(c->out + c->at, c->j->ipart, (c->at + n <= c->cap ? n : c->cap - c->at) * 4);
    return NULL;
}

static void add_stats(orc_geo_stats *to, const orc_geo_stats *s) {
    to->records += s->records;
    for (int k = 0; k < 2; k++) {
        to->values[k] += s->values[k];
        to->checksum[k] += s->checksum[k];
        to->sum_e6[k] = (int64_t)((uint64_t)to->sum_e6[k] + (uint64_t)s->sum_e6[k]);
        to->inexact[k] += s->inexact[k];
        to->fold[k] += s->fold[k];
    }
}

int orc_par_parse(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t *idx, uint64_t idx_cap,
                  uint64_t *n_idx, orc_col *cols, int ncols, uint64_t rows_cap, uint64_t *rows_out, uint64_t *fields,
                  uint64_t *bytes, uint32_t sf0, uint32_t sf1, orc_geo_stats *stats) {
    plan_t *pl = (plan_t *)malloc(sizeof(plan_t));
    make_plan(pl, dialect, d, n, threads);
    sink_job *jobs = (sink_job *)calloc((size_t)pl->threads, sizeof(sink_job));
    for (int t = 0; t < pl->threads; t++) {
        jobs[t].pl = pl;
        jobs[t].t = t;
        jobs[t].ncols = ncols;
        jobs[t].want_cols = ncols > 0;
        jobs[t].want_fb = fields != NULL;
        jobs[t].want_idx = n_idx != NULL;
        jobs[t].want_stats = stats != NULL;
        jobs[t].sf[0] = sf0;
        jobs[t].sf[1] = sf1;
        for (int k = 0; k < ncols; k++) {
            jobs[t].cols[k].field = cols[k].field;
            jobs[t].cols[k].type = cols[k].type;
        }
    }
    run_threads(pl->threads, sink_chunk, jobs, sizeof(sink_job));
    int over = 0;
    if (n_idx) {
        icopy_job ic[256];
        uint64_t total = 0;
        for (int t = 0; t < pl->threads; t++) {
            ic[t].j = &jobs[t];
            ic[t].out = idx;
            ic[t].at = total;
            ic[t].cap = idx_cap;
            total += jobs[t].icnt;
        }
        run_threads(pl->threads, icopy, ic, sizeof(icopy_job));
        *n_idx = total;
        if (total > idx_cap) over = 1;
    }
    if (fields) {
        uint64_t f = 0, b = 0;
        for (int t = 0; t < pl->threads; t++) {
            f += jobs[t].fields;
            b += jobs[t].bytes;
        }
        *fields = f;
        *bytes = b;
    }
    if (stats) {
        memset(stats, 0, sizeof *stats);
        for (int t = 0; t < pl->threads; t++) add_stats(stats, &jobs[t].st);
    }
    uint64_t rows = 0;
    if (ncols > 0) {
        uint64_t *arena_at = (uint64_t *)calloc((size_t)pl->threads * 32, 8);
        uint64_t alen[32] = {0};
        for (int k = 0; k < ncols; k++) {
            if (cols[k].valid) memset(cols[k].valid, 0, ((rows_cap + 63) / 64) * 8);
            if (cols[k].type == ORC_STR && cols[k].values) ((int32_t *)cols[k].values)[0] = 0;
        }
        for (int t = 0; t < pl->threads; t++) {
            jobs[t].row_at = rows;
            jobs[t].arena_at = arena_at + 32 * t;
            jobs[t].out = cols;
            jobs[t].rows_cap = rows_cap;
            for (int k = 0; k < ncols; k++) {
                jobs[t].arena_at[k] = alen[k];
                alen[k] += jobs[t].cols[k].alen;
            }
            rows += jobs[t].rows;
        }
        for (int k = 0; k < ncols; k++) {
            cols[k].str_len = alen[k];
            if (cols[k].type == ORC_STR && alen[k] > cols[k].str_cap) over = 1;
        }
        if (rows > rows_cap) over = 1;
        run_threads(pl->threads, sink_copy, jobs, sizeof(sink_job));
        free(arena_at);
    }
    if (rows_out) *rows_out = rows;
    for (int t = 0; t < pl->threads; t++) free_job(&jobs[t]);
    free(jobs);
    free(pl);
    return over ? -1 : 0;
}

void orc_par_geo_stats(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t f0, uint32_t f1,
                       orc_geo_stats *out) {
    orc_par_parse(dialect, d, n, threads, NULL, 0, NULL, NULL, 0, 0, NULL, NULL, NULL, f0, f1, out);
}
