/*
 * CPU oracle: serial restatement of the reference's structural-index and
 * column-materialisation semantics. TEST INFRASTRUCTURE ONLY (see oracle.h):
 * the product never links or calls this file.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Dialects (formats.rs:56-185).                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    const char *structural; /* NUL-terminated byte set */
    int quote;              /* -1 = none */
    int escape;             /* -1 = none */
    int comment;            /* -1 = none */
} orc_dialect;

static orc_dialect dialect_of(int d) {
    orc_dialect r;
    switch (d) {
    case ORC_CSV: r.structural = ",\n"; r.quote = '"'; r.escape = -1; r.comment = -1; break;
    case ORC_CSV_HASH: r.structural = ",\n"; r.quote = '"'; r.escape = -1; r.comment = '#'; break;
    case ORC_TSV: r.structural = "\t\n"; r.quote = -1; r.escape = -1; r.comment = -1; break;
    case ORC_LOGFMT: r.structural = " =\n"; r.quote = '"'; r.escape = '\\'; r.comment = -1; break;
    default: r.structural = "\n"; r.quote = '"'; r.escape = '\\'; r.comment = -1; break; /* NDJSON */
    }
    return r;
}

static int in_set(const char *set, uint8_t b) {
    for (; *set; set++)
        if ((uint8_t)*set == b) return 1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Byte-serial ground truth (scalar.rs:23-59).                                */
/* ------------------------------------------------------------------------- */

uint64_t orc_index_spec(int dialect, const uint8_t *d, uint64_t n, uint32_t *out, uint64_t cap) {
    orc_dialect dl = dialect_of(dialect);
    int in_quotes = 0, in_comment = 0, line_start = 1;
    uint64_t escape_run = 0, cnt = 0;
    for (uint64_t i = 0; i < n; i++) {
        uint8_t b = d[i];
        int escaped = (escape_run & 1) == 1;
        if (dl.escape >= 0 && b == (uint8_t)dl.escape) escape_run++;
        else escape_run = 0;
        if (in_comment) {
            if (b == '\n') {
                in_comment = 0;
                if (in_set(dl.structural, '\n')) {
                    if (cnt < cap) out[cnt] = (uint32_t)i;
                    cnt++;
                }
            }
        } else if (dl.quote >= 0 && b == (uint8_t)dl.quote) {
            if (!escaped) in_quotes = !in_quotes;
        } else if (!in_quotes && dl.comment >= 0 && b == (uint8_t)dl.comment && line_start) {
            in_comment = 1;
        } else if (!in_quotes && in_set(dl.structural, b)) {
            if (cnt < cap) out[cnt] = (uint32_t)i;
            cnt++;
        }
        line_start = b == '\n';
    }
    return cnt;
}

/* Seeded serial pass over one shard of a file (index_structurals_seeded,
 * csv_geo.rs:1855-1873; csv_hash seeds `line_start | region << 1`,
 * csv_hash.rs:1877, codegen.rs:1097-1106). `state` is the automaton state
 * before the shard in the engine's encoding (csv: in quotes; csv_hash: 0
 * normal, 1 quote, 2 comment; logfmt / ndjson: escape carry | quote parity
 * << 1), `prev_byte` the byte before it (-1: file start). Positions are
 * written plus pos_base. Returns the structural count; reports the exit
 * state, terminators and rows (record starts inside the shard, csv_hash
 * comment records excluded). */
uint64_t orc_index_seeded(int dialect, const uint8_t *d, uint64_t n, uint32_t state, int prev_byte,
                          uint64_t pos_base, uint32_t *out, uint64_t cap, uint32_t *exit_state, uint64_t *terms,
                          uint64_t *rows) {
    orc_dialect dl = dialect_of(dialect);
    int in_quotes, in_comment = 0;
    uint64_t escape_run = 0, cnt = 0, nterm = 0, nrows = 0;
    if (dialect == 1) {
        in_quotes = state == 1;
        in_comment = state == 2;
    } else if (dialect == 3 || dialect == 4) {
        escape_run = state & 1;
        in_quotes = (state >> 1) & 1;
    } else {
        in_quotes = (int)(state & 1);
    }
    int line_start = prev_byte < 0 || prev_byte == '\n';
    /* position 0 starts a record at the file start, or after a structural newline */
    int rec = prev_byte < 0 || (prev_byte == '\n' && !in_quotes && !in_comment);
    for (uint64_t i = 0; i < n; i++) {
        uint8_t b = d[i];
        if (rec) {
            if (!(dialect == 1 && b == '#')) nrows++;
            rec = 0;
        }
        int escaped = (escape_run & 1) == 1;
        if (dl.escape >= 0 && b == (uint8_t)dl.escape) escape_run++;
        else escape_run = 0;
        int st = 0;
        if (in_comment) {
            if (b == '\n') {
                in_comment = 0;
                st = in_set(dl.structural, '\n');
            }
        } else if (dl.quote >= 0 && b == (uint8_t)dl.quote) {
            if (!escaped) in_quotes = !in_quotes;
        } else if (!in_quotes && dl.comment >= 0 && b == (uint8_t)dl.comment && line_start) {
            in_comment = 1;
        } else if (!in_quotes && in_set(dl.structural, b)) {
            st = 1;
        }
        if (st) {
            if (cnt < cap) out[cnt] = (uint32_t)(pos_base + i);
            cnt++;
            if (b == '\n') {
                nterm++;
                rec = 1;
            }
        }
        line_start = b == '\n';
    }
    if (exit_state) {
        if (dialect == 1) *exit_state = in_comment ? 2u : in_quotes ? 1u : 0u;
        else if (dialect == 3 || dialect == 4) *exit_state = (uint32_t)((escape_run & 1) | ((uint64_t)in_quotes << 1));
        else if (dialect == 2) *exit_state = 0;
        else *exit_state = (uint32_t)in_quotes;
    }
    if (terms) *terms = nterm;
    if (rows) *rows = nrows;
    return cnt;
}

/* ------------------------------------------------------------------------- */
/* Blockwise restatement of the generated `step` functions.                   */
/* ------------------------------------------------------------------------- */

static uint64_t eq_mask(const uint8_t *blk, uint8_t c) {
    uint64_t m = 0;
    for (int i = 0; i < 64; i++) m |= (uint64_t)(blk[i] == c) << i;
    return m;
}

/* Bit i = XOR of bits 0..=i (interp.rs:143-151). */
static uint64_t prefix_xor(uint64_t x) {
    x ^= x << 1; x ^= x << 2; x ^= x << 4; x ^= x << 8; x ^= x << 16; x ^= x << 32;
    return x;
}

/* Bits [from, to) set (interp.rs:136-141). */
static uint64_t range_mask(unsigned from, unsigned to) {
    uint64_t hi = to >= 64 ? ~0ull : ((1ull << to) - 1);
    return hi & ~((1ull << from) - 1);
}

/* Three-state NORMAL/QUOTE/COMMENT resolver (interp.rs:93-133). */
static uint64_t resolve_regions(uint64_t q, uint64_t s, uint64_t nl, uint64_t *state) {
    uint64_t inert = 0, events = q | s | nl;
    unsigned run_start = 0;
    while (events) {
        unsigned p = (unsigned)__builtin_ctzll(events);
        uint64_t bit = 1ull << p;
        if (*state == 1) {
            if (q & bit) { inert |= range_mask(run_start, p); *state = 0; }
        } else if (*state == 2) {
            if (nl & bit) { inert |= range_mask(run_start, p); *state = 0; }
        } else {
            if (q & bit) { *state = 1; run_start = p; }
            else if (s & bit) { *state = 2; run_start = p; }
        }
        events &= events - 1;
    }
    if (*state != 0) inert |= range_mask(run_start, 64);
    return inert;
}

/* One 64-byte block -> (structural, terminator) masks; carries in c[2]. */
static void step_block(int dialect, const uint8_t *blk, uint64_t c[2], uint64_t *st, uint64_t *term) {
    const uint64_t EVEN = 0x5555555555555555ull;
    uint64_t nl = eq_mask(blk, '\n');
    uint64_t s;
    switch (dialect) {
    case ORC_CSV: {
        uint64_t par = prefix_xor(eq_mask(blk, '"')) ^ c[0];
        c[0] = (uint64_t)((int64_t)par >> 63);
        s = (nl | eq_mask(blk, ',')) & ~par;
        break;
    }
    case ORC_CSV_HASH: {
        uint64_t ls = (nl << 1) | c[0];
        c[0] = nl >> 63;
        uint64_t h = eq_mask(blk, '#') & ls;
        uint64_t inert = resolve_regions(eq_mask(blk, '"'), h, nl, &c[1]);
        s = (nl | eq_mask(blk, ',')) & ~inert;
        break;
    }
    case ORC_TSV:
        s = nl | eq_mask(blk, '\t');
        break;
    default: { /* LOGFMT, NDJSON: backslash escapes + quote parity */
        uint64_t bs = eq_mask(blk, '\\');
        uint64_t v2 = EVEN ^ bs;
        uint64_t partial = EVEN + v2;
        uint64_t c1 = partial < EVEN;
        uint64_t sum = partial + c[0];
        uint64_t c2 = sum < partial;
        c[0] = c1 | c2;
        uint64_t not_escaped = EVEN ^ sum;
        uint64_t uq = eq_mask(blk, '"') & not_escaped;
        uint64_t par = prefix_xor(uq) ^ c[1];
        c[1] = (uint64_t)((int64_t)par >> 63);
        uint64_t cls = nl;
        if (dialect == ORC_LOGFMT) cls |= eq_mask(blk, ' ') | eq_mask(blk, '=');
        s = cls & ~par;
        break;
    }
    }
    *st = s;
    *term = s & nl;
}

static void carry_init(int dialect, uint64_t c[2]) {
    c[0] = dialect == ORC_CSV_HASH ? 1 : 0; /* csv_hash CARRY_INIT = [1, 0] */
    c[1] = 0;
}

uint64_t orc_index_blocks(int dialect, const uint8_t *d, uint64_t n, uint32_t *out, uint64_t cap) {
    uint64_t c[2], cnt = 0;
    carry_init(dialect, c);
    uint8_t blk[64];
    for (uint64_t off = 0; off < n; off += 64) {
        uint64_t rem = n - off, live = ~0ull;
        const uint8_t *p = d + off;
        if (rem < 64) {
            memset(blk, 0, 64);
            memcpy(blk, p, rem);
            p = blk;
            live = (1ull << rem) - 1;
        }
        uint64_t st, term;
        step_block(dialect, p, c, &st, &term);
        st &= live;
        while (st) {
            if (cnt < cap) out[cnt] = (uint32_t)(off + __builtin_ctzll(st));
            cnt++;
            st &= st - 1;
        }
    }
    return cnt;
}

/* ------------------------------------------------------------------------- */
/* Tape (csv_geo.rs:1838-1849).                                               */
/* ------------------------------------------------------------------------- */

void orc_parse_tape(int dialect, const uint8_t *d, uint64_t n, uint32_t *seps, uint64_t seps_cap,
                    uint64_t *ends, uint64_t ends_cap, uint64_t *n_seps, uint64_t *n_ends) {
    uint64_t total = orc_index_spec(dialect, d, n, NULL, 0);
    uint32_t *idx = (uint32_t *)malloc((total ? total : 1) * sizeof(uint32_t));
    orc_index_spec(dialect, d, n, idx, total);
    uint64_t ns = 0, ne = 0;
    for (uint64_t i = 0; i < total; i++) {
        uint32_t p = idx[i];
        if (d[p] == '\n') {
            if (ne < ends_cap) ends[ne] = (ns << 32) | p;
            ne++;
        } else {
            if (ns < seps_cap) seps[ns] = p;
            ns++;
        }
    }
    free(idx);
    *n_seps = ns;
    *n_ends = ne;
}

/* ------------------------------------------------------------------------- */
/* Cell decoders.                                                             */
/* ------------------------------------------------------------------------- */

/* Strip outer quotes (len >= 2, both ends '"') and collapse doubled quotes
 * (csv_geo.rs:875-895). Returns the cleaned length written to `out`. */
static uint64_t clean_into(const uint8_t *raw, uint64_t len, uint8_t *out) {
    if (len >= 2 && raw[0] == '"' && raw[len - 1] == '"') {
        const uint8_t *in = raw + 1;
        uint64_t il = len - 2, o = 0, i = 0;
        while (i < il) {
            out[o++] = in[i];
            if (in[i] == '"' && i + 1 < il && in[i + 1] == '"') i += 2;
            else i += 1;
        }
        return o;
    }
    memcpy(out, raw, len);
    return len;
}

/* Length of the cleaned cell (csv_hash.rs:1207-1230). */
static uint64_t field_byte_len(const uint8_t *raw, uint64_t len) {
    if (len >= 2 && raw[0] == '"' && raw[len - 1] == '"') {
        uint64_t il = len - 2, o = 0, i = 0;
        const uint8_t *in = raw + 1;
        while (i < il) {
            o++;
            if (in[i] == '"' && i + 1 < il && in[i + 1] == '"') i += 2;
            else i += 1;
        }
        return o;
    }
    return len;
}

static int is_digit(uint8_t b) { return b >= '0' && b <= '9'; }

static int ieq(const uint8_t *s, uint64_t len, const char *lit) {
    uint64_t l = strlen(lit);
    if (len != l) return 0;
    for (uint64_t i = 0; i < l; i++) {
        uint8_t c = s[i];
        if (c >= 'A' && c <= 'Z') c = (uint8_t)(c + 32);
        if (c != (uint8_t)lit[i]) return 0;
    }
    return 1;
}

/* str::parse::<f64> grammar (core::num::dec2flt): [+-]? then either a decimal
 * with at least one mantissa digit and an optional exponent with at least one
 * digit, or inf / infinity / nan (ASCII case-insensitive). The value is the
 * correctly rounded IEEE double, taken from glibc strtod on the validated
 * text. */
int orc_parse_f64(const uint8_t *s, uint64_t len, double *out) {
    if (len == 0) return 0;
    int neg = 0;
    const uint8_t *p = s;
    uint64_t l = len;
    if (p[0] == '-' || p[0] == '+') { neg = p[0] == '-'; p++; l--; }
    if (l == 0) return 0;
    uint64_t i = 0, nd = 0;
    while (i < l && is_digit(p[i])) { i++; nd++; }
    if (i < l && p[i] == '.') {
        i++;
        while (i < l && is_digit(p[i])) { i++; nd++; }
    }
    int ok = nd > 0;
    if (ok && i < l && (p[i] == 'e' || p[i] == 'E')) {
        i++;
        if (i < l && (p[i] == '+' || p[i] == '-')) i++;
        uint64_t ed = 0;
        while (i < l && is_digit(p[i])) { i++; ed++; }
        if (ed == 0) ok = 0;
    }
    if (ok && i == l) {
        char stackbuf[128];
        char *buf = len < sizeof stackbuf ? stackbuf : (char *)malloc(len + 1);
        memcpy(buf, s, len);
        buf[len] = 0;
        *out = strtod(buf, NULL);
        if (buf != stackbuf) free(buf);
        return 1;
    }
    union { uint64_t u; double f; } v;
    if (ieq(p, l, "inf") || ieq(p, l, "infinity")) v.u = 0x7FF0000000000000ull;
    else if (ieq(p, l, "nan")) v.u = 0x7FF8000000000000ull;
    else return 0;
    if (neg) v.u |= 0x8000000000000000ull;
    *out = v.f;
    return 1;
}

/* str::parse::<i64>: optional sign (not alone), ASCII digits, no overflow. */
int orc_parse_i64(const uint8_t *s, uint64_t len, int64_t *out) {
    if (len == 0) return 0;
    int neg = 0;
    uint64_t i = 0;
    if (s[0] == '+' || s[0] == '-') {
        if (len == 1) return 0;
        neg = s[0] == '-';
        i = 1;
    }
    /* accumulate negatively so INT64_MIN parses */
    int64_t v = 0;
    for (; i < len; i++) {
        if (!is_digit(s[i])) return 0;
        int64_t dg = s[i] - '0';
        if (v < (INT64_MIN + dg) / 10) return 0;
        if (v * 10 < INT64_MIN + dg) return 0;
        v = v * 10 - dg;
    }
    if (!neg) {
        if (v == INT64_MIN) return 0;
        v = -v;
    }
    *out = v;
    return 1;
}

/* str::parse::<u32>: optional '+' (not alone), ASCII digits, <= u32::MAX. */
int orc_parse_u32(const uint8_t *s, uint64_t len, uint32_t *out) {
    if (len == 0) return 0;
    uint64_t i = 0;
    if (s[0] == '+') {
        if (len == 1) return 0;
        i = 1;
    }
    uint64_t v = 0;
    for (; i < len; i++) {
        if (!is_digit(s[i])) return 0;
        v = v * 10 + (uint64_t)(s[i] - '0');
        if (v > 0xFFFFFFFFull) return 0;
    }
    *out = (uint32_t)v;
    return 1;
}

/* Cells are cleaned first only when they start with a quote
 * (csv_geo.rs:1480-1486, csv_hash.rs:1784-1791). */
static const uint8_t *numeric_view(const uint8_t *raw, uint64_t len, uint8_t *scratch, uint64_t *ol) {
    if (len > 0 && raw[0] == '"') {
        *ol = clean_into(raw, len, scratch);
        return scratch;
    }
    *ol = len;
    return raw;
}

/* Exact value*1e6 for cells of the form [+-]?d*(.d{0,6})? with at least one
 * digit and |value*1e6| < 2^63. Returns 0 when the cell is not exact in
 * micro-units (more fraction digits, an exponent, inf/nan, overflow). */
static int exact_e6(const uint8_t *s, uint64_t len, int64_t *out) {
    uint64_t i = 0;
    int neg = 0;
    if (len && (s[0] == '+' || s[0] == '-')) { neg = s[0] == '-'; i = 1; }
    uint64_t ip = 0, nd = 0;
    int over = 0;
    while (i < len && is_digit(s[i])) {
        if (ip > 922337203684ull) over = 1;
        ip = ip * 10 + (uint64_t)(s[i] - '0');
        i++; nd++;
    }
    uint64_t fr = 0, nf = 0;
    if (i < len && s[i] == '.') {
        i++;
        while (i < len && is_digit(s[i])) {
            if (nf == 6) return 0;
            fr = fr * 10 + (uint64_t)(s[i] - '0');
            i++; nf++; nd++;
        }
    }
    if (nd == 0 || i != len || over) return 0;
    for (; nf < 6; nf++) fr *= 10;
    if (ip > 9223372036853ull) return 0;
    uint64_t m = ip * 1000000ull + fr;
    if (m > (uint64_t)INT64_MAX) return 0;
    *out = neg ? -(int64_t)m : (int64_t)m;
    return 1;
}

/* ------------------------------------------------------------------------- */
/* Record walker shared by the sinks: drives structurals in order like the    */
/* generated ColumnSink::drive / flush / finish (csv_geo.rs:952-1101).         */
/* ------------------------------------------------------------------------- */

typedef struct {
    uint64_t record_start;
    uint64_t end;     /* terminator position or n */
    uint64_t to;      /* end with a trailing \r trimmed */
    uint32_t nfields;
    uint32_t *fstart; /* nfields entries */
    uint32_t *fend;
} orc_record;

typedef void (*record_fn)(void *ctx, const uint8_t *d, const orc_record *r);

static void walk_records(int dialect, const uint8_t *d, uint64_t n, record_fn fn, void *ctx) {
    uint64_t total = orc_index_spec(dialect, d, n, NULL, 0);
    uint32_t *idx = (uint32_t *)malloc((total ? total : 1) * sizeof(uint32_t));
    orc_index_spec(dialect, d, n, idx, total);
    uint64_t fcap = 64;
    uint32_t *fs = (uint32_t *)malloc(fcap * 4), *fe = (uint32_t *)malloc(fcap * 4);
    uint64_t record_start = 0, field_start = 0, nf = 0;
    orc_record r;
    for (uint64_t k = 0; k <= total; k++) {
        int last = k == total;
        uint64_t p = last ? n : idx[k];
        int is_term = !last && d[p] == '\n';
        if (last && record_start >= n) break; /* no trailing record */
        if (nf + 1 >= fcap) {
            fcap *= 2;
            fs = (uint32_t *)realloc(fs, fcap * 4);
            fe = (uint32_t *)realloc(fe, fcap * 4);
        }
        if (is_term || last) {
            uint64_t to = (p > record_start && d[p - 1] == '\r') ? p - 1 : p;
            fs[nf] = (uint32_t)field_start;
            fe[nf] = (uint32_t)to;
            nf++;
            r.record_start = record_start;
            r.end = p;
            r.to = to;
            r.nfields = (uint32_t)nf;
            r.fstart = fs;
            r.fend = fe;
            fn(ctx, d, &r);
            record_start = p + 1;
            field_start = p + 1;
            nf = 0;
        } else {
            fs[nf] = (uint32_t)field_start;
            fe[nf] = (uint32_t)p;
            nf++;
            field_start = p + 1;
        }
    }
    free(fs);
    free(fe);
    free(idx);
}

/* Comment record: first byte '#' and end > record_start (csv_hash.rs:1381). */
static int is_comment(int dialect, const uint8_t *d, const orc_record *r) {
    return dialect == ORC_CSV_HASH && r->end > r->record_start && d[r->record_start] == '#';
}

/* --------------------------- columns ------------------------------------- */

typedef struct {
    int dialect;
    orc_col *cols;
    int ncols;
    uint64_t rows_cap;
    uint64_t rows;
    int overflow;
    uint8_t *scratch;
    uint64_t scratch_cap;
} cols_ctx;

static void cols_record(void *vctx, const uint8_t *d, const orc_record *r) {
    cols_ctx *c = (cols_ctx *)vctx;
    if (is_comment(c->dialect, d, r)) return;
    uint64_t row = c->rows;
    if (row >= c->rows_cap) { c->overflow = 1; c->rows++; return; }
    for (int k = 0; k < c->ncols; k++) {
        orc_col *col = &c->cols[k];
        int present = col->field < r->nfields;
        const uint8_t *raw = present ? d + r->fstart[col->field] : NULL;
        uint64_t len = present ? r->fend[col->field] - r->fstart[col->field] : 0;
        if (present && len > c->scratch_cap) {
            c->scratch_cap = len * 2;
            c->scratch = (uint8_t *)realloc(c->scratch, c->scratch_cap);
        }
        int ok = 0;
        switch (col->type) {
        case ORC_I64: {
            int64_t v = 0;
            if (present) {
                uint64_t vl;
                const uint8_t *vs = numeric_view(raw, len, c->scratch, &vl);
                ok = orc_parse_i64(vs, vl, &v);
            }
            ((int64_t *)col->values)[row] = ok ? v : 0;
            break;
        }
        case ORC_U32: {
            uint32_t v = 0;
            if (present) {
                uint64_t vl;
                const uint8_t *vs = numeric_view(raw, len, c->scratch, &vl);
                ok = orc_parse_u32(vs, vl, &v);
            }
            ((uint32_t *)col->values)[row] = ok ? v : 0;
            break;
        }
        case ORC_F64: {
            double v = 0.0;
            if (present) {
                uint64_t vl;
                const uint8_t *vs = numeric_view(raw, len, c->scratch, &vl);
                ok = orc_parse_f64(vs, vl, &v);
            }
            ((double *)col->values)[row] = ok ? v : 0.0;
            break;
        }
        case ORC_STR: {
            int32_t *offs = (int32_t *)col->values;
            if (row == 0) offs[0] = 0;
            if (present) {
                uint64_t cl = clean_into(raw, len, c->scratch);
                if (col->str_len + cl <= col->str_cap) memcpy(col->str_data + col->str_len, c->scratch, cl);
                else c->overflow = 1;
                col->str_len += cl;
                ok = 1;
            }
            offs[row + 1] = (int32_t)col->str_len;
            break;
        }
        default: { /* BYTES: raw span, valid iff present and non-empty */
            uint32_t *sp = (uint32_t *)col->values;
            ok = present && len > 0;
            sp[2 * row] = ok ? r->fstart[col->field] : 0;
            sp[2 * row + 1] = ok ? r->fend[col->field] : 0;
            break;
        }
        }
        if (ok) col->valid[row >> 6] |= 1ull << (row & 63);
    }
    c->rows++;
}

int orc_parse_columns(int dialect, const uint8_t *d, uint64_t n, orc_col *cols, int ncols,
                      uint64_t rows_cap, uint64_t *rows_out) {
    cols_ctx c = {dialect, cols, ncols, rows_cap, 0, 0, NULL, 0};
    for (int k = 0; k < ncols; k++) {
        cols[k].str_len = 0;
        if (cols[k].valid) memset(cols[k].valid, 0, ((rows_cap + 63) / 64) * 8);
        if (cols[k].type == ORC_STR && cols[k].values) ((int32_t *)cols[k].values)[0] = 0;
    }
    walk_records(dialect, d, n, cols_record, &c);
    free(c.scratch);
    *rows_out = c.rows;
    return c.overflow ? -1 : 0;
}

/* --------------------------- stats --------------------------------------- */

typedef struct {
    int dialect;
    uint32_t f[2];
    orc_geo_stats *st;
    uint8_t *scratch;
    uint64_t scratch_cap;
} stats_ctx;

static void stats_record(void *vctx, const uint8_t *d, const orc_record *r) {
    stats_ctx *c = (stats_ctx *)vctx;
    if (is_comment(c->dialect, d, r)) return;
    c->st->records++;
    for (int k = 0; k < 2; k++) {
        if (c->f[k] >= r->nfields) continue;
        const uint8_t *raw = d + r->fstart[c->f[k]];
        uint64_t len = r->fend[c->f[k]] - r->fstart[c->f[k]];
        if (len > c->scratch_cap) {
            c->scratch_cap = len * 2;
            c->scratch = (uint8_t *)realloc(c->scratch, c->scratch_cap);
        }
        uint64_t vl;
        const uint8_t *vs = numeric_view(raw, len, c->scratch, &vl);
        double v;
        if (!orc_parse_f64(vs, vl, &v)) continue;
        union { double f; uint64_t u; } b;
        b.f = v;
        c->st->values[k]++;
        c->st->checksum[k] += b.u;
        c->st->fold[k] += v;
        int64_t e6;
        if (exact_e6(vs, vl, &e6)) c->st->sum_e6[k] = (int64_t)((uint64_t)c->st->sum_e6[k] + (uint64_t)e6);
        else c->st->inexact[k]++;
    }
}

/* One count / sum cell (the stats sink's per-cell work). */
int orc_stats_cell(const uint8_t *raw, uint64_t len, uint64_t *bits, int64_t *e6, int *exact) {
    uint8_t small[256];
    uint8_t *scratch = len <= sizeof small ? small : (uint8_t *)malloc(len);
    uint64_t vl;
    const uint8_t *vs = numeric_view(raw, len, scratch, &vl);
    double v;
    int ok = orc_parse_f64(vs, vl, &v);
    if (ok) {
        union { double f; uint64_t u; } b;
        b.f = v;
        *bits = b.u;
        *exact = exact_e6(vs, vl, e6);
    }
    if (scratch != small) free(scratch);
    return ok;
}

void orc_geo_stats_run(int dialect, const uint8_t *d, uint64_t n, uint32_t field0, uint32_t field1,
                       orc_geo_stats *out) {
    memset(out, 0, sizeof *out);
    stats_ctx c = {dialect, {field0, field1}, out, NULL, 0};
    walk_records(dialect, d, n, stats_record, &c);
    free(c.scratch);
}

/* --------------------------- City text lane ------------------------------ */
/* CsvGeoTextStats (csv_geo_text.rs:1845-1937): per record, the city cell's
 * presence, cleaned length and the wrapping sum of its cleaned byte values;
 * the lat / lon cells' values and wrapping sums of their f64 bit patterns
 * (numeric cells cleaned first when they open with a quote). */
typedef struct {
    int dialect;
    uint32_t f[3];
    orc_text_stats *st;
} text_ctx;

static void text_record(void *vctx, const uint8_t *d, const orc_record *r) {
    text_ctx *c = (text_ctx *)vctx;
    if (is_comment(c->dialect, d, r)) return;
    c->st->records++;
    if (c->f[0] < r->nfields) {
        const uint8_t *raw = d + r->fstart[c->f[0]];
        const uint64_t len = r->fend[c->f[0]] - r->fstart[c->f[0]];
        uint64_t bytes = 0, sum = 0;
        if (len >= 2 && raw[0] == '"' && raw[len - 1] == '"') {
            const uint8_t *in = raw + 1;
            const uint64_t il = len - 2;
            uint64_t i = 0;
            while (i < il) {
                bytes++;
                sum += in[i];
                i += (in[i] == '"' && i + 1 < il && in[i + 1] == '"') ? 2 : 1;
            }
        } else {
            bytes = len;
            for (uint64_t i = 0; i < len; i++) sum += raw[i];
        }
        c->st->city_values++;
        c->st->city_bytes += bytes;
        c->st->city_checksum += sum;
    }
    for (int k = 0; k < 2; k++) {
        const uint32_t f = c->f[1 + k];
        if (f >= r->nfields) continue;
        uint64_t bits;
        int64_t e6;
        int exact;
        if (!orc_stats_cell(d + r->fstart[f], r->fend[f] - r->fstart[f], &bits, &e6, &exact)) continue;
        c->st->values[k]++;
        c->st->checksum[k] += bits;
    }
}

void orc_geo_text_stats(int dialect, const uint8_t *d, uint64_t n, uint32_t city, uint32_t lat, uint32_t lon,
                        orc_text_stats *out) {
    memset(out, 0, sizeof *out);
    text_ctx c = {dialect, {city, lat, lon}, out};
    walk_records(dialect, d, n, text_record, &c);
}

/* --------------------------- field bytes --------------------------------- */

typedef struct {
    int dialect;
    uint64_t fields, bytes;
} fb_ctx;

static void fb_record(void *vctx, const uint8_t *d, const orc_record *r) {
    fb_ctx *c = (fb_ctx *)vctx;
    if (is_comment(c->dialect, d, r)) return;
    for (uint32_t k = 0; k < r->nfields; k++) {
        c->fields++;
        c->bytes += field_byte_len(d + r->fstart[k], r->fend[k] - r->fstart[k]);
    }
}

void orc_field_bytes(int dialect, const uint8_t *d, uint64_t n, uint64_t *fields, uint64_t *bytes) {
    fb_ctx c = {dialect, 0, 0};
    walk_records(dialect, d, n, fb_record, &c);
    *fields = c.fields;
    *bytes = c.bytes;
}

/* ------------------------------------------------------------------------- */
/* NDJSON literal sink (ndjson.rs:679-880).                                    */
/* ------------------------------------------------------------------------- */

static int parse_ndjson_i64_at(const uint8_t *d, uint64_t n, uint64_t i, int64_t *v, uint64_t *after) {
    if (i >= n) return 0;
    int neg = d[i] == '-';
    if (neg) i++;
    if (i >= n || !is_digit(d[i])) return 0;
    uint64_t val = 0;
    while (i < n && is_digit(d[i])) {
        val = val * 10 + (uint64_t)(d[i] - '0');
        i++;
    }
    *v = neg ? (int64_t)(0 - val) : (int64_t)val;
    *after = i;
    return 1;
}

int orc_ndjson_literal(const uint8_t *d, uint64_t n, uint64_t *records, int64_t *sum) {
    static const char ID[] = "{\"id\":";
    static const char SC[] = "],\"nested\":{\"score\":";
    uint64_t recs = 0, s = 0, i = 0;
    const uint64_t lid = sizeof ID - 1, lsc = sizeof SC - 1;
    while (i < n) {
        while (i < n && (d[i] == '\n' || d[i] == '\r')) i++;
        if (i >= n) break;
        if (n - i < lid || memcmp(d + i, ID, lid) != 0) return -1;
        int64_t id, score;
        uint64_t after;
        if (!parse_ndjson_i64_at(d, n, i + lid, &id, &after)) return -1;
        const uint8_t *hit = (const uint8_t *)memmem(d + after, n - after, SC, lsc);
        if (!hit) return -1;
        uint64_t key = (uint64_t)(hit - d);
        uint64_t after_score;
        if (!parse_ndjson_i64_at(d, n, key + lsc, &score, &after_score)) return -1;
        recs++;
        s += (uint64_t)id + (uint64_t)score;
        const uint8_t *nlp = (const uint8_t *)memchr(d + after_score, '\n', n - after_score);
        i = nlp ? (uint64_t)(nlp - d) + 1 : n;
    }
    *records = recs;
    *sum = (int64_t)s;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* JSON-aware id + nested.score sink.                                         */
/* Each line (records separated by raw '\n'; blank and '\r'-only lines are     */
/* skipped, as the literal sink does) must hold one JSON object whose member   */
/* "id" is an integer and whose member "nested" is an object holding a member  */
/* "score" that is a decimal with at most 6 fraction digits and no exponent.   */
/* Any other shape is a schema error (-1).                                     */
/* ------------------------------------------------------------------------- */

static void skip_ws(const uint8_t *d, uint64_t e, uint64_t *i) {
    while (*i < e && (d[*i] == ' ' || d[*i] == '\t' || d[*i] == '\r')) (*i)++;
}

/* Skip a JSON string starting at the opening quote; returns 0 on error. */
static int skip_string(const uint8_t *d, uint64_t e, uint64_t *i) {
    (*i)++;
    while (*i < e) {
        uint8_t c = d[*i];
        if (c == '\\') { *i += 2; continue; }
        (*i)++;
        if (c == '"') return 1;
    }
    return 0;
}

static int skip_value(const uint8_t *d, uint64_t e, uint64_t *i);

static int skip_composite(const uint8_t *d, uint64_t e, uint64_t *i) {
    int depth = 0;
    while (*i < e) {
        uint8_t c = d[*i];
        if (c == '"') { if (!skip_string(d, e, i)) return 0; continue; }
        if (c == '{' || c == '[') depth++;
        else if (c == '}' || c == ']') {
            depth--;
            if (depth == 0) { (*i)++; return 1; }
        }
        (*i)++;
    }
    return 0;
}

static int skip_value(const uint8_t *d, uint64_t e, uint64_t *i) {
    skip_ws(d, e, i);
    if (*i >= e) return 0;
    uint8_t c = d[*i];
    if (c == '"') return skip_string(d, e, i);
    if (c == '{' || c == '[') return skip_composite(d, e, i);
    while (*i < e && d[*i] != ',' && d[*i] != '}' && d[*i] != ']' && d[*i] != ' ' && d[*i] != '\t' &&
           d[*i] != '\r')
        (*i)++;
    return 1;
}

static int key_is(const uint8_t *d, uint64_t ks, uint64_t ke, const char *k) {
    uint64_t l = strlen(k);
    return ke - ks == l + 2 && memcmp(d + ks + 1, k, l) == 0;
}

/* JSON integer: -?(0|[1-9]d*), no fraction or exponent. */
static int json_int(const uint8_t *d, uint64_t e, uint64_t *i, int64_t *out) {
    uint64_t j = *i;
    int neg = 0;
    if (j < e && d[j] == '-') { neg = 1; j++; }
    if (j >= e || !is_digit(d[j])) return 0;
    uint64_t v = 0, nd = 0;
    while (j < e && is_digit(d[j])) { v = v * 10 + (uint64_t)(d[j] - '0'); j++; nd++; }
    if (nd > 19) return 0;
    *out = neg ? (int64_t)(0 - v) : (int64_t)v;
    *i = j;
    return 1;
}

/* JSON decimal with at most 6 fraction digits, as an exact x1e6 integer. */
static int json_dec_e6(const uint8_t *d, uint64_t e, uint64_t *i, int64_t *out) {
    uint64_t j = *i;
    int neg = 0;
    if (j < e && d[j] == '-') { neg = 1; j++; }
    if (j >= e || !is_digit(d[j])) return 0;
    uint64_t ip = 0, nd = 0;
    while (j < e && is_digit(d[j])) { ip = ip * 10 + (uint64_t)(d[j] - '0'); j++; nd++; }
    if (nd > 12) return 0;
    uint64_t fr = 0, nf = 0;
    if (j < e && d[j] == '.') {
        j++;
        if (j >= e || !is_digit(d[j])) return 0;
        while (j < e && is_digit(d[j])) {
            if (nf == 6) return 0;
            fr = fr * 10 + (uint64_t)(d[j] - '0');
            j++; nf++;
        }
    }
    if (j < e && (d[j] == 'e' || d[j] == 'E')) return 0;
    for (; nf < 6; nf++) fr *= 10;
    uint64_t m = ip * 1000000ull + fr;
    *out = neg ? -(int64_t)m : (int64_t)m;
    *i = j;
    return 1;
}

/* Find member `key` of the object whose '{' is at *i; leave *i at its value. */
static int find_member(const uint8_t *d, uint64_t e, uint64_t *i, const char *key) {
    uint64_t j = *i;
    if (j >= e || d[j] != '{') return 0;
    j++;
    for (;;) {
        skip_ws(d, e, &j);
        if (j >= e || d[j] != '"') return 0;
        uint64_t ks = j;
        if (!skip_string(d, e, &j)) return 0;
        uint64_t ke = j;
        skip_ws(d, e, &j);
        if (j >= e || d[j] != ':') return 0;
        j++;
        skip_ws(d, e, &j);
        if (key_is(d, ks, ke, key)) { *i = j; return 1; }
        if (!skip_value(d, e, &j)) return 0;
        skip_ws(d, e, &j);
        if (j < e && d[j] == ',') { j++; continue; }
        return 0;
    }
}

/* Parallel form: chunks snapped to the byte after a newline, totals added
 * (records are independent lines, ndjson.rs:857-880). */
typedef struct {
    const uint8_t *d;
    uint64_t lo, hi;
    orc_ndjson_stats st;
    int rc;
} nd_job;

static void *nd_part(void *arg) {
    nd_job *j = (nd_job *)arg;
    j->rc = orc_ndjson_json(j->d + j->lo, j->hi - j->lo, &j->st);
    return NULL;
}

int orc_par_ndjson_json(const uint8_t *d, uint64_t n, int threads, orc_ndjson_stats *out) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    nd_job jobs[256];
    pthread_t th[256];
    uint64_t b[257];
    b[0] = 0;
    for (int t = 1; t < threads; t++) {
        uint64_t x = n / (uint64_t)threads * (uint64_t)t;
        if (x < b[t - 1]) x = b[t - 1];
        const uint8_t *nl = x < n ? (const uint8_t *)memchr(d + x, '\n', n - x) : NULL;
        b[t] = nl ? (uint64_t)(nl - d) + 1 : n;
    }
    b[threads] = n;
    for (int t = 0; t < threads; t++) {
        jobs[t].d = d;
        jobs[t].lo = b[t];
        jobs[t].hi = b[t + 1];
        pthread_create(&th[t], NULL, nd_part, &jobs[t]);
    }
    __int128 total = 0;
    int rc = 0;
    memset(out, 0, sizeof *out);
    for (int t = 0; t < threads; t++) {
        pthread_join(th[t], NULL);
        if (jobs[t].rc) rc = -1;
        out->records += jobs[t].st.records;
        out->sum_id = (int64_t)((uint64_t)out->sum_id + (uint64_t)jobs[t].st.sum_id);
        out->sum_score_e6 = (int64_t)((uint64_t)out->sum_score_e6 + (uint64_t)jobs[t].st.sum_score_e6);
        total += ((__int128)jobs[t].st.total_e6_hi << 64) | (__int128)(uint64_t)jobs[t].st.total_e6_lo;
    }
    out->total_e6_lo = (int64_t)(uint64_t)total;
    out->total_e6_hi = (int64_t)(total >> 64);
    out->total_f64 = (double)total / 1e6;
    return rc;
}

int orc_ndjson_json(const uint8_t *d, uint64_t n, orc_ndjson_stats *out) {
    memset(out, 0, sizeof *out);
    __int128 total = 0;
    uint64_t i = 0;
    while (i < n) {
        const uint8_t *nlp = (const uint8_t *)memchr(d + i, '\n', n - i);
        uint64_t e = nlp ? (uint64_t)(nlp - d) : n;
        uint64_t j = i;
        skip_ws(d, e, &j);
        if (j < e) {
            uint64_t a = j, b = j;
            int64_t id, sc;
            if (!find_member(d, e, &a, "id") || !json_int(d, e, &a, &id)) return -1;
            if (!find_member(d, e, &b, "nested") || !find_member(d, e, &b, "score") ||
                !json_dec_e6(d, e, &b, &sc))
                return -1;
            out->records++;
            out->sum_id = (int64_t)((uint64_t)out->sum_id + (uint64_t)id);
            out->sum_score_e6 = (int64_t)((uint64_t)out->sum_score_e6 + (uint64_t)sc);
            total += (__int128)id * 1000000 + sc;
        }
        i = e + 1;
    }
    out->total_e6_lo = (int64_t)(uint64_t)total;
    out->total_e6_hi = (int64_t)(total >> 64);
    out->total_f64 = (double)total / 1e6;
    return 0;
}
