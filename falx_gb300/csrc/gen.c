/*
 * Seeded synthetic inputs for the benchmark and test workloads.
 *
 * Output depends only on (kind, seed, target bytes): the document is cut into
 * a fixed number of segments, each generated from its own xorshift64* stream
 * (the generator of the reference's tests/common/mod.rs:6-16 and
 * examples/make_datasets.rs), then concatenated. Integer arithmetic only, so
 * x86 and Arm produce identical bytes.
 *
 *  FALX_GEN_CSV_GEO   id,City,Country,Population,Latitude,Longitude (LF, header row);
 *                     5% of City cells quoted with an embedded comma and a doubled quote.
 *  FALX_GEN_CSV_HASH  same columns; 2% whole-line '#' comments (1% of them with an
 *                     unmatched '"'); 3% of City cells quoted and holding '#'.
 *  FALX_GEN_NDJSON    {"id": u40, "name": ..., "nested": {"score": d.dddddd, "tags": [...]},
 *                     "active": bool} with 0-2 spaces around ':' and ','.
 *  FALX_GEN_TSV       the CSV_GEO columns tab-separated, no quoting.
 *  FALX_GEN_LOGFMT    id= city= country= population= lat= lon=, 3% quoted values.
 *  FALX_GEN_ADVERSARIAL csv_hash with 20% quoted cells up to 4 KiB holding '#', ',' and
 *                     newlines; 5% of comment lines with '"'.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum {
    FALX_GEN_CSV_GEO = 0,
    FALX_GEN_CSV_HASH = 1,
    FALX_GEN_NDJSON = 2,
    FALX_GEN_TSV = 3,
    FALX_GEN_LOGFMT = 4,
    FALX_GEN_ADVERSARIAL = 5
};

#define NSEG 64

typedef struct {
    uint64_t s;
} rng_t;

static uint64_t rnext(rng_t *r) {
    r->s ^= r->s >> 12;
    r->s ^= r->s << 25;
    r->s ^= r->s >> 27;
    return r->s * 0x2545F4914F6CDD1Dull;
}
static uint64_t below(rng_t *r, uint64_t n) { return rnext(r) % n; }

typedef struct {
    uint8_t *p;
    uint64_t n, cap;
} buf_t;

static void put(buf_t *b, uint8_t c) {
    if (b->n < b->cap) b->p[b->n] = c;
    b->n++;
}
static void puts_(buf_t *b, const char *s) {
    while (*s) put(b, (uint8_t)*s++);
}
static void put_u64(buf_t *b, uint64_t v) {
    char t[24];
    int k = 0;
    do {
        t[k++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (k) put(b, (uint8_t)t[--k]);
}
/* micro-units -> [-]d+.dddddd */
static void put_fixed6(buf_t *b, int64_t micro) {
    if (micro < 0) {
        put(b, '-');
        micro = -micro;
    }
    put_u64(b, (uint64_t)micro / 1000000);
    put(b, '.');
    uint64_t f = (uint64_t)micro % 1000000;
    char t[6];
    for (int k = 5; k >= 0; k--) {
        t[k] = (char)('0' + f % 10);
        f /= 10;
    }
    for (int k = 0; k < 6; k++) put(b, (uint8_t)t[k]);
}
static void put_letters(buf_t *b, rng_t *r, int lo, int hi, int with_space) {
    int n = lo + (int)below(r, (uint64_t)(hi - lo + 1));
    for (int i = 0; i < n; i++) {
        uint64_t c = below(r, with_space ? 53 : 52);
        put(b, c == 52 ? ' ' : (uint8_t)(c < 26 ? 'A' + c : 'a' + (c - 26)));
    }
}
static void put_upper(buf_t *b, rng_t *r, int n) {
    for (int i = 0; i < n; i++) put(b, (uint8_t)('A' + below(r, 26)));
}
static int64_t uniform_micro(rng_t *r, int64_t lim) { /* [-lim, lim] in 1e-6 */
    return (int64_t)below(r, (uint64_t)(2 * lim * 1000000 + 1)) - lim * 1000000;
}

static void city_cell(buf_t *b, rng_t *r, int hash_dialect) {
    uint64_t pct = below(r, 100);
    if (!hash_dialect && pct < 5) {
        put(b, '"');
        put_letters(b, r, 1, 8, 1);
        puts_(b, ", ");
        put_letters(b, r, 1, 6, 0);
        puts_(b, "\"\"");
        put_letters(b, r, 1, 5, 0);
        put(b, '"');
    } else if (hash_dialect && pct < 3) {
        put(b, '"');
        put_letters(b, r, 1, 6, 1);
        puts_(b, " #");
        put_letters(b, r, 1, 5, 0);
        if (below(r, 2)) {
            puts_(b, ", ");
            put_letters(b, r, 1, 5, 0);
        }
        if (below(r, 2)) {
            puts_(b, "\"\"");
            put_letters(b, r, 1, 4, 0);
        }
        put(b, '"');
    } else {
        put_letters(b, r, 3, 20, 1);
    }
}

static void geo_row(buf_t *b, rng_t *r, uint64_t id, char sep, int hash_dialect, int tsv) {
    put_u64(b, id);
    put(b, (uint8_t)sep);
    if (tsv) put_letters(b, r, 3, 20, 1);
    else city_cell(b, r, hash_dialect);
    put(b, (uint8_t)sep);
    put_upper(b, r, 2);
    put(b, (uint8_t)sep);
    put_u64(b, below(r, 10000001));
    put(b, (uint8_t)sep);
    put_fixed6(b, uniform_micro(r, 90));
    put(b, (uint8_t)sep);
    put_fixed6(b, uniform_micro(r, 180));
    put(b, '\n');
}

static void comment_line(buf_t *b, rng_t *r, int quote_pct_x10) {
    puts_(b, "# ");
    put_letters(b, r, 3, 12, 1);
    puts_(b, ", note");
    if ((int)below(r, 1000) < quote_pct_x10) {
        puts_(b, " \"");
        put_letters(b, r, 1, 8, 0);
    }
    put(b, '\n');
}

static void logfmt_key(buf_t *b, const char *key) {
    puts_(b, key);
    put(b, '=');
}

static void logfmt_row(buf_t *b, rng_t *r, uint64_t id) {
    int q;
    logfmt_key(b, "id");
    put_u64(b, id);
    put(b, ' ');
    logfmt_key(b, "city");
    q = below(r, 100) < 3;
    if (q) {
        put(b, '"');
        put_letters(b, r, 1, 8, 1);
        if (below(r, 2)) puts_(b, " \\\"x\\\" ");
        puts_(b, " a=b");
        put(b, '"');
    } else {
        put_letters(b, r, 3, 20, 0);
    }
    put(b, ' ');
    logfmt_key(b, "country");
    put_upper(b, r, 2);
    put(b, ' ');
    logfmt_key(b, "population");
    put_u64(b, below(r, 10000001));
    put(b, ' ');
    logfmt_key(b, "lat");
    put_fixed6(b, uniform_micro(r, 90));
    put(b, ' ');
    logfmt_key(b, "lon");
    put_fixed6(b, uniform_micro(r, 180));
    put(b, '\n');
}

static void spaces(buf_t *b, rng_t *r) {
    uint64_t n = below(r, 3);
    for (uint64_t i = 0; i < n; i++) put(b, ' ');
}

static void ndjson_row(buf_t *b, rng_t *r) {
    put(b, '{');
    puts_(b, "\"id\"");
    spaces(b, r);
    put(b, ':');
    spaces(b, r);
    put_u64(b, rnext(r) & ((1ull << 40) - 1));
    spaces(b, r);
    put(b, ',');
    spaces(b, r);
    puts_(b, "\"name\"");
    spaces(b, r);
    put(b, ':');
    spaces(b, r);
    put(b, '"');
    int nl = 4 + (int)below(r, 21);
    int esc = below(r, 100) < 2;
    int at = esc ? (int)below(r, (uint64_t)nl) : -1;
    for (int i = 0; i < nl; i++) {
        if (i == at) {
            static const char *E[] = {"\\\"", "\\\\", "\\n", "\\/"};
            puts_(b, E[below(r, 4)]);
        } else {
            put(b, (uint8_t)('a' + below(r, 26)));
        }
    }
    put(b, '"');
    spaces(b, r);
    put(b, ',');
    spaces(b, r);
    puts_(b, "\"nested\"");
    spaces(b, r);
    put(b, ':');
    spaces(b, r);
    put(b, '{');
    puts_(b, "\"score\"");
    spaces(b, r);
    put(b, ':');
    spaces(b, r);
    {
        int fd = 1 + (int)below(r, 6);
        uint64_t scale = 1;
        for (int i = 0; i < fd; i++) scale *= 10;
        int64_t v = (int64_t)below(r, 2000 * scale + 1) - (int64_t)(1000 * scale);
        if (v < 0) {
            put(b, '-');
            v = -v;
        }
        put_u64(b, (uint64_t)v / scale);
        put(b, '.');
        uint64_t f = (uint64_t)v % scale;
        char t[8];
        for (int k = fd - 1; k >= 0; k--) {
            t[k] = (char)('0' + f % 10);
            f /= 10;
        }
        for (int k = 0; k < fd; k++) put(b, (uint8_t)t[k]);
    }
    spaces(b, r);
    put(b, ',');
    spaces(b, r);
    puts_(b, "\"tags\"");
    spaces(b, r);
    put(b, ':');
    spaces(b, r);
    put(b, '[');
    int nt = (int)below(r, 6);
    for (int i = 0; i < nt; i++) {
        if (i) {
            put(b, ',');
            spaces(b, r);
        }
        put(b, '"');
        put_letters(b, r, 1, 6, 0);
        put(b, '"');
    }
    put(b, ']');
    put(b, '}');
    spaces(b, r);
    put(b, ',');
    spaces(b, r);
    puts_(b, "\"active\"");
    spaces(b, r);
    put(b, ':');
    spaces(b, r);
    puts_(b, below(r, 2) ? "true" : "false");
    put(b, '}');
    put(b, '\n');
}

static void adversarial_row(buf_t *b, rng_t *r, uint64_t id) {
    if (below(r, 100) < 2) {
        comment_line(b, r, 50);
        return;
    }
    for (int f = 0; f < 6; f++) {
        if (f) put(b, ',');
        if (below(r, 100) < 20) {
            put(b, '"');
            uint64_t n = below(r, 100) < 10 ? below(r, 4096) : below(r, 48);
            for (uint64_t i = 0; i < n; i++) {
                uint64_t c = below(r, 40);
                if (c == 0) put(b, '#');
                else if (c == 1) put(b, ',');
                else if (c == 2) put(b, '\n');
                else if (c == 3) puts_(b, "\"\"");
                else if (c == 4) puts_(b, "\n#");
                else put(b, (uint8_t)('a' + below(r, 26)));
            }
            put(b, '"');
        } else if (f == 0) {
            put_u64(b, id);
        } else {
            put_letters(b, r, 1, 12, 0);
        }
    }
    put(b, '\n');
}

typedef struct {
    int kind;
    uint64_t seed;
    uint64_t budget;
    int seg;
    buf_t out;
} seg_job;

static void *seg_run(void *arg) {
    seg_job *j = (seg_job *)arg;
    rng_t r = {j->seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(j->seg + 1))};
    if (r.s == 0) r.s = 1;
    for (int i = 0; i < 4; i++) rnext(&r);
    buf_t *b = &j->out;
    uint64_t id = (uint64_t)j->seg << 26;
    if (j->seg == 0) {
        if (j->kind == FALX_GEN_CSV_GEO || j->kind == FALX_GEN_CSV_HASH)
            puts_(b, "id,City,Country,Population,Latitude,Longitude\n");
        else if (j->kind == FALX_GEN_TSV)
            puts_(b, "id\tCity\tCountry\tPopulation\tLatitude\tLongitude\n");
        else if (j->kind == FALX_GEN_ADVERSARIAL)
            puts_(b, "# adversarial quoted cells\n");
    }
    while (b->n < j->budget) {
        switch (j->kind) {
        case FALX_GEN_CSV_GEO: geo_row(b, &r, id, ',', 0, 0); break;
        case FALX_GEN_CSV_HASH:
            if (below(&r, 100) < 2) comment_line(b, &r, 10);
            else geo_row(b, &r, id, ',', 1, 0);
            break;
        case FALX_GEN_NDJSON: ndjson_row(b, &r); break;
        case FALX_GEN_TSV: geo_row(b, &r, id, '\t', 0, 1); break;
        case FALX_GEN_LOGFMT: logfmt_row(b, &r, id); break;
        default: adversarial_row(b, &r, id); break;
        }
        id++;
    }
    return NULL;
}

/* Generate about `target` bytes into `out` (capacity `cap`); returns the
 * number of bytes the document has (written only up to `cap`). */
uint64_t falx_gen(int kind, uint64_t seed, uint64_t target, uint8_t *out, uint64_t cap, int threads) {
    seg_job jobs[NSEG];
    uint64_t per = target / NSEG;
    for (int k = 0; k < NSEG; k++) {
        jobs[k].kind = kind;
        jobs[k].seed = seed;
        jobs[k].budget = k == NSEG - 1 ? target - per * (NSEG - 1) : per;
        jobs[k].seg = k;
        jobs[k].out.cap = jobs[k].budget + 131072; /* slack for the row that crosses the budget */
        jobs[k].out.p = (uint8_t *)malloc(jobs[k].out.cap);
        jobs[k].out.n = 0;
    }
    if (threads < 1) threads = 1;
    if (threads > NSEG) threads = NSEG;
    for (int base = 0; base < NSEG; base += threads) {
        pthread_t th[NSEG];
        int n = 0;
        for (int k = base; k < NSEG && k < base + threads; k++, n++) pthread_create(&th[n], NULL, seg_run, &jobs[k]);
        for (int i = 0; i < n; i++) pthread_join(th[i], NULL);
    }
    uint64_t total = 0;
    for (int k = 0; k < NSEG; k++) {
        uint64_t n = jobs[k].out.n;
        if (n > jobs[k].out.cap) n = jobs[k].out.cap; /* a row overflowed the slack: cut it */
        if (total < cap) memcpy(out + total, jobs[k].out.p, (total + n <= cap) ? n : cap - total);
        total += n;
        free(jobs[k].out.p);
    }
    return total;
}
