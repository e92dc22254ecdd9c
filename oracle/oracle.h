/*
 * CPU oracle for the falx structural-index / column-materialisation path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product (falx_gb300/, include/)
 * links, loads or calls this code. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it, and only as the checker or as the timed
 * CPU baseline.
 *
 * It restates, in plain C, the serial semantics of the reference's generated
 * Rust parsers (Mapika/falx, the src/kernels/ modules) and of its byte-serial ground
 * truth (src/scalar.rs). The reference cannot be compiled here (no Rust
 * toolchain), so parity is pinned through the known-answer vectors held in
 * the reference's own tests (tests/ndjson_id_score.rs, tests/comments.rs,
 * tests/csv_hash_fused_par.rs, tests/columns.rs, src/lib.rs), committed as
 * fixtures under tests/golden/. The JSON-aware NDJSON sink (orc_ndjson_json)
 * covers input the reference rejects; beyond the reference's one integer
 * known answer its parity is unpinned.
 */
#ifndef FALX_ORACLE_H
#define FALX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Dialects: same numbering as include/falx_gpu.h. */
enum { ORC_CSV = 0, ORC_CSV_HASH = 1, ORC_TSV = 2, ORC_LOGFMT = 3, ORC_NDJSON = 4 };
/* Column types: same numbering as include/falx_gpu.h. */
enum { ORC_I64 = 0, ORC_U32 = 1, ORC_F64 = 2, ORC_STR = 3, ORC_BYTES = 4 };

/* Byte-serial structural index (src/scalar.rs:23-59). Returns the number of
 * structurals; writes at most `cap` of them. */
uint64_t orc_index_spec(int dialect, const uint8_t *d, uint64_t n, uint32_t *out, uint64_t cap);
uint64_t orc_index_seeded(int dialect, const uint8_t *d, uint64_t n, uint32_t state, int prev_byte,
                          uint64_t pos_base, uint32_t *out, uint64_t cap, uint32_t *exit_state, uint64_t *terms,
                          uint64_t *rows);

/* Blockwise restatement of the generated `step` kernels: 64-byte blocks,
 * zero-padded tail, carried state between blocks (csv_geo.rs:2117-2127,
 * csv_hash.rs:2125-2222, tsv.rs:1302-1308, logfmt.rs:994-1012,
 * ndjson.rs:1017-1033). Must equal orc_index_spec. */
uint64_t orc_index_blocks(int dialect, const uint8_t *d, uint64_t n, uint32_t *out, uint64_t cap);

/* Tape behind parse()/records() (csv_geo.rs:1809-1849): separator positions
 * and record ends `(cumulative_separators << 32) | position`. */
void orc_parse_tape(int dialect, const uint8_t *d, uint64_t n, uint32_t *seps, uint64_t seps_cap,
                    uint64_t *ends, uint64_t ends_cap, uint64_t *n_seps, uint64_t *n_ends);

/* One projected column (codegen Column: index + type). Buffers are caller
 * owned and sized for `rows_cap` rows. */
typedef struct {
    uint32_t field;
    uint32_t type;
    void *values;       /* I64: int64[rows]; U32: uint32[rows]; F64: double[rows];
                           BYTES: uint32[2*rows] (from,to); STR: int32 offsets[rows+1] */
    uint8_t *str_data;  /* STR arena */
    uint64_t str_cap;
    uint64_t str_len;   /* out */
    uint64_t *valid;    /* LSB-first validity words, ceil(rows_cap/64) */
} orc_col;

/* ColumnSink restatement (csv_geo.rs:952-1101, csv_hash.rs:1277-1435,
 * csv_typed.rs:1084-1138). Returns 0, or -1 if a capacity is too small
 * (rows_out is still set). */
int orc_parse_columns(int dialect, const uint8_t *d, uint64_t n, orc_col *cols, int ncols,
                      uint64_t rows_cap, uint64_t *rows_out);

/* Fused count/sum sink over two f64 fields (csv_geo.rs:1491-1770), extended
 * with an exact fixed-point (x1e6) sum and a sequential f64 fold. */
typedef struct {
    uint64_t records;
    uint64_t values[2];
    uint64_t checksum[2];   /* wrapping sum of f64 bit patterns */
    int64_t sum_e6[2];      /* exact sum of value*1e6 over cells that are exact in 1e-6 units */
    uint64_t inexact[2];    /* valid cells excluded from sum_e6 */
    double fold[2];         /* sequential left fold of the valid values, row order */
} orc_geo_stats;
void orc_geo_stats_run(int dialect, const uint8_t *d, uint64_t n, uint32_t field0, uint32_t field1,
                       orc_geo_stats *out);

/* Field-byte sink (csv_hash.rs:965-1230). */
void orc_field_bytes(int dialect, const uint8_t *d, uint64_t n, uint64_t *fields, uint64_t *bytes);

/* Literal-prefix NDJSON id+score sink (ndjson.rs:662-750). Returns 0, or -1
 * where the reference would panic on a schema mismatch. */
int orc_ndjson_literal(const uint8_t *d, uint64_t n, uint64_t *records, int64_t *sum);

/* JSON-aware id + nested.score sink for decimal scores. */
typedef struct {
    uint64_t records;
    int64_t sum_id;        /* wrapping */
    int64_t sum_score_e6;  /* wrapping */
    int64_t total_e6_lo;   /* exact 128-bit sum of id*1e6 + score_e6 */
    int64_t total_e6_hi;
    double total_f64;      /* (double)total_e6 / 1e6 */
} orc_ndjson_stats;
int orc_ndjson_json(const uint8_t *d, uint64_t n, orc_ndjson_stats *out);
int orc_par_ndjson_json(const uint8_t *d, uint64_t n, int threads, orc_ndjson_stats *out);
/* One count / sum cell: 1 if it holds a value (bits, and its exact x1e6
 * value when it has one). */
int orc_stats_cell(const uint8_t *raw, uint64_t len, uint64_t *bits, int64_t *e6, int *exact);

/* Cell decoders with str::parse semantics. */
int orc_parse_f64(const uint8_t *s, uint64_t len, double *out);
int orc_parse_i64(const uint8_t *s, uint64_t len, int64_t *out);
int orc_parse_u32(const uint8_t *s, uint64_t len, uint32_t *out);

/* City text lane (csv_geo_text.rs:1607-1640 CsvGeoTextStats). */
typedef struct {
    uint64_t records;
    uint64_t city_values, city_bytes, city_checksum; /* checksum: wrapping sum of cleaned byte values */
    uint64_t values[2];                             /* latitude, longitude */
    uint64_t checksum[2];                           /* wrapping sums of their f64 bit patterns */
} orc_text_stats;
void orc_geo_text_stats(int dialect, const uint8_t *d, uint64_t n, uint32_t city, uint32_t lat, uint32_t lon,
                        orc_text_stats *out);

/* Multi-threaded port of the reference's `_par` drivers, used as the timed
 * CPU baseline (csv_hash.rs:345-399 three-phase index, :1507-1601 columns,
 * :984-1051 field bytes; csv_geo.rs:1513-1561 stats; ndjson.rs:726-750). */
uint64_t orc_par_index(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t *out, uint64_t cap);
int orc_par_columns(int dialect, const uint8_t *d, uint64_t n, int threads, orc_col *cols, int ncols,
                    uint64_t rows_cap, uint64_t *rows_out);
void orc_par_field_bytes(int dialect, const uint8_t *d, uint64_t n, int threads, uint64_t *fields,
                         uint64_t *bytes);
/* Index, field bytes, columns and count / sum over fields sf0, sf1 from one
 * pass per chunk (any of n_idx, fields, ncols, stats may be absent / 0).
 * Returns -1 if an output was too small. */
int orc_par_parse(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t *idx, uint64_t idx_cap,
                  uint64_t *n_idx, orc_col *cols, int ncols, uint64_t rows_cap, uint64_t *rows_out, uint64_t *fields,
                  uint64_t *bytes, uint32_t sf0, uint32_t sf1, orc_geo_stats *stats);
/* Count / sum over fields f0, f1 (csv_geo.rs:1513-1561 parse_csv_geo_stats_par):
 * per chunk, then added; `fold` is the chunks' folds added in order. */
void orc_par_geo_stats(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t f0, uint32_t f1,
                       orc_geo_stats *out);

/* Raw DEFLATE and bgzf (inflate.c). Status codes, shared with the GPU
 * decoder's per-block status: */
#define ORC_Z_TRUNCATED 1
#define ORC_Z_BLOCK_TYPE 2
#define ORC_Z_STORED_LEN 3
#define ORC_Z_CODES 4
#define ORC_Z_SYMBOL 5
#define ORC_Z_DISTANCE 6
#define ORC_Z_OVERFLOW 7
#define ORC_Z_SIZE 8
typedef struct {
    uint64_t in_off, out_off;
    uint32_t in_len, out_len;
} orc_gz_block;
/* 0, or a status above: in[0, n) inflated to exactly out_len bytes */
int orc_inflate(const uint8_t *in, uint64_t n, uint8_t *out, uint64_t out_len);
/* the non-empty members; -1 if malformed; *total = inflated bytes */
int64_t orc_bgzf_scan(const uint8_t *c, uint64_t n, orc_gz_block *out, uint64_t cap, uint64_t *total);
uint64_t orc_bgzf_inflate_par(const uint8_t *comp, const orc_gz_block *blocks, uint64_t nb, uint8_t *out,
                              int32_t *status, int threads);

#ifdef __cplusplus
}
#endif
#endif
