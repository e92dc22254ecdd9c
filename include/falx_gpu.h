/*
 * falx_gpu.h — C ABI of the GB300 structural-index / column-materialisation
 * engine. Drop-in boundary for the generated falx parser modules
 * (Mapika/falx src/kernels/{csv_geo,csv_hash,csv_typed,tsv,logfmt,ndjson}.rs):
 * each entry point below cites the reference function it replaces.
 *
 * Conventions
 *  - Plain pointers and sizes only. Unless a name says `_host`, data and
 *    output buffers are device pointers in the context's device, owned by the
 *    caller; the library never frees them.
 *  - Every call is stream-ordered on the context's stream and returns after
 *    the stream has drained, so counts are valid on return.
 *  - Return 0 (FALX_OK) or a negative FALX_ERR_* code; nothing traps.
 *    On FALX_ERR_CAPACITY the counts are still reported, so callers can
 *    resize and retry (the reference's Vec outputs grow instead).
 *  - Offsets are u32, so inputs must be shorter than 4 GiB
 *    (the reference's limit as well: csv_geo.rs push_indexes stores u32).
 *  - A context is single-stream and not thread-safe; use one per host thread.
 *  - Device input is read in whole 16-byte-aligned chunks (bulk copies), so
 *    the bytes of the chunks that hold data[0] and data[len-1] are read too;
 *    they stay inside the allocation (CUDA allocations are at least 256-byte
 *    aligned and granular) and never affect the results.
 */
#ifndef FALX_GPU_H
#define FALX_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FALX_OK 0
#define FALX_ERR_INVALID (-1)          /* null pointer, unknown dialect, bad schema */
#define FALX_ERR_CAPACITY (-2)         /* an output buffer is too small; counts reported */
#define FALX_ERR_INPUT_TOO_LARGE (-3)  /* len >= 4 GiB */
#define FALX_ERR_SCHEMA (-4)           /* NDJSON record outside the id+score schema */
#define FALX_ERR_TIMEOUT (-5)          /* a device-side wait gave up; outputs undefined */
#define FALX_ERR_CUDA (-6)             /* CUDA runtime error */
#define FALX_ERR_OVERFLOW (-7)         /* string arena beyond i32 offsets (2 GiB) */
#define FALX_ERR_FORMAT (-8)           /* not a bgzf stream, or a block that does not inflate */

/* Dialects (formats.rs:56-185). */
typedef enum {
    FALX_CSV = 0,      /* ',' '\n', doubled-quote regions          (csv_dialect) */
    FALX_CSV_HASH = 1, /* as CSV plus '#' comment lines             (csv_hash_dialect) */
    FALX_TSV = 2,      /* '\t' '\n', no quoting                     (tsv_dialect) */
    FALX_LOGFMT = 3,   /* ' ' '=' '\n', backslash-escaped quotes    (logfmt_dialect) */
    FALX_NDJSON = 4    /* '\n' outside backslash-escaped strings    (ndjson_dialect) */
} falx_dialect;

/* Column types (codegen.rs:78-93 ColumnType, plus U32). */
typedef enum {
    FALX_I64 = 0,   /* str::parse::<i64> */
    FALX_U32 = 1,   /* str::parse::<u32> */
    FALX_F64 = 2,   /* str::parse::<f64>, bit-exact */
    FALX_STR = 3,   /* cleaned bytes, Arrow varbinary (i32 offsets + arena) */
    FALX_BYTES = 4  /* raw (from,to) span, valid iff present and non-empty */
} falx_col_type;

#define FALX_MAX_COLUMNS 32 /* codegen.rs:198-205 */

typedef struct falx_ctx falx_ctx;

/* Context: device, stream, look-back scratch, tuned launch parameters. */
int falx_create(int device, falx_ctx **out);
void falx_destroy(falx_ctx *ctx);
/* Options. FALX_OPT_ROWS_PATH: how rows (columns, field bytes, count/sum)
 * are made: 0 (default) index + tape pass, then a record-parallel pass over
 * the tape; 1 one fused tile pass. Same outputs either way.
 * FALX_OPT_CTAS_PER_SM caps the persistent grids (0 = as many as fit). */
#define FALX_OPT_ROWS_PATH 1
#define FALX_OPT_CTAS_PER_SM 2
#define FALX_OPT_TIMING 3 /* 1: time each launch of the rows path with CUDA events */
/* FALX_OPT_PIPELINE (default 1): falx_parse_host with columns over 64 MiB or
 * more runs as a pipeline of input chunks (16 MiB first and last, about 96
 * MiB in the middle):
 * each chunk is copied in,
 * indexed and its records decoded while later chunks are still being copied
 * in, and its outputs are copied back while later chunks are parsed (host to
 * device and device to host transfers overlap). 0: one copy in, the whole
 * parse, the copies back. Same outputs either way. */
#define FALX_OPT_PIPELINE 4
int falx_set_option(falx_ctx *ctx, int option, int value);
/* Device times (ms) of the last rows call's launches, in order: index + tape,
 * columns. Returns how many were recorded (0 unless FALX_OPT_TIMING is on
 * and the default rows path ran). */
int falx_last_timings(const falx_ctx *ctx, float *ms, int n);

/* Use `stream` (a cudaStream_t; NULL = the legacy default stream). */
int falx_set_stream(falx_ctx *ctx, void *stream);
const char *falx_strerror(int code);

/* Structural index: offsets of every structural byte, byte-identical to the
 * serial path. Replaces index_structurals / index_structurals_par
 * (csv_geo.rs:24, :95; csv_hash.rs:345; tsv.rs:20, :64; logfmt.rs;
 * ndjson.rs). Writes min(n, cap) entries; *n_out = n. */
int falx_index_structurals(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len,
                           uint32_t *out, uint64_t cap, uint64_t *n_out);

/* Tape behind parse() / parse_par() (csv_geo.rs:394, :215, push_tape
 * :1838-1849): separator offsets, and per terminated record an end entry
 * `(separators_before << 32) | terminator_offset`. Records / fields views
 * are built on these two arrays by the host API. */
int falx_parse_tape(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len,
                    uint32_t *seps, uint64_t seps_cap, uint64_t *ends, uint64_t ends_cap,
                    uint64_t *n_seps, uint64_t *n_ends);

typedef struct {
    uint32_t field; /* 0-based field ordinal within the record */
    uint32_t type;  /* falx_col_type */
} falx_column;

typedef struct {
    int32_t dialect;
    uint32_t ncols;
    falx_column cols[FALX_MAX_COLUMNS];
} falx_schema;

typedef struct {
    void *values;      /* I64 int64[rows_cap]; U32 uint32[rows_cap]; F64 double[rows_cap];
                          BYTES uint32[2*rows_cap] (from,to); STR int32 offsets[rows_cap+1] */
    uint64_t *valid;   /* LSB-first validity bitmap, ceil(rows_cap/64) words */
    uint8_t *str_data; /* STR arena */
    uint64_t str_cap;
    uint64_t str_len;  /* out: arena bytes used (STR) */
} falx_column_out;

typedef struct {
    uint64_t rows_cap;
    uint64_t rows; /* out */
    falx_column_out cols[FALX_MAX_COLUMNS];
} falx_columns;

/* Typed columns (Arrow-compatible). Replaces parse_columns /
 * parse_columns_par / parse_columns_chunks_par (csv_geo.rs:1112, :1216,
 * :1167; csv_hash.rs:1451, :1570, :1507; csv_typed.rs). Comment records
 * (csv_hash) are not rows. */
int falx_parse_columns(falx_ctx *ctx, const falx_schema *schema, const uint8_t *data, uint64_t len,
                       falx_columns *out);

/* Test hook for failure detection (no reference counterpart): as
 * falx_parse_columns, but only record block 1 of the columns pass runs, so
 * its look-back waits for a block 0 that never publishes; the wait gives up
 * after wait_ns and the call returns FALX_ERR_TIMEOUT with the context still
 * usable. The input must hold more than 512 records. Outputs are undefined. */
int falx_test_stalled_lookback(falx_ctx *ctx, const falx_schema *schema, const uint8_t *data, uint64_t len,
                               falx_columns *out, uint64_t wait_ns);

typedef struct {
    uint64_t records;
    uint64_t values[2];
    uint64_t checksum[2]; /* wrapping sum of f64 bit patterns (csv_geo.rs:1735-1750) */
    int64_t sum_e6[2];    /* exact sum of value*1e6 over cells exact in micro-units */
    uint64_t inexact[2];  /* valid cells not exact in micro-units */
    double sum_f64[2];    /* sum_e6 / 1e6 */
} falx_geo_stats;

/* Fused count / sum over two f64 fields without materialising columns.
 * Replaces parse_csv_geo_stats / parse_csv_geo_stats_par
 * (csv_geo.rs:1505, :1513). */
int falx_stats_count_sum(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len, uint32_t field0,
                         uint32_t field1, falx_geo_stats *out);

typedef struct {
    uint64_t records;
    uint64_t city_values;        /* rows whose city field is present */
    uint64_t city_bytes;         /* cleaned bytes of those cells */
    uint64_t city_checksum;      /* wrapping sum of their cleaned byte values */
    uint64_t latitude_values;
    uint64_t longitude_values;
    uint64_t latitude_checksum;  /* wrapping sum of f64 bit patterns */
    uint64_t longitude_checksum;
} falx_geo_text_stats;

/* City text lane with the lat / lon count and checksums, without
 * materialising columns. Replaces parse_csv_geo_text_stats /
 * parse_csv_geo_text_stats_par (csv_geo_text.rs:1627, :1637; sink
 * :1845-1937). csv_hash comment records are not rows. */
int falx_csv_geo_text_stats(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len, uint32_t city_field,
                            uint32_t lat_field, uint32_t lon_field, falx_geo_text_stats *out);

typedef struct {
    uint64_t fields;
    uint64_t bytes;
} falx_field_byte_stats;

/* Field count and total cleaned field bytes. Replaces parse_field_bytes /
 * parse_field_bytes_par (csv_hash.rs:976, :984). */
int falx_field_bytes(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len,
                     falx_field_byte_stats *out);

/* Everything above from one pass over the input; NULL / zero-capacity
 * members are skipped. The fused form of the entry points above. */
typedef struct {
    uint32_t *index;
    uint64_t index_cap;
    uint64_t n_index; /* out */
    uint32_t *seps;
    uint64_t seps_cap;
    uint64_t n_seps; /* out */
    uint64_t *ends;
    uint64_t ends_cap;
    uint64_t n_ends; /* out */
    falx_columns *columns;
    falx_field_byte_stats *field_bytes;
    falx_geo_stats *stats;
    uint32_t stats_fields[2];
} falx_outputs;

int falx_parse(falx_ctx *ctx, const falx_schema *schema, const uint8_t *data, uint64_t len,
               falx_outputs *out);

typedef struct {
    uint64_t records;
    int64_t sum_id;       /* wrapping */
    int64_t sum_score_e6; /* wrapping */
    int64_t total_e6_lo;  /* exact 128-bit sum of id*1e6 + score_e6 */
    int64_t total_e6_hi;
    double total_f64;     /* (double)total_e6 / 1e6 */
} falx_ndjson_stats;

/* sum(id + nested.score) over NDJSON records, JSON-aware (any key order,
 * whitespace, escapes, decimal scores with up to 6 fraction digits). The
 * generalisation of parse_ndjson_id_score(_par) (ndjson.rs:679, :726); a
 * record outside the schema returns FALX_ERR_SCHEMA where the reference
 * panics (ndjson.rs:721-724). */
int falx_ndjson_id_score(falx_ctx *ctx, const uint8_t *data, uint64_t len, falx_ndjson_stats *out);

/* Host-buffer forms for callers without device memory: copy `data` in,
 * run, copy the results out, all on the context's stream. */
int falx_index_structurals_host(falx_ctx *ctx, int dialect, const uint8_t *host_data, uint64_t len,
                                uint32_t *host_out, uint64_t cap, uint64_t *n_out);
int falx_parse_host(falx_ctx *ctx, const falx_schema *schema, const uint8_t *host_data, uint64_t len,
                    falx_outputs *host_out);

/* ---------------------------------------------------------------------------
 * Shards of one file on several GPUs (one process per GPU). Each rank
 * summarises its shard independently of the state it starts in, the ranks
 * exchange the summaries (a few dozen bytes each, through the host), every
 * rank folds the summaries of the ranks before it into its true entry state
 * and output offsets, then runs a seeded pass that writes its own range of
 * the global index / tape. The reference runs the same three steps across
 * threads (csv_hash.rs:152-214 region_scan3 phases; csv_geo.rs:95-149
 * chunk parities; seeded pass index_structurals_seeded, csv_geo.rs:1855-1873).
 * `prev_byte` is the byte before the shard (-1 at the start of the file); it
 * decides whether the shard starts a line (csv_hash comments) and a record.
 * ------------------------------------------------------------------------- */
typedef struct {
    uint32_t states;          /* entry states of the dialect's automaton */
    uint32_t exit[4];         /* exit state for each entry state */
    uint64_t structurals[4];  /* counts for each entry state */
    uint64_t terminators[4];
    uint64_t rows[4];         /* record starts inside the shard (csv_hash comments excluded) */
    int32_t last_byte;        /* the shard's last byte, -1 if empty */
} falx_shard_summary;

int falx_summarize_shard(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len, int prev_byte,
                       falx_shard_summary *out);
/* Seeded pass: structural index and / or tape of the shard as part of the
 * whole file. Positions get pos_base (the shard's file offset) added, tape
 * ends count separators from sep_base; entry_state comes from the summaries
 * of the shards before it. NULL / zero-capacity outputs are skipped. */
int falx_parse_tape_seeded(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len, int prev_byte,
                           uint32_t entry_state, uint64_t pos_base, uint64_t sep_base, uint32_t *index,
                           uint64_t index_cap, uint32_t *seps, uint64_t seps_cap, uint64_t *ends, uint64_t ends_cap,
                           uint64_t *n_index, uint64_t *n_seps, uint64_t *n_ends);

/* ---------------------------------------------------------------------------
 * Learned speculation. The reference's parallel drivers guess each chunk's
 * entry state ("outside quotes") and re-index chunks whose guess was wrong
 * (csv_geo.rs:95-149 speculative parity; csv_hash.rs:152-214 instead runs a
 * full transfer-function prepass). Here a small MLP predicts every 16 KiB
 * tile's entry region from its 256 leading bytes; the speculative index scans
 * each tile under its predicted entry only, the exact look-back verifies every
 * prediction, and a tile whose prediction was wrong re-derives its masks from
 * the true entry before it publishes. Output is identical to
 * falx_index_structurals whatever the predictions are.
 *
 * Model: 256 bytes -> one-hot over 8 byte classes ('"' '#' '\n' ',' '\r'
 * digit letter other) -> 256 ReLU -> 256 ReLU -> 3 (NORMAL / QUOTE /
 * COMMENT), BF16 operands, FP32 accumulation and softmax. Parameters are one
 * FP32 vector: W1[2048][256] (row = byte * 8 + class), b1[256],
 * W2[256][256] (in, out), b2[256], W3[256][3], b3[3].
 * ------------------------------------------------------------------------- */
#define FALX_MLP_BYTES 256
#define FALX_SPEC_TILE 16384
typedef struct falx_model falx_model;

typedef struct {
    uint64_t tiles;
    uint64_t mispredicted; /* tiles re-derived from their true entry state */
} falx_spec_stats;

uint64_t falx_model_param_count(void);
/* Random initial weights (uniform, scaled by fan-in) from `seed`. */
int falx_model_create(falx_ctx *ctx, uint64_t seed, falx_model **out);
void falx_model_destroy(falx_model *model);
/* Tiles whose predicted state has softmax probability below `min_prob`
 * assume nothing: they count under every entry state, like the plain scan,
 * and can never be mispredicted (default 0: always take the arg-max). */
int falx_model_set_confidence(falx_model *model, float min_prob);
/* Copy the FP32 parameter vector out / in (host buffers of
 * falx_model_param_count() floats). Setting resets the optimiser. */
int falx_model_get(falx_ctx *ctx, const falx_model *model, float *host, uint64_t n);
int falx_model_set(falx_ctx *ctx, falx_model *model, const float *host, uint64_t n);
/* Byte classes of the FALX_MLP_BYTES bytes from each of n start offsets
 * (device int64 array) into cls[n][256]; bytes outside the input are class 7. */
int falx_byte_classes(falx_ctx *ctx, const uint8_t *data, uint64_t len, const int64_t *starts, uint32_t n,
                      uint8_t *cls);
/* Forward pass: logits[n][3] and/or the arg-max state (either may be NULL);
 * `cls` 16-byte aligned. */
int falx_model_forward(falx_ctx *ctx, const falx_model *model, const uint8_t *cls, uint32_t n, float *logits,
                       uint8_t *pred);
/* Gradient of the mean softmax cross-entropy over n labelled samples into
 * grad[falx_model_param_count()] (device); *loss = the mean loss. */
int falx_model_grad(falx_ctx *ctx, const falx_model *model, const uint8_t *cls, const uint8_t *labels, uint32_t n,
                    float *grad, float *loss);
/* Adam over `epochs` passes of n samples in minibatches of `batch`. */
int falx_model_train(falx_ctx *ctx, falx_model *model, const uint8_t *cls, const uint8_t *labels, uint64_t n,
                     uint32_t batch, uint32_t epochs, float lr, float *last_loss);
/* Labels from the exact scan: the region state at the start of every
 * 64-byte block, entry k for file position 64k - (data & 15). */
int falx_region_states(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len, uint8_t *states,
                       uint64_t cap, uint64_t *n_out);
/* Predicted entry state of every tile (tile t starts at 16384t - (data & 15)). */
int falx_predict_tiles(falx_ctx *ctx, const falx_model *model, const uint8_t *data, uint64_t len, uint8_t *pred,
                       uint64_t cap, uint64_t *n_tiles);
/* Speculative structural index under caller-supplied assumed entry states
 * (device array, one per tile; 0xFF = no assumption, count every entry
 * state; other values outside the dialect's states read as 0; tile 0 always
 * assumes the initial state). */
int falx_index_structurals_assumed(falx_ctx *ctx, int dialect, const uint8_t *data, uint64_t len,
                                   const uint8_t *assumed, uint32_t *out, uint64_t cap, uint64_t *n_out,
                                   falx_spec_stats *stats);
/* Speculative structural index; `model` NULL assumes every tile starts
 * outside any region (the reference's guess). */
int falx_index_structurals_speculative(falx_ctx *ctx, const falx_model *model, int dialect, const uint8_t *data,
                                       uint64_t len, uint32_t *out, uint64_t cap, uint64_t *n_out,
                                       falx_spec_stats *stats);

/* ---------------------------------------------------------------------------
 * Batched documents: many documents of uneven sizes in one persistent launch
 * from a device work queue, replayed from a CUDA graph. The reference parses
 * one document per call (parse_columns_par / index_structurals_par per file,
 * csv_geo.rs:1216-1284, :95-149); here a batch is planned once and each run
 * gives every document the same outputs as falx_index_structurals plus two
 * f64 columns (falx_parse_columns with two FALX_F64 columns).
 * ------------------------------------------------------------------------- */
typedef struct {
    const uint8_t *data;  /* device, 16-byte aligned */
    uint64_t len;
    int32_t dialect;      /* FALX_CSV, FALX_TSV or FALX_LOGFMT */
    uint32_t field0;      /* ordinals of the two f64 columns (e.g. lat, lon) */
    uint32_t field1;
    uint32_t *index;      /* structural index, index_cap entries (NULL / 0: none) */
    uint64_t index_cap;
    double *col0;         /* f64 columns and LSB-first validity, rows_cap rows (0: none) */
    double *col1;
    uint64_t *valid0;
    uint64_t *valid1;
    uint64_t rows_cap;
    uint64_t n_index;     /* out */
    uint64_t rows;        /* out */
    int32_t status;       /* out: FALX_OK or an error of this document */
} falx_doc;

typedef struct {
    uint32_t chunk_bytes; /* documents up to this size run whole on one CTA; larger ones tile by tile */
    uint32_t ctas_per_sm; /* 0: as many as fit */
    uint32_t staging;     /* tile buffers in flight per CTA: 2 or 3 */
} falx_batch_config;

typedef struct falx_batch falx_batch;

/* Plan a batch on `docs` (device buffers stay the caller's; the batch
 * records their addresses). cfg NULL: the context's last falx_batch_tune
 * result, else defaults (1 MiB, all CTAs that fit, 2 buffers). */
int falx_batch_create(falx_ctx *ctx, const falx_doc *docs, uint32_t ndocs, const falx_batch_config *cfg,
                      falx_batch **out);
/* One run of the planned batch (graph replay on the context's stream);
 * fills n_index / rows / status of `docs` when not NULL. Returns the first
 * document error, if any. */
int falx_batch_run(falx_batch *batch, falx_doc *docs);
int falx_batch_info(const falx_batch *batch, falx_batch_config *cfg, uint32_t *n_items, uint32_t *grid,
                    int *graph);
void falx_batch_destroy(falx_batch *batch);
/* Time every candidate configuration (chunk 64 KiB..4 MiB, CTAs per SM,
 * staging 2 / 3) on this batch; keep the fastest in the context. */
int falx_batch_tune(falx_ctx *ctx, falx_doc *docs, uint32_t ndocs, falx_batch_config *best, float *best_ms);
/* The work queue a batch would run (host only): items[3k..3k+2] =
 * (document, first tile, end tile) for document lengths `lens`. */
int falx_batch_plan(const uint64_t *lens, uint32_t ndocs, uint32_t chunk_bytes, uint32_t *items, uint32_t cap,
                    uint32_t *n_items);

/* ---------------------------------------------------------------------------
 * bgzf input (bgzf.rs): a stream of gzip members of at most 64 KiB, each a
 * raw DEFLATE payload with its uncompressed size (ISIZE) in the trailer.
 * falx_bgzf_scan walks the member headers on the host (bgzf.rs:61 scan) and
 * lists every non-empty block with its place in the inflated output;
 * falx_bgzf_inflate inflates all of them on the GPU at once (one warp per
 * block; bgzf.rs:201 decompress, :209 decompress_par) into one contiguous
 * buffer, which the parse entry points then read in place, so the text
 * never crosses the host link (bgzf.rs:538 parse_gz_par,
 * examples/gpu_pipeline.rs:1-8). As in the reference, ISIZE must equal the
 * inflated length and the CRC is not checked.
 * ------------------------------------------------------------------------- */
typedef struct {
    uint64_t in_off;   /* raw DEFLATE payload: offset in the compressed stream */
    uint64_t out_off;  /* offset of the block's bytes in the inflated output */
    uint32_t in_len;   /* payload bytes */
    uint32_t out_len;  /* ISIZE */
} falx_gz_block;

/* Host only. FALX_ERR_FORMAT for a malformed stream; FALX_ERR_CAPACITY (with
 * *n_blocks and *out_len set) when `cap` is too small. */
int falx_bgzf_scan(const uint8_t *comp, uint64_t len, falx_gz_block *blocks, uint64_t cap, uint64_t *n_blocks,
                   uint64_t *out_len);
/* `comp` and `out` are device pointers, `blocks` host memory (copied to the
 * device). Returns FALX_ERR_FORMAT when a block fails to inflate;
 * block_status (host, n_blocks entries, optional) then says which: 0 ok,
 * 1 truncated, 2 reserved block type, 3 stored length mismatch, 4 bad code
 * lengths, 5 invalid symbol, 6 distance before the block start, 7 more
 * output than ISIZE, 8 less output than ISIZE, 9 block outside the buffers.
 * Synchronous on the context's stream. */
int falx_bgzf_inflate(falx_ctx *ctx, const uint8_t *comp, uint64_t comp_len, const falx_gz_block *blocks,
                      uint64_t n_blocks, uint8_t *out, uint64_t out_cap, int32_t *block_status, uint64_t *n_failed);
/* bgzf.rs:538 parse_gz_par with host buffers: falx_parse_host over the text
 * of the bgzf stream `comp` (host memory; pinned for the copy to overlap),
 * whose blocks (host, from falx_bgzf_scan: texts end to end from 0) are
 * inflated on the GPU into device memory, never crossing the host link.
 * The parse and the copies back are those of falx_parse_host (pipelined for
 * columns over 64 MiB: the outputs go back chunk by chunk while the parse
 * goes on). FALX_ERR_FORMAT when a block fails to inflate (the outputs are then
 * undefined; falx_bgzf_inflate tells which block); FALX_ERR_INVALID when
 * the blocks' texts are not end to end. */
int falx_parse_gz_host(falx_ctx *ctx, const falx_schema *schema, const uint8_t *comp, uint64_t comp_len,
                       const falx_gz_block *blocks, uint64_t n_blocks, falx_outputs *host_out);

/* Structural index without any allocation (no counterpart in the
 * reference, whose callers are Rust code that allocates freely). For callers
 * that may not allocate device memory: the look-back scratch is a fixed
 * array inside the library (about 1 MiB per GPU that loads it, held until the
 * process exits), so inputs are limited to FALX_NOALLOC_MAX_BYTES
 * (FALX_ERR_INPUT_TOO_LARGE beyond). `data` and `out` are device pointers in
 * `device`; `stream` is a cudaStream_t (NULL = legacy default stream); the
 * call synchronises `stream` and returns after it has drained. The first
 * call on a device also sets that device up (looks up the scratch address,
 * sets kernel attributes), so make it before any stream capture. Under
 * CUDA's default lazy module loading the driver places the scratch array in
 * device memory during that first call, which can therefore still fail for
 * lack of memory: make it early, before memory is full or frozen; later
 * calls allocate nothing. All calls share the
 * one scratch array: calls whose work can overlap on a GPU (other host
 * threads, other streams) race and must be serialised by the caller.
 * Output is identical to falx_index_structurals. */
#define FALX_NOALLOC_MAX_BYTES (256ull << 20)
int falx_index_structurals_noalloc(int device, int dialect, const uint8_t *data, uint64_t len, uint32_t *out,
                                   uint64_t cap, uint64_t *n_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
