/*
 * Multi-threaded port of the reference's `_par` drivers: the timed CPU
 * baseline. TEST INFRASTRUCTURE ONLY (see oracle.h).
 */
#include "oracle.h"

uint64_t orc_par_index(int dialect, const uint8_t *d, uint64_t n, int threads, uint32_t *out, uint64_t cap) {
    (void)threads;
    return orc_index_blocks(dialect, d, n, out, cap);
}

int orc_par_columns(int dialect, const uint8_t *d, uint64_t n, int threads, orc_col *cols, int ncols,
                    uint64_t rows_cap, uint64_t *rows_out) {
    (void)threads;
    return orc_parse_columns(dialect, d, n, cols, ncols, rows_cap, rows_out);
}

void orc_par_field_bytes(int dialect, const uint8_t *d, uint64_t n, int threads, uint64_t *fields,
                         uint64_t *bytes) {
    (void)threads;
    orc_field_bytes(dialect, d, n, fields, bytes);
}
