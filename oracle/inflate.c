/* Test infrastructure (the oracle): a serial restatement of raw DEFLATE
 * decoding (RFC 1951) and of the bgzf member walk, used to check the GPU
 * inflate kernel and timed as the CPU baseline of the bgzf path. The
 * reference inflates with flate2 (miniz_oxide) or libdeflate, neither of
 * which is under the reference tree (Cargo.toml:16-18; bgzf.rs:22-160); this
 * file restates the published format instead: canonical Huffman codes
 * decoded one bit at a time, the fixed and dynamic code sets, the length and
 * distance tables, stored blocks. Rules shared with the GPU decoder so that
 * both accept and reject the same streams: an over-subscribed code set is an
 * error, an incomplete one is accepted (an unused pattern is an error when
 * met), a dynamic block must code the end-of-block symbol, distances may not
 * reach before the member's first byte, and the output must have exactly
 * ISIZE bytes (bgzf.rs:125-160). */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
    const uint8_t *in;
    uint64_t n, at; /* input bytes, next byte */
    uint32_t bits;  /* unused bits of in[at - 1], low first */
    int nbits;
    uint8_t *out;
    uint64_t cap, len;
    int err;
} orc_z;

typedef struct {
    uint16_t count[16];
    uint16_t symbol[320];
} orc_huff;

static int z_bit(orc_z *z) {
    if (z->nbits == 0) {
        if (z->at >= z->n) {
            z->err = 1;
            return 0;
        }
        z->bits = z->in[z->at++];
        z->nbits = 8;
    }
    int b = (int)(z->bits & 1u);
    z->bits >>= 1;
    z->nbits--;
    return b;
}

static uint32_t z_bits(orc_z *z, int k) {
    uint32_t v = 0;
    for (int i = 0; i < k; i++) v |= (uint32_t)z_bit(z) << i;
    return v;
}

/* 0 ok, -1 over-subscribed */
static int huff_make(orc_huff *h, const uint8_t *len, int n) {
    uint16_t offs[16];
    memset(h->count, 0, sizeof h->count);
    for (int s = 0; s < n; s++) h->count[len[s]]++;
    int left = 1;
    for (int l = 1; l <= 15; l++) {
        left *= 2;
        left -= h->count[l];
        if (left < 0) return -1;
    }
    offs[1] = 0;
    for (int l = 1; l < 15; l++) offs[l + 1] = (uint16_t)(offs[l] + h->count[l]);
    for (int s = 0; s < n; s++)
        if (len[s] != 0) h->symbol[offs[len[s]]++] = (uint16_t)s;
    return 0;
}

/* canonical decode, most significant code bit first in the code value */
static int huff_decode(orc_z *z, const orc_huff *h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l <= 15; l++) {
        code |= z_bit(z);
        if (z->err) return -1;
        int cnt = h->count[l];
        if (code - first < cnt) return h->symbol[index + (code - first)];
        index += cnt;
        first += cnt;
        first <<= 1;
        code <<= 1;
    }
    return -2;
}

static const uint16_t LBASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
static const uint8_t LEXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
static const uint16_t DBASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                   193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
static const uint8_t DEXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

/* symbols of one Huffman-coded block */
static int z_codes(orc_z *z, const orc_huff *lit, const orc_huff *dist) {
    for (;;) {
        int s = huff_decode(z, lit);
        if (z->err) return ORC_Z_TRUNCATED;
        if (s < 0) return ORC_Z_SYMBOL;
        if (s < 256) {
            if (z->len >= z->cap) return ORC_Z_OVERFLOW;
            z->out[z->len++] = (uint8_t)s;
        } else if (s == 256) {
            return 0;
        } else {
            s -= 257;
            if (s >= 29) return ORC_Z_SYMBOL;
            uint64_t len = LBASE[s] + z_bits(z, LEXTRA[s]);
            int d = huff_decode(z, dist);
            if (z->err) return ORC_Z_TRUNCATED;
            if (d < 0 || d >= 30) return ORC_Z_SYMBOL;
            uint64_t back = DBASE[d] + z_bits(z, DEXTRA[d]);
            if (z->err) return ORC_Z_TRUNCATED;
            if (back > z->len) return ORC_Z_DISTANCE;
            if (z->cap - z->len < len) return ORC_Z_OVERFLOW;
            for (uint64_t k = 0; k < len; k++, z->len++) z->out[z->len] = z->out[z->len - back];
        }
    }
}

static int z_fixed(orc_z *z) {
    uint8_t len[320];
    orc_huff lit, dist;
    for (int s = 0; s < 288; s++) len[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
    huff_make(&lit, len, 288);
    for (int s = 0; s < 32; s++) len[s] = 5;
    huff_make(&dist, len, 32);
    return z_codes(z, &lit, &dist);
}

static int z_dynamic(orc_z *z) {
    static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    uint8_t len[320];
    orc_huff lit, dist;
    int nlen = (int)z_bits(z, 5) + 257, ndist = (int)z_bits(z, 5) + 1, ncode = (int)z_bits(z, 4) + 4;
    if (z->err) return ORC_Z_TRUNCATED;
    if (nlen > 286 || ndist > 30) return ORC_Z_CODES;
    memset(len, 0, sizeof len);
    for (int i = 0; i < ncode; i++) len[order[i]] = (uint8_t)z_bits(z, 3);
    if (z->err) return ORC_Z_TRUNCATED;
    if (huff_make(&lit, len, 19) != 0) return ORC_Z_CODES;
    int i = 0;
    while (i < nlen + ndist) {
        int s = huff_decode(z, &lit);
        if (z->err) return ORC_Z_TRUNCATED;
        if (s < 0) return ORC_Z_SYMBOL;
        if (s < 16) {
            len[i++] = (uint8_t)s;
            continue;
        }
        int v = 0, rep;
        if (s == 16) {
            if (i == 0) return ORC_Z_CODES;
            v = len[i - 1];
            rep = 3 + (int)z_bits(z, 2);
        } else if (s == 17) {
            rep = 3 + (int)z_bits(z, 3);
        } else {
            rep = 11 + (int)z_bits(z, 7);
        }
        if (z->err) return ORC_Z_TRUNCATED;
        if (i + rep > nlen + ndist) return ORC_Z_CODES;
        while (rep--) len[i++] = (uint8_t)v;
    }
    if (len[256] == 0) return ORC_Z_CODES;
    if (huff_make(&lit, len, nlen) != 0) return ORC_Z_CODES;
    if (huff_make(&dist, len + nlen, ndist) != 0) return ORC_Z_CODES;
    return z_codes(z, &lit, &dist);
}

int orc_inflate(const uint8_t *in, uint64_t n, uint8_t *out, uint64_t out_len) {
    orc_z z = {in, n, 0, 0, 0, out, out_len, 0, 0};
    int last;
    do {
        last = z_bit(&z);
        int type = (int)z_bits(&z, 2);
        if (z.err) return ORC_Z_TRUNCATED;
        int rc;
        if (type == 0) {
            z.nbits = 0; /* the rest of the current byte */
            if (z.n - z.at < 4) return ORC_Z_TRUNCATED;
            uint32_t len = z.in[z.at] | (z.in[z.at + 1] << 8), nl = z.in[z.at + 2] | (z.in[z.at + 3] << 8);
            if (len != (~nl & 0xFFFFu)) return ORC_Z_STORED_LEN;
            z.at += 4;
            if (z.n - z.at < len) return ORC_Z_TRUNCATED;
            if (z.cap - z.len < len) return ORC_Z_OVERFLOW;
            memcpy(z.out + z.len, z.in + z.at, len);
            z.at += len;
            z.len += len;
            rc = 0;
        } else if (type == 1) {
            rc = z_fixed(&z);
        } else if (type == 2) {
            rc = z_dynamic(&z);
        } else {
            rc = ORC_Z_BLOCK_TYPE;
        }
        if (rc) return rc;
    } while (!last);
    return z.len == out_len ? 0 : ORC_Z_SIZE;
}

static uint32_t rd16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
static uint32_t rd32(const uint8_t *p) { return rd16(p) | (rd16(p + 2) << 16); }

/* bgzf members (bgzf.rs:42-108): the same walk as the GPU path's host scan */
int64_t orc_bgzf_scan(const uint8_t *c, uint64_t n, orc_gz_block *out, uint64_t cap, uint64_t *total) {
    uint64_t pos = 0, k = 0, tot = 0;
    while (pos < n) {
        if (n - pos < 12) return -1;
        const uint8_t *h = c + pos;
        if (h[0] != 31 || h[1] != 139 || h[2] != 8 || (h[3] & 4) == 0) return -1;
        uint64_t xlen = rd16(h + 10);
        if (n - pos - 12 < xlen) return -1;
        int64_t bsize = -1;
        uint64_t i = 0;
        while (i + 4 <= xlen) {
            uint64_t slen = rd16(h + 12 + i + 2);
            if (h[12 + i] == 66 && h[12 + i + 1] == 67 && slen == 2 && i + 6 <= xlen) {
                bsize = rd16(h + 12 + i + 4);
                break;
            }
            i += 4 + slen;
        }
        if (bsize < 0) return -1;
        uint64_t blen = (uint64_t)bsize + 1;
        if (blen <= 12 + xlen + 8 || blen > n - pos) return -1;
        uint32_t isize = rd32(h + blen - 4);
        if (isize) {
            if (k < cap) {
                out[k].in_off = pos + 12 + xlen;
                out[k].in_len = blen - 12 - xlen - 8;
                out[k].out_off = tot;
                out[k].out_len = isize;
            }
            k++;
            tot += isize;
        }
        pos += blen;
    }
    *total = tot;
    return (int64_t)k;
}

typedef struct {
    const uint8_t *comp;
    const orc_gz_block *blocks;
    uint64_t lo, hi;
    uint8_t *out;
    int32_t *status;
} z_job;

static void *z_worker(void *arg) {
    z_job *j = (z_job *)arg;
    for (uint64_t b = j->lo; b < j->hi; b++) {
        const orc_gz_block *g = &j->blocks[b];
        j->status[b] = orc_inflate(j->comp + g->in_off, g->in_len, j->out + g->out_off, g->out_len);
    }
    return NULL;
}

/* every block, contiguous block groups on `threads` threads (decompress_par,
 * bgzf.rs:209-240); returns the number of failed blocks */
uint64_t orc_bgzf_inflate_par(const uint8_t *comp, const orc_gz_block *blocks, uint64_t nb, uint8_t *out,
                              int32_t *status, int threads) {
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > nb) threads = nb ? (int)nb : 1;
    pthread_t tid[256];
    z_job jobs[256];
    if (threads > 256) threads = 256;
    for (int t = 0; t < threads; t++) {
        jobs[t] = (z_job){comp, blocks, nb * t / threads, nb * (t + 1) / threads, out, status};
        if (t) pthread_create(&tid[t], NULL, z_worker, &jobs[t]);
    }
    z_worker(&jobs[0]);
    for (int t = 1; t < threads; t++) pthread_join(tid[t], NULL);
    uint64_t failed = 0;
    for (uint64_t b = 0; b < nb; b++) failed += status[b] != 0;
    return failed;
}
