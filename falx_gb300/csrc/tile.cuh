// Tile machinery shared by the persistent kernels: per-tile look-back
// status, launch parameters, shared-memory layout, bulk-copy issue, the
// warp look-back and the full tile pass (classify, region scan, counts,
// look-back, staging, index / tape writes, rows).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/falx_gpu.h"
#include "rows.cuh"
#include "scan_core.cuh"

namespace falx {

constexpr uint64_t kWaitNs = 4000000000ull;  // every device-side wait gives up after 4 s

// One per tile. Level 1 publishes the tile's aggregate: its transfer function
// and, for every possible entry state, its counts (structurals, terminators,
// rows packed 21 bits apart). Level 2 publishes the inclusive prefix: the
// absolute exit state and the counts of the whole file up to the tile end.
// Every field is written once per launch, before the release of its level.
struct TileStatus {      // 64 bytes
    uint32_t flag;       // epoch * 4 + level
    uint32_t func;       // transfer function (level 1)
    uint64_t agg[4];     // packed counts per entry state (level 1)
    uint32_t exit;       // exit state (level 2)
    uint32_t incl[3];    // inclusive structurals, terminators, rows (level 2)
    uint32_t pad[2];
};

struct ArenaStatus {  // 48 bytes: prefix of string-arena bytes for up to kMaxStr columns
    uint32_t flag;    // epoch * 4 + level (1: aggregate, 2: inclusive)
    uint32_t pad[3];
    uint32_t agg[kMaxStr];
    uint32_t incl[kMaxStr];
};

struct DevHeader {
    uint32_t ticket;
    uint32_t abort;
    uint32_t error;
    uint32_t exit_state;  // the index pass's exit state at the end of its input
    unsigned long long n_struct, n_terms, n_rows;
    unsigned long long arena[kMaxStr];
    unsigned long long fb_fields, fb_bytes;
    unsigned long long st_records, st_values[2], st_checksum[2], st_sum_e6[2], st_inexact[2];
    unsigned long long st_text[3];  // City text lane: values, cleaned bytes, wrapping byte checksum
    unsigned long long spec_repairs;  // speculative tiles whose assumed entry state was wrong
    uint32_t col_ticket;              // record blocks taken by the columns pass
    uint32_t pad2;
};

// Where a launch over one chunk of a pipelined call ends (the exit state and
// the structurals / terminators through the chunk), written by the chunk's
// index pass for the next chunk. `error` is not used.
struct SeedRec {
    uint32_t error;
    uint32_t exit_state;
    unsigned long long n_struct, n_terms;  // through the chunk
};
static_assert(sizeof(SeedRec) == 24, "seed record");

// ERR_TAPE: the tape outgrew the buffers it was written to (the host sizes
// them exactly and runs again)
enum : uint32_t { ERR_TIMEOUT = 1, ERR_ARENA = 2, ERR_TMA = 4, ERR_TAPE = 8 };

struct Params {
    const uint8_t *data;
    const uint8_t *abase;  // data rounded down to 16 bytes
    uint64_t len;
    uint32_t shift;        // data - abase
    uint32_t num_tiles;
    uint32_t epoch;
    uint32_t halo;         // halo bytes staged after each tile (rows only)
    TileStatus *status;
    ArenaStatus *astatus;
    DevHeader *hdr;
    uint32_t *index;
    uint64_t index_cap;
    uint32_t *seps;
    uint64_t seps_cap;
    uint64_t *ends;
    uint64_t ends_cap;
    int32_t dialect;       // batched launches: the document's dialect
    // Seeded launches over one shard of a file: the automaton state and the
    // byte before the shard, and what to add to output positions and to the
    // separator counts of tape ends. Zero: the data is a whole file.
    uint32_t seeded;
    uint32_t prev_byte;
    uint32_t entry0;
    uint64_t pos_base;
    uint64_t sep_base;
    const uint8_t *pred;   // speculative index: assumed entry state of every tile
    uint8_t *states64;     // optional: entry state of every 64-byte block
    // optional: input still arriving in chunks of chunk_tiles tiles; chunk k
    // is in device memory once arrive[k] == arrive_tag
    const uint32_t *arrive;
    uint32_t arrive_tag;
    uint32_t chunk_tiles;
    // Index-pass launches over consecutive chunks of one input (pipelined
    // host-buffer calls): the entry state and the structurals / terminators
    // before the chunk, from the previous chunk's seed record.
    const SeedRec *seed_in;
    SeedRec *seed_out;  // optional: where the launch ends (exit state, totals), for the next chunk
    // seeded launches over a chunk of input already in device memory: the
    // byte before the chunk is read there (prev_byte is then unused)
    const uint8_t *prev_ptr;
    RowSpec rows;
};

// Shared state of the block-wide look-back.

// Shared state of the block-wide look-back.
struct LookbackSmem {
    uint32_t wf[kWarps];
    unsigned long long wc[kWarps][4];
    uint32_t first_incl[3], first_wait[3], stop, entry, pre[3], restart;
};

// Shared-memory layout (dynamic); NB tile buffers in flight.
template <bool ROWS, int NB = 2>
struct Smem {
    static constexpr int kHalo = ROWS ? kHaloBytes : 0;
    static constexpr int kBuf = kPre + kTile + kHalo;  // multiple of 16
    alignas(128) uint8_t buf[NB][kBuf];
    uint16_t stage[ROWS ? kStageCap + kHalo : kTile];
    uint64_t bar[NB];
    uint32_t warp_f[kWarps];
    unsigned long long warp_c[kWarps];
    unsigned long long warp_agg[kWarps][4];
    uint32_t entry_state;
    uint32_t tile_f;
    uint32_t base[3];       // global structural / terminator / row offsets of the tile
    unsigned long long tile_c;
    LookbackSmem lb;
    RowShared<ROWS> rs;
};

__device__ __forceinline__ bool aborted(const DevHeader *h) {
    return *(volatile const uint32_t *)&h->abort != 0;
}

__device__ __forceinline__ void fail(DevHeader *h, uint32_t bits) {
    atomicOr(&h->error, bits);
    atomicExch(&h->abort, 1u);
}

// Issue the bulk copy of tile `t` into `dst` (thread 0 only).
template <bool ROWS>
__device__ __forceinline__ void issue_tile(const Params &p, uint32_t t, uint8_t *dst, uint64_t *bar) {
    constexpr int kBuf = Smem<ROWS>::kBuf;
    const uint8_t *lo_full = p.abase + (uint64_t)t * kTile - kPre;  // address of dst[0]
    const uint8_t *lo = t == 0 ? p.abase : lo_full;
    const uint8_t *end16 = p.abase + ((p.shift + p.len + 15) & ~15ull);
    const uint8_t *hi = lo_full + kBuf;
    if (hi > end16) hi = end16;
    uint32_t bytes = (uint32_t)(hi - lo);
    mbar_expect_tx(bar, bytes);
    bulk_g2s(dst + (lo - lo_full), lo, bytes, bar);
}

// Bulk copy of tile `t` (plus the kPre bytes before it) for the index kernel.
// Input arriving in chunks (host-buffer calls): wait, bounded, until tile t's
// chunk has landed. The flag is written by the copy stream after the chunk's
// copy, behind a memory fence; chunks land in order, so the 16 bytes before
// the tile (previous chunk) are there too.
static __device__ __noinline__ bool wait_arrival(const Params &p, uint32_t t) {
    const uint32_t k = t / p.chunk_tiles;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t i = 0;; i++) {
        if (ld_acquire(p.arrive + k) == p.arrive_tag) return true;
        if ((i & 63) == 63 && globaltimer_ns() - t0 > kWaitNs) return false;
        __nanosleep(256);
    }
}

__device__ __forceinline__ void issue_tile_ix(const Params &p, uint32_t t, uint8_t *dst, uint64_t *bar) {
    if (p.arrive && !wait_arrival(p, t)) fail(p.hdr, ERR_TIMEOUT);
    constexpr int kBuf = kPre + kTile;
    const uint8_t *lo_full = p.abase + (uint64_t)t * kTile - kPre;
    const uint8_t *lo = t == 0 ? p.abase : lo_full;
    const uint8_t *end16 = p.abase + ((p.shift + p.len + 15) & ~15ull);
    const uint8_t *hi = lo_full + kBuf;
    if (hi > end16) hi = end16;
    const uint32_t bytes = (uint32_t)(hi - lo);
    mbar_expect_tx(bar, bytes);
    bulk_g2s(dst + (lo - lo_full), lo, bytes, bar);
}

// Inclusive warp scan of transfer functions.
__device__ __forceinline__ uint32_t warp_scan_f(uint32_t f, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, f, d);
        if (lane >= d) f = fcompose(o, f);
    }
    return f;
}

__device__ __forceinline__ unsigned long long warp_scan_sum(unsigned long long v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        unsigned long long o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

// Count fields packed 21 bits apart: structurals | terminators << 21 | rows << 42.
__device__ __forceinline__ uint32_t cfield(unsigned long long c, int k) {
    return (uint32_t)((c >> (21 * k)) & 0x1FFFFFull);
}

// Number of region states of each dialect's automaton.
template <int D>
struct NStates {
    static constexpr int value = D == D_TSV ? 1 : D == D_CSV ? 2 : D == D_CSV_HASH ? 3 : 4;
};

__device__ __forceinline__ uint64_t ld_relaxed64(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Combine an older aggregate (gf, gc) into a newer one (f, c), in place:
// (f . gf, gc[s] + c[gf(s)]).
template <int NS>
__device__ __forceinline__ void agg_prepend(uint32_t gf, const uint64_t (&gc)[4], uint32_t &f, uint64_t (&c)[4]) {
    uint64_t r[4];
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const uint32_t m = fapply(gf, s);
        uint64_t cm = c[0];
#pragma unroll
        for (int t = 1; t < NS; t++) cm = m == (uint32_t)t ? c[t] : cm;
        r[s] = gc[s] + cm;
    }
#pragma unroll
    for (int s = 0; s < NS; s++) c[s] = r[s];
    f = fcompose(gf, f);
}

// Counts packed 21 bits apart hold one tile (at most 16384 each); sums over
// longer spans are kept unpacked. In speculative aggregates bit 63 marks
// counts that are not known (entry states the tile did not assume).
constexpr uint64_t kUnknown = 1ull << 63;
// Assumed entry of a speculative tile that counted under every entry state.
constexpr uint32_t kAllStates = 0xFF;

// Transfer function that sends every state to x.
__device__ __forceinline__ uint32_t fconst(uint32_t x) { return x * 0x55u; }

// Prepend an older packed aggregate (gf, gc) of at most 128 tiles to a wide
// one (f, c, unknown-state mask u): (f . gf, gc[s] + c[gf(s)]).
template <int NS>
__device__ __forceinline__ void wide_prepend(uint32_t gf, const unsigned long long (&gc)[4], uint32_t &f,
                                             uint32_t (&c)[4][3], uint32_t &u) {
    uint32_t r[4][3], ru = 0;
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const uint32_t m = fapply(gf, s);
        uint32_t c0 = c[0][0], c1 = c[0][1], c2 = c[0][2];
#pragma unroll
        for (int t = 1; t < NS; t++)
            if (m == (uint32_t)t) { c0 = c[t][0]; c1 = c[t][1]; c2 = c[t][2]; }
        r[s][0] = cfield(gc[s], 0) + c0;
        r[s][1] = cfield(gc[s], 1) + c1;
        r[s][2] = cfield(gc[s], 2) + c2;
        ru |= (((uint32_t)(gc[s] >> 63) | (u >> m)) & 1u) << s;
    }
#pragma unroll
    for (int s = 0; s < NS; s++) {
        c[s][0] = r[s][0];
        c[s][1] = r[s][1];
        c[s][2] = r[s][2];
    }
    u = ru;
    f = fcompose(gf, f);
}

// As agg_prepend, keeping the unknown mark (speculative aggregates).
template <int NS>
__device__ __forceinline__ void agg_prepend_spec(uint32_t gf, const uint64_t (&gc)[4], uint32_t &f,
                                                 uint64_t (&c)[4]) {
    uint64_t r[4];
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const uint32_t m = fapply(gf, s);
        uint64_t cm = c[0];
#pragma unroll
        for (int t = 1; t < NS; t++) cm = m == (uint32_t)t ? c[t] : cm;
        r[s] = (((gc[s] & ~kUnknown) + (cm & ~kUnknown)) | ((gc[s] | cm) & kUnknown));
    }
#pragma unroll
    for (int s = 0; s < NS; s++) c[s] = r[s];
    f = fcompose(gf, f);
}

// Block-wide look-back (all threads): thread t watches predecessor
// tile - 1 - t. Waits only for the predecessors nearer than the nearest
// published inclusive prefix (level kIncl); returns the tile's entry state,
// the counts of the file before it and, for speculative aggregates, whether
// some of those counts are not known yet.
//
// Speculative status levels: 1 = the tile's full transfer function, the
// entry state it assumed and its counts under that assumption; 2 = its true
// exit state and its counts under its true entry (published by a tile whose
// assumption was wrong, as soon as its look-back knows its entry); 3 = its
// inclusive prefix. The entry state never waits on counts: it follows from
// the transfer functions alone. A level-1 tile that assumed the wrong entry
// makes the counts unknown until it reaches level 2.
template <int NS, bool SPEC>
__device__ void lookback_cta(const Params &p, LookbackSmem &L, uint32_t tile, uint32_t &entry, uint32_t pre[3],
                             bool &unknown) {
    constexpr uint32_t kIncl = SPEC ? 3 : 2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t af = kIdentity;  // thread 0: aggregate between the window and `tile`
    uint32_t ac[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    uint32_t au = 0;
    const uint64_t t0 = globaltimer_ns();
    unknown = false;
    if (tile == 0) {
        entry = p.entry0;
        pre[0] = pre[1] = pre[2] = 0;
        return;
    }
    for (int64_t hi = (int64_t)tile - 1; hi >= 0; hi -= kThreads) {
        const int64_t j = hi - tid;
        const bool in = j >= 0;
        uint32_t flag = 0;
        uint32_t sidx;
        // Three rotating slots for the block-wide minima: in poll iteration
        // `it` thread 0 resets slot it+1 before the barrier, every thread
        // updates slot it before it and reads slot it after it. No slot is
        // reset while a thread may still read it.
        if (tid == 0) {
            L.first_incl[0] = L.first_wait[0] = kThreads;
        }
        __syncthreads();
        for (uint32_t it = 0;; it++) {
            const uint32_t sl = it % 3, nx = (it + 1) % 3;
            if (tid == 0) L.first_incl[nx] = L.first_wait[nx] = kThreads;
            if (in) flag = ld_acquire(&p.status[j].flag);
            const bool cur = (flag >> 2) == p.epoch;
            const bool waitv = in && !(cur && (flag & 3) >= 1);
            const bool incl = in && cur && (flag & 3) >= kIncl;
            const uint32_t bw = __ballot_sync(0xffffffffu, waitv), bi = __ballot_sync(0xffffffffu, incl);
            if (lane == 0 && bw) atomicMin(&L.first_wait[sl], (uint32_t)(warp * 32 + __ffs(bw) - 1));
            if (lane == 0 && bi) atomicMin(&L.first_incl[sl], (uint32_t)(warp * 32 + __ffs(bi) - 1));
            __syncthreads();
            const uint32_t fw = L.first_wait[sl], fi = L.first_incl[sl];
            sidx = fi;
            if (fw > fi || fw == (uint32_t)kThreads) break;
            if ((it & 15) == 15) {
                const bool stop = tid == 0 && (aborted(p.hdr) || globaltimer_ns() - t0 > kWaitNs);
                if (__syncthreads_or(stop)) {
                    if (tid == 0) fail(p.hdr, ERR_TIMEOUT);
                    entry = 0;
                    pre[0] = pre[1] = pre[2] = 0;
                    return;
                }
            }
            __nanosleep(64);
        }
        uint32_t f = kIdentity;
        uint64_t c[4] = {0, 0, 0, 0};
        // warps whose predecessors all lie at or past the inclusive prefix
        // contribute nothing: they skip the fold (warp-uniform)
        const bool active = (uint32_t)(warp * 32) < sidx;
        if (in && (uint32_t)tid < sidx) {
            if (!SPEC) {
                f = ld_relaxed(&p.status[j].func);
#pragma unroll
                for (int s0 = 0; s0 < NS; s0++) c[s0] = ld_relaxed64(&p.status[j].agg[s0]);
            } else if ((flag & 3) >= 2) {
                f = fconst(ld_relaxed(&p.status[j].exit));
                const uint64_t v = ld_relaxed64(&p.status[j].agg[1]);
#pragma unroll
                for (int s0 = 0; s0 < NS; s0++) c[s0] = v;
            } else {
                const uint32_t pf = ld_relaxed(&p.status[j].func);
                f = pf & 0xFF;
                if ((pf >> 8) == kAllStates) {
#pragma unroll
                    for (int s0 = 0; s0 < NS; s0++) c[s0] = ld_relaxed64(&p.status[j].agg[s0]);
                } else {
                    const uint64_t v = ld_relaxed64(&p.status[j].agg[0]);
#pragma unroll
                    for (int s0 = 0; s0 < NS; s0++) c[s0] = (uint32_t)s0 == (pf >> 8) ? v : kUnknown;
                }
            }
        }
        if (active) {
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t gf = __shfl_down_sync(0xffffffffu, f, d);
                uint64_t gc[4];
#pragma unroll
                for (int s0 = 0; s0 < NS; s0++) gc[s0] = __shfl_down_sync(0xffffffffu, c[s0], d);
                if (lane + d < 32) {
                    if (SPEC) agg_prepend_spec<NS>(gf, gc, f, c);
                    else agg_prepend<NS>(gf, gc, f, c);
                }
            }
        }
        if (lane == 0 && active) {
            L.wf[warp] = f;
#pragma unroll
            for (int s0 = 0; s0 < NS; s0++) L.wc[warp][s0] = c[s0];
        }
        if ((uint32_t)tid == sidx) {
            L.entry = ld_relaxed(&p.status[j].exit);
            L.pre[0] = ld_relaxed(&p.status[j].incl[0]);
            L.pre[1] = ld_relaxed(&p.status[j].incl[1]);
            L.pre[2] = ld_relaxed(&p.status[j].incl[2]);
        }
        __syncthreads();
        if (tid == 0) {
            const int nw = sidx >= (uint32_t)kThreads ? kWarps : (int)((sidx + 31) / 32);
            for (int w = 0; w < nw; w++) {
                unsigned long long g[4];
#pragma unroll
                for (int s0 = 0; s0 < NS; s0++) g[s0] = L.wc[w][s0];
                wide_prepend<NS>(L.wf[w], g, af, ac, au);
            }
            const bool found = sidx < (uint32_t)kThreads;
            const bool at_start = hi - kThreads < 0;
            L.stop = found || at_start;
            if (found || at_start) {
                const uint32_t ex = found ? L.entry : p.entry0;
                uint32_t c0 = ac[0][0], c1 = ac[0][1], c2 = ac[0][2];
#pragma unroll
                for (int t = 1; t < NS; t++)
                    if (ex == (uint32_t)t) { c0 = ac[t][0]; c1 = ac[t][1]; c2 = ac[t][2]; }
                L.pre[0] = (found ? L.pre[0] : 0u) + c0;
                L.pre[1] = (found ? L.pre[1] : 0u) + c1;
                L.pre[2] = (found ? L.pre[2] : 0u) + c2;
                L.entry = fapply(af, ex);
                L.restart = (au >> ex) & 1u;
            }
        }
        __syncthreads();
        if (L.stop) break;
    }
    entry = L.entry;
    pre[0] = L.pre[0];
    pre[1] = L.pre[1];
    pre[2] = L.pre[2];
    unknown = SPEC && L.restart;
}

// The byte before position 0 of a launch: -1 at the start of a file.
__device__ __forceinline__ int prev_of(const Params &p) {
    return p.seeded ? (p.prev_ptr ? (int)*p.prev_ptr : (int)p.prev_byte) : -1;
}
// Position 0 starts a line: at a file start, or after a '\n'.
__device__ __forceinline__ bool starts_line(int prev) { return prev < 0 || prev == '\n'; }

// Record starts among this thread's 64 bytes for entry state s_in: position
// 0 (at a file start, or after a structural newline before a shard) and
// every byte after a structural newline, inside the data; csv_hash records
// opening with '#' are comments, not rows.
template <int D>
__device__ __forceinline__ uint64_t row_starts(const Masks &m, uint64_t term, bool prev_nl, uint32_t s_in,
                                               int64_t base_t, int64_t len, int prev) {
    uint64_t rs = (term << 1) | (uint64_t)(prev_nl && state_outside<D>(s_in));
    if (base_t <= 0 && base_t + kThreadBytes > 0 && (prev < 0 || (prev == '\n' && state_outside<D>(s_in))))
        rs |= 1ull << (-base_t);
    const int64_t live = len - base_t;
    if (live < kThreadBytes) rs &= live <= 0 ? 0 : ((1ull << live) - 1);
    if (base_t < 0) rs &= ~((1ull << (-base_t)) - 1);
    if (D == D_CSV_HASH) rs &= ~(m.x);
    return rs;
}

template <int D, bool ROWS>
__device__ __forceinline__ unsigned long long thread_counts(const Masks &m, uint64_t ls, bool prev_nl, uint32_t s,
                                                            int64_t base_t, int64_t len, int prev) {
    const uint64_t st = structural_mask<D>(m, ls, s);
    const uint64_t term = st & m.nl;
    unsigned long long c = (unsigned long long)__popcll(st) | ((unsigned long long)__popcll(term) << 21);
    if (ROWS) c |= (unsigned long long)__popcll(row_starts<D>(m, term, prev_nl, s, base_t, len, prev)) << 42;
    return c;
}

template <int D, bool ROWS, int NB = 2>
__device__ __forceinline__ void process_tile(const Params &p, Smem<ROWS, NB> &S, uint32_t tile, uint8_t *b) {
    constexpr int kBuf = Smem<ROWS, NB>::kBuf;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t vs = (int64_t)tile * kTile - (int64_t)p.shift;  // file position of b[kPre]
    const int64_t len = (int64_t)p.len;

    // Bytes outside the file read as zero (the reference zero-pads its tail).
    if (vs - kPre < 0 || vs - kPre + kBuf > len) {
        for (int i = tid; i < kBuf; i += kThreads) {
            int64_t v = vs - kPre + i;
            if (v < 0 || v >= len) b[i] = 0;
        }
        __syncthreads();
    }

    // ---- classify this thread's 64 bytes (rotated chunks: conflict-free LDS.128)
    const int r = (lane >> 1) & 3;
    uint32_t w[16];
    const uint4 *src = reinterpret_cast<const uint4 *>(b + kPre + tid * kThreadBytes);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint4 v = src[(k + r) & 3];
        w[4 * k] = v.x; w[4 * k + 1] = v.y; w[4 * k + 2] = v.z; w[4 * k + 3] = v.w;
    }
    const Masks m = classify<D>(w, r);
    const int64_t base_t = vs + (int64_t)tid * kThreadBytes;
    const bool prev_nl = b[kPre + tid * kThreadBytes - 1] == '\n';
    uint64_t ls = (m.nl << 1) | (uint64_t)prev_nl;
    if (base_t <= 0 && base_t + kThreadBytes > 0 && starts_line(prev_of(p))) ls |= 1ull << (-base_t);

    // ---- transfer functions: thread -> warp -> block
    const uint32_t f = thread_function<D>(m, ls);
    uint32_t incl = warp_scan_f(f, lane);
    if (lane == 31) S.warp_f[warp] = incl;
    uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = kIdentity;
    __syncthreads();
    if (warp == 0) {
        uint32_t wf = lane < kWarps ? S.warp_f[lane] : kIdentity;
        uint32_t wi = warp_scan_f(wf, lane);
        uint32_t we = __shfl_up_sync(0xffffffffu, wi, 1);
        if (lane == 0) we = kIdentity;
        if (lane < kWarps) S.warp_f[lane] = we;
        if (lane == kWarps - 1) S.tile_f = wi;
    }
    __syncthreads();
    excl = fcompose(S.warp_f[warp], excl);

    // ---- tile aggregate: function + counts for every entry state
    constexpr int NS = NStates<D>::value;
    unsigned long long cv[NS];
#pragma unroll
    for (int e = 0; e < NS; e++) cv[e] = thread_counts<D, ROWS>(m, ls, prev_nl, e, base_t, len, prev_of(p));
    {
        unsigned long long v[NS];
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++) {
            const uint32_t e = fapply(excl, s0);
            unsigned long long x = cv[0];
#pragma unroll
            for (int t = 1; t < NS; t++) x = e == (uint32_t)t ? cv[t] : x;
            v[s0] = x;
        }
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++) {
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) v[s0] += __shfl_xor_sync(0xffffffffu, v[s0], d);
            if (lane == 0) S.warp_agg[warp][s0] = v[s0];
        }
    }
    __syncthreads();

    // ---- publish the aggregate; one look-back gives entry state and offsets
    unsigned long long agg[4] = {0, 0, 0, 0};
#pragma unroll
    for (int s0 = 0; s0 < NS; s0++)
        for (int w2 = 0; w2 < kWarps; w2++) agg[s0] += S.warp_agg[w2][s0];
    TileStatus *const tst = &p.status[tile];
    if (tid == 0) {
        tst->func = S.tile_f;
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++) tst->agg[s0] = agg[s0];
        st_release(&tst->flag, p.epoch * 4 + 1);
    }
    {
        uint32_t pre[3], e;
        bool unknown;
        lookback_cta<NS, false>(p, S.lb, tile, e, pre, unknown);
        if (tid == 0) {
            unsigned long long mine = agg[0];
#pragma unroll
            for (int t = 1; t < NS; t++) mine = e == (uint32_t)t ? agg[t] : mine;
            tst->exit = fapply(S.tile_f, e);
            tst->incl[0] = pre[0] + cfield(mine, 0);
            tst->incl[1] = pre[1] + cfield(mine, 1);
            tst->incl[2] = pre[2] + cfield(mine, 2);
            st_release(&tst->flag, p.epoch * 4 + 2);
            S.entry_state = e;
            S.base[0] = pre[0]; S.base[1] = pre[1]; S.base[2] = pre[2];
            S.tile_c = mine;
            if (tile == p.num_tiles - 1) {
                p.hdr->n_struct = pre[0] + cfield(mine, 0);
                p.hdr->n_terms = pre[1] + cfield(mine, 1);
                p.hdr->n_rows = pre[2] + cfield(mine, 2);
            }
        }
    }
    __syncthreads();
    const uint32_t entry = S.entry_state;
    const uint32_t s_in = fapply(excl, entry);

    // ---- this thread's masks for its true entry state, ranks within the tile
    const uint64_t stm = structural_mask<D>(m, ls, s_in);
    const uint64_t term = stm & m.nl;
    uint64_t rows_m = 0;
    if (ROWS) rows_m = row_starts<D>(m, term, prev_nl, s_in, base_t, len, prev_of(p));
    unsigned long long c = cv[0];
#pragma unroll
    for (int t = 1; t < NS; t++) c = s_in == (uint32_t)t ? cv[t] : c;
    unsigned long long ci = warp_scan_sum(c, lane);
    if (lane == 31) S.warp_c[warp] = ci;
    unsigned long long ce = ci - c;
    __syncthreads();
    if (warp == 0) {
        unsigned long long wc = lane < kWarps ? S.warp_c[lane] : 0ull;
        unsigned long long wi = warp_scan_sum(wc, lane);
        if (lane < kWarps) S.warp_c[lane] = wi - wc;
    }
    __syncthreads();
    ce += S.warp_c[warp];

    // ---- stage positions (tile-relative, bit 15 = terminator) in rank order
    {
        uint32_t k = cfield(ce, 0);
        uint64_t mm = stm;
        while (mm) {
            unsigned bpos = __ffsll((long long)mm) - 1;
            uint32_t rel = (uint32_t)(tid * kThreadBytes + bpos);
            if (k < (uint32_t)(ROWS ? kStageCap : kTile)) S.stage[k] = (uint16_t)(rel | (((term >> bpos) & 1) << 15));
            k++;
            mm &= mm - 1;
        }
    }
    __syncthreads();
    const uint32_t n_tile = cfield(S.tile_c, 0);
    const uint32_t sbase = S.base[0];
    const bool overflow = ROWS && n_tile > (uint32_t)kStageCap;

    // ---- structural index: coalesced from the staging list, or straight
    // from the masks when the tile is too dense to stage
    if (p.index && !overflow) {
        for (uint32_t i = tid; i < n_tile; i += kThreads) {
            uint64_t g = (uint64_t)sbase + i;
            if (g < p.index_cap) p.index[g] = (uint32_t)(p.pos_base + vs + (S.stage[i] & 0x7FFF));
        }
    } else if (p.index) {
        uint64_t g = (uint64_t)sbase + cfield(ce, 0);
        uint64_t mm = stm;
        while (mm) {
            const unsigned bpos = __ffsll((long long)mm) - 1;
            if (g < p.index_cap) p.index[g] = (uint32_t)(p.pos_base + base_t + bpos);
            g++;
            mm &= mm - 1;
        }
    }
    // ---- tape: separators and record ends
    if (p.seps || p.ends) {
        const uint32_t tbase = S.base[1];
        const uint32_t my_s = cfield(ce, 0), my_t = cfield(ce, 1);
        uint64_t sep_before = (uint64_t)(sbase - tbase) + (my_s - my_t);  // separators before this thread
        uint64_t term_before = (uint64_t)tbase + my_t;
        uint64_t mm = stm;
        while (mm) {
            unsigned bpos = __ffsll((long long)mm) - 1;
            uint64_t pos = (uint64_t)(p.pos_base + base_t + bpos);
            if ((term >> bpos) & 1) {
                if (p.ends && term_before < p.ends_cap) p.ends[term_before] = ((p.sep_base + sep_before) << 32) | pos;
                term_before++;
            } else {
                if (p.seps && sep_before < p.seps_cap) p.seps[sep_before] = (uint32_t)pos;
                sep_before++;
            }
            mm &= mm - 1;
        }
    }

    if constexpr (ROWS) {
        RowCtx rc;
        rc.vs = vs;
        rc.len = len;
        rc.buf = b;
        rc.buf_end = vs - kPre + kBuf;
        rc.n_tile = n_tile;
        rc.row_base = S.base[2];
        rc.exit_state = fapply(S.tile_f, entry);
        rc.tile = tile;
        rc.epoch = p.epoch;
        rc.data = p.data;
        rc.astatus = reinterpret_cast<void *>(p.astatus);
        rc.hdr_arena = p.hdr->arena;
        rc.hdr_fb = &p.hdr->fb_fields;
        rc.hdr_st = &p.hdr->st_records;
        rc.hdr_error = &p.hdr->error;
        rc.hdr_abort = &p.hdr->abort;
        rc.last_tile = tile == p.num_tiles - 1;
        // does the tile's first byte start a record (comment records included)?
        const bool rec0 = vs <= 0 || (b[kPre - 1] == '\n' && state_outside<D>(entry));
        rows_phase<D>(p.rows, rc, S.rs, S.stage, rows_m, stm, term, cfield(ce, 0), cfield(ce, 1), cfield(ce, 2),
                      cfield(S.tile_c, 1), cfield(S.tile_c, 2), rec0, overflow, base_t, tid);
    }
}


}  // namespace falx
