// Structural index and tape in one persistent pass (index_pass_kernel).
//
// The input is cut into 16 KiB tiles and the tiles into groups of
// kIxGroup consecutive tiles; a group is the unit of the look-back. Each CTA
// takes the groups c, c + G, c + 2G, ... (G = resident CTAs, cooperative
// launch) and splits the work between two kinds of warps that never meet at
// a CTA-wide barrier:
//
//  8 compute warps   local pass of each tile of group i: classify its bytes
//                    (64 per thread), scan the dialect's region automaton as
//                    transfer functions (thread -> warp) and count
//                    structurals and terminators for every warp entry state;
//                    the masks go to a ring of two groups of tiles in shared
//                    memory. The last warp to finish a tile composes its
//                    aggregate (transfer function, counts per entry state)
//                    and refills the tile buffer; after the group's last
//                    tile it publishes the group's aggregate (level 1). Then
//                    the output of group i - 1: masks under their true entry
//                    states, index and tape entries.
//  1 scheduler warp  the look-backs, group after group: entry state and
//                    output offsets of each tile, the group's inclusive
//                    prefix published at level 2. (More scheduler warps
//                    measured slower: their polling competes for the same
//                    status lines in L2.)
//
// A look-back costs a few dependent round trips to L2 whatever the size of
// the unit it places; with single 16 KiB tiles the scheduler warp took
// longer per tile than the compute warps and set the pace. A group of two
// tiles halves the look-backs per byte, and with one whole group between a
// local pass and its output a CTA runs ahead of its look-backs, so the
// rounds' jitter averages out. The warps hand over through mbarriers in
// shared memory (tile bytes landed; aggregate published; look-back done).
// Transfer functions are kept in byte form (byte s = exit state for entry
// state s), so composing two is one byte permute; warp sums of counts are
// one redux each. Every wait is bounded.
//
// Reference mapping (Mapika/falx): step + prefix_xor + push_indexes
// (csv_geo.rs:2117-2170, csv_hash.rs:2125-2222, tsv.rs:1302-1308,
// logfmt.rs:994-1012, ndjson.rs:1017-1033); the three-phase region scan
// and seeded pass of the parallel drivers (csv_hash.rs:152-214, :345-399;
// csv_geo.rs:95-149, :1855-1873); push_tape (csv_geo.rs:1838-1849).
#pragma once

#include <cstdint>

#include "scan_core.cuh"
#include "tile.cuh"

namespace falx {

constexpr int kIxScheds = 1;                           // scheduler warps
constexpr int kIxThreads = kThreads + 32 * kIxScheds;  // 8 compute warps + the scheduler warp
constexpr int kIxSched = kWarps;                       // warp index of the scheduler
constexpr int kIxGroup = 2;                // tiles per look-back
constexpr int kIxSlots = 2 * kIxGroup;     // ring of tile slots: two groups (slot 2 g + k: tile k of group slot g)
constexpr int kIxStage = 256;              // staged structurals per warp and batch
constexpr int kLbPer = 8;                  // look-back: predecessors watched per lane
constexpr int kLbWin = 32 * kLbPer;        // look-back: predecessors per round of loads

// ---------------------------------------------------------------------------
// Transfer functions in byte form.
// ---------------------------------------------------------------------------
constexpr uint32_t kIdB = 0x03020100u;

__device__ __forceinline__ uint32_t fb_apply(uint32_t f, uint32_t s) { return (f >> (8u * s)) & 0xFFu; }

// Apply a, then b: byte s of the result is b[a[s]]. The byte values of a
// (each below 4) become the byte selectors of one permute.
__device__ __forceinline__ uint32_t fb_compose(uint32_t a, uint32_t b) {
    const uint32_t t = (a | (a >> 4)) & 0x00FF00FFu;
    return __byte_perm(b, 0u, t | (t >> 8));
}

// ---------------------------------------------------------------------------
// Byte classes of one thread's 64 bytes (16 words in rotated chunk order r,
// see classify in scan_core.cuh). Separators | newlines and newlines come
// from per-byte SWAR tests; the dialect's special bytes (quote, '#',
// backslash) from one combined test, then sorted into quote and other by
// reading the few bytes the combined mask marks.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ Masks ix_classify(const uint32_t (&w)[16], int r, const uint8_t *bytes) {
    Masks m;
    uint32_t sm[4], nm[4], pm[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t fs[4], fn[4], fp[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t v = w[4 * k + j];
            const uint32_t n = eq_flags(v, '\n');
            uint32_t s;
            if (D == D_TSV) s = n | eq_flags(v, '\t');
            else if (D == D_LOGFMT) s = n | eq_flags(v, ' ') | eq_flags(v, '=');
            else if (D == D_NDJSON) s = n;
            else s = n | eq_flags(v, ',');
            uint32_t sp = 0;
            if (D == D_CSV) sp = eq_flags(v, '"');
            else if (D == D_CSV_HASH) sp = zero_flags((v | 0x01010101u) ^ 0x23232323u);  // '"' or '#'
            else if (D == D_LOGFMT || D == D_NDJSON) sp = eq_flags(v, '"') | eq_flags(v, '\\');
            fs[j] = s;
            fn[j] = n;
            fp[j] = sp;
        }
        sm[k] = gather16(fs[0], fs[1], fs[2], fs[3]);
        nm[k] = gather16(fn[0], fn[1], fn[2], fn[3]);
        pm[k] = D == D_TSV ? 0u : gather16(fp[0], fp[1], fp[2], fp[3]);
    }
    m.s = assemble64(sm[0], sm[1], sm[2], sm[3], r);
    m.nl = assemble64(nm[0], nm[1], nm[2], nm[3], r);
    m.q = 0;
    m.x = 0;
    if (D == D_TSV) {
        m.special = false;
        return m;
    }
    const uint64_t sp = assemble64(pm[0], pm[1], pm[2], pm[3], r);
    m.special = sp != 0;
    if (D == D_CSV) {
        m.q = sp;
        return m;
    }
    // quote, or the dialect's other special byte ('#' or backslash)
    uint64_t q = 0, rest = sp;
    while (rest) {
        const int i = __ffsll((long long)rest) - 1;
        if (bytes[i] == '"') q |= 1ull << i;
        rest &= rest - 1;
    }
    m.q = q;
    m.x = sp & ~q;
    return m;
}

// Transfer function (byte form) and counts (structurals | terminators << 16)
// of one thread's 64 bytes for every entry state.
template <int D>
__device__ __forceinline__ uint32_t ix_function_counts(const Masks &m, uint64_t ls_bits, uint32_t (&cv)[4]) {
    auto cnt = [&](uint64_t st) { return (uint32_t)__popcll(st) | ((uint32_t)__popcll(st & m.nl) << 16); };
    if (D == D_TSV) {
        cv[0] = cnt(m.s);
        return kIdB;
    }
    if (D == D_CSV) {
        if (!m.special) {
            cv[0] = cnt(m.s);
            cv[1] = 0;
            return kIdB;
        }
        const uint64_t inq = prefix_xor64(m.q);
        cv[0] = cnt(m.s & ~inq);
        cv[1] = cnt(m.s & inq);
        return (__popcll(m.q) & 1) ? 0x03020001u : kIdB;
    }
    if (D == D_CSV_HASH) {
        if (!m.special) {
            // NORMAL: everything; QUOTE: nothing; COMMENT: from the first newline
            cv[0] = cnt(m.s);
            cv[1] = 0;
            cv[2] = m.nl ? cnt(m.s & ~((1ull << (__ffsll((long long)m.nl) - 1)) - 1)) : 0u;
            return R_N | (R_Q << 8) | ((m.nl ? R_N : R_C) << 16) | (3u << 24);
        }
        const uint64_t h = m.x & ls_bits;
        uint32_t fn, fq, fc;
        if (h == 0) {
            // no comment starts: quote parity decides, a comment ends at the
            // first newline and parity restarts there
            const uint64_t inq = prefix_xor64(m.q);
            const uint32_t par = (uint32_t)(inq >> 63);
            fn = par ? R_Q : R_N;
            fq = par ? R_N : R_Q;
            cv[0] = cnt(m.s & ~inq);
            cv[1] = cnt(m.s & inq);
            if (m.nl == 0) {
                fc = R_C;
                cv[2] = 0;
            } else {
                const uint64_t from = ~0ull << (__ffsll((long long)m.nl) - 1);
                const uint64_t before = (uint64_t)(__popcll(m.q & ~from) & 1);
                const uint64_t inq_c = inq ^ (0ull - before);
                fc = (uint32_t)(inq_c >> 63) ? R_Q : R_N;
                cv[2] = cnt(m.s & from & ~inq_c);
            }
        } else {
            fn = R_N;
            cv[0] = cnt(m.s & ~resolve_regions(m.q, h, m.nl, fn));
            fq = R_Q;
            cv[1] = cnt(m.s & ~resolve_regions(m.q, h, m.nl, fq));
            fc = R_C;
            cv[2] = cnt(m.s & ~resolve_regions(m.q, h, m.nl, fc));
        }
        return fn | (fq << 8) | (fc << 16) | (3u << 24);
    }
    // LOGFMT / NDJSON: state = escape carry | quote parity << 1
    if (!m.special) {
        cv[0] = cv[1] = cnt(m.s);
        cv[2] = cv[3] = 0;
        return 0x02020000u;  // escape carry cleared, parity kept
    }
    uint32_t r = 0;
#pragma unroll
    for (uint32_t e = 0; e < 2; e++) {
        uint32_t eo = e;
        const uint64_t ne = not_escaped64(m.x, eo);
        const uint64_t inq = prefix_xor64(m.q & ne);
        const uint32_t par = (uint32_t)(inq >> 63);
        cv[e] = cnt(m.s & ~inq);
        cv[e | 2] = cnt(m.s & inq);
#pragma unroll
        for (uint32_t pq = 0; pq < 2; pq++) r |= (eo | ((pq ^ par) << 1)) << (8u * (e | (pq << 1)));
    }
    return r;
}

// ---------------------------------------------------------------------------
// Look-back record of one group (64 bytes, in the context's tile-status
// array). Each field is written once per launch before the release of its
// level; the flag carries the launch epoch, so the array is never cleared
// between launches.
// ---------------------------------------------------------------------------
struct IxStatus {
    uint32_t flag;    // epoch * 4 + level
    uint32_t exit;    // level 2: exit state
    uint32_t incl_s;  // level 2: structurals up to the group's end
    uint32_t incl_t;  // level 2: terminators up to the group's end
    uint32_t func;    // level 1: transfer function (byte form)
    uint32_t agg[4];  // level 1: per entry state, structurals | terminators << 16 (below 2^16 each)
    uint32_t pad[7];
};
static_assert(sizeof(IxStatus) == sizeof(TileStatus), "tile status records share one array");

struct IxSmem {
    alignas(128) uint8_t buf[2][kPre + kTile];
    // per ring slot, per thread: the masks kept for the output, and the
    // function of the threads before it in its warp (bit 31: the byte before
    // its 64 is a newline)
    uint64_t ms[kIxSlots][kThreads], mnl[kIxSlots][kThreads], mq[kIxSlots][kThreads], mx[kIxSlots][kThreads];
    uint32_t mex[kIxSlots][kThreads];
    uint16_t stage[kWarps][kIxStage];       // per warp: a batch of its structurals in rank order
    uint64_t full[2];                       // per buffer (tile k of a group): its bytes have landed (bulk copy)
    uint64_t pub[2];                        // per group slot: the group's aggregate is published
    uint64_t lb[2];                         // per group slot: the group's look-back is done
    uint32_t wf[kIxSlots][kWarps];          // warp-inclusive transfer functions
    uint32_t wc[kIxSlots][kWarps][4];       // warp counts per warp entry state
    uint32_t wx[kIxSlots][kWarps];          // function of the warps before, within the tile
    uint32_t tf[kIxSlots];                  // the tile's transfer function
    uint32_t tc[kIxSlots][4];               // the tile's counts per entry state
    uint32_t cnt[kIxSlots];                 // compute warps done with the tile's local pass
    uint32_t base_s[kIxSlots], base_t[kIxSlots];  // structurals / terminators before the tile
    uint32_t went[kIxSlots][kWarps];        // entry state of each warp
    uint32_t woff[kIxSlots][kWarps];        // counts before each warp within the tile
    uint32_t issued[2], used[2];            // bulk copies per buffer: issued, waited for
    uint32_t stop;                          // a wait gave up: every warp leaves
};

__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bytes of the thread's 16 words outside [0, len) read as zero (the
// reference zero-pads its tail block, interp.rs:155-183). Word 4k + j holds
// bytes 16 ((k + r) & 3) + 4 j of the thread's 64.
__device__ __forceinline__ void mask_outside(uint32_t (&w)[16], int r, int64_t base_t, int64_t len) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int64_t a = base_t + 16 * ((k + r) & 3) + 4 * j;
            uint32_t keep = 0xFFFFFFFFu;
            if (a < 0) keep = a <= -4 ? 0u : keep << (8 * (int)(-a));
            const int64_t rem = len - a;
            if (rem < 4) keep &= rem <= 0 ? 0u : 0xFFFFFFFFu >> (8 * (int)(4 - rem));
            w[4 * k + j] &= keep;
        }
    }
}

// Line starts of the thread's 64 bytes: after each newline, after a newline
// just before them, and at file position 0 when the launch starts a line.
__device__ __forceinline__ uint64_t ix_line_starts(const Params &p, uint64_t nl, bool prev_nl, int64_t base_t) {
    uint64_t ls = (nl << 1) | (uint64_t)prev_nl;
    if (base_t <= 0 && base_t + kThreadBytes > 0 && starts_line(prev_of(p))) ls |= 1ull << (-base_t);
    return ls;
}

// Local pass of one tile (compute threads): masks into ring slot `rs`, the
// warp's function and counts per warp entry state into shared memory.
template <int D>
__device__ __forceinline__ void ix_local(const Params &p, IxSmem &S, uint32_t tile, int bs, int rs) {
    constexpr int NS = NStates<D>::value;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint8_t *b = S.buf[bs];
    const int64_t vs = (int64_t)tile * kTile - (int64_t)p.shift;  // file position of b[kPre]
    const int64_t len = (int64_t)p.len;
    const int64_t base_t = vs + (int64_t)tid * kThreadBytes;
    const int r = (lane >> 1) & 3;
    uint32_t w[16];
    const uint8_t *mine = b + kPre + tid * kThreadBytes;
    const uint4 *src = reinterpret_cast<const uint4 *>(mine);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint4 v = src[(k + r) & 3];
        w[4 * k] = v.x;
        w[4 * k + 1] = v.y;
        w[4 * k + 2] = v.z;
        w[4 * k + 3] = v.w;
    }
    if (base_t < 0 || base_t + kThreadBytes > len) mask_outside(w, r, base_t, len);
    const int64_t pp = base_t - 1;
    const bool prev_nl = pp >= 0 && pp < len && mine[-1] == '\n';
    const Masks m = ix_classify<D>(w, r, mine);
    const uint64_t ls = ix_line_starts(p, m.nl, prev_nl, base_t);
    uint32_t cv[4];
    const uint32_t f = ix_function_counts<D>(m, ls, cv);
    uint32_t incl = f;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl = fb_compose(o, incl);
    }
    uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = kIdB;
    uint32_t wc[4];
#pragma unroll
    for (int e = 0; e < NS; e++) {
        const uint32_t ts = fb_apply(excl, (uint32_t)e);
        uint32_t c = cv[0];
#pragma unroll
        for (int t = 1; t < NS; t++) c = ts == (uint32_t)t ? cv[t] : c;
        wc[e] = __reduce_add_sync(0xffffffffu, c);  // at most 2048 of each per warp: no carry between halves
    }
    S.ms[rs][tid] = m.s;
    S.mnl[rs][tid] = m.nl;
    S.mq[rs][tid] = m.q;
    S.mx[rs][tid] = m.x;
    S.mex[rs][tid] = excl | ((uint32_t)prev_nl << 31);
    if (lane == 31) S.wf[rs][warp] = incl;
    if (lane == 0) {
#pragma unroll
        for (int e = 0; e < NS; e++) S.wc[rs][warp][e] = wc[e];
    }
}

// The last compute warp of a local pass: the tile's transfer function and
// counts per entry state from the eight warps', into shared memory.
template <int D>
__device__ __forceinline__ void ix_tile_agg(IxSmem &S, int rs, int lane) {
    constexpr int NS = NStates<D>::value;
    const int w = lane & (kWarps - 1);
    const uint32_t wf = lane < kWarps ? S.wf[rs][w] : kIdB;
    uint32_t incl = wf;
#pragma unroll
    for (int d = 1; d < kWarps; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl = fb_compose(o, incl);
    }
    uint32_t wx = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) wx = kIdB;
    const uint32_t tf = __shfl_sync(0xffffffffu, incl, kWarps - 1);
    uint32_t tot[4];
#pragma unroll
    for (int e = 0; e < NS; e++) {
        const uint32_t we = fb_apply(wx, (uint32_t)e);
        const uint32_t c = lane < kWarps ? S.wc[rs][w][we & 3] : 0u;
        tot[e] = __reduce_add_sync(0xffffffffu, c);  // at most 16384 of each per tile
    }
    if (lane < kWarps) S.wx[rs][w] = wx;
    if (lane == 0) {
        S.tf[rs] = tf;
#pragma unroll
        for (int e = 0; e < NS; e++) S.tc[rs][e] = tot[e];
    }
}

// The group's aggregate from its tiles' (slots rs0 .. rs0 + nt - 1),
// published at level 1 (one thread).
template <int D>
__device__ __forceinline__ void ix_group_publish(const Params &p, IxSmem &S, IxStatus *st, uint32_t group, int rs0,
                                                 int nt) {
    constexpr int NS = NStates<D>::value;
    IxStatus *me = st + group;
    uint32_t f = kIdB;
    uint32_t agg[4] = {0, 0, 0, 0};
    for (int k = 0; k < nt; k++) {
#pragma unroll
        for (int e = 0; e < NS; e++) agg[e] += S.tc[rs0 + k][fb_apply(f, (uint32_t)e)];
        f = fb_compose(f, S.tf[rs0 + k]);
    }
    me->func = f;
#pragma unroll
    for (int e = 0; e < NS; e++) me->agg[e] = agg[e];
    st_release(&me->flag, p.epoch * 4 + 1);
}

// Scheduler warp: entry state of group `tile` and the structurals /
// terminators before it, by a look-back over the group records. Returns false if a wait gave up (the error is
// recorded in the header).
//
// Two phases. (1) Flags only, newest first, kLbWin per round of relaxed
// loads (lane l watches tile-1-kLbPer*l-k): find the nearest tile j* with
// its inclusive prefix published, waiting until every tile after it has
// its aggregate; one fence then orders those loads before the loads of the
// data. (2) Forward from j*, whose exit state and counts are known, kLbWin
// tiles per round (lane l takes kLbPer consecutive tiles): each lane
// composes its tiles' transfer functions, a warp scan gives the state
// entering every lane's run, and each lane adds the counts of its tiles
// under the states they are entered in. No count vector per entry state is
// carried.
template <int D>
__device__ __forceinline__ bool ix_lookback(const Params &p, IxStatus *st, uint32_t tile, int lane, uint32_t e0,
                                            uint32_t b0s, uint32_t b0t, uint32_t &entry, uint32_t &bs, uint32_t &bt) {
    constexpr int NS = NStates<D>::value;
    // e0, b0s, b0t: the launch's entry state and the counts before it
    entry = e0;
    bs = b0s;
    bt = b0t;
    if (tile > 0) {
        // ---- (1) the nearest inclusive prefix
        const uint64_t t0 = globaltimer_ns();
        int64_t jstar = -1;
        for (int64_t hi = (int64_t)tile - 1; hi >= 0; hi -= kLbWin) {
            uint32_t fi;
            for (uint32_t it = 0;; it++) {
                uint32_t inc = 0, notr = 0;
#pragma unroll
                for (int k = 0; k < kLbPer; k++) {
                    const int64_t j = hi - kLbPer * lane - k;
                    if (j < 0) {
                        inc |= 1u << k;  // before the file: the launch's entry state, nothing counted
                    } else {
                        const uint32_t f = ld_relaxed(&st[j].flag);
                        const bool cur = (f >> 2) == p.epoch;
                        if (cur && (f & 3) >= 2) inc |= 1u << k;
                        if (!(cur && (f & 3) >= 1)) notr |= 1u << k;
                    }
                }
                fi = __reduce_min_sync(0xffffffffu, inc ? kLbPer * lane + __ffs(inc) - 1 : (uint32_t)kLbWin);
                const uint32_t fw =
                    __reduce_min_sync(0xffffffffu, notr ? kLbPer * lane + __ffs(notr) - 1 : (uint32_t)kLbWin);
                if (fw >= fi) break;  // every tile nearer than the nearest inclusive prefix has its aggregate
                if ((it & 7) == 7) {
                    const bool stop = lane == 0 && (aborted(p.hdr) || globaltimer_ns() - t0 > kWaitNs);
                    if (__any_sync(0xffffffffu, stop)) {
                        if (lane == 0) fail(p.hdr, ERR_TIMEOUT);
                        return false;
                    }
                }
                __nanosleep(32);
            }
            if (fi < (uint32_t)kLbWin) {
                jstar = hi - (int64_t)fi;
                break;
            }
        }
        fence_acq_rel_gpu();  // the relaxed flag loads above happen before the data loads below
        uint32_t s = e0;
        if (jstar >= 0) {
            s = ld_relaxed(&st[jstar].exit);
            bs = ld_relaxed(&st[jstar].incl_s);
            bt = ld_relaxed(&st[jstar].incl_t);
        }
        // ---- (2) fold forward over tiles jstar+1 .. tile-1
        for (int64_t lo = jstar + 1; lo < (int64_t)tile; lo += kLbWin) {
            uint32_t g[kLbPer], a[kLbPer][NS];
            uint32_t fl = kIdB;  // the lane's run, oldest tile first
#pragma unroll
            for (int k = 0; k < kLbPer; k++) {
                const int64_t j = lo + kLbPer * lane + k;
                g[k] = kIdB;
#pragma unroll
                for (int e = 0; e < NS; e++) a[k][e] = 0;
                if (j < (int64_t)tile) {
                    g[k] = ld_relaxed(&st[j].func);
#pragma unroll
                    for (int e = 0; e < NS; e++) a[k][e] = ld_relaxed(&st[j].agg[e]);
                }
                fl = fb_compose(fl, g[k]);
            }
            // state entering each lane's run: the runs of the lanes before it
            uint32_t x = fl;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x = fb_compose(o, x);
            }
            uint32_t ex = __shfl_up_sync(0xffffffffu, x, 1);
            if (lane == 0) ex = kIdB;
            uint32_t q = fb_apply(ex, s), cs = 0, ct = 0;
#pragma unroll
            for (int k = 0; k < kLbPer; k++) {
                uint32_t c = a[k][0];
#pragma unroll
                for (int e = 1; e < NS; e++) c = q == (uint32_t)e ? a[k][e] : c;
                cs += c & 0xFFFFu;
                ct += c >> 16;
                q = fb_apply(g[k], q);
            }
            bs += __reduce_add_sync(0xffffffffu, cs);  // a window's counts stay below 2^32
            bt += __reduce_add_sync(0xffffffffu, ct);
            s = fb_apply(__shfl_sync(0xffffffffu, x, 31), s);
        }
        entry = s;
    }
    return true;
}

// Scheduler warp, once the group's aggregate is in: per-warp entry states and
// offsets of one of its tiles into shared memory. Returns the tile's counts
// (structurals | terminators << 16) under its entry state.
template <int D>
__device__ __forceinline__ uint32_t ix_place(IxSmem &S, int slot, int lane, uint32_t entry, uint32_t bs,
                                             uint32_t bt) {
    const int w = lane & (kWarps - 1);
    const uint32_t wx = lane < kWarps ? S.wx[slot][w] : kIdB;
    const uint32_t we = fb_apply(wx, entry);
    const uint32_t wc = lane < kWarps ? S.wc[slot][w][we & 3] : 0u;
    uint32_t x = wc;
#pragma unroll
    for (int d = 1; d < kWarps; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += o;
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, x, kWarps - 1);
    if (lane < kWarps) {
        S.went[slot][w] = we;
        S.woff[slot][w] = x - wc;
    }
    if (lane == 0) {
        S.base_s[slot] = bs;
        S.base_t[slot] = bt;
    }
    return tot;
}

__device__ __forceinline__ uint32_t cap32(uint64_t cap) { return cap > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)cap; }

// Output of a tile (compute threads, after its look-back): the thread's
// masks under its true entry state, ranks within the warp, then the warp's
// index and tape entries from a staged list, coalesced.
template <int D>
__device__ __forceinline__ void ix_output(const Params &p, IxSmem &S, uint32_t tile, int rs) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t vs = (int64_t)tile * kTile - (int64_t)p.shift;
    const int64_t base_t = vs + (int64_t)tid * kThreadBytes;
    Masks m;
    m.s = S.ms[rs][tid];
    m.nl = S.mnl[rs][tid];
    m.q = S.mq[rs][tid];
    m.x = S.mx[rs][tid];
    m.special = (m.q | m.x) != 0;
    const uint32_t mex = S.mex[rs][tid];
    const uint64_t ls = ix_line_starts(p, m.nl, (mex >> 31) != 0, base_t);
    const uint32_t s_in = fb_apply(mex & 0x7FFFFFFFu, S.went[rs][warp]);
    if (p.states64) p.states64[(uint64_t)tile * kThreads + tid] = (uint8_t)s_in;
    const uint64_t stm = structural_mask<D>(m, ls, s_in);
    const uint64_t term = stm & m.nl;
    const uint32_t c = (uint32_t)__popcll(stm) | ((uint32_t)__popcll(term) << 16);
    uint32_t x = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += o;
    }
    const uint32_t woff = S.woff[rs][warp], ce = x - c;
    const uint32_t n = __shfl_sync(0xffffffffu, x, 31) & 0xFFFFu;  // the warp's structurals
    const uint32_t my0 = ce & 0xFFFFu, my1 = my0 + (c & 0xFFFFu);   // my ranks within the warp
    // Ordinals and positions in 32 bits: a launch's input is shorter than
    // 4 GiB, so its counts and positions (base included) fit.
    const uint32_t gs0 = S.base_s[rs] + (woff & 0xFFFFu);  // structurals before the warp's run
    uint32_t gt = S.base_t[rs] + (woff >> 16);              // terminators before the batch
    const uint32_t pbase = (uint32_t)(p.pos_base + vs);
    const uint32_t sbase = (uint32_t)p.sep_base;            // ends keep the low 32 bits of the separator count
    const uint32_t icap = p.index ? cap32(p.index_cap) : 0u;
    const uint32_t scap = p.seps ? cap32(p.seps_cap) : 0u;
    const uint32_t ecap = p.ends ? cap32(p.ends_cap) : 0u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t at = (uint32_t)tid * kThreadBytes;
    uint16_t *stage = S.stage[warp];
    // batches of kIxStage ranks: stage (tile offset, bit 15 = terminator) in
    // rank order, then write index and tape entries coalesced
    for (uint32_t lo = 0; lo < n; lo += kIxStage) {
        const uint32_t hi = min(lo + (uint32_t)kIxStage, n);
        if (n <= (uint32_t)kIxStage) {
            // one batch (the usual case): all of the thread's structurals
            uint64_t mm = stm;
            uint32_t k = my0;
            while (mm) {
                const uint32_t b = (uint32_t)__ffsll((long long)mm) - 1u;
                stage[k++] = (uint16_t)((at + b) | ((uint32_t)(term >> b) & 1u) << 15);
                mm &= mm - 1;
            }
        } else if (my1 > lo && my0 < hi) {
            uint32_t k = my0;
            uint64_t mm = stm;
            while (mm && k < hi) {
                const uint32_t b = (uint32_t)__ffsll((long long)mm) - 1u;
                if (k >= lo) stage[k - lo] = (uint16_t)((at + b) | ((uint32_t)(term >> b) & 1u) << 15);
                k++;
                mm &= mm - 1;
            }
        }
        __syncwarp();
        for (uint32_t q = lo; q < hi; q += 32) {
            const uint32_t kk = q + lane;
            const bool in = kk < hi;
            const uint32_t e = in ? stage[kk - lo] : 0u;
            const bool is_t = in && (e >> 15);
            const uint32_t bt_mask = __ballot_sync(0xffffffffu, is_t);
            const uint32_t gs = gs0 + kk;                    // structural ordinal
            const uint32_t gtt = gt + __popc(bt_mask & lt);  // terminators before it
            const uint32_t gsep = gs - gtt;                  // separators before it
            const uint32_t pos = pbase + (e & 0x7FFFu);
            if (in && gs < icap) p.index[gs] = pos;
            if (is_t) {
                if (gtt < ecap) p.ends[gtt] = ((uint64_t)(sbase + gsep) << 32) | pos;
            } else if (in && gsep < scap) {
                p.seps[gsep] = pos;
            }
            gt += __popc(bt_mask);
        }
        __syncwarp();  // the batch is read before the next one is staged
    }
}

// Bulk copy of tile t into buffer b (one thread), counted for the drain.
__device__ __forceinline__ void ix_issue(const Params &p, IxSmem &S, uint32_t t, int b) {
    issue_tile_ix(p, t, S.buf[b], &S.full[b]);
    S.issued[b]++;
}

__device__ __forceinline__ bool ix_stopped(IxSmem &S) { return *(volatile uint32_t *)&S.stop != 0; }
__device__ __forceinline__ void ix_set_stop(IxSmem &S) { *(volatile uint32_t *)&S.stop = 1; }

// SEED: the launch's entry state and counts come from p.seed_in (chunks of
// a pipelined call); without it they are p.entry0 and zero.
template <int D, bool SEED = false>
__global__ void __launch_bounds__(kIxThreads, 3) index_pass_kernel(const __grid_constant__ Params p) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    IxSmem &S = *reinterpret_cast<IxSmem *>(smem_raw);
    IxStatus *const st = reinterpret_cast<IxStatus *>(p.status);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t G = gridDim.x;
    const uint32_t groups = (p.num_tiles + kIxGroup - 1) / kIxGroup;
    const uint32_t own = (groups - blockIdx.x + G - 1) / G;  // groups of this CTA (grid <= groups)
    // tiles of group g that exist (the last group may be short)
    auto tiles_of = [&](uint32_t g) -> int {
        const uint32_t t0 = g * kIxGroup;
        return (int)min((uint32_t)kIxGroup, p.num_tiles - t0);
    };
    if (tid == 0) {
        mbar_init(&S.full[0], 1);
        mbar_init(&S.full[1], 1);
        for (int k = 0; k < 2; k++) {
            mbar_init(&S.pub[k], 1);
            mbar_init(&S.lb[k], 1);
        }
        for (int k = 0; k < kIxSlots; k++) S.cnt[k] = 0;
        S.issued[0] = S.issued[1] = S.used[0] = S.used[1] = 0;
        S.stop = 0;
        fence_mbar_init();
        if (own > 0) {
            const uint32_t g = blockIdx.x;
            for (int k = 0; k < tiles_of(g); k++) ix_issue(p, S, g * kIxGroup + k, k);
        }
    }
    __syncthreads();
    if (warp >= kIxSched) {
        // ---- scheduler warp: the look-backs, in group order
        const uint32_t e0 = SEED ? p.seed_in->exit_state : p.entry0;
        const uint32_t b0s = SEED ? (uint32_t)p.seed_in->n_struct : 0u;
        const uint32_t b0t = SEED ? (uint32_t)p.seed_in->n_terms : 0u;
        for (uint32_t j = (uint32_t)(warp - kIxSched); j < own; j += kIxScheds) {
            const uint32_t g = blockIdx.x + j * G;
            const int gs = (int)(j & 1);
            // the look-back starts once this CTA's own group is published, by
            // which time the groups before it in the round mostly are too
            // (starting earlier only adds polling traffic)
            const bool pub_ok = mbar_wait(&S.pub[gs], (j >> 1) & 1, kWaitNs);
            uint32_t entry = 0, bs = 0, bt = 0;
            const bool lb_ok =
                __all_sync(0xffffffffu, pub_ok) && ix_lookback<D>(p, st, g, lane, e0, b0s, b0t, entry, bs, bt);
            const bool ok = pub_ok && lb_ok;
            if (!__all_sync(0xffffffffu, ok) || ix_stopped(S)) {
                if (lane == 0) {
                    if (!pub_ok) fail(p.hdr, ERR_TIMEOUT);
                    ix_set_stop(S);
                    mbar_arrive(&S.lb[gs]);  // the compute warps see stop
                }
                break;
            }
            // each tile of the group: entry state and offsets, in order
            const int nt = tiles_of(g);
            uint32_t s = entry, cs = bs, ct = bt;
            for (int k = 0; k < nt; k++) {
                const int slot = 2 * gs + k;
                const uint32_t tot = ix_place<D>(S, slot, lane, s, cs, ct);
                s = fb_apply(S.tf[slot], s);
                cs += tot & 0xFFFFu;
                ct += tot >> 16;
            }
            if (lane == 0) {
                IxStatus *me = st + g;
                me->exit = s;
                me->incl_s = cs;
                me->incl_t = ct;
                st_release(&me->flag, p.epoch * 4 + 2);
                if (g == groups - 1) {
                    p.hdr->n_struct = cs;
                    p.hdr->n_terms = ct;
                    p.hdr->exit_state = s;
                    if (p.seed_out) {
                        p.seed_out->exit_state = s;
                        p.seed_out->n_struct = cs;
                        p.seed_out->n_terms = ct;
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.lb[gs]);
        }
    } else {
        // ---- compute warps: local passes of group i, output of group i - 1
        for (uint32_t i = 0; i < own + 1; i++) {
            bool quit = false;
            if (i < own) {
                const uint32_t g = blockIdx.x + i * G;
                const int gs = (int)(i & 1), nt = tiles_of(g);
                for (int k = 0; k < nt && !quit; k++) {
                    const uint32_t tile = g * kIxGroup + k;
                    const int rs = 2 * gs + k;
                    const bool ok = mbar_wait(&S.full[k], i & 1, kWaitNs);
                    // the abort flag is read every 16th group: every wait is bounded
                    const bool ab = lane == 0 && k == 0 && (i & 15) == 15 && aborted(p.hdr);
                    if (!__all_sync(0xffffffffu, ok) || __any_sync(0xffffffffu, ab) || ix_stopped(S)) {
                        if (lane == 0) {
                            if (!ok) fail(p.hdr, ERR_TMA);
                            ix_set_stop(S);
                        }
                        quit = true;
                        break;
                    }
                    ix_local<D>(p, S, tile, k, rs);
                    __syncwarp();
                    uint32_t last = 0;
                    if (lane == 0) {
                        __threadfence_block();  // this warp's shared-memory results before the count
                        last = atomicAdd(&S.cnt[rs], 1u) == kWarps - 1;
                    }
                    if (__shfl_sync(0xffffffffu, last, 0)) {
                        __threadfence_block();  // every warp's results are visible to the last one
                        ix_tile_agg<D>(S, rs, lane);
                        if (lane == 0) {
                            S.cnt[rs] = 0;
                            S.used[k]++;
                            // every warp has read buf[k]: refill it with tile k of
                            // this CTA's next group
                            if (i + 1 < own) {
                                const uint32_t g2 = g + G;
                                if (k < tiles_of(g2)) {
                                    fence_proxy_async();
                                    ix_issue(p, S, g2 * kIxGroup + k, k);
                                }
                            }
                            if (k == nt - 1) {
                                ix_group_publish<D>(p, S, st, g, 2 * gs, nt);
                                mbar_arrive(&S.pub[gs]);
                            }
                        }
                    }
                }
            }
            if (quit) break;
            if (i >= 1) {
                const uint32_t o = i - 1;  // group whose output is due
                const uint32_t g = blockIdx.x + o * G;
                const int gs = (int)(o & 1);
                const bool ok = mbar_wait(&S.lb[gs], (o >> 1) & 1, kWaitNs);
                if (!__all_sync(0xffffffffu, ok) || ix_stopped(S)) {
                    if (lane == 0 && !ok) {
                        fail(p.hdr, ERR_TIMEOUT);
                        ix_set_stop(S);
                    }
                    break;
                }
                const int nt = tiles_of(g);
                for (int k = 0; k < nt; k++) ix_output<D>(p, S, g * kIxGroup + k, 2 * gs + k);
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        // never leave a bulk copy in flight into this CTA's shared memory
        for (int b = 0; b < 2; b++)
            if (S.issued[b] > S.used[b]) mbar_wait(&S.full[b], S.used[b] & 1, kWaitNs);
    }
}

}  // namespace falx
