// GB300 engine for the falx structural-index / column-materialisation path.
//
// One persistent kernel per call. CTAs take 16 KiB tiles from an atomic
// ticket counter, stage each tile (plus a few bytes before it and, when rows
// are materialised, a halo after it) into shared memory with a TMA bulk copy
// that is issued one tile ahead, classify bytes with 4-byte SWAR tests, scan
// the dialect's region automaton as packed transfer functions (thread ->
// warp -> block), and chain tiles with a bounded decoupled look-back: first
// the region state (so every tile resolves quotes / comments / escapes
// without a second read of the input), then the output offsets. Positions
// are compacted with popc ranks through shared memory and written coalesced.
//
// Reference mapping (Mapika/falx):
//   step() + prefix_xor + push_indexes    csv_geo.rs:2117-2170, csv_hash.rs:2125-2222,
//                                          tsv.rs:1302-1308, logfmt.rs:994-1012, ndjson.rs:1017-1033
//   three-phase region scan (csv_hash)    csv_hash.rs:152-214, :345-399, :1921-1955
//   speculative quote parity (csv)        csv_geo.rs:95-149
//   tape (parse / records / fields)       csv_geo.rs:394-686, :1838-1849
//   ColumnSink / stats / field bytes      csv_geo.rs:952-1101, :1491-1770; csv_hash.rs:965-1435
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "../../include/falx_gpu.h"
#include "mlp.cuh"
#include "ndjson.cuh"
#include "rows.cuh"
#include "scan_core.cuh"

#include "tile.cuh"
#include "columns.cuh"
#include "index_pass.cuh"

namespace falx {

// ===========================================================================
// Index / tape kernel with deferred look-back.
//
// Without rows, a tile's input is only read during its local pass, so its
// buffer is refilled right after that pass and the tile's look-back and
// output are deferred by one round: iteration i runs the local pass of tile
// c + iG, then the look-back and output of tile c + (i-1)G. By then every
// aggregate the look-back needs has been published, so it never waits on a
// tile that is still classifying.
// ===========================================================================
struct LocalState {
    Masks m;
    uint64_t ls;
    int64_t base_t;
    uint32_t excl;
    bool prev_nl;
    unsigned long long cv[4];
    uint64_t stm;  // speculative: structural mask under the assumed entry
};

struct SmemIx {
    alignas(128) uint8_t buf[2][kPre + kTile];
    uint16_t stage[kTile];
    uint64_t bar[2];
    uint32_t warp_f[kWarps];
    unsigned long long warp_agg[kWarps][4];
    unsigned long long warp_c[kWarps];
    // per-tile results of the local pass, two slots: the local pass of tile
    // i writes slot i & 1 while the deferred output of tile i - 1 reads the
    // other, so no hand-over copy (and no barrier pair) is needed
    uint32_t tile_f[2];
    unsigned long long agg[2][4];
    LookbackSmem lb;  // block-wide look-back
    uint32_t base[3];
    unsigned long long tile_c;
    // speculative index: entry state assumed by the tile in its local pass
    // and by the deferred one; counts of the look-back not known yet
    uint32_t spec_p[2];
};

// Local pass of one tile: classify, scan transfer functions, publish the
// aggregate. Leaves the per-thread state needed by the deferred output.
// SPEC: the tile assumes the entry state p.pred[tile] (tile 0 assumes the
// file's initial state), counts only under that assumption and publishes
// its full transfer function, the assumed entry and those counts.
template <int D, bool SPEC, bool CROWS = false>
__device__ __forceinline__ void local_pass(const Params &p, SmemIx &S, uint32_t tile, uint8_t *b, LocalState &L,
                                           int slot) {
    constexpr int kBuf = kPre + kTile;
    constexpr int NS = NStates<D>::value;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t vs = (int64_t)tile * kTile - (int64_t)p.shift;
    const int64_t len = (int64_t)p.len;
    if (vs - kPre < 0 || vs - kPre + kBuf > len) {
        for (int i = tid; i < kBuf; i += kThreads) {
            const int64_t v = vs - kPre + i;
            if (v < 0 || v >= len) b[i] = 0;
        }
        __syncthreads();
    }
    const int r = (lane >> 1) & 3;
    uint32_t w[16];
    const uint4 *src = reinterpret_cast<const uint4 *>(b + kPre + tid * kThreadBytes);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint4 v = src[(k + r) & 3];
        w[4 * k] = v.x; w[4 * k + 1] = v.y; w[4 * k + 2] = v.z; w[4 * k + 3] = v.w;
    }
    L.m = classify<D>(w, r);
    L.base_t = vs + (int64_t)tid * kThreadBytes;
    L.prev_nl = b[kPre + tid * kThreadBytes - 1] == '\n';
    L.ls = (L.m.nl << 1) | (uint64_t)L.prev_nl;
    if (L.base_t <= 0 && L.base_t + kThreadBytes > 0 && starts_line(prev_of(p))) L.ls |= 1ull << (-L.base_t);
    const uint32_t f = thread_function<D>(L.m, L.ls);
    uint32_t incl = warp_scan_f(f, lane);
    if (lane == 31) S.warp_f[warp] = incl;
    uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = kIdentity;
    if (!SPEC) {
#pragma unroll
        for (int e = 0; e < NS; e++) L.cv[e] = thread_counts<D, CROWS>(L.m, L.ls, L.prev_nl, e, L.base_t, len, prev_of(p));
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t wf = lane < kWarps ? S.warp_f[lane] : kIdentity;
        const uint32_t wi = warp_scan_f(wf, lane);
        uint32_t we = __shfl_up_sync(0xffffffffu, wi, 1);
        if (lane == 0) we = kIdentity;
        if (lane < kWarps) S.warp_f[lane] = we;
        if (lane == kWarps - 1) S.tile_f[slot] = wi;
    }
    __syncthreads();
    L.excl = fcompose(S.warp_f[warp], excl);
    uint32_t pk = kAllStates;
    if (SPEC) {
        pk = tile == 0 ? p.entry0 : !p.pred ? 0u : (uint32_t)p.pred[tile];
        if (pk >= (uint32_t)NS && pk != kAllStates) pk = 0;
    }
    if (SPEC && pk == kAllStates) {
        // no assumption: count under every entry state, as the plain scan does
#pragma unroll
        for (int e = 0; e < NS; e++) L.cv[e] = thread_counts<D, CROWS>(L.m, L.ls, L.prev_nl, e, L.base_t, len, prev_of(p));
    }
    if (SPEC && pk != kAllStates) {
        const uint32_t s_in = fapply(L.excl, pk);
        L.stm = structural_mask<D>(L.m, L.ls, s_in);
        unsigned long long v = (unsigned long long)__popcll(L.stm) |
                               ((unsigned long long)__popcll(L.stm & L.m.nl) << 21);
        L.cv[0] = v;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
        if (lane == 0) S.warp_agg[warp][0] = v;
        __syncthreads();
        if (tid == 0) {
            TileStatus *tst = &p.status[tile];
            unsigned long long agg = 0;
            for (int w2 = 0; w2 < kWarps; w2++) agg += S.warp_agg[w2][0];
            tst->func = S.tile_f[slot] | (pk << 8);
            tst->agg[0] = agg;
            st_release(&tst->flag, p.epoch * 4 + 1);
            S.agg[slot][0] = agg;
            S.spec_p[slot] = pk;
        }
        return;
    }
    {
        unsigned long long v[NS];
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++) {
            const uint32_t e = fapply(L.excl, s0);
            unsigned long long x = L.cv[0];
#pragma unroll
            for (int t = 1; t < NS; t++) x = e == (uint32_t)t ? L.cv[t] : x;
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
    if (tid == 0) {
        TileStatus *tst = &p.status[tile];
        unsigned long long agg[4] = {0, 0, 0, 0};
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++)
            for (int w2 = 0; w2 < kWarps; w2++) agg[s0] += S.warp_agg[w2][s0];
        tst->func = SPEC ? (S.tile_f[slot] | (kAllStates << 8)) : S.tile_f[slot];
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++) tst->agg[s0] = agg[s0];
        st_release(&tst->flag, p.epoch * 4 + 1);
        for (int s0 = 0; s0 < 4; s0++) S.agg[slot][s0] = agg[s0];
        S.spec_p[slot] = kAllStates;
    }
}

// Deferred output of one tile: inclusive prefix, staged index, tape.
// SPEC: a tile whose true entry (from the look-back) equals the one it
// assumed reuses its local-pass masks; otherwise it re-derives them from
// the true entry (the classified bytes are still in registers), publishes
// its true exit and counts at once (level 2), and then its inclusive prefix
// when every count before it is known.
template <int D, bool SPEC>
__device__ __forceinline__ void output_pass(const Params &p, SmemIx &S, uint32_t tile, const LocalState &L,
                                            int slot) {
    constexpr int NS = NStates<D>::value;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t vs = (int64_t)tile * kTile - (int64_t)p.shift;
    uint32_t entry, pre[3];
    bool unknown;
    lookback_cta<NS, SPEC>(p, S.lb, tile, entry, pre, unknown);
    const bool full = !SPEC || S.spec_p[slot] == kAllStates;  // counted under every entry
    const bool hit = full || entry == S.spec_p[slot];         // block-uniform
    if (tid == 0 && hit && !unknown) {
        TileStatus *tst = &p.status[tile];
        unsigned long long mine = S.agg[slot][0];
        if (full) {
#pragma unroll
            for (int t = 1; t < NS; t++) mine = entry == (uint32_t)t ? S.agg[slot][t] : mine;
        }
        tst->exit = fapply(S.tile_f[slot], entry);
        tst->incl[0] = pre[0] + cfield(mine, 0);
        tst->incl[1] = pre[1] + cfield(mine, 1);
        tst->incl[2] = pre[2] + cfield(mine, 2);
        st_release(&tst->flag, p.epoch * 4 + (SPEC ? 3 : 2));
        S.tile_c = mine;
        if (tile == p.num_tiles - 1) {
            p.hdr->n_struct = pre[0] + cfield(mine, 0);
            p.hdr->n_terms = pre[1] + cfield(mine, 1);
            p.hdr->n_rows = pre[2] + cfield(mine, 2);
        }
    }
    const uint32_t s_in = fapply(L.excl, entry);
    if (p.states64) p.states64[(uint64_t)tile * kThreads + tid] = (uint8_t)s_in;
    uint64_t stm;
    unsigned long long c;
    if (!full && hit) {
        stm = L.stm;
        c = L.cv[0];
    } else {
        stm = structural_mask<D>(L.m, L.ls, s_in);
        if (!full) {
            c = (unsigned long long)__popcll(stm) | ((unsigned long long)__popcll(stm & L.m.nl) << 21);
        } else {
            c = L.cv[0];
#pragma unroll
            for (int t = 1; t < NS; t++) c = s_in == (uint32_t)t ? L.cv[t] : c;
        }
    }
    const uint64_t term = stm & L.m.nl;
    const unsigned long long ci = warp_scan_sum(c, lane);
    if (lane == 31) S.warp_c[warp] = ci;
    unsigned long long ce = ci - c;
    __syncthreads();
    if (warp == 0) {
        const unsigned long long wc = lane < kWarps ? S.warp_c[lane] : 0ull;
        const unsigned long long wi = warp_scan_sum(wc, lane);
        if (lane < kWarps) S.warp_c[lane] = wi - wc;
        if (SPEC && !hit && lane == kWarps - 1) {
            // wrong assumption: true exit and recount for the successors
            TileStatus *tst = &p.status[tile];
            tst->exit = fapply(S.tile_f[slot], entry);
            tst->agg[1] = wi;
            st_release(&tst->flag, p.epoch * 4 + 2);
            atomicAdd(&p.hdr->spec_repairs, 1ull);
        }
        if (SPEC && lane == kWarps - 1) S.tile_c = wi;
    }
    __syncthreads();
    if (SPEC && (!hit || unknown)) {
        // wait until every count before the tile is known, then publish
        const uint64_t t0 = globaltimer_ns();
        while (unknown) {
            if (__syncthreads_or(tid == 0 && (aborted(p.hdr) || globaltimer_ns() - t0 > kWaitNs))) {
                if (tid == 0) fail(p.hdr, ERR_TIMEOUT);
                break;
            }
            __nanosleep(128);
            uint32_t e2;
            lookback_cta<NS, SPEC>(p, S.lb, tile, e2, pre, unknown);
        }
        if (tid == 0) {
            const unsigned long long mine = S.tile_c;
            TileStatus *tst = &p.status[tile];
            if (hit) tst->exit = fapply(S.tile_f[slot], entry);
            tst->incl[0] = pre[0] + cfield(mine, 0);
            tst->incl[1] = pre[1] + cfield(mine, 1);
            tst->incl[2] = pre[2] + cfield(mine, 2);
            st_release(&tst->flag, p.epoch * 4 + 3);
            if (tile == p.num_tiles - 1) {
                p.hdr->n_struct = pre[0] + cfield(mine, 0);
                p.hdr->n_terms = pre[1] + cfield(mine, 1);
                p.hdr->n_rows = pre[2] + cfield(mine, 2);
            }
        }
        __syncthreads();
    }
    ce += S.warp_c[warp];
    // Stage the thread's structurals (tile offset, bit 15 = terminator). A
    // warp's threads are consecutive, so its entries are one contiguous run
    // of the staging list and the warp writes index, separators and ends
    // from it alone, coalesced, after a warp barrier.
    {
        uint32_t k = cfield(ce, 0);
        uint64_t mm = stm;
        while (mm) {
            const unsigned bpos = __ffsll((long long)mm) - 1;
            if (k < (uint32_t)kTile)
                S.stage[k] = (uint16_t)(tid * kThreadBytes + bpos) | (uint16_t)(((term >> bpos) & 1) << 15);
            k++;
            mm &= mm - 1;
        }
    }
    __syncwarp();
    {
        const unsigned long long cend = ce + c;  // the thread's inclusive counts
        const uint32_t k0 = cfield(__shfl_sync(0xffffffffu, ce, 0), 0);
        const uint32_t k1 = min(cfield(__shfl_sync(0xffffffffu, cend, 31), 0), (uint32_t)kTile);
        uint32_t t = cfield(__shfl_sync(0xffffffffu, ce, 0), 1);  // tile terminators before the chunk
        const uint32_t lt = (1u << lane) - 1u;
        const bool tape = p.seps || p.ends;
        for (uint32_t k = k0; k < k1; k += 32) {
            const uint32_t kk = k + lane;
            const bool in = kk < k1;
            const uint32_t e = in ? S.stage[kk] : 0u;
            const bool is_t = in && (e >> 15);
            const uint32_t bt = __ballot_sync(0xffffffffu, is_t);
            const uint64_t gs = (uint64_t)pre[0] + kk;                     // structural ordinal
            const uint64_t gt = (uint64_t)pre[1] + t + __popc(bt & lt);    // terminators before it
            const uint32_t pos = (uint32_t)(p.pos_base + vs + (e & 0x7FFFu));
            if (in && p.index && gs < p.index_cap) p.index[gs] = pos;
            if (in && tape) {
                const uint64_t gsep = gs - gt;  // separators before it
                if (is_t) {
                    if (p.ends && gt < p.ends_cap) p.ends[gt] = ((p.sep_base + gsep) << 32) | pos;
                } else if (p.seps && gsep < p.seps_cap) {
                    p.seps[gsep] = pos;
                }
            }
            t += __popc(bt);
        }
    }
}

template <int D, bool SPEC = false>
__global__ void __launch_bounds__(kThreads, 3) index_kernel(const __grid_constant__ Params p) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    SmemIx &S = *reinterpret_cast<SmemIx *>(smem_raw);
    const int tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_mbar_init();
        for (int s = 0; s < 2; s++) {
            const uint32_t t = blockIdx.x + (uint32_t)s * G;
            if (t < p.num_tiles) issue_tile_ix(p, t, S.buf[s], &S.bar[s]);
        }
    }
    __syncthreads();
    uint32_t phase[2] = {0, 0};
    LocalState prev;
    bool have_prev = false;
    uint32_t prev_tile = 0;
    for (uint32_t i = 0;; i++) {
        const uint32_t tile = blockIdx.x + i * G;
        const int s = i & 1;
        const bool has_cur = tile < p.num_tiles;
        LocalState cur;
        if (has_cur) {
            const bool ok = mbar_wait(&S.bar[s], phase[s], kWaitNs);
            // the abort flag (set by a CTA whose wait gave up) is read every
            // 16th tile: every wait is bounded, so a late exit only costs time
            if (__syncthreads_or(!ok || (tid == 0 && (i & 15) == 15 && aborted(p.hdr)))) {
                if (tid == 0) {
                    if (!ok) fail(p.hdr, ERR_TMA);
                    else if (tile + G < p.num_tiles) mbar_wait(&S.bar[s ^ 1], phase[s ^ 1], kWaitNs);
                }
                break;
            }
            phase[s] ^= 1;
            local_pass<D, SPEC>(p, S, tile, S.buf[s], cur, s);
            __syncthreads();  // buf[s] fully read
            if (tid == 0 && tile + 2 * G < p.num_tiles) {
                fence_proxy_async();
                issue_tile_ix(p, tile + 2 * G, S.buf[s], &S.bar[s]);
            }
        }
        if (have_prev) output_pass<D, SPEC>(p, S, prev_tile, prev, s ^ 1);
        if (!has_cur) break;
        prev = cur;
        prev_tile = tile;
        have_prev = true;
    }
}

// ===========================================================================
// Shard summaries (several GPUs over one file): every tile's aggregate
// (transfer function, counts per entry state) from a local pass alone, then
// their composition in tile order. Nothing waits on another CTA.
// ===========================================================================
struct ShardSummaryDev {
    uint32_t func;
    uint32_t pad;
    unsigned long long counts[4][3];  // per entry state: structurals, terminators, rows
};

template <int D>
__global__ void __launch_bounds__(kThreads) summary_tiles_kernel(const __grid_constant__ Params p) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    SmemIx &S = *reinterpret_cast<SmemIx *>(smem_raw);
    const int tid = threadIdx.x;
    for (uint32_t tile = blockIdx.x; tile < p.num_tiles; tile += gridDim.x) {
        // plain 16-byte loads of the bytes a bulk copy of the tile would bring
        const uint8_t *lo_full = p.abase + (uint64_t)tile * kTile - kPre;
        const uint8_t *lo = tile == 0 ? p.abase : lo_full;
        const uint8_t *end16 = p.abase + ((p.shift + p.len + 15) & ~15ull);
        const uint8_t *hi = lo_full + kPre + kTile;
        if (hi > end16) hi = end16;
        uint8_t *dst = S.buf[0];
        const uint32_t first = (uint32_t)(lo - lo_full), n16 = (uint32_t)(hi - lo) / 16;
        for (uint32_t i = tid; i < n16; i += kThreads)
            *reinterpret_cast<uint4 *>(dst + first + 16 * i) = reinterpret_cast<const uint4 *>(lo)[i];
        __syncthreads();
        LocalState L;
        local_pass<D, false, true>(p, S, tile, S.buf[0], L, 0);
        __syncthreads();
    }
}

constexpr int kSumThreads = 256;

// Compose the tile aggregates of one shard in order (one CTA): each thread
// folds a run of tiles, thread 0 folds the runs. With backslash escapes
// (NS == 4) the tiles' functions carry the escape bit through the zero
// padding after the last byte, which consumes it; the shard's exit escape
// bit comes from its trailing run of backslashes instead.
template <int NS>
__global__ void __launch_bounds__(kSumThreads) summary_reduce(const TileStatus *status, uint32_t tiles,
                                                       const uint8_t *data, uint64_t len, ShardSummaryDev *out) {
    __shared__ uint32_t sf[kSumThreads];
    __shared__ unsigned long long sc[kSumThreads][4][3];
    const int t = threadIdx.x;
    const uint32_t per = (tiles + kSumThreads - 1) / kSumThreads;
    uint32_t f = kIdentity;
    unsigned long long c[4][3] = {};
    for (uint32_t j = t * per; j < tiles && j < (uint32_t)(t + 1) * per; j++) {
        const uint32_t g = status[j].func;
        unsigned long long r[4][3];
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++) {
            const unsigned long long v = status[j].agg[fapply(f, s0)];
#pragma unroll
            for (int k = 0; k < 3; k++) r[s0][k] = c[s0][k] + cfield(v, k);
        }
#pragma unroll
        for (int s0 = 0; s0 < NS; s0++)
#pragma unroll
            for (int k = 0; k < 3; k++) c[s0][k] = r[s0][k];
        f = fcompose(f, g);
    }
    sf[t] = f;
#pragma unroll
    for (int s0 = 0; s0 < 4; s0++)
#pragma unroll
        for (int k = 0; k < 3; k++) sc[t][s0][k] = c[s0][k];
    __syncthreads();
    if (t == 0) {
        uint32_t af = kIdentity;
        unsigned long long ac[4][3] = {};
        for (int i = 0; i < kSumThreads; i++) {
            unsigned long long r[4][3];
            for (int s0 = 0; s0 < NS; s0++) {
                const uint32_t m = fapply(af, s0);
                for (int k = 0; k < 3; k++) r[s0][k] = ac[s0][k] + sc[i][m][k];
            }
            for (int s0 = 0; s0 < NS; s0++)
                for (int k = 0; k < 3; k++) ac[s0][k] = r[s0][k];
            af = fcompose(af, sf[i]);
        }
        if (NS == 4) {
            uint64_t k = 0;
            while (k < len && data[len - 1 - k] == '\\') k++;
            uint32_t fixed = 0;
            for (uint32_t s0 = 0; s0 < 4; s0++) {
                const uint32_t esc = k < len ? (uint32_t)(k & 1) : (uint32_t)((len + (s0 & 1)) & 1);
                fixed |= ((fapply(af, s0) & 2u) | esc) << (2 * s0);
            }
            af = fixed;
        }
        out->func = af;
        for (int s0 = 0; s0 < 4; s0++)
            for (int k = 0; k < 3; k++) out->counts[s0][k] = s0 < NS ? ac[s0][k] : 0ull;
    }
}

// Persistent kernel, launched cooperatively so every CTA is resident. CTA c
// takes tiles c, c + G, c + 2G, ... (G = grid size): each round of G
// consecutive tiles is in flight at once and every look-back waits only on
// tiles of the same or an earlier round, which resident CTAs are already
// processing. The bulk copy of a CTA's next tile is issued one round ahead.
template <int D, bool ROWS>
__global__ void __launch_bounds__(kThreads, 3) scan_kernel(const __grid_constant__ Params p) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    Smem<ROWS> &S = *reinterpret_cast<Smem<ROWS> *>(smem_raw);
    const int tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_mbar_init();
        for (int s = 0; s < 2; s++) {
            const uint32_t t = blockIdx.x + (uint32_t)s * G;
            if (t < p.num_tiles) issue_tile<ROWS>(p, t, S.buf[s], &S.bar[s]);
        }
    }
    __syncthreads();
    uint32_t phase[2] = {0, 0};
    int s = 0;
    for (uint32_t tile = blockIdx.x; tile < p.num_tiles; tile += G) {
        const bool ok = mbar_wait(&S.bar[s], phase[s], kWaitNs);
        // One decision for the whole CTA: a timed-out copy or an abort stops it.
        if (__syncthreads_or(!ok || (tid == 0 && aborted(p.hdr)))) {
            if (tid == 0) {
                if (!ok) fail(p.hdr, ERR_TMA);
                // never leave a bulk copy in flight into this CTA's shared memory
                else if (tile + G < p.num_tiles) mbar_wait(&S.bar[s ^ 1], phase[s ^ 1], kWaitNs);
            }
            break;
        }
        phase[s] ^= 1;
        process_tile<D, ROWS>(p, S, tile, S.buf[s]);
        __syncthreads();  // every read of buf[s] and S.* for this tile is done
        if (tid == 0) {
            const uint32_t t = tile + 2 * G;
            if (t < p.num_tiles) {
                fence_proxy_async();
                issue_tile<ROWS>(p, t, S.buf[s], &S.bar[s]);
            }
        }
        s ^= 1;
    }
}

}  // namespace falx

// ===========================================================================
// Host side.
// ===========================================================================
using namespace falx;

#include "context.h"

namespace {

int cuda_fail(cudaError_t e) {
    if (e == cudaSuccess) return FALX_OK;
    (void)cudaGetLastError();
    return FALX_ERR_CUDA;
}
#define FALX_CUDA(x)                         \
    do {                                     \
        cudaError_t e_ = (x);                \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)

template <int D>
int setup_spec_kernel(falx_ctx *c) {
    const void *fn = (const void *)index_kernel<D, true>;
    FALX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemIx)));
    int nb = 0;
    FALX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, sizeof(SmemIx)));
    c->blocks_per_sm_spec[D] = nb > 0 ? nb : 1;
    return FALX_OK;
}

template <int D>
int setup_pass_kernel(falx_ctx *c) {
    const void *fn = (const void *)index_pass_kernel<D, false>;
    FALX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(IxSmem)));
    FALX_CUDA(cudaFuncSetAttribute((const void *)index_pass_kernel<D, true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(IxSmem)));
    int nb = 0;
    FALX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kIxThreads, sizeof(IxSmem)));
    c->blocks_per_sm_pass[D] = nb > 0 ? nb : 1;
    return FALX_OK;
}

template <int D, bool ROWS>
int setup_kernel(falx_ctx *c) {
    const void *fn = ROWS ? (const void *)scan_kernel<D, true> : (const void *)index_kernel<D>;
    const size_t smem = ROWS ? sizeof(Smem<true>) : sizeof(SmemIx);
    FALX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    FALX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, smem));
    c->blocks_per_sm[D][ROWS] = nb > 0 ? nb : 1;
    return FALX_OK;
}

int ensure_status(falx_ctx *c, uint32_t tiles) {
    if (tiles <= c->status_cap && c->epoch < (1u << 28)) {
        c->epoch++;
        return FALX_OK;
    }
    if (tiles > c->status_cap) {
        if (c->status) cudaFree(c->status);
        if (c->astatus) cudaFree(c->astatus);
        c->status = nullptr;
        c->astatus = nullptr;
        uint32_t cap = tiles < 1024 ? 1024 : tiles + tiles / 4;
        FALX_CUDA(cudaMalloc(&c->status, sizeof(TileStatus) * (size_t)cap));
        FALX_CUDA(cudaMalloc(&c->astatus, sizeof(ArenaStatus) * (size_t)cap));
        c->status_cap = cap;
    }
    FALX_CUDA(cudaMemsetAsync(c->status, 0, sizeof(TileStatus) * (size_t)c->status_cap, c->stream));
    FALX_CUDA(cudaMemsetAsync(c->astatus, 0, sizeof(ArenaStatus) * (size_t)c->status_cap, c->stream));
    c->epoch = 1;
    return FALX_OK;
}

bool valid_dialect(int d) { return d >= FALX_CSV && d <= FALX_NDJSON; }

// Launch the scan over [data, data+len) with the outputs in `P` (device);
// the header (counts, error bits) is final once the stream reaches this point.
int launch_scan(falx_ctx *c, int dialect, bool rows, const uint8_t *data, uint64_t len, Params P, bool spec = false,
                bool keep_hdr = false) {
    uint64_t shift = (uint64_t)((uintptr_t)data & 15u);
    uint64_t tiles64 = (len + shift + kTile - 1) / kTile;
    uint32_t tiles = (uint32_t)tiles64;
    int rc = ensure_status(c, tiles);
    if (rc) return rc;
    if (!keep_hdr) FALX_CUDA(cudaMemsetAsync(c->hdr, 0, sizeof(DevHeader), c->stream));
    P.data = data;
    P.abase = data - shift;
    P.len = len;
    P.shift = (uint32_t)shift;
    P.num_tiles = tiles;
    P.epoch = c->epoch;
    P.status = c->status;
    P.astatus = c->astatus;
    P.hdr = c->hdr;
    P.halo = rows ? kHaloBytes : 0;
    const bool pass = !rows && !spec && !c->old_index;
    int nb = spec ? c->blocks_per_sm_spec[dialect] : pass ? c->blocks_per_sm_pass[dialect]
                                                         : c->blocks_per_sm[dialect][rows ? 1 : 0];
    if (c->ctas_per_sm > 0 && c->ctas_per_sm < nb) nb = c->ctas_per_sm;
    uint64_t grid = (uint64_t)c->sm_count * (uint64_t)nb;
    // the index pass takes its tiles in groups of kIxGroup
    const uint64_t units = pass ? (tiles + kIxGroup - 1) / kIxGroup : tiles;
    if (grid > units) grid = units;
    if (grid == 0) grid = 1;
#define FALX_LAUNCH(D)                                                                            \
    do {                                                                                          \
        void *args_[] = {(void *)&P};                                                             \
        if (rows)                                                                                 \
            err = cudaLaunchCooperativeKernel((const void *)scan_kernel<D, true>, dim3((unsigned)grid), \
                                              dim3(kThreads), args_, sizeof(Smem<true>), c->stream);     \
        else if (spec)                                                                            \
            err = cudaLaunchCooperativeKernel((const void *)index_kernel<D, true>, dim3((unsigned)grid), \
                                              dim3(kThreads), args_, sizeof(SmemIx), c->stream);         \
        else if (pass)                                                                            \
            err = cudaLaunchCooperativeKernel(P.seed_in ? (const void *)index_pass_kernel<D, true>        \
                                                        : (const void *)index_pass_kernel<D, false>,     \
                                              dim3((unsigned)grid), dim3(kIxThreads), args_,             \
                                              sizeof(IxSmem), c->stream);                                \
        else                                                                                      \
            err = cudaLaunchCooperativeKernel((const void *)index_kernel<D>, dim3((unsigned)grid),     \
                                              dim3(kThreads), args_, sizeof(SmemIx), c->stream);         \
    } while (0)
    cudaError_t err = cudaSuccess;
    switch (dialect) {
    case FALX_CSV: FALX_LAUNCH(D_CSV); break;
    case FALX_CSV_HASH: FALX_LAUNCH(D_CSV_HASH); break;
    case FALX_TSV: FALX_LAUNCH(D_TSV); break;
    case FALX_LOGFMT: FALX_LAUNCH(D_LOGFMT); break;
    default: FALX_LAUNCH(D_NDJSON); break;
    }
    FALX_CUDA(err);
#undef FALX_LAUNCH
    return FALX_OK;
}

// Header back to the host, then the call's error status.
int finish_scan(falx_ctx *c) {
    FALX_CUDA(cudaMemcpyAsync(c->hhdr, c->hdr, sizeof(DevHeader), cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    if (c->hhdr->error & ERR_TIMEOUT) return FALX_ERR_TIMEOUT;
    if (c->hhdr->error & ERR_TMA) return FALX_ERR_TIMEOUT;
    if (c->hhdr->error & ERR_ARENA) return FALX_ERR_OVERFLOW;
    return FALX_OK;
}

int run_scan(falx_ctx *c, int dialect, bool rows, const uint8_t *data, uint64_t len, Params P, bool spec = false) {
    const int rc = launch_scan(c, dialect, rows, data, len, P, spec);
    return rc ? rc : finish_scan(c);
}

int check_common(falx_ctx *c, int dialect, const void *data, uint64_t len) {
    if (!c || !valid_dialect(dialect)) return FALX_ERR_INVALID;
    if (len && !data) return FALX_ERR_INVALID;
    if (len >= (1ull << 32)) return FALX_ERR_INPUT_TOO_LARGE;
    return FALX_OK;
}

int validate_schema(const falx_schema *s, RowSpec &rs, uint64_t rows_cap, const falx_columns *cols) {
    if (s->ncols > FALX_MAX_COLUMNS) return FALX_ERR_INVALID;
    rs.ncols = (int)s->ncols;
    int nstr = 0;
    rs.max_field = 0;
    for (uint32_t k = 0; k < s->ncols; k++) {
        uint32_t ty = s->cols[k].type;
        if (ty > FALX_BYTES) return FALX_ERR_INVALID;
        rs.field[k] = s->cols[k].field;
        rs.type[k] = ty;
        if (s->cols[k].field + 1 > rs.max_field) rs.max_field = s->cols[k].field + 1;
        rs.str_slot[k] = -1;
        if (ty == FALX_STR) {
            if (nstr >= kMaxStr) return FALX_ERR_INVALID;
            rs.str_slot[k] = nstr++;
        }
        if (cols) {
            const falx_column_out &o = cols->cols[k];
            if (rows_cap && (!o.values || !o.valid)) return FALX_ERR_INVALID;
            if (ty == FALX_STR && o.str_cap && !o.str_data) return FALX_ERR_INVALID;
            rs.values[k] = o.values;
            rs.valid[k] = o.valid;
            rs.str_data[k] = o.str_data;
            rs.str_cap[k] = o.str_cap;
        }
    }
    rs.nstr = nstr;
    rs.rows_cap = rows_cap;
    return FALX_OK;
}

// Grow a device scratch buffer to `need` bytes (contents not kept).
int grow_scratch(void **p, uint64_t *cap, uint64_t need) {
    if (need <= *cap) return FALX_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const uint64_t want = need + need / 8;
    FALX_CUDA(cudaMalloc(p, want));
    *cap = want;
    return FALX_OK;
}

// Rows, field bytes and count / sum from the tape: the index kernel writes
// the tape (the caller's buffers when it gives them, else scratch), then
// columns_kernel decodes the records. The columns kernel reads the record
// counts on the device, so the host waits once, after both launches, except
// for host-buffer calls, which copy the index back while the columns kernel
// runs and so need its size first. A tape that outgrew its buffers is
// flagged by the columns kernel; both passes then run again with buffers of
// the exact size. P carries the caller's index and tape outputs; rs the
// columns and sinks.
template <int D, bool STATS>
int columns_grid(falx_ctx *c) {
    int &g = c->col_grid[D][STATS ? 1 : 0];
    if (!g) {
        const void *fn = (const void *)columns_kernel<D, STATS>;
        FALX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ColSmem)));
        int nb = 0;
        FALX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, sizeof(ColSmem)));
        g = c->sm_count * (nb > 0 ? nb : 1);
    }
    return FALX_OK;
}

int rows_two_pass(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, Params P) {
    const bool own = !P.seps || !P.ends;
    const RowSpec rs = P.rows;
    memset(&P.rows, 0, sizeof P.rows);
    if (c->pend_arrive) {
        P.arrive = c->pend_arrive;
        P.arrive_tag = c->pend_tag;
        P.chunk_tiles = c->pend_chunk_tiles;
        c->pend_arrive = nullptr;
    }
    c->last_n = 0;
    // tape scratch: a first guess from the input size, the exact size after
    // a pass that did not fit
    uint64_t want_seps = (len / 6 + 1024) * 4, want_ends = (len / 24 + 1024) * 8;
    for (int attempt = 0; attempt < 2; attempt++) {
        if (own) {
            int rc = grow_scratch((void **)&c->tape_seps, &c->tape_seps_cap, want_seps);
            if (!rc) rc = grow_scratch((void **)&c->tape_ends, &c->tape_ends_cap, want_ends);
            if (rc) return rc;
            P.seps = c->tape_seps;
            P.seps_cap = c->tape_seps_cap / 4;
            P.ends = c->tape_ends;
            P.ends_cap = c->tape_ends_cap / 8;
        }
        if (c->timing) FALX_CUDA(cudaEventRecord(c->ev[0], c->stream));
        int rc = launch_scan(c, dialect, false, data, len, P);
        if (rc) return rc;
        if (c->timing) FALX_CUDA(cudaEventRecord(c->ev[1], c->stream));
        if (c->host_index && P.index) {
            // host-buffer call: the index is final once the index kernel is
            // done; copy it back while the columns kernel runs
            rc = finish_scan(c);
            if (rc) return rc;
            const uint64_t n_struct = c->hhdr->n_struct;
            const uint64_t ni = n_struct < c->host_index_cap ? n_struct : c->host_index_cap;
            if (ni) FALX_CUDA(cudaMemcpyAsync(c->host_index, P.index, ni * 4, cudaMemcpyDeviceToHost, c->copy_stream));
            c->host_index_done = true;
        }
        ColParams cp;
        memset(&cp, 0, sizeof cp);
        cp.data = data;
        cp.shift = (uint32_t)((uintptr_t)data & 15u);
        cp.abase = data - cp.shift;
        cp.len = len;
        cp.seps = P.seps;
        cp.seps_cap = P.seps_cap;
        cp.ends = P.ends;
        cp.ends_cap = P.ends_cap;
        cp.hdr = c->hdr;
        cp.rows = rs;
        // look-back records for every block the tape's capacity allows,
        // tagged with a per-call epoch: cleared only when (re)allocated and
        // when the epoch wraps
        const uint64_t blocks = (P.ends_cap + 1 + kRecBlock - 1) / kRecBlock;
        if (blocks * sizeof(BlkStatus) > c->rec_sums_cap || c->col_epoch >= (1u << 29)) {
            rc = grow_scratch(&c->rec_sums, &c->rec_sums_cap, blocks * sizeof(BlkStatus));
            if (rc) return rc;
            FALX_CUDA(cudaMemsetAsync(c->rec_sums, 0, c->rec_sums_cap, c->stream));
            c->col_epoch = 0;
        }
        cp.status = static_cast<BlkStatus *>(c->rec_sums);
        cp.epoch = ++c->col_epoch;
        cp.wait_ns = kWaitNs;
        const size_t smem_cells = sizeof(ColSmem);
#define FALX_COLS(D)                                                                                       \
    do {                                                                                                   \
        rc = rs.want_stats ? columns_grid<D, true>(c) : columns_grid<D, false>(c);                         \
        if (rc) return rc;                                                                                 \
        unsigned grid_ = (unsigned)c->col_grid[D][rs.want_stats ? 1 : 0];                                  \
        if (c->stall_test_ns) {                                                                            \
            /* test hook: one CTA starting at record block 1, so its look-back                          \
               waits for a block 0 that never publishes and gives up after the                          \
               given limit */                                                                              \
            cp.blk0 = 1;                                                                                   \
            cp.wait_ns = c->stall_test_ns;                                                                 \
            grid_ = 1;                                                                                     \
        }                                                                                                  \
        if (rs.want_stats) columns_kernel<D, true><<<grid_, kThreads, smem_cells, c->stream>>>(cp);       \
        else columns_kernel<D, false><<<grid_, kThreads, smem_cells, c->stream>>>(cp);                    \
    } while (0)
        switch (dialect) {
        case FALX_CSV: FALX_COLS(D_CSV); break;
        case FALX_CSV_HASH: FALX_COLS(D_CSV_HASH); break;
        case FALX_TSV: FALX_COLS(D_TSV); break;
        default: FALX_COLS(D_LOGFMT); break;
        }
#undef FALX_COLS
        FALX_CUDA(cudaGetLastError());
        if (c->timing) FALX_CUDA(cudaEventRecord(c->ev[2], c->stream));
        FALX_CUDA(cudaMemcpyAsync(c->hhdr, c->hdr, sizeof(DevHeader), cudaMemcpyDeviceToHost, c->stream));
        FALX_CUDA(cudaStreamSynchronize(c->stream));
        if (c->hhdr->error & (ERR_TIMEOUT | ERR_TMA)) return FALX_ERR_TIMEOUT;
        if (!(c->hhdr->error & ERR_TAPE)) break;
        if (!own || attempt == 1) return FALX_ERR_CAPACITY;  // the caller's tape buffers are too small
        // the tape did not fit the scratch: size it exactly and run again
        const uint64_t n_struct = c->hhdr->n_struct, n_terms = c->hhdr->n_terms;
        want_seps = (n_struct - n_terms + 1) * 4;
        want_ends = (n_terms + 1) * 8;
        P.arrive = nullptr;  // the input is in place now
        c->host_index_done = false;
        for (int k = 0; k < rs.ncols; k++) {
            const uint64_t words = (rs.rows_cap + 63) / 64;
            if (words) FALX_CUDA(cudaMemsetAsync(rs.valid[k], 0, words * 8, c->stream));
        }
    }
    if (c->timing) {
        for (int k = 0; k < 2; k++) cudaEventElapsedTime(&c->last_ms[k], c->ev[k], c->ev[k + 1]);
        c->last_n = 2;
    }
    for (int k = 0; k < kMaxStr; k++)
        if (c->hhdr->arena[k] > 0x7FFFFFFFull) return FALX_ERR_OVERFLOW;  // i32 string offsets
    return FALX_OK;
}

// Chunk k of a pipelined call is done: its seed record and totals stored to
// mapped host memory (one warp).
__global__ void pipe_publish_kernel(const SeedRec *seed, const unsigned long long *out, SeedRec *h_seed,
                                    unsigned long long *h_out) {
    const int t = threadIdx.x;
    if (t == 0) {
        h_seed->error = seed->error;
        h_seed->exit_state = seed->exit_state;
        h_seed->n_struct = seed->n_struct;
        h_seed->n_terms = seed->n_terms;
    }
    if (t < 6) h_out[t] = out[t];
}

// Host buffers of a pipelined falx_parse_host call.
struct HostPipe {
    const uint8_t *in;      // the input (host); NULL: already in device memory (inflated bgzf)
    const falx_outputs *ho;  // the caller's host outputs
    const falx_schema *schema;
};

constexpr int kPipeChunks = 16;                    // at most
constexpr uint64_t kPipeFirstBytes = 16ull << 20;  // the first and last chunks
constexpr uint64_t kPipeChunkBytes = 96ull << 20;  // the middle chunks, about
constexpr int kPipeRetry = 1;  // the tape outgrew its scratch: run the whole-input path instead

// Rows of a host-buffer call as a pipeline over input chunks of whole tiles
// (ramping from kPipeFirstBytes up to about kPipeChunkBytes and back down,
// at most kPipeChunks): copy stream H2D chunk k; compute stream: index pass
// over chunk k seeded from chunk k - 1's exit state and counts (device
// records, no host round trip), columns kernel over the record blocks that
// end inside chunks 0..k; out stream: chunk k's index, tape, column values,
// offsets, arena and full validity words copied back once the host sees
// chunk k's totals. The tape and the look-back records of the columns pass
// are shared by all launches, so outputs are those of one whole-input call.
int rows_pipelined(falx_ctx *c, int dialect, const uint8_t *dev_in, uint64_t len, Params P, const HostPipe &hp) {
    const RowSpec rs = P.rows;
    memset(&P.rows, 0, sizeof P.rows);
    c->last_n = 0;
    const falx_outputs *ho = hp.ho;
    const falx_columns *hc = ho->columns;
    if (!c->copy_stream) FALX_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    if (!c->out_stream) FALX_CUDA(cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking));
    if (!c->in_free) FALX_CUDA(cudaEventCreateWithFlags(&c->in_free, cudaEventDisableTiming));
    for (int k = 0; k < 2 * kPipeChunks; k++)
        if (!c->pipe_ev[k]) FALX_CUDA(cudaEventCreateWithFlags(&c->pipe_ev[k], cudaEventDisableTiming));
    // device: seed records (kPipeChunks + 1) | tickets | per-chunk totals 6 u64 each
    static_assert(offsetof(DevHeader, error) == 8 && offsetof(DevHeader, exit_state) == 12 &&
                      offsetof(DevHeader, n_struct) == 16 && offsetof(DevHeader, n_terms) == 24,
                  "a seed record is bytes [8, 32) of the header");
    constexpr size_t kSeedB = (kPipeChunks + 1) * sizeof(SeedRec), kTickOff = 416, kOutB = kPipeChunks * 6 * 8;
    constexpr size_t kPipeB = 512 + kOutB;
    static_assert(kSeedB <= kTickOff && kTickOff + kPipeChunks * 4 <= 512, "pipeline records");
    if (!c->pipe_dev) FALX_CUDA(cudaMalloc(&c->pipe_dev, kPipeB));
    if (!c->pipe_host) FALX_CUDA(cudaHostAlloc(&c->pipe_host, kPipeB, cudaHostAllocMapped));
    SeedRec *seeds = reinterpret_cast<SeedRec *>(c->pipe_dev);
    uint32_t *tickets = reinterpret_cast<uint32_t *>(reinterpret_cast<uint8_t *>(c->pipe_dev) + kTickOff);
    unsigned long long *chunk_out = reinterpret_cast<unsigned long long *>(reinterpret_cast<uint8_t *>(c->pipe_dev) + 512);
    const volatile SeedRec *h_seeds = reinterpret_cast<const volatile SeedRec *>(c->pipe_host);
    const volatile unsigned long long *h_out = c->pipe_host + 64;
    // the same host records as the kernels see them (mapped pinned memory)
    unsigned long long *host_map = nullptr;
    FALX_CUDA(cudaHostGetDevicePointer((void **)&host_map, c->pipe_host, 0));
    SeedRec *host_seeds = reinterpret_cast<SeedRec *>(host_map);
    unsigned long long *host_out = host_map + 64;
    // chunks of whole tiles (the device input is 256-byte aligned)
    const uint64_t tiles = (len + kTile - 1) / kTile;
    // Chunk sizes ramp up from kPipeFirstBytes (doubling) and back down at
    // the end, with chunks of about kPipeChunkBytes between: the first
    // outputs start back early and the last chunk's copies are short, so
    // little of the transfer time falls outside the full pipeline.
    uint64_t bounds[kPipeChunks + 1];
    int nk = 0;
    {
        uint64_t ramp[4];
        int nr = 0;
        uint64_t sum = 0;
        for (uint64_t step = kPipeFirstBytes / kTile; nr < 4 && step < kPipeChunkBytes / kTile &&
                                                      2 * (sum + step) <= tiles;
             step *= 2)
            ramp[nr++] = step, sum += step;
        const uint64_t mid = tiles - 2 * sum;
        uint64_t nm = mid ? (mid + kPipeChunkBytes / kTile - 1) / (kPipeChunkBytes / kTile) : 0;
        if (nm > (uint64_t)(kPipeChunks - 2 * nr)) nm = kPipeChunks - 2 * nr;
        uint64_t t = 0;
        bounds[0] = 0;
        for (int i = 0; i < nr; i++) bounds[++nk] = t += ramp[i];
        for (uint64_t i = 0; i < nm; i++) bounds[++nk] = t += mid / nm + (i < mid % nm ? 1 : 0);
        for (int i = nr - 1; i >= 0; i--) bounds[++nk] = t += ramp[i];
    }
    auto off = [&](int k) { return std::min(len, bounds[k] * kTile); };
    // tape scratch sized from the input; a tape that outgrows it sends the
    // call to the whole-input path
    const uint64_t want_seps = (len / 6 + 1024) * 4, want_ends = (len / 24 + 1024) * 8;
    int rc = grow_scratch((void **)&c->tape_seps, &c->tape_seps_cap, want_seps);
    if (!rc) rc = grow_scratch((void **)&c->tape_ends, &c->tape_ends_cap, want_ends);
    if (rc) return rc;
    P.seps = c->tape_seps;
    P.seps_cap = c->tape_seps_cap / 4;
    P.ends = c->tape_ends;
    P.ends_cap = c->tape_ends_cap / 8;
    const uint64_t blocks = (P.ends_cap + 1 + kRecBlock - 1) / kRecBlock;
    if (blocks * sizeof(BlkStatus) > c->rec_sums_cap || c->col_epoch >= (1u << 29)) {
        rc = grow_scratch(&c->rec_sums, &c->rec_sums_cap, blocks * sizeof(BlkStatus));
        if (rc) return rc;
        FALX_CUDA(cudaMemsetAsync(c->rec_sums, 0, c->rec_sums_cap, c->stream));
        c->col_epoch = 0;
    }
    const uint32_t col_epoch = ++c->col_epoch;
    FALX_CUDA(cudaMemsetAsync(c->hdr, 0, sizeof(DevHeader), c->stream));
    FALX_CUDA(cudaMemsetAsync(c->pipe_dev, 0, kPipeB, c->stream));
    if (hp.in) {
        // the input buffer is overwritten only after earlier work on the stream
        FALX_CUDA(cudaEventRecord(c->in_free, c->stream));
        FALX_CUDA(cudaStreamWaitEvent(c->copy_stream, c->in_free, 0));
        for (int k = 0; k < nk; k++) {
            FALX_CUDA(cudaMemcpyAsync(const_cast<uint8_t *>(dev_in) + off(k), hp.in + off(k), off(k + 1) - off(k),
                                      cudaMemcpyHostToDevice, c->copy_stream));
            FALX_CUDA(cudaEventRecord(c->pipe_ev[k], c->copy_stream));
        }
    }
    for (int k = 0; k < nk; k++) {
        if (hp.in) FALX_CUDA(cudaStreamWaitEvent(c->stream, c->pipe_ev[k], 0));
        Params Pk = P;
        Pk.seeded = k > 0;
        Pk.prev_byte = k > 0 && hp.in ? hp.in[off(k) - 1] : 0u;
        Pk.prev_ptr = k > 0 && !hp.in ? dev_in + off(k) - 1 : nullptr;
        Pk.entry0 = 0;
        Pk.pos_base = off(k);
        Pk.sep_base = 0;
        Pk.seed_in = k > 0 ? seeds + k : nullptr;
        Pk.seed_out = seeds + k + 1;  // where chunk k ends: its exit state and the totals through it
        rc = launch_scan(c, dialect, false, dev_in + off(k), off(k + 1) - off(k), Pk, false, true);
        if (rc) return rc;
        ColParams cp;
        memset(&cp, 0, sizeof cp);
        cp.data = dev_in;
        cp.abase = dev_in;
        cp.len = len;
        cp.seps = P.seps;
        cp.seps_cap = P.seps_cap;
        cp.ends = P.ends;
        cp.ends_cap = P.ends_cap;
        cp.hdr = c->hdr;
        cp.rows = rs;
        cp.status = static_cast<BlkStatus *>(c->rec_sums);
        cp.epoch = col_epoch;
        cp.wait_ns = kWaitNs;
        cp.seed_lo = k > 0 ? seeds + k : nullptr;
        cp.seed_hi = seeds + k + 1;
        cp.ticket = tickets + k;
        cp.chunk_out = chunk_out + 6 * k;
        cp.last = k == nk - 1;
#define FALX_COLS(D)                                                                                        \
    do {                                                                                                    \
        rc = rs.want_stats ? columns_grid<D, true>(c) : columns_grid<D, false>(c);                          \
        if (rc) return rc;                                                                                  \
        const unsigned grid_ = (unsigned)c->col_grid[D][rs.want_stats ? 1 : 0];                             \
        if (rs.want_stats) columns_kernel<D, true><<<grid_, kThreads, sizeof(ColSmem), c->stream>>>(cp);   \
        else columns_kernel<D, false><<<grid_, kThreads, sizeof(ColSmem), c->stream>>>(cp);                \
    } while (0)
        switch (dialect) {
        case FALX_CSV: FALX_COLS(D_CSV); break;
        case FALX_CSV_HASH: FALX_COLS(D_CSV_HASH); break;
        case FALX_TSV: FALX_COLS(D_TSV); break;
        default: FALX_COLS(D_LOGFMT); break;
        }
#undef FALX_COLS
        // chunk k's seed record and totals to the host by a store kernel (a
        // copy on this stream would queue behind the out stream's copies
        // back on the copy engine, and hold up the next chunk's kernels)
        pipe_publish_kernel<<<1, 32, 0, c->stream>>>(seeds + k + 1, chunk_out + 6 * k, host_seeds + k + 1,
                                                     host_out + 6 * k);
        FALX_CUDA(cudaGetLastError());
        FALX_CUDA(cudaEventRecord(c->pipe_ev[kPipeChunks + k], c->stream));
    }
    // copy each chunk's outputs back as soon as its totals are in
    uint64_t ps = 0, pt = 0, prow = 0, pw = 0, poff = 0, parena[kMaxStr] = {0, 0, 0, 0};
    auto back = [&](void *dst, const void *src, uint64_t bytes) -> int {
        if (bytes && dst) FALX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->out_stream));
        return FALX_OK;
    };
    auto clampu = [](uint64_t v, uint64_t cap) { return v < cap ? v : cap; };
    for (int k = 0; k < nk; k++) {
        FALX_CUDA(cudaEventSynchronize(c->pipe_ev[kPipeChunks + k]));
        const uint64_t s_k = h_seeds[k + 1].n_struct, t_k = h_seeds[k + 1].n_terms;
        const bool wrote = h_out[6 * k + 5] != 0;
        const uint64_t rows_k = wrote ? h_out[6 * k] : prow;
        uint64_t arena_k[kMaxStr];
        for (int j = 0; j < kMaxStr; j++) arena_k[j] = wrote ? h_out[6 * k + 1 + j] : parena[j];
        if (ho->index && P.index) {
            const uint64_t a = clampu(ps, ho->index_cap), b = clampu(s_k, ho->index_cap);
            if (b > a && (rc = back(ho->index + a, P.index + a, (b - a) * 4))) return rc;
        }
        if (ho->seps && ho->seps_cap) {
            const uint64_t a = clampu(ps - pt, ho->seps_cap), b = clampu(s_k - t_k, ho->seps_cap);
            if (b > a && (rc = back(ho->seps + a, P.seps + a, (b - a) * 4))) return rc;
        }
        if (ho->ends && ho->ends_cap) {
            const uint64_t a = clampu(pt, ho->ends_cap), b = clampu(t_k, ho->ends_cap);
            if (b > a && (rc = back(ho->ends + a, P.ends + a, (b - a) * 8))) return rc;
        }
        if (hc) {
            const uint64_t rcap = hc->rows_cap, wcap = (rcap + 63) / 64;
            const uint64_t wk = clampu(rows_k / 64, wcap);
            for (int j = 0; j < rs.ncols; j++) {
                const uint32_t ty = rs.type[j];
                const uint8_t *dv = static_cast<const uint8_t *>(rs.values[j]);
                uint8_t *hv = static_cast<uint8_t *>(hc->cols[j].values);
                if (ty == FALX_STR) {
                    // offsets [0, rows_k] are final once a row exists (offset 0
                    // is written by record block 0)
                    const uint64_t a = clampu(poff, rcap + 1), b = rows_k ? clampu(rows_k + 1, rcap + 1) : a;
                    if (b > a && (rc = back(hv + 4 * a, dv + 4 * a, (b - a) * 4))) return rc;
                    const int sl = rs.str_slot[j];
                    const uint64_t cap = hc->cols[j].str_cap;
                    const uint64_t x = clampu(parena[sl], cap), y = clampu(arena_k[sl], cap);
                    if (y > x && (rc = back(hc->cols[j].str_data + x, rs.str_data[j] + x, y - x))) return rc;
                } else {
                    const uint64_t es = ty == FALX_U32 ? 4 : 8;
                    const uint64_t a = clampu(prow, rcap), b = clampu(rows_k, rcap);
                    if (b > a && (rc = back(hv + es * a, dv + es * a, (b - a) * es))) return rc;
                }
                // validity words every fourth chunk (small copies cost the
                // copy engine about as much as large ones)
                if ((k & 3) == 3 && wk > pw && (rc = back(hc->cols[j].valid + pw, rs.valid[j] + pw, (wk - pw) * 8)))
                    return rc;
            }
            if ((k & 3) == 3) pw = wk > pw ? wk : pw;
            if (rows_k) poff = rows_k + 1;
        }
        ps = s_k;
        pt = t_k;
        prow = rows_k;
        for (int j = 0; j < kMaxStr; j++) parena[j] = arena_k[j];
    }
    // the header (totals, errors), then the validity words not yet copied
    FALX_CUDA(cudaMemcpyAsync(c->hhdr, c->hdr, sizeof(DevHeader), cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    if (c->hhdr->error & (ERR_TIMEOUT | ERR_TMA)) {
        FALX_CUDA(cudaStreamSynchronize(c->out_stream));
        return FALX_ERR_TIMEOUT;
    }
    if (c->hhdr->error & ERR_TAPE) {
        FALX_CUDA(cudaStreamSynchronize(c->out_stream));
        return kPipeRetry;
    }
    if (hc) {
        const uint64_t wcap = (hc->rows_cap + 63) / 64;
        const uint64_t wend = clampu((c->hhdr->n_rows + 63) / 64, wcap);
        for (int j = 0; j < rs.ncols; j++) {
            if (wend > pw && (rc = back(hc->cols[j].valid + pw, rs.valid[j] + pw, (wend - pw) * 8))) return rc;
            // no rows at all: the string offsets array is the one 0
            if (rs.type[j] == FALX_STR && poff == 0 && hc->rows_cap + 1 > 0 &&
                (rc = back(hc->cols[j].values, rs.values[j], 4)))
                return rc;
        }
    }
    FALX_CUDA(cudaStreamSynchronize(c->out_stream));
    c->pipe_done = true;
    for (int k = 0; k < kMaxStr; k++)
        if (c->hhdr->arena[k] > 0x7FFFFFFFull) return FALX_ERR_OVERFLOW;  // i32 string offsets
    return FALX_OK;
}

// text_field: the City text lane's field (with o->stats: lat / lon), or
// negative for none.
int parse_device(falx_ctx *c, const falx_schema *schema, const uint8_t *data, uint64_t len, falx_outputs *o,
                 int64_t text_field = -1) {
    if (!schema || !o) return FALX_ERR_INVALID;
    int dialect = schema->dialect;
    int rc = check_common(c, dialect, data, len);
    if (rc) return rc;
    if (dialect == FALX_NDJSON && (o->columns || o->field_bytes || o->stats)) return FALX_ERR_INVALID;
    Params P;
    memset(&P, 0, sizeof P);
    P.index = o->index_cap ? o->index : nullptr;
    P.index_cap = o->index_cap;
    P.seps = o->seps_cap ? o->seps : nullptr;
    P.seps_cap = o->seps_cap;
    P.ends = o->ends_cap ? o->ends : nullptr;
    P.ends_cap = o->ends_cap;
    if ((o->index_cap && !o->index) || (o->seps_cap && !o->seps) || (o->ends_cap && !o->ends))
        return FALX_ERR_INVALID;
    bool rows = o->columns || o->field_bytes || o->stats;
    RowSpec &rs = P.rows;
    rs.ncols = 0;
    rs.nstr = 0;
    rs.max_field = 0;
    rs.rows_cap = 0;
    if (o->columns) {
        rc = validate_schema(schema, rs, o->columns->rows_cap, o->columns);
        if (rc) return rc;
        for (int k = 0; k < rs.ncols; k++) {
            uint64_t words = (o->columns->rows_cap + 63) / 64;
            if (words) FALX_CUDA(cudaMemsetAsync(rs.valid[k], 0, words * 8, c->stream));
        }
    }
    rs.want_fb = o->field_bytes != nullptr;
    rs.want_stats = o->stats != nullptr;
    rs.stats_field[0] = o->stats_fields[0];
    rs.stats_field[1] = o->stats_fields[1];
    if (rs.want_stats) {
        uint32_t mf = (o->stats_fields[0] > o->stats_fields[1] ? o->stats_fields[0] : o->stats_fields[1]) + 1;
        if (mf > rs.max_field) rs.max_field = mf;
    }
    rs.want_text = text_field >= 0 && rs.want_stats;
    rs.text_field = rs.want_text ? (uint32_t)text_field : 0u;
    if (rs.want_text && rs.text_field + 1 > rs.max_field) rs.max_field = rs.text_field + 1;
    o->n_index = o->n_seps = o->n_ends = 0;
    if (o->columns) o->columns->rows = 0;
    if (len == 0) {
        if (o->columns) {
            for (int k = 0; k < rs.ncols; k++) {
                o->columns->cols[k].str_len = 0;
                if (rs.type[k] == FALX_STR && o->columns->rows_cap + 1 > 0 && rs.values[k])
                    FALX_CUDA(cudaMemsetAsync(rs.values[k], 0, 4, c->stream));
            }
            FALX_CUDA(cudaStreamSynchronize(c->stream));
        }
        if (o->field_bytes) o->field_bytes->fields = o->field_bytes->bytes = 0;
        if (o->stats) memset(o->stats, 0, sizeof *o->stats);
        return FALX_OK;
    }
    if (rows && c->pipe) {
        rc = rows_pipelined(c, dialect, data, len, P, *static_cast<const HostPipe *>(c->pipe));
        if (rc == kPipeRetry) return rc;
    } else if (rows && (c->rows_path == 0 || rs.want_text)) {
        rc = rows_two_pass(c, dialect, data, len, P);
    } else {
        rc = run_scan(c, dialect, rows, data, len, P);
    }
    if (rc && rc != FALX_ERR_CAPACITY) return rc;  // on CAPACITY the counts are still reported
    const DevHeader &h = *c->hhdr;
    o->n_index = h.n_struct;
    o->n_ends = h.n_terms;
    o->n_seps = h.n_struct - h.n_terms;
    bool cap_err = (o->index_cap && h.n_struct > o->index_cap) || (o->ends_cap && o->n_ends > o->ends_cap) ||
                   (o->seps_cap && o->n_seps > o->seps_cap);
    if (o->columns) {
        o->columns->rows = h.n_rows;
        if (h.n_rows > o->columns->rows_cap) cap_err = true;
        for (int k = 0; k < rs.ncols; k++) {
            if (rs.str_slot[k] >= 0) {
                o->columns->cols[k].str_len = h.arena[rs.str_slot[k]];
                if (h.arena[rs.str_slot[k]] > o->columns->cols[k].str_cap) cap_err = true;
            } else {
                o->columns->cols[k].str_len = 0;
            }
        }
    }
    if (o->field_bytes) {
        o->field_bytes->fields = h.fb_fields;
        o->field_bytes->bytes = h.fb_bytes;
    }
    if (o->stats) {
        falx_geo_stats &s = *o->stats;
        s.records = h.st_records;
        for (int k = 0; k < 2; k++) {
            s.values[k] = h.st_values[k];
            s.checksum[k] = h.st_checksum[k];
            s.sum_e6[k] = (int64_t)h.st_sum_e6[k];
            s.inexact[k] = h.st_inexact[k];
            s.sum_f64[k] = (double)(int64_t)h.st_sum_e6[k] / 1e6;
        }
    }
    return cap_err || rc ? FALX_ERR_CAPACITY : FALX_OK;
}

}  // namespace

extern "C" {

const char *falx_strerror(int code) {
    switch (code) {
    case FALX_OK: return "ok";
    case FALX_ERR_INVALID: return "invalid argument";
    case FALX_ERR_CAPACITY: return "output capacity too small";
    case FALX_ERR_INPUT_TOO_LARGE: return "input must be shorter than 4 GiB";
    case FALX_ERR_SCHEMA: return "record outside the expected schema";
    case FALX_ERR_TIMEOUT: return "device-side wait gave up";
    case FALX_ERR_CUDA: return "CUDA runtime error";
    case FALX_ERR_OVERFLOW: return "string arena exceeds 2 GiB";
    case FALX_ERR_FORMAT: return "malformed bgzf stream or DEFLATE block";
    default: return "unknown error";
    }
}

int falx_create(int device, falx_ctx **out) {
    if (!out) return FALX_ERR_INVALID;
    *out = nullptr;
    FALX_CUDA(cudaSetDevice(device));
    falx_ctx *c = new (std::nothrow) falx_ctx;
    if (!c) return FALX_ERR_INVALID;
    c->device = device;
    if (const char *e = getenv("FALX_CTAS_PER_SM")) c->ctas_per_sm = atoi(e);
    if (const char *e = getenv("FALX_INDEX_KERNEL")) c->old_index = strcmp(e, "tile") == 0;
    int rc = FALX_OK;
    if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) rc = FALX_ERR_CUDA;
#define FALX_SETUP(D)                                  \
    if (!rc) rc = setup_kernel<D, false>(c);           \
    if (!rc) rc = setup_kernel<D, true>(c);            \
    if (!rc) rc = setup_spec_kernel<D>(c);             \
    if (!rc) rc = setup_pass_kernel<D>(c);
    FALX_SETUP(D_CSV) FALX_SETUP(D_CSV_HASH) FALX_SETUP(D_TSV) FALX_SETUP(D_LOGFMT) FALX_SETUP(D_NDJSON)
#undef FALX_SETUP
    if (!rc && cudaMalloc(&c->hdr, sizeof(DevHeader)) != cudaSuccess) rc = FALX_ERR_CUDA;
    if (!rc && cudaMallocHost(&c->hhdr, sizeof(DevHeader)) != cudaSuccess) rc = FALX_ERR_CUDA;
    if (!rc) rc = ndjson_setup(c->device);
    if (!rc && cudaMalloc(&c->nd_acc, sizeof(NdjsonAcc)) != cudaSuccess) rc = FALX_ERR_CUDA;
    if (!rc && cudaMallocHost(&c->nd_host, sizeof(NdjsonAcc)) != cudaSuccess) rc = FALX_ERR_CUDA;
    if (rc) {
        falx_destroy(c);
        (void)cudaGetLastError();
        return rc;
    }
    *out = c;
    return FALX_OK;
}

void falx_destroy(falx_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->status) cudaFree(c->status);
    if (c->astatus) cudaFree(c->astatus);
    if (c->hdr) cudaFree(c->hdr);
    if (c->hhdr) cudaFreeHost(c->hhdr);
    if (c->dev_in) cudaFree(c->dev_in);
    if (c->dev_out) cudaFree(c->dev_out);
    if (c->nd_acc) cudaFree(c->nd_acc);
    if (c->nd_host) cudaFreeHost(c->nd_host);
    if (c->mlp_scratch) cudaFree(c->mlp_scratch);
    if (c->pred) cudaFree(c->pred);
    if (c->summary_dev) cudaFree(c->summary_dev);
    if (c->tape_seps) cudaFree(c->tape_seps);
    if (c->tape_ends) cudaFree(c->tape_ends);
    if (c->rec_sums) cudaFree(c->rec_sums);
    if (c->gz_scratch) cudaFree(c->gz_scratch);
    if (c->gz_comp) cudaFree(c->gz_comp);
    if (c->gz_host) cudaFreeHost(c->gz_host);
    if (c->pipe_dev) cudaFree(c->pipe_dev);
    if (c->pipe_host) cudaFreeHost(c->pipe_host);
    if (c->out_stream) cudaStreamDestroy(c->out_stream);
    for (int k = 0; k < 32; k++)
        if (c->pipe_ev[k]) cudaEventDestroy(c->pipe_ev[k]);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->arrive) cudaFree(c->arrive);
    if (c->in_free) cudaEventDestroy(c->in_free);
    for (int k = 0; k < 5; k++)
        if (c->ev[k]) cudaEventDestroy(c->ev[k]);
    delete c;
}

int falx_set_option(falx_ctx *c, int option, int value) {
    if (!c) return FALX_ERR_INVALID;
    switch (option) {
    case FALX_OPT_ROWS_PATH:
        if (value != 0 && value != 1) return FALX_ERR_INVALID;
        c->rows_path = value;
        return FALX_OK;
    case FALX_OPT_CTAS_PER_SM:
        if (value < 0) return FALX_ERR_INVALID;
        c->ctas_per_sm = value;
        return FALX_OK;
    case FALX_OPT_PIPELINE:
        if (value != 0 && value != 1) return FALX_ERR_INVALID;
        c->pipeline = value;
        return FALX_OK;
    case FALX_OPT_TIMING:
        if (value && !c->ev[0])
            for (int k = 0; k < 5; k++) FALX_CUDA(cudaEventCreate(&c->ev[k]));
        c->timing = value != 0;
        return FALX_OK;
    default:
        return FALX_ERR_INVALID;
    }
}

int falx_test_stalled_lookback(falx_ctx *c, const falx_schema *schema, const uint8_t *data, uint64_t len,
                                falx_columns *out, uint64_t wait_ns) {
    if (!c || !schema || !out || !wait_ns) return FALX_ERR_INVALID;
    c->stall_test_ns = wait_ns;
    const int rc = falx_parse_columns(c, schema, data, len, out);
    c->stall_test_ns = 0;
    return rc;
}

int falx_last_timings(const falx_ctx *c, float *ms, int n) {
    if (!c || (n && !ms)) return FALX_ERR_INVALID;
    for (int k = 0; k < n && k < c->last_n; k++) ms[k] = c->last_ms[k];
    return c->last_n;
}

int falx_set_stream(falx_ctx *c, void *stream) {
    if (!c) return FALX_ERR_INVALID;
    c->stream = (cudaStream_t)stream;
    return FALX_OK;
}

int falx_index_structurals(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, uint32_t *out,
                           uint64_t cap, uint64_t *n_out) {
    if (!n_out) return FALX_ERR_INVALID;
    falx_schema s;
    memset(&s, 0, sizeof s);
    s.dialect = dialect;
    falx_outputs o;
    memset(&o, 0, sizeof o);
    o.index = out;
    o.index_cap = cap;
    int rc = parse_device(c, &s, data, len, &o);
    *n_out = o.n_index;
    if (!rc && !cap && o.n_index) rc = FALX_ERR_CAPACITY;
    return rc;
}

int falx_parse_tape(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, uint32_t *seps,
                    uint64_t seps_cap, uint64_t *ends, uint64_t ends_cap, uint64_t *n_seps, uint64_t *n_ends) {
    if (!n_seps || !n_ends) return FALX_ERR_INVALID;
    falx_schema s;
    memset(&s, 0, sizeof s);
    s.dialect = dialect;
    falx_outputs o;
    memset(&o, 0, sizeof o);
    o.seps = seps;
    o.seps_cap = seps_cap;
    o.ends = ends;
    o.ends_cap = ends_cap;
    // Counts come from the structural scan even when a capacity is zero.
    int rc = parse_device(c, &s, data, len, &o);
    *n_seps = o.n_seps;
    *n_ends = o.n_ends;
    if (!rc && ((!seps_cap && o.n_seps) || (!ends_cap && o.n_ends))) rc = FALX_ERR_CAPACITY;
    return rc;
}

int falx_parse_columns(falx_ctx *c, const falx_schema *schema, const uint8_t *data, uint64_t len,
                       falx_columns *out) {
    if (!schema || !out) return FALX_ERR_INVALID;
    falx_outputs o;
    memset(&o, 0, sizeof o);
    o.columns = out;
    return parse_device(c, schema, data, len, &o);
}

int falx_stats_count_sum(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, uint32_t field0,
                         uint32_t field1, falx_geo_stats *out) {
    if (!out) return FALX_ERR_INVALID;
    falx_schema s;
    memset(&s, 0, sizeof s);
    s.dialect = dialect;
    falx_outputs o;
    memset(&o, 0, sizeof o);
    o.stats = out;
    o.stats_fields[0] = field0;
    o.stats_fields[1] = field1;
    return parse_device(c, &s, data, len, &o);
}

int falx_csv_geo_text_stats(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, uint32_t city_field,
                            uint32_t lat_field, uint32_t lon_field, falx_geo_text_stats *out) {
    if (!out || dialect == FALX_NDJSON) return FALX_ERR_INVALID;
    falx_schema s;
    memset(&s, 0, sizeof s);
    s.dialect = dialect;
    falx_geo_stats st;
    falx_outputs o;
    memset(&o, 0, sizeof o);
    o.stats = &st;
    o.stats_fields[0] = lat_field;
    o.stats_fields[1] = lon_field;
    memset(out, 0, sizeof *out);
    const int rc = parse_device(c, &s, data, len, &o, (int64_t)city_field);
    if (rc) return rc;
    out->records = st.records;
    out->city_values = len ? c->hhdr->st_text[0] : 0;
    out->city_bytes = len ? c->hhdr->st_text[1] : 0;
    out->city_checksum = len ? c->hhdr->st_text[2] : 0;
    out->latitude_values = st.values[0];
    out->longitude_values = st.values[1];
    out->latitude_checksum = st.checksum[0];
    out->longitude_checksum = st.checksum[1];
    return FALX_OK;
}

int falx_field_bytes(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, falx_field_byte_stats *out) {
    if (!out) return FALX_ERR_INVALID;
    falx_schema s;
    memset(&s, 0, sizeof s);
    s.dialect = dialect;
    falx_outputs o;
    memset(&o, 0, sizeof o);
    o.field_bytes = out;
    return parse_device(c, &s, data, len, &o);
}

int falx_parse(falx_ctx *c, const falx_schema *schema, const uint8_t *data, uint64_t len, falx_outputs *out) {
    return parse_device(c, schema, data, len, out);
}

int falx_ndjson_id_score(falx_ctx *c, const uint8_t *data, uint64_t len, falx_ndjson_stats *out) {
    if (!c || !out) return FALX_ERR_INVALID;
    if (len && !data) return FALX_ERR_INVALID;
    if (len >= (1ull << 32)) return FALX_ERR_INPUT_TOO_LARGE;
    FALX_CUDA(cudaSetDevice(c->device));
    return ndjson_run(data, len, out, c->nd_acc, c->nd_host, c->stream);
}

static int grow(void **p, uint64_t *cap, uint64_t need) {
    if (need <= *cap) return FALX_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    uint64_t n = need + need / 8 + 4096;
    FALX_CUDA(cudaMalloc(p, n));
    *cap = n;
    return FALX_OK;
}

int falx_index_structurals_host(falx_ctx *c, int dialect, const uint8_t *host_data, uint64_t len,
                                uint32_t *host_out, uint64_t cap, uint64_t *n_out) {
    if (!c || !n_out || (len && !host_data) || (cap && !host_out)) return FALX_ERR_INVALID;
    FALX_CUDA(cudaSetDevice(c->device));
    int rc = grow((void **)&c->dev_in, &c->dev_in_cap, len);
    if (rc) return rc;
    rc = grow(&c->dev_out, &c->dev_out_cap, cap * 4);
    if (rc) return rc;
    if (len) FALX_CUDA(cudaMemcpyAsync(c->dev_in, host_data, len, cudaMemcpyHostToDevice, c->stream));
    rc = falx_index_structurals(c, dialect, c->dev_in, len, (uint32_t *)c->dev_out, cap, n_out);
    if (rc && rc != FALX_ERR_CAPACITY) return rc;
    uint64_t n = *n_out < cap ? *n_out : cap;
    if (n) FALX_CUDA(cudaMemcpyAsync(host_out, c->dev_out, n * 4, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    return rc;
}

// Host-buffer form of falx_parse: `host_out` holds HOST pointers (index,
// seps, ends, column buffers); they are staged through device buffers that
// the context owns and reuses across calls.
}  // extern "C"

namespace {
constexpr uint64_t kChunkedInMin = 64ull << 20;  // smaller inputs: one copy
constexpr uint32_t kMaxArriveChunks = 64;
constexpr uint32_t kArriveChunks = 8;
typedef int (*WriteValue32Fn)(void *stream, unsigned long long addr, unsigned int value, unsigned int flags);

// Copy host_data into c->dev_in as chunks on the copy stream, each followed
// by a flag write (cuStreamWriteValue32: the driver fences the copy before
// the write). Returns 1 when the chunks are queued and the first index
// launch should wait on them, 2 when the whole input is already on the
// device (a flag write failed and the rest was copied synchronously), 0
// when the caller should copy as usual.
// cuStreamWriteValue32 through the driver entry point (flags written by the
// copy stream after each chunk of input); false when it is not available.
bool write_value_ready(falx_ctx *c) {
    if (c->write_value_state == 0) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        c->write_value_state = -1;
        if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess && fn) {
            c->write_value = fn;
            c->write_value_state = 1;
        }
        cudaGetLastError();
    }
    return c->write_value_state == 1;
}

int start_chunked_input(falx_ctx *c, const uint8_t *host_data, uint64_t len) {
    if (!write_value_ready(c)) return 0;
    if (!c->copy_stream) FALX_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    if (!c->in_free) FALX_CUDA(cudaEventCreateWithFlags(&c->in_free, cudaEventDisableTiming));
    if (!c->arrive || c->arrive_tag >= 0x7FFFFFFFu) {
        if (!c->arrive) FALX_CUDA(cudaMalloc(&c->arrive, kMaxArriveChunks * sizeof(uint32_t)));
        FALX_CUDA(cudaMemsetAsync(c->arrive, 0, kMaxArriveChunks * sizeof(uint32_t), c->stream));
        c->arrive_tag = 0;
    }
    const uint32_t tag = ++c->arrive_tag;
    // the input buffer is overwritten only after earlier work on the stream
    FALX_CUDA(cudaEventRecord(c->in_free, c->stream));
    FALX_CUDA(cudaStreamWaitEvent(c->copy_stream, c->in_free, 0));
    const uint64_t tiles = (len + kTile - 1) / kTile;  // dev_in is 256-byte aligned: no shift
    const uint64_t ct = (tiles + kArriveChunks - 1) / kArriveChunks;
    const WriteValue32Fn wv = (WriteValue32Fn)c->write_value;
    for (uint32_t k = 0; k * ct < tiles; k++) {
        const uint64_t lo = (uint64_t)k * ct * kTile, hi = std::min(len, (uint64_t)(k + 1) * ct * kTile);
        FALX_CUDA(cudaMemcpyAsync(c->dev_in + lo, host_data + lo, hi - lo, cudaMemcpyHostToDevice, c->copy_stream));
        if (wv((void *)c->copy_stream, (unsigned long long)(uintptr_t)(c->arrive + k), tag, 0) != 0) {
            // no flag for this chunk: finish the copy before the kernel starts
            FALX_CUDA(cudaMemcpyAsync(c->dev_in + hi, host_data + hi, len - hi, cudaMemcpyHostToDevice,
                                      c->copy_stream));
            FALX_CUDA(cudaStreamSynchronize(c->copy_stream));
            c->write_value_state = -1;
            return 2;
        }
    }
    c->pend_arrive = c->arrive;
    c->pend_tag = tag;
    c->pend_chunk_tiles = (uint32_t)ct;
    return 1;
}
// A bgzf stream in host memory whose text is the input of a host-buffer
// parse (falx_parse_gz_host).
struct GzIn {
    const uint8_t *comp;
    uint64_t comp_len;
    const falx_gz_block *blocks;
    uint64_t n_blocks;
};

// The compressed stream in, then the inflate into c->dev_in; its failure
// count comes back to c->gz_host once it is done. (Copying the stream in
// chunks while the inflate kernel waited for each member's chunk measured
// slower: 50.5 against 44.5 ms to the end of the inflate for 1 GiB of text.)
int gz_input(falx_ctx *c, const GzIn &gz, uint64_t len) {
    int rc = grow((void **)&c->gz_comp, &c->gz_comp_cap, gz.comp_len);
    if (rc) return rc;
    if (!c->gz_host) FALX_CUDA(cudaHostAlloc(&c->gz_host, 64, cudaHostAllocDefault));
    if (gz.comp_len) FALX_CUDA(cudaMemcpyAsync(c->gz_comp, gz.comp, gz.comp_len, cudaMemcpyHostToDevice, c->stream));
    unsigned long long *counters = nullptr;
    int32_t *status = nullptr;
    rc = gz_launch(c, c->gz_comp, gz.comp_len, gz.blocks, gz.n_blocks, c->dev_in, len, &counters, &status);
    if (rc) return rc;
    FALX_CUDA(cudaMemcpyAsync(c->gz_host, counters, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    return FALX_OK;
}

// falx_parse_host, and falx_parse_gz_host (gz: the input is the text of a
// bgzf stream, inflated into device memory; host_data is NULL).
int parse_host_impl(falx_ctx *c, const falx_schema *schema, const uint8_t *host_data, uint64_t len,
                    falx_outputs *host_out, const GzIn *gz) {
    if (!c || !schema || !host_out || (len && !host_data && !gz)) return FALX_ERR_INVALID;
    FALX_CUDA(cudaSetDevice(c->device));
    const falx_columns *hc = host_out->columns;
    // Device layout: [index][seps][ends][per column: values | valid | str]
    uint64_t need = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t at = (need + 255) & ~255ull;
        need = at + bytes;
        return at;
    };
    uint64_t o_index = take(host_out->index_cap * 4), o_seps = take(host_out->seps_cap * 4),
             o_ends = take(host_out->ends_cap * 8);
    uint64_t o_vals[FALX_MAX_COLUMNS], o_valid[FALX_MAX_COLUMNS], o_str[FALX_MAX_COLUMNS];
    uint64_t vbytes[FALX_MAX_COLUMNS];
    if (hc) {
        if (schema->ncols > FALX_MAX_COLUMNS) return FALX_ERR_INVALID;
        for (uint32_t k = 0; k < schema->ncols; k++) {
            uint32_t ty = schema->cols[k].type;
            uint64_t rc_ = hc->rows_cap;
            vbytes[k] = ty == FALX_I64 || ty == FALX_F64 ? rc_ * 8 : ty == FALX_U32 ? rc_ * 4
                        : ty == FALX_BYTES ? rc_ * 8 : (rc_ + 1) * 4;
            o_vals[k] = take(vbytes[k]);
            o_valid[k] = take((rc_ + 63) / 64 * 8);
            o_str[k] = take(ty == FALX_STR ? hc->cols[k].str_cap : 0);
        }
    }
    int rc = grow((void **)&c->dev_in, &c->dev_in_cap, len);
    if (rc) return rc;
    rc = grow(&c->dev_out, &c->dev_out_cap, need);
    if (rc) return rc;
    uint8_t *dout = (uint8_t *)c->dev_out;
    if (gz) {
        rc = gz_input(c, *gz, len);
        if (rc) return rc;
    }
    // Large inputs on the default rows path: copy in chunks on the copy
    // stream and let the index kernel start on the first chunk.
    const bool rows_call = hc || host_out->field_bytes || host_out->stats;
    // columns over a large input: the pipelined form (copies in and out
    // overlap the parse, rows_pipelined)
    const bool pipelined = c->pipeline && hc && len >= kChunkedInMin && c->rows_path == 0 && !c->old_index &&
                           schema->dialect != FALX_NDJSON;
    bool chunked = false, copied = pipelined || gz;
    if (!copied && len >= kChunkedInMin && rows_call && c->rows_path == 0 && schema->dialect != FALX_NDJSON) {
        rc = start_chunked_input(c, host_data, len);
        if (rc < 0) return rc;
        chunked = rc == 1;
        copied = rc == 2;
    }
    if (len && !chunked && !copied) FALX_CUDA(cudaMemcpyAsync(c->dev_in, host_data, len, cudaMemcpyHostToDevice, c->stream));
    falx_outputs d = *host_out;
    falx_columns dc;
    if (host_out->index_cap) d.index = (uint32_t *)(dout + o_index);
    if (host_out->seps_cap) d.seps = (uint32_t *)(dout + o_seps);
    if (host_out->ends_cap) d.ends = (uint64_t *)(dout + o_ends);
    if (hc) {
        dc = *hc;
        for (uint32_t k = 0; k < schema->ncols; k++) {
            dc.cols[k].values = dout + o_vals[k];
            dc.cols[k].valid = (uint64_t *)(dout + o_valid[k]);
            dc.cols[k].str_data = schema->cols[k].type == FALX_STR ? dout + o_str[k] : nullptr;
        }
        d.columns = &dc;
    }
    if (!pipelined && host_out->index_cap && host_out->index && hc) {
        if (!c->copy_stream) FALX_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        c->host_index = host_out->index;
        c->host_index_cap = host_out->index_cap;
        c->host_index_done = false;
    }
    HostPipe hp{gz ? nullptr : host_data, host_out, schema};
    c->pipe = pipelined ? &hp : nullptr;
    c->pipe_done = false;
    rc = parse_device(c, schema, c->dev_in, len, &d);
    c->pipe = nullptr;
    if (rc == kPipeRetry) {
        // the tape outgrew the pipeline's scratch: the whole-input path on
        // the input already in device memory (it sizes the tape exactly)
        if (hc)
            for (uint32_t k = 0; k < schema->ncols; k++) dc.cols[k].str_len = 0;
        rc = parse_device(c, schema, c->dev_in, len, &d);
    }
    const bool pipe_done = c->pipe_done;
    c->pipe_done = false;
    const bool index_done = c->host_index_done;
    c->host_index = nullptr;
    c->host_index_done = false;
    // an early return inside parse_device leaves the chunk hand-off unused;
    // either way the copies from host_data end before this call returns
    c->pend_arrive = nullptr;
    if (index_done || chunked) FALX_CUDA(cudaStreamSynchronize(c->copy_stream));
    if (gz) {
        // a member that failed to inflate makes the text, and so every
        // output, undefined
        FALX_CUDA(cudaStreamSynchronize(c->stream));
        if (c->gz_host[0]) return FALX_ERR_FORMAT;
    }
    if (rc && rc != FALX_ERR_CAPACITY) return rc;
    auto back = [&](void *dst, const void *src, uint64_t bytes) -> int {
        if (bytes && dst) FALX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
        return FALX_OK;
    };
    int r2 = FALX_OK;
    uint64_t ni = d.n_index < host_out->index_cap ? d.n_index : host_out->index_cap;
    uint64_t ns = d.n_seps < host_out->seps_cap ? d.n_seps : host_out->seps_cap;
    uint64_t ne = d.n_ends < host_out->ends_cap ? d.n_ends : host_out->ends_cap;
    if (!pipe_done) {  // (the pipeline copied every output back chunk by chunk)
        if (!r2 && !index_done) r2 = back(host_out->index, d.index, ni * 4);
        if (!r2) r2 = back(host_out->seps, d.seps, ns * 4);
        if (!r2) r2 = back(host_out->ends, d.ends, ne * 8);
    }
    if (hc) {
        falx_columns *ho = host_out->columns;
        uint64_t rows = dc.rows < hc->rows_cap ? dc.rows : hc->rows_cap;
        for (uint32_t k = 0; k < schema->ncols && !r2; k++) {
            uint32_t ty = schema->cols[k].type;
            uint64_t vb = ty == FALX_I64 || ty == FALX_F64 || ty == FALX_BYTES ? rows * 8
                          : ty == FALX_U32 ? rows * 4 : (rows + 1) * 4;
            if (!pipe_done) {
                r2 = back(ho->cols[k].values, dc.cols[k].values, vb);
                if (!r2) r2 = back(ho->cols[k].valid, dc.cols[k].valid, (rows + 63) / 64 * 8);
                if (!r2 && ty == FALX_STR) {
                    uint64_t sl =
                        dc.cols[k].str_len < hc->cols[k].str_cap ? dc.cols[k].str_len : hc->cols[k].str_cap;
                    r2 = back(ho->cols[k].str_data, dc.cols[k].str_data, sl);
                }
            }
            ho->cols[k].str_len = dc.cols[k].str_len;
        }
        ho->rows = dc.rows;
    }
    if (!r2) FALX_CUDA(cudaStreamSynchronize(c->stream));
    host_out->n_index = d.n_index;
    host_out->n_seps = d.n_seps;
    host_out->n_ends = d.n_ends;
    return r2 ? r2 : rc;
}
}  // namespace

extern "C" {

int falx_parse_host(falx_ctx *c, const falx_schema *schema, const uint8_t *host_data, uint64_t len,
                    falx_outputs *host_out) {
    return parse_host_impl(c, schema, host_data, len, host_out, nullptr);
}

int falx_parse_gz_host(falx_ctx *c, const falx_schema *schema, const uint8_t *comp, uint64_t comp_len,
                       const falx_gz_block *blocks, uint64_t n_blocks, falx_outputs *host_out) {
    if (!c || !schema || !host_out || (comp_len && !comp) || (n_blocks && !blocks) || n_blocks > 0xFFFFFFFFull)
        return FALX_ERR_INVALID;
    // the blocks' texts lie end to end from 0 (as falx_bgzf_scan lists them)
    uint64_t len = 0;
    for (uint64_t k = 0; k < n_blocks; k++) {
        if (blocks[k].out_off != len) return FALX_ERR_INVALID;
        len += blocks[k].out_len;
    }
    if (len >= (1ull << 32)) return FALX_ERR_INPUT_TOO_LARGE;
    if (len == 0) {
        static const uint8_t none = 0;
        return parse_host_impl(c, schema, &none, 0, host_out, nullptr);
    }
    const GzIn gz{comp, comp_len, blocks, n_blocks};
    return parse_host_impl(c, schema, nullptr, len, host_out, &gz);
}

// ---------------------------------------------------------------------------
// Shards of one file (one per GPU): summary, then a seeded pass.
// ---------------------------------------------------------------------------
int falx_summarize_shard(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, int prev_byte,
                       falx_shard_summary *out) {
    int rc = check_common(c, dialect, data, len);
    if (rc) return rc;
    if (!out || prev_byte > 255) return FALX_ERR_INVALID;
    memset(out, 0, sizeof *out);
    static const uint32_t ns[5] = {2, 3, 1, 4, 4};
    out->states = ns[dialect];
    out->last_byte = -1;
    for (uint32_t s0 = 0; s0 < 4; s0++) out->exit[s0] = s0;
    if (len == 0) return FALX_OK;  // an empty shard passes every state through and counts nothing
    const uint64_t shift = (uint64_t)((uintptr_t)data & 15u);
    const uint32_t tiles = (uint32_t)((len + shift + kTile - 1) / kTile);
    rc = ensure_status(c, tiles);
    if (rc) return rc;
    if (!c->summary_dev) FALX_CUDA(cudaMalloc(&c->summary_dev, sizeof(ShardSummaryDev)));
    Params P;
    memset(&P, 0, sizeof P);
    P.data = data;
    P.abase = data - shift;
    P.len = len;
    P.shift = (uint32_t)shift;
    P.num_tiles = tiles;
    P.epoch = c->epoch;
    P.status = c->status;
    P.hdr = c->hdr;
    P.seeded = prev_byte >= 0;
    P.prev_byte = prev_byte >= 0 ? (uint32_t)prev_byte : 0u;
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)c->sm_count * 2);
    ShardSummaryDev *sd = static_cast<ShardSummaryDev *>(c->summary_dev);
#define FALX_SUMMARY(D)                                                                                     \
    do {                                                                                                    \
        FALX_CUDA(cudaFuncSetAttribute((const void *)summary_tiles_kernel<D>,                               \
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemIx)));  \
        summary_tiles_kernel<D><<<grid, kThreads, sizeof(SmemIx), c->stream>>>(P);                          \
        summary_reduce<NStates<D>::value><<<1, kSumThreads, 0, c->stream>>>(c->status, tiles, data, len, sd); \
    } while (0)
    switch (dialect) {
    case FALX_CSV: FALX_SUMMARY(D_CSV); break;
    case FALX_CSV_HASH: FALX_SUMMARY(D_CSV_HASH); break;
    case FALX_TSV: FALX_SUMMARY(D_TSV); break;
    case FALX_LOGFMT: FALX_SUMMARY(D_LOGFMT); break;
    default: FALX_SUMMARY(D_NDJSON); break;
    }
#undef FALX_SUMMARY
    FALX_CUDA(cudaGetLastError());
    ShardSummaryDev h;
    uint8_t last = 0;
    FALX_CUDA(cudaMemcpyAsync(&h, sd, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaMemcpyAsync(&last, data + len - 1, 1, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    for (uint32_t s0 = 0; s0 < out->states; s0++) {
        out->exit[s0] = (h.func >> (2 * s0)) & 3u;
        out->structurals[s0] = h.counts[s0][0];
        out->terminators[s0] = h.counts[s0][1];
        out->rows[s0] = h.counts[s0][2];
    }
    out->last_byte = last;
    return FALX_OK;
}

int falx_parse_tape_seeded(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, int prev_byte,
                           uint32_t entry_state, uint64_t pos_base, uint64_t sep_base, uint32_t *index,
                           uint64_t index_cap, uint32_t *seps, uint64_t seps_cap, uint64_t *ends, uint64_t ends_cap,
                           uint64_t *n_index, uint64_t *n_seps, uint64_t *n_ends) {
    int rc = check_common(c, dialect, data, len);
    if (rc) return rc;
    static const uint32_t ns[5] = {2, 3, 1, 4, 4};
    if (prev_byte > 255 || entry_state >= ns[dialect] || pos_base + len > (1ull << 32)) return FALX_ERR_INVALID;
    if ((index_cap && !index) || (seps_cap && !seps) || (ends_cap && !ends)) return FALX_ERR_INVALID;
    uint64_t ni = 0, nt = 0;
    if (len) {
        Params P;
        memset(&P, 0, sizeof P);
        P.index = index_cap ? index : nullptr;
        P.index_cap = index_cap;
        P.seps = seps_cap ? seps : nullptr;
        P.seps_cap = seps_cap;
        P.ends = ends_cap ? ends : nullptr;
        P.ends_cap = ends_cap;
        P.seeded = prev_byte >= 0;
        P.prev_byte = prev_byte >= 0 ? (uint32_t)prev_byte : 0u;
        P.entry0 = entry_state;
        P.pos_base = pos_base;
        P.sep_base = sep_base;
        rc = run_scan(c, dialect, false, data, len, P);
        if (rc) return rc;
        ni = c->hhdr->n_struct;
        nt = c->hhdr->n_terms;
    }
    if (n_index) *n_index = ni;
    if (n_seps) *n_seps = ni - nt;
    if (n_ends) *n_ends = nt;
    if ((index_cap && ni > index_cap) || (seps_cap && ni - nt > seps_cap) || (ends_cap && nt > ends_cap))
        return FALX_ERR_CAPACITY;
    return FALX_OK;
}

}  // extern "C"

// ===========================================================================
// Learned speculation: the entry-region predictor and the speculative index.
// ===========================================================================
struct falx_model {
    int device = 0;
    falx::mlp::Model m;
    float *grad = nullptr;  // gradient scratch [kParams]
    float *loss = nullptr;  // device scalar
    float min_prob = 0.f;   // tile predictions less likely than this assume nothing
};

namespace {

using namespace falx::mlp;

// Scratch for n samples: classes, activations, gradients.
struct MlpScratch {
    uint8_t *cls, *label;
    Acts a;
};

uint64_t mlp_bytes(uint64_t n) {
    auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
    return al(n * kPos) + al(n) + 4 * al(n * kHid * 4) + 2 * al(n * kHid * 2) + 2 * al(n * kOut * 4) + al(4);
}

int mlp_scratch(falx_ctx *c, uint64_t n, MlpScratch &s) {
    const uint64_t need = mlp_bytes(n);
    if (need > c->mlp_cap) {
        if (c->mlp_scratch) cudaFree(c->mlp_scratch);
        c->mlp_scratch = nullptr;
        c->mlp_cap = 0;
        FALX_CUDA(cudaMalloc(&c->mlp_scratch, need));
        c->mlp_cap = need;
    }
    uint8_t *p = c->mlp_scratch;
    auto take = [&](uint64_t b) {
        uint8_t *r = p;
        p += (b + 255) & ~255ull;
        return r;
    };
    s.cls = take(n * kPos);
    s.label = take(n);
    s.a.a1 = (float *)take(n * kHid * 4);
    s.a.a2 = (float *)take(n * kHid * 4);
    s.a.d2 = (float *)take(n * kHid * 4);
    s.a.d1 = (float *)take(n * kHid * 4);
    s.a.h1 = (__nv_bfloat16 *)take(n * kHid * 2);
    s.a.h2 = (__nv_bfloat16 *)take(n * kHid * 2);
    s.a.z = (float *)take(n * kOut * 4);
    s.a.dz = (float *)take(n * kOut * 4);
    s.a.loss = (float *)take(4);
    return FALX_OK;
}

unsigned blocks(uint64_t n, unsigned per) { return (unsigned)((n + per - 1) / per); }

int refresh(falx_ctx *c, falx_model *md) {
    refresh_bf16<<<blocks((uint64_t)kIn * kHid, 256), 256, 0, c->stream>>>(md->m.w, md->m.w1, md->m.w1t, md->m.w2,
                                                                          md->m.w2t, md->m.w3);
    return cuda_fail(cudaGetLastError());
}

// Forward pass of n samples whose classes are in `cls`; keeps the
// pre-activations when `train`.
int mlp_forward(falx_ctx *c, const falx_model *md, const uint8_t *cls, uint32_t n, Acts &a, bool train, uint8_t *pred) {
    if (n == 0) return FALX_OK;
    l1_forward<<<blocks(n, kL1Samples), kHid, 0, c->stream>>>(cls, n, md->m.w1, md->m.w + kOffB1,
                                                              train ? a.a1 : nullptr, a.h1);
    l2_forward<<<blocks(n, kL2Samples), kHid, 0, c->stream>>>(a.h1, n, md->m.w2, md->m.w + kOffB2,
                                                              train ? a.a2 : nullptr, a.h2);
    l3_forward<<<blocks((uint64_t)n * 32, 256), 256, 0, c->stream>>>(a.h2, n, md->m.w3, md->m.w + kOffB3, a.z, pred);
    return cuda_fail(cudaGetLastError());
}

// Inference on the tensor cores: samples are the 256 bytes at
// first + s * stride of `data`, or the classes in `cls`.
int mlp_infer(falx_ctx *c, const falx_model *md, const uint8_t *data, uint64_t len, int64_t first, int64_t stride,
              const uint8_t *cls, uint32_t n, Acts &a, float *z, uint8_t *pred, float min_prob) {
    if (n == 0) return FALX_OK;
    const unsigned grid = blocks(n, kMmaRows);
    mma_layer<true><<<grid, kMmaThreads, sizeof(MmaSmem), c->stream>>>(data, len, first, stride, cls, nullptr, n,
                                                                        md->m.w1t, md->m.w + kOffB1, a.h1);
    mma_layer<false><<<grid, kMmaThreads, sizeof(MmaSmem), c->stream>>>(nullptr, 0, 0, 0, nullptr, a.h1, n, md->m.w2t,
                                                                         md->m.w + kOffB2, a.h2);
    l3_forward<<<blocks((uint64_t)n * 32, 256), 256, 0, c->stream>>>(a.h2, n, md->m.w3, md->m.w + kOffB3, z, pred,
                                                                      min_prob);
    return cuda_fail(cudaGetLastError());
}

// Gradient of the mean cross-entropy of n labelled samples into g.
int mlp_grad(falx_ctx *c, const falx_model *md, const uint8_t *cls, const uint8_t *label, uint32_t n, Acts &a,
             float *g) {
    int rc = mlp_forward(c, md, cls, n, a, true, nullptr);
    if (rc) return rc;
    FALX_CUDA(cudaMemsetAsync(a.loss, 0, 4, c->stream));
    xent_kernel<<<blocks(n, 256), 256, 0, c->stream>>>(a.z, label, n, a.dz, a.loss);
    const unsigned g3 = n < 1024 ? n : 1024;
    l3_backward<<<g3, kHid, 0, c->stream>>>(a.h2, a.a2, a.dz, n, md->m.w3, g, a.d2);
    l2_wgrad<<<kHid, kHid, 0, c->stream>>>(a.h1, a.d2, n, g);
    l2_dgrad<<<blocks(n, kL2Samples), kHid, 0, c->stream>>>(a.d2, a.a1, n, md->m.w2t, a.d1);
    l1_wgrad<<<kPos, kHid, 0, c->stream>>>(cls, a.d1, n, g);
    return cuda_fail(cudaGetLastError());
}

// splitmix64 for the initial weights.
uint64_t mix64(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int tile_count(const uint8_t *data, uint64_t len, uint32_t &tiles, uint64_t &shift) {
    shift = (uint64_t)((uintptr_t)data & 15u);
    tiles = (uint32_t)((len + shift + kTile - 1) / kTile);
    return FALX_OK;
}

}  // namespace

extern "C" {

uint64_t falx_model_param_count(void) { return kParams; }

int falx_model_create(falx_ctx *c, uint64_t seed, falx_model **out) {
    if (!c || !out) return FALX_ERR_INVALID;
    *out = nullptr;
    FALX_CUDA(cudaSetDevice(c->device));
    falx_model *md = new (std::nothrow) falx_model;
    if (!md) return FALX_ERR_INVALID;
    md->device = c->device;
    float *host = (float *)calloc(kParams, sizeof(float));
    int rc = host ? FALX_OK : FALX_ERR_INVALID;
    if (!rc) {
        // uniform(-r, r) with r = sqrt(6 / active inputs); biases zero
        uint64_t x = seed;
        auto fill = [&](uint64_t off, uint64_t count, float r) {
            for (uint64_t i = 0; i < count; i++) {
                const double u = (double)(mix64(x) >> 11) * (1.0 / 9007199254740992.0);
                host[off + i] = (float)((2.0 * u - 1.0) * r);
            }
        };
        fill(kOffW1, (uint64_t)kIn * kHid, sqrtf(6.f / kPos));
        fill(kOffW2, (uint64_t)kHid * kHid, sqrtf(6.f / kHid));
        fill(kOffW3, (uint64_t)kHid * kOut, sqrtf(6.f / (kHid + kOut)));
    }
    auto alloc = [&](void **p, uint64_t b) {
        if (!rc && cudaMalloc(p, b) != cudaSuccess) rc = FALX_ERR_CUDA;
    };
    alloc((void **)&md->m.w, kParams * 4);
    alloc((void **)&md->m.m, kParams * 4);
    alloc((void **)&md->m.v, kParams * 4);
    alloc((void **)&md->grad, kParams * 4);
    alloc((void **)&md->loss, 4);
    alloc((void **)&md->m.w1, (uint64_t)kIn * kHid * 2);
    alloc((void **)&md->m.w1t, (uint64_t)kIn * kHid * 2);
    if (!rc && (cudaFuncSetAttribute((const void *)mma_layer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(MmaSmem)) != cudaSuccess ||
                cudaFuncSetAttribute((const void *)mma_layer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(MmaSmem)) != cudaSuccess))
        rc = FALX_ERR_CUDA;
    alloc((void **)&md->m.w2, (uint64_t)kHid * kHid * 2);
    alloc((void **)&md->m.w2t, (uint64_t)kHid * kHid * 2);
    alloc((void **)&md->m.w3, (uint64_t)kHid * kOut * 2);
    if (!rc && cudaMemcpyAsync(md->m.w, host, kParams * 4, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
        rc = FALX_ERR_CUDA;
    if (!rc && cudaMemsetAsync(md->m.m, 0, kParams * 4, c->stream) != cudaSuccess) rc = FALX_ERR_CUDA;
    if (!rc && cudaMemsetAsync(md->m.v, 0, kParams * 4, c->stream) != cudaSuccess) rc = FALX_ERR_CUDA;
    if (!rc) rc = refresh(c, md);
    if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = FALX_ERR_CUDA;
    free(host);
    if (rc) {
        falx_model_destroy(md);
        (void)cudaGetLastError();
        return rc;
    }
    *out = md;
    return FALX_OK;
}

void falx_model_destroy(falx_model *md) {
    if (!md) return;
    cudaSetDevice(md->device);
    void *ps[] = {md->m.w, md->m.m, md->m.v, md->grad, md->loss, md->m.w1, md->m.w1t, md->m.w2, md->m.w2t, md->m.w3};
    for (void *p : ps)
        if (p) cudaFree(p);
    delete md;
}

int falx_model_set_confidence(falx_model *md, float min_prob) {
    if (!md || !(min_prob >= 0.f && min_prob <= 1.f)) return FALX_ERR_INVALID;
    md->min_prob = min_prob;
    return FALX_OK;
}

int falx_model_get(falx_ctx *c, const falx_model *md, float *host, uint64_t n) {
    if (!c || !md || !host || n != kParams) return FALX_ERR_INVALID;
    FALX_CUDA(cudaMemcpyAsync(host, md->m.w, kParams * 4, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    return FALX_OK;
}

int falx_model_set(falx_ctx *c, falx_model *md, const float *host, uint64_t n) {
    if (!c || !md || !host || n != kParams) return FALX_ERR_INVALID;
    FALX_CUDA(cudaMemcpyAsync(md->m.w, host, kParams * 4, cudaMemcpyHostToDevice, c->stream));
    FALX_CUDA(cudaMemsetAsync(md->m.m, 0, kParams * 4, c->stream));
    FALX_CUDA(cudaMemsetAsync(md->m.v, 0, kParams * 4, c->stream));
    md->m.step = 0;
    int rc = refresh(c, md);
    if (rc) return rc;
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    return FALX_OK;
}

int falx_byte_classes(falx_ctx *c, const uint8_t *data, uint64_t len, const int64_t *starts, uint32_t n,
                      uint8_t *cls) {
    if (!c || (len && !data) || (n && (!starts || !cls))) return FALX_ERR_INVALID;
    if (n == 0) return FALX_OK;
    classes_kernel<<<blocks((uint64_t)n * kPos, 256), 256, 0, c->stream>>>(data, len, starts, 0, 0, n, cls);
    FALX_CUDA(cudaGetLastError());
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    return FALX_OK;
}

int falx_model_forward(falx_ctx *c, const falx_model *md, const uint8_t *cls, uint32_t n, float *logits,
                       uint8_t *pred) {
    if (!c || !md || (n && !cls) || ((uintptr_t)cls & 15)) return FALX_ERR_INVALID;
    MlpScratch s;
    int rc = mlp_scratch(c, n, s);
    if (rc) return rc;
    rc = mlp_infer(c, md, nullptr, 0, 0, 0, cls, n, s.a, s.a.z, pred, 0.f);
    if (rc) return rc;
    if (logits && n) FALX_CUDA(cudaMemcpyAsync(logits, s.a.z, (uint64_t)n * kOut * 4, cudaMemcpyDeviceToDevice,
                                               c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    return FALX_OK;
}

int falx_model_grad(falx_ctx *c, const falx_model *md, const uint8_t *cls, const uint8_t *labels, uint32_t n,
                    float *grad, float *loss) {
    if (!c || !md || !cls || !labels || !grad || n == 0) return FALX_ERR_INVALID;
    MlpScratch s;
    int rc = mlp_scratch(c, n, s);
    if (rc) return rc;
    rc = mlp_grad(c, md, cls, labels, n, s.a, grad);
    if (rc) return rc;
    float l = 0;
    FALX_CUDA(cudaMemcpyAsync(&l, s.a.loss, 4, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    if (loss) *loss = l;
    return FALX_OK;
}

int falx_model_train(falx_ctx *c, falx_model *md, const uint8_t *cls, const uint8_t *labels, uint64_t n,
                     uint32_t batch, uint32_t epochs, float lr, float *last_loss) {
    if (!c || !md || !cls || !labels || n == 0 || batch == 0) return FALX_ERR_INVALID;
    MlpScratch s;
    int rc = mlp_scratch(c, batch, s);
    if (rc) return rc;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float l = 0;
    for (uint32_t e = 0; e < epochs; e++) {
        for (uint64_t at = 0; at + batch <= n; at += batch) {
            rc = mlp_grad(c, md, cls + at * kPos, labels + at, batch, s.a, md->grad);
            if (rc) return rc;
            md->m.step++;
            const float c1 = 1.f - powf(b1, (float)md->m.step), c2 = 1.f - powf(b2, (float)md->m.step);
            adam_kernel<<<blocks(kParams, 256), 256, 0, c->stream>>>(md->m.w, md->m.m, md->m.v, md->grad, kParams,
                                                                      lr, b1, b2, eps, c1, c2);
            rc = refresh(c, md);
            if (rc) return rc;
        }
    }
    FALX_CUDA(cudaMemcpyAsync(&l, s.a.loss, 4, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    if (last_loss) *last_loss = l;
    return FALX_OK;
}

int falx_region_states(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len, uint8_t *states, uint64_t cap,
                       uint64_t *n_out) {
    int rc = check_common(c, dialect, data, len);
    if (rc) return rc;
    if (!n_out) return FALX_ERR_INVALID;
    uint32_t tiles;
    uint64_t shift;
    tile_count(data, len, tiles, shift);
    *n_out = (uint64_t)tiles * kThreads;
    if (len == 0) return FALX_OK;
    if (cap < *n_out || !states) return FALX_ERR_CAPACITY;
    Params P;
    memset(&P, 0, sizeof P);
    P.states64 = states;
    return run_scan(c, dialect, false, data, len, P);
}

int falx_predict_tiles(falx_ctx *c, const falx_model *md, const uint8_t *data, uint64_t len, uint8_t *pred,
                       uint64_t cap, uint64_t *n_tiles) {
    if (!c || !md || !n_tiles || (len && !data)) return FALX_ERR_INVALID;
    uint32_t tiles;
    uint64_t shift;
    tile_count(data, len, tiles, shift);
    *n_tiles = tiles;
    if (tiles == 0) return FALX_OK;
    if (cap < tiles || !pred) return FALX_ERR_CAPACITY;
    MlpScratch s;
    int rc = mlp_scratch(c, tiles, s);
    if (rc) return rc;
    rc = mlp_infer(c, md, data, len, -(int64_t)shift, kTile, nullptr, tiles, s.a, nullptr, pred, md->min_prob);
    if (rc) return rc;
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    return FALX_OK;
}

int falx_index_structurals_assumed(falx_ctx *c, int dialect, const uint8_t *data, uint64_t len,
                                   const uint8_t *assumed, uint32_t *out, uint64_t cap, uint64_t *n_out,
                                   falx_spec_stats *stats) {
    int rc = check_common(c, dialect, data, len);
    if (rc) return rc;
    if (!n_out || (cap && !out)) return FALX_ERR_INVALID;
    uint32_t tiles;
    uint64_t shift;
    tile_count(data, len, tiles, shift);
    *n_out = 0;
    if (stats) memset(stats, 0, sizeof *stats);
    if (len == 0) return FALX_OK;
    Params P;
    memset(&P, 0, sizeof P);
    P.index = cap ? out : nullptr;
    P.index_cap = cap;
    P.pred = assumed;
    rc = run_scan(c, dialect, false, data, len, P, true);
    if (rc) return rc;
    const DevHeader &h = *c->hhdr;
    *n_out = h.n_struct;
    if (stats) {
        stats->tiles = tiles;
        stats->mispredicted = h.spec_repairs;
    }
    if (h.n_struct > cap) return FALX_ERR_CAPACITY;
    return FALX_OK;
}

int falx_index_structurals_speculative(falx_ctx *c, const falx_model *md, int dialect, const uint8_t *data,
                                       uint64_t len, uint32_t *out, uint64_t cap, uint64_t *n_out,
                                       falx_spec_stats *stats) {
    int rc = check_common(c, dialect, data, len);
    if (rc) return rc;
    if (!n_out || (cap && !out)) return FALX_ERR_INVALID;
    uint32_t tiles;
    uint64_t shift;
    tile_count(data, len, tiles, shift);
    *n_out = 0;
    if (stats) memset(stats, 0, sizeof *stats);
    if (len == 0) return FALX_OK;
    Params P;
    memset(&P, 0, sizeof P);
    P.index = cap ? out : nullptr;
    P.index_cap = cap;
    if (md) {
        if (tiles > c->pred_cap) {
            if (c->pred) cudaFree(c->pred);
            c->pred = nullptr;
            c->pred_cap = 0;
            FALX_CUDA(cudaMalloc(&c->pred, tiles));
            c->pred_cap = tiles;
        }
        MlpScratch s;
        rc = mlp_scratch(c, tiles, s);
        if (rc) return rc;
        rc = mlp_infer(c, md, data, len, -(int64_t)shift, kTile, nullptr, tiles, s.a, nullptr, c->pred,
                       md->min_prob);
        if (rc) return rc;
        P.pred = c->pred;
    }
    rc = run_scan(c, dialect, false, data, len, P, true);
    if (rc) return rc;
    const DevHeader &h = *c->hhdr;
    *n_out = h.n_struct;
    if (stats) {
        stats->tiles = tiles;
        stats->mispredicted = h.spec_repairs;
    }
    if (h.n_struct > cap) return FALX_ERR_CAPACITY;
    return FALX_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free structural index.
//
// Some callers cannot allocate device memory at all: code running under an
// allocator that forbids it (a memory pool that is already full, a process
// that must not grow its footprint while serving), plugins called from a
// host that owns every allocation, or code paths that must not take the
// driver's allocation locks. For them this entry point runs the same index
// kernel as falx_index_structurals without a context: its look-back scratch
// (one status record per 16 KiB tile plus a small header) lives in the
// file-scope array below. Under CUDA's default lazy module loading the
// driver places that array in device memory on the first call on each
// device (the cudaGetSymbolAddress in noalloc_setup), so that first call
// can still fail for lack of memory: callers make one call early, before
// memory is full or frozen. From then on the device holds those bytes until
// the process exits, and no call allocates.
// ===========================================================================
namespace {

constexpr uint64_t kNoAllocMaxBytes = FALX_NOALLOC_MAX_BYTES;
// Tiles are cut on the buffer's 16-byte address grid, so a misaligned
// buffer can span one tile more than len / kTile rounded up.
constexpr uint32_t kNoAllocMaxTiles = (uint32_t)((kNoAllocMaxBytes + 15 + kTile - 1) / kTile) + 1;

struct NoAllocScratch {
    DevHeader hdr;
    alignas(64) TileStatus status[kNoAllocMaxTiles];
};

struct NoAllocDevice {
    bool ready;
    NoAllocScratch *scratch;  // device address of g_noalloc_scratch on this device
    int sm_count;
    int blocks_per_sm[5];
    uint32_t epoch;
};

constexpr int kNoAllocMaxDevices = 64;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

}  // namespace

// The scratch itself. In host code this name is only a stand-in for the
// symbol; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

namespace {

template <int D>
int noalloc_setup_kernel(NoAllocDevice &dv) {
    const void *fn = (const void *)index_kernel<D>;
    FALX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemIx)));
    int nb = 0;
    FALX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, sizeof(SmemIx)));
    dv.blocks_per_sm[D] = nb > 0 ? nb : 1;
    return FALX_OK;
}

// Once per device, with that device current.
int noalloc_setup(int device) {
    NoAllocDevice &dv = g_noalloc_dev[device];
    void *ptr = nullptr;
    FALX_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    FALX_CUDA(cudaDeviceGetAttribute(&dv.sm_count, cudaDevAttrMultiProcessorCount, device));
    int rc = noalloc_setup_kernel<D_CSV>(dv);
    if (!rc) rc = noalloc_setup_kernel<D_CSV_HASH>(dv);
    if (!rc) rc = noalloc_setup_kernel<D_TSV>(dv);
    if (!rc) rc = noalloc_setup_kernel<D_LOGFMT>(dv);
    if (!rc) rc = noalloc_setup_kernel<D_NDJSON>(dv);
    if (rc) return rc;
    dv.scratch = static_cast<NoAllocScratch *>(ptr);
    // FALX_NOALLOC_EPOCH_START (tests only) starts the epoch near its wrap
    // so the clearing path below runs within a few calls.
    const char *e0 = getenv("FALX_NOALLOC_EPOCH_START");
    dv.epoch = e0 ? (uint32_t)strtoul(e0, nullptr, 0) : 0;
    if (dv.epoch >= (1u << 28)) dv.epoch = 0;
    dv.ready = true;
    return FALX_OK;
}

int noalloc_run(int device, int dialect, const uint8_t *data, uint64_t len, uint32_t *out, uint64_t cap,
                uint64_t *n_out, cudaStream_t stream) {
    NoAllocDevice &dv = g_noalloc_dev[device];
    if (!dv.ready) {
        int rc = noalloc_setup(device);
        if (rc) return rc;
    }
    // Status records are tagged with a launch epoch, so only the header must
    // start at zero; the whole array is cleared when the epoch wraps.
    if (++dv.epoch >= (1u << 28)) {
        FALX_CUDA(cudaMemsetAsync(dv.scratch, 0, sizeof(NoAllocScratch), stream));
        dv.epoch = 1;
    }
    FALX_CUDA(cudaMemsetAsync(&dv.scratch->hdr, 0, sizeof(DevHeader), stream));
    Params P;
    memset(&P, 0, sizeof P);
    const uint64_t shift = (uint64_t)((uintptr_t)data & 15u);
    P.data = data;
    P.abase = data - shift;
    P.len = len;
    P.shift = (uint32_t)shift;
    P.num_tiles = (uint32_t)((len + shift + kTile - 1) / kTile);
    P.epoch = dv.epoch;
    P.status = dv.scratch->status;
    P.hdr = &dv.scratch->hdr;
    P.index = cap ? out : nullptr;
    P.index_cap = cap;
    uint64_t grid = (uint64_t)dv.sm_count * (uint64_t)dv.blocks_per_sm[dialect];
    if (grid > P.num_tiles) grid = P.num_tiles;
    void *args[] = {(void *)&P};
    const void *fn = dialect == FALX_CSV        ? (const void *)index_kernel<D_CSV>
                     : dialect == FALX_CSV_HASH ? (const void *)index_kernel<D_CSV_HASH>
                     : dialect == FALX_TSV      ? (const void *)index_kernel<D_TSV>
                     : dialect == FALX_LOGFMT   ? (const void *)index_kernel<D_LOGFMT>
                                                : (const void *)index_kernel<D_NDJSON>;
    FALX_CUDA(cudaLaunchCooperativeKernel(fn, dim3((unsigned)grid), dim3(kThreads), args, sizeof(SmemIx), stream));
    DevHeader h;
    FALX_CUDA(cudaMemcpyAsync(&h, &dv.scratch->hdr, sizeof(DevHeader), cudaMemcpyDeviceToHost, stream));
    FALX_CUDA(cudaStreamSynchronize(stream));
    *n_out = h.n_struct;
    if (h.error) return FALX_ERR_TIMEOUT;
    return h.n_struct > cap ? FALX_ERR_CAPACITY : FALX_OK;
}

}  // namespace

extern "C" int falx_index_structurals_noalloc(int device, int dialect, const uint8_t *data, uint64_t len,
                                              uint32_t *out, uint64_t cap, uint64_t *n_out, void *stream) {
    if (!n_out || !valid_dialect(dialect) || device < 0 || device >= kNoAllocMaxDevices) return FALX_ERR_INVALID;
    if ((len && !data) || (cap && !out)) return FALX_ERR_INVALID;
    *n_out = 0;
    if (len > kNoAllocMaxBytes) return FALX_ERR_INPUT_TOO_LARGE;
    if (len == 0) return FALX_OK;
    int prev = 0;
    FALX_CUDA(cudaGetDevice(&prev));
    if (prev != device) FALX_CUDA(cudaSetDevice(device));
    const int rc = noalloc_run(device, dialect, data, len, out, cap, n_out, (cudaStream_t)stream);
    if (prev != device) cudaSetDevice(prev);
    return rc;
}
