// NDJSON sum(id + nested.score): JSON-aware sink over newline-delimited
// records (generalises ndjson.rs:662-750, which only accepts the literal
// prefixes `{"id":` and `],"nested":{"score":` with integer scores).
//
// Records are owned by line: a valid NDJSON record holds no raw newline
// inside a string, so every raw '\n' ends a record and tiles need no carried
// state (the reference's parallel driver snaps chunks to raw newlines the same
// way, ndjson.rs:857-880). A tile owns the lines that start inside it; each
// thread parses the lines starting in its 64 bytes from shared memory (the
// tile plus a 4 KiB halo after it).
//
// Per record: member "id" of the top-level object must be a JSON integer;
// member "nested" must be an object whose member "score" is a JSON number
// with at most 6 fraction digits and no exponent. Anything else sets the
// schema error. Blank lines (spaces, tabs, '\r' only) are skipped.
#pragma once
#include <cuda_runtime.h>

#include "scan_core.cuh"

namespace falx {

struct NdjsonAcc {
    unsigned long long records;
    unsigned long long sum_id;
    unsigned long long sum_score;
    unsigned long long total_lo;
    unsigned long long total_hi;
    uint32_t error;
    uint32_t ticket;
};

struct LineView {
    const uint8_t *sm;  // shared copy of [s0, s1)
    int64_t s0, s1;
    const uint8_t *g;   // global data
    __device__ __forceinline__ uint8_t at(int64_t i) const { return (i >= s0 && i < s1) ? sm[i - s0] : g[i]; }
};

// A line staged whole in shared memory: positions relative to the staged
// window, 32-bit, no per-byte range test (nearly every line).
struct SmemView {
    const uint8_t *sm;
    __device__ __forceinline__ uint8_t at(int i) const { return sm[i]; }
};

// The scanner below takes either view: V (LineView or SmemView) and the
// position type I (int64_t or int).
template <class V, typename I>
__device__ __forceinline__ void j_ws(const V &v, I e, I &i) {
    while (i < e) {
        uint8_t c = v.at(i);
        if (c != ' ' && c != '\t' && c != '\r') break;
        i++;
    }
}

template <class V, typename I>
__device__ __forceinline__ bool j_string(const V &v, I e, I &i) {
    i++;
    while (i < e) {
        uint8_t c = v.at(i);
        if (c == '\\') { i += 2; continue; }
        i++;
        if (c == '"') return true;
    }
    return false;
}

template <class V, typename I>
__device__ inline bool j_skip_value(const V &v, I e, I &i) {
    j_ws(v, e, i);
    if (i >= e) return false;
    uint8_t c = v.at(i);
    if (c == '"') return j_string(v, e, i);
    if (c == '{' || c == '[') {
        int depth = 0;
        while (i < e) {
            uint8_t x = v.at(i);
            if (x == '"') {
                if (!j_string(v, e, i)) return false;
                continue;
            }
            if (x == '{' || x == '[') depth++;
            else if (x == '}' || x == ']') {
                if (--depth == 0) { i++; return true; }
            }
            i++;
        }
        return false;
    }
    while (i < e) {
        uint8_t x = v.at(i);
        if (x == ',' || x == '}' || x == ']' || x == ' ' || x == '\t' || x == '\r') break;
        i++;
    }
    return true;
}

// Position *i on the value of member `key` of the object opening at *i.
template <class V, typename I>
__device__ inline bool j_member(const V &v, I e, I &i, const char *key, int klen) {
    if (i >= e || v.at(i) != '{') return false;
    i++;
    for (;;) {
        j_ws(v, e, i);
        if (i >= e || v.at(i) != '"') return false;
        const I ks = i;
        if (!j_string(v, e, i)) return false;
        const I ke = i;
        bool match = ke - ks == klen + 2;
        for (int k = 0; match && k < klen; k++) match = v.at(ks + 1 + k) == (uint8_t)key[k];
        j_ws(v, e, i);
        if (i >= e || v.at(i) != ':') return false;
        i++;
        j_ws(v, e, i);
        if (match) return true;
        if (!j_skip_value(v, e, i)) return false;
        j_ws(v, e, i);
        if (i < e && v.at(i) == ',') { i++; continue; }
        return false;
    }
}

template <class V, typename I>
__device__ inline bool j_int(const V &v, I e, I i, int64_t &out) {
    bool neg = false;
    if (i < e && v.at(i) == '-') { neg = true; i++; }
    if (i >= e) return false;
    uint64_t val = 0;
    int nd = 0;
    while (i < e) {
        uint32_t d = (uint8_t)(v.at(i) - '0');
        if (d >= 10) break;
        val = val * 10 + d;
        i++;
        nd++;
    }
    if (nd == 0 || nd > 19) return false;
    out = neg ? (int64_t)(0 - val) : (int64_t)val;
    return true;
}

template <class V, typename I>
__device__ inline bool j_dec_e6(const V &v, I e, I i, int64_t &out) {
    bool neg = false;
    if (i < e && v.at(i) == '-') { neg = true; i++; }
    uint64_t ip = 0;
    int nd = 0;
    while (i < e) {
        uint32_t d = (uint8_t)(v.at(i) - '0');
        if (d >= 10) break;
        ip = ip * 10 + d;
        i++;
        nd++;
    }
    if (nd == 0 || nd > 12) return false;
    uint64_t fr = 0;
    int nf = 0;
    if (i < e && v.at(i) == '.') {
        i++;
        while (i < e) {
            uint32_t d = (uint8_t)(v.at(i) - '0');
            if (d >= 10) break;
            if (nf == 6) return false;
            fr = fr * 10 + d;
            i++;
            nf++;
        }
        if (nf == 0) return false;
    }
    if (i < e && (v.at(i) | 0x20) == 'e') return false;
    for (; nf < 6; nf++) fr *= 10;
    uint64_t m = ip * 1000000ull + fr;
    out = neg ? -(int64_t)m : (int64_t)m;
    return true;
}

// One line [j, e): 1 and its id and score, 0 outside the schema, -1 blank.
template <class V, typename I>
__device__ __forceinline__ int nd_line(const V &v, I j, I e, int64_t &id, int64_t &sc) {
    j_ws(v, e, j);
    if (j >= e) return -1;
    I a = j, b = j;
    if (!j_member(v, e, a, "id", 2) || !j_int(v, e, a, id) || !j_member(v, e, b, "nested", 6) ||
        !j_member(v, e, b, "score", 5) || !j_dec_e6(v, e, b, sc))
        return 0;
    return 1;
}

constexpr int kNdTile = 16384;  // a tile owns the lines that start inside it
constexpr int kNdHalo = 4096;   // bytes staged after the tile for the lines that cross its end
constexpr int kNdSpan = kNdTile + kNdHalo;
constexpr int kNdWords = kNdSpan / 64;

struct NdSmem {
    alignas(16) uint8_t buf[16 + kNdSpan];  // 16 bytes before the tile, the tile, the halo
    uint64_t nl[kNdWords];                  // newline bitmap of the tile and the halo
    unsigned long long red[kWarps][5];
    uint32_t s_tile;
};

// Tiles sit on the 16-byte address grid of the input: tile t starts at file
// position kNdTile t - shift, so every staging load is an aligned 16-byte
// load. A thread finds the line starts among its 64 bytes of the tile from
// the newline bitmap, the end of each line from the bitmap too (lines
// crossing into the halo included), and parses each line from shared
// memory; only a line longer than the halo reads global memory past it.
__global__ void __launch_bounds__(kThreads) ndjson_kernel(const uint8_t *data, uint64_t len, uint32_t ntiles,
                                                           NdjsonAcc *acc) {
    __shared__ NdSmem S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t shift = (uint32_t)((uintptr_t)data & 15u);
    const uint8_t *abase = data - shift;
    const uint64_t end16 = (shift + len + 15) & ~15ull;  // staged bytes stay inside [abase, abase + end16)
    for (;;) {
        if (tid == 0) S.s_tile = atomicAdd(&acc->ticket, 1u);
        __syncthreads();
        const uint32_t tile = S.s_tile;
        if (tile >= ntiles) break;
        const uint64_t a0 = (uint64_t)tile * kNdTile;     // address offset of the tile
        const int64_t t0 = (int64_t)a0 - (int64_t)shift;  // its file position
        // ---- stage [a0 - 16, a0 + kNdSpan) with aligned 16-byte loads
        for (int i = tid; i < (16 + kNdSpan) / 16; i += kThreads) {
            const int64_t o = (int64_t)a0 - 16 + 16 * i;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (o >= 0 && (uint64_t)o < end16) v = *reinterpret_cast<const uint4 *>(abase + o);
            *reinterpret_cast<uint4 *>(S.buf + 16 * i) = v;
        }
        __syncthreads();
        // ---- newline bitmap (positions outside the input are not newlines)
        for (int k = tid; k < kNdWords; k += kThreads) {
            const uint32_t *w = reinterpret_cast<const uint32_t *>(S.buf + 16 + 64 * k);
            uint64_t m = 0;
#pragma unroll
            for (int c = 0; c < 4; c++)
                m |= (uint64_t)gather16(eq_flags(w[4 * c], '\n'), eq_flags(w[4 * c + 1], '\n'),
                                        eq_flags(w[4 * c + 2], '\n'), eq_flags(w[4 * c + 3], '\n'))
                     << (16 * c);
            const int64_t p0 = t0 + 64 * k;
            if (p0 < 0) m &= p0 <= -64 ? 0ull : ~0ull << (-p0);
            if (p0 + 64 > (int64_t)len) m &= p0 >= (int64_t)len ? 0ull : (1ull << ((int64_t)len - p0)) - 1;
            S.nl[k] = m;
        }
        __syncthreads();
        LineView v{S.buf + 16, t0, t0 + kNdSpan, data};
        unsigned long long recs = 0, sid = 0, ssc = 0;
        __int128 tot = 0;
        bool bad = false;
        // line starts among this thread's 64 bytes of the tile
        const int64_t b0 = t0 + 64 * tid;
        uint64_t starts = S.nl[tid] << 1;
        if (tid > 0) starts |= S.nl[tid - 1] >> 63;
        else if (b0 > 0 && S.buf[15] == '\n') starts |= 1;
        if (b0 <= 0 && b0 + 64 > 0) starts |= 1ull << (-b0);  // file position 0
        if (b0 < 0) starts &= b0 <= -64 ? 0ull : ~0ull << (-b0);
        if (b0 + 64 > (int64_t)len) starts &= b0 >= (int64_t)len ? 0ull : (1ull << ((int64_t)len - b0)) - 1;
        while (starts) {
            const int bpos = __ffsll((long long)starts) - 1;
            starts &= starts - 1;
            const int64_t p = b0 + bpos;
            // end of the line: the next newline in the bitmap, else past the halo
            int wi = tid;
            uint64_t m = S.nl[wi] & (~0ull << bpos);
            while (!m && wi + 1 < kNdWords) m = S.nl[++wi];
            int64_t e;
            if (m) {
                e = t0 + 64 * wi + (__ffsll((long long)m) - 1);
            } else {
                e = t0 + kNdSpan;
                while (e < (int64_t)len && data[e] != '\n') e++;
                if (e > (int64_t)len) e = (int64_t)len;
            }
            int64_t id, sc;
            int st;
            if (e <= t0 + kNdSpan) {
                // the whole line is staged
                const SmemView sv{S.buf + 16};
                st = nd_line(sv, (int)(p - t0), (int)(e - t0), id, sc);
            } else {
                st = nd_line(v, p, e, id, sc);
            }
            if (st < 0) continue;  // a blank line
            if (st == 0) {
                bad = true;
                continue;
            }
            recs++;
            sid += (unsigned long long)id;
            ssc += (unsigned long long)sc;
            tot += (__int128)id * 1000000 + sc;
        }
        unsigned long long vals[5] = {recs, sid, ssc, (unsigned long long)(uint64_t)tot,
                                      (unsigned long long)(uint64_t)(tot >> 64)};
        // lo/hi reduction with carries: reduce lo in 64 bits, count carries into hi
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            unsigned long long olo = __shfl_down_sync(0xffffffffu, vals[3], d);
            unsigned long long ohi = __shfl_down_sync(0xffffffffu, vals[4], d);
            unsigned long long nlo = vals[3] + olo;
            vals[4] += ohi + (nlo < vals[3] ? 1 : 0);
            vals[3] = nlo;
#pragma unroll
            for (int k = 0; k < 3; k++) vals[k] += __shfl_down_sync(0xffffffffu, vals[k], d);
        }
        if (lane == 0)
            for (int k = 0; k < 5; k++) S.red[warp][k] = vals[k];
        if (__syncthreads_or(bad) && tid == 0) atomicOr(&acc->error, 1u);
        if (tid == 0) {
            unsigned long long r[5] = {0, 0, 0, 0, 0};
            for (int w = 0; w < kWarps; w++) {
                for (int k = 0; k < 3; k++) r[k] += S.red[w][k];
                unsigned long long nlo = r[3] + S.red[w][3];
                r[4] += S.red[w][4] + (nlo < r[3] ? 1 : 0);
                r[3] = nlo;
            }
            atomicAdd(&acc->records, r[0]);
            atomicAdd(&acc->sum_id, r[1]);
            atomicAdd(&acc->sum_score, r[2]);
            unsigned long long old = atomicAdd(&acc->total_lo, r[3]);
            unsigned long long carry = (old + r[3] < old) ? 1 : 0;
            atomicAdd(&acc->total_hi, r[4] + carry);
        }
        __syncthreads();
    }
}

static int g_nd_sm_count = 0;

inline int ndjson_setup(int device) {
    if (cudaDeviceGetAttribute(&g_nd_sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return FALX_ERR_CUDA;
    return FALX_OK;
}

inline int ndjson_run(const uint8_t *data, uint64_t len, falx_ndjson_stats *out, NdjsonAcc *acc, NdjsonAcc *host,
                      cudaStream_t stream) {
    memset(out, 0, sizeof *out);
    if (len == 0) return FALX_OK;
    const uint64_t shift = (uint64_t)((uintptr_t)data & 15u);
    uint32_t ntiles = (uint32_t)((len + shift + kNdTile - 1) / kNdTile);
    uint32_t grid = (uint32_t)(g_nd_sm_count * 4);
    if (grid > ntiles) grid = ntiles;
    if (cudaMemsetAsync(acc, 0, sizeof(NdjsonAcc), stream) != cudaSuccess) return FALX_ERR_CUDA;
    ndjson_kernel<<<grid, kThreads, 0, stream>>>(data, len, ntiles, acc);
    if (cudaGetLastError() != cudaSuccess) return FALX_ERR_CUDA;
    if (cudaMemcpyAsync(host, acc, sizeof(NdjsonAcc), cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        return FALX_ERR_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return FALX_ERR_CUDA;
    if (host->error) return FALX_ERR_SCHEMA;
    out->records = host->records;
    out->sum_id = (int64_t)host->sum_id;
    out->sum_score_e6 = (int64_t)host->sum_score;
    out->total_e6_lo = (int64_t)host->total_lo;
    out->total_e6_hi = (int64_t)host->total_hi;
    __int128 t = ((__int128)(int64_t)host->total_hi << 64) | (__int128)(unsigned long long)host->total_lo;
    out->total_f64 = (double)t / 1e6;
    return FALX_OK;
}

}  // namespace falx
