// NDJSON sum(id + nested.score): JSON-aware sink over newline-delimited
// records (generalises ndjson.rs:662-750, which only accepts the literal
// prefixes `{"id":` and `],"nested":{"score":` with integer scores).
//
// Records are owned by line: a valid NDJSON record holds no raw newline
// inside a string, so every raw '\n' ends a record and tiles need no carried
// state (the reference's parallel driver snaps chunks to raw newlines the same
// way, ndjson.rs:857-880). A tile owns the lines that start inside it; each
// thread parses the lines starting in its 64 bytes, reading the tile from
// shared memory and the tail of its last line from global memory.
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

__device__ __forceinline__ void j_ws(const LineView &v, int64_t e, int64_t &i) {
    while (i < e) {
        uint8_t c = v.at(i);
        if (c != ' ' && c != '\t' && c != '\r') break;
        i++;
    }
}

__device__ __forceinline__ bool j_string(const LineView &v, int64_t e, int64_t &i) {
    i++;
    while (i < e) {
        uint8_t c = v.at(i);
        if (c == '\\') { i += 2; continue; }
        i++;
        if (c == '"') return true;
    }
    return false;
}

__device__ inline bool j_skip_value(const LineView &v, int64_t e, int64_t &i) {
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
__device__ inline bool j_member(const LineView &v, int64_t e, int64_t &i, const char *key, int klen) {
    if (i >= e || v.at(i) != '{') return false;
    i++;
    for (;;) {
        j_ws(v, e, i);
        if (i >= e || v.at(i) != '"') return false;
        int64_t ks = i;
        if (!j_string(v, e, i)) return false;
        int64_t ke = i;
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

__device__ inline bool j_int(const LineView &v, int64_t e, int64_t i, int64_t &out) {
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

__device__ inline bool j_dec_e6(const LineView &v, int64_t e, int64_t i, int64_t &out) {
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

constexpr int kNdTile = 16384;

__global__ void __launch_bounds__(kThreads) ndjson_kernel(const uint8_t *data, uint64_t len, uint32_t ntiles,
                                                           NdjsonAcc *acc) {
    __shared__ __align__(16) uint8_t sm[kNdTile + 16];
    __shared__ unsigned long long red[kWarps][5];
    __shared__ uint32_t s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(&acc->ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const int64_t t0 = (int64_t)tile * kNdTile;
        const int64_t t1 = t0 + kNdTile < (int64_t)len ? t0 + kNdTile : (int64_t)len;
        // stage [t0 - 1, t1): one byte before the tile for the line-start test
        const int64_t s0 = t0 > 0 ? t0 - 1 : 0;
        for (int64_t i = s0 + tid; i < t1; i += kThreads) sm[i - s0] = data[i];
        __syncthreads();
        LineView v{sm, s0, t1, data};
        unsigned long long recs = 0, sid = 0, ssc = 0;
        __int128 tot = 0;
        bool bad = false;
        const int64_t b0 = t0 + (int64_t)tid * kThreadBytes;
        const int64_t b1 = b0 + kThreadBytes < t1 ? b0 + kThreadBytes : t1;
        for (int64_t p = b0; p < b1; p++) {
            if (!(p == 0 || v.at(p - 1) == '\n')) continue;
            int64_t e = p;
            while (e < (int64_t)len && v.at(e) != '\n') e++;
            int64_t j = p;
            j_ws(v, e, j);
            if (j >= e) continue;
            int64_t a = j, b = j, id, sc;
            if (!j_member(v, e, a, "id", 2) || !j_int(v, e, a, id) || !j_member(v, e, b, "nested", 6) ||
                !j_member(v, e, b, "score", 5) || !j_dec_e6(v, e, b, sc)) {
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
            for (int k = 0; k < 5; k++) red[warp][k] = vals[k];
        if (__syncthreads_or(bad) && tid == 0) atomicOr(&acc->error, 1u);
        if (tid == 0) {
            unsigned long long r[5] = {0, 0, 0, 0, 0};
            for (int w = 0; w < kWarps; w++) {
                for (int k = 0; k < 3; k++) r[k] += red[w][k];
                unsigned long long nlo = r[3] + red[w][3];
                r[4] += red[w][4] + (nlo < r[3] ? 1 : 0);
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
    uint32_t ntiles = (uint32_t)((len + kNdTile - 1) / kNdTile);
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
