// bgzf inflate on the GPU: the host walks the gzip member headers (a few
// bytes per 64 KiB block), the kernel inflates every block at once, one
// warp per block, into one contiguous output buffer that the index and
// columns kernels then read in place (bgzf.rs:61-108 scan, :180-240
// inflate_blocks_into / decompress_par; examples/gpu_pipeline.rs:1-8).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "../../include/falx_gpu.h"
#include "context.h"
#include "inflate_core.h"

namespace falx {
namespace gz {
namespace {

constexpr int kGzWarps = 8;
constexpr int kGzThreads = 32 * kGzWarps;

// The warp's view of the decoder's output: a literal is stored by lane 0;
// a match (after a barrier that makes lane 0's stores visible to the warp)
// and a stored run are copied by all lanes.
struct WarpSink {
    uint8_t *out;
    uint32_t lane;

    __device__ __forceinline__ void sync() { __syncwarp(); }
    __device__ __forceinline__ void flush() { __syncwarp(); }
    __device__ __forceinline__ void literal(uint32_t pos, uint32_t c) {
        if (lane == 0) out[pos] = (uint8_t)c;
    }
    __device__ __forceinline__ void match(uint32_t pos, uint32_t dist, uint32_t len) {
        __syncwarp();
        const uint8_t *src = out + (pos - dist);
        if (dist >= len) {
            for (uint32_t k = lane; k < len; k += 32) out[pos + k] = src[k];
        } else {
            for (uint32_t k = lane; k < len; k += 32) out[pos + k] = src[k % dist];
        }
        __syncwarp();
    }
    __device__ __forceinline__ void stored(const uint8_t *s, uint32_t pos, uint32_t len) {
        __syncwarp();
        for (uint32_t k = lane; k < len; k += 32) out[pos + k] = s[k];
        __syncwarp();
    }
    __device__ __forceinline__ void fill_fast(uint16_t *fast, int F, const uint16_t *count, const uint16_t *sym) {
        __syncwarp();
        for (uint32_t i = lane; i < (1u << F); i += 32) fast[i] = fast_entry(i, F, count, sym);
        __syncwarp();
    }
};

// Members are taken from an atomic ticket, one per warp at a time
// (members differ in decode time; a static split left warps idle at the
// end). `counters`: [0] failed members, [1] the ticket.
__global__ void __launch_bounds__(kGzThreads) inflate_kernel(const uint8_t *comp, uint64_t comp_len,
                                                              const Block *blocks, uint32_t nblocks, uint8_t *out,
                                                              uint64_t out_cap, int32_t *status,
                                                              unsigned long long *counters) {
    __shared__ Tables T[kGzWarps];
    __shared__ Consts K;
    if (threadIdx.x == 0) make_consts(K);
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (;;) {
        uint32_t b = 0;
        if (lane == 0) b = (uint32_t)atomicAdd(counters + 1, 1ull);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= nblocks) break;
        const Block B = blocks[b];
        int rc;
        if (B.in_off > comp_len || B.in_len > comp_len - B.in_off || B.out_off > out_cap ||
            B.out_len > out_cap - B.out_off) {
            rc = ERR_BOUNDS;
        } else {
            Bits bits{comp + B.in_off, B.in_len, 0u, 0ull, 0, false};
            WarpSink sink{out + B.out_off, lane};
            rc = inflate_stream(bits, T[warp], K, sink, B.out_len);
        }
        if (lane == 0) {
            status[b] = rc;
            if (rc) atomicAdd(counters, 1ull);
        }
        __syncwarp();
    }
}

int cuda_fail(cudaError_t e) {
    (void)cudaGetLastError();
    return e == cudaSuccess ? FALX_OK : FALX_ERR_CUDA;
}
#define FALX_CUDA(x)                                 \
    do {                                             \
        cudaError_t e_ = (x);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)

uint16_t le16(const uint8_t *p) { return (uint16_t)(p[0] | (p[1] << 8)); }
uint32_t le32(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }

}  // namespace
}  // namespace gz
}  // namespace falx

using namespace falx::gz;

namespace falx {
int gz_launch(falx_ctx *c, const uint8_t *comp, uint64_t comp_len, const falx_gz_block *blocks, uint64_t n_blocks,
              uint8_t *out, uint64_t out_cap, unsigned long long **counters, int32_t **status) {
    static_assert(sizeof(falx_gz_block) == sizeof(Block), "block layout");
    // scratch: the block table, then per-block status and the counters
    const uint64_t tbytes = n_blocks * sizeof(Block), sbytes = n_blocks * 4;
    const uint64_t need = ((tbytes + 255) & ~255ull) + ((sbytes + 255) & ~255ull) + 256;  // + counters
    if (need > c->gz_cap) {
        // earlier launches may still read the old scratch
        FALX_CUDA(cudaStreamSynchronize(c->stream));
        if (c->gz_scratch) cudaFree(c->gz_scratch);
        c->gz_scratch = nullptr;
        c->gz_cap = 0;
        FALX_CUDA(cudaMalloc(&c->gz_scratch, need));
        c->gz_cap = need;
    }
    uint8_t *base = static_cast<uint8_t *>(c->gz_scratch);
    Block *dblocks = reinterpret_cast<Block *>(base);
    int32_t *dstatus = reinterpret_cast<int32_t *>(base + ((tbytes + 255) & ~255ull));
    unsigned long long *dcounters =
        reinterpret_cast<unsigned long long *>(base + ((tbytes + 255) & ~255ull) + ((sbytes + 255) & ~255ull));
    FALX_CUDA(cudaMemcpyAsync(dblocks, blocks, tbytes, cudaMemcpyHostToDevice, c->stream));
    FALX_CUDA(cudaMemsetAsync(dcounters, 0, 2 * sizeof(unsigned long long), c->stream));
    if (!c->gz_grid) {
        int nb = 0;
        FALX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, inflate_kernel, kGzThreads, 0));
        c->gz_grid = std::max(1, nb) * c->sm_count;
    }
    const uint64_t want = (n_blocks + kGzWarps - 1) / kGzWarps;
    const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)c->gz_grid);
    inflate_kernel<<<grid, kGzThreads, 0, c->stream>>>(comp, comp_len, dblocks, (uint32_t)n_blocks, out, out_cap,
                                                       dstatus, dcounters);
    FALX_CUDA(cudaGetLastError());
    *counters = dcounters;
    *status = dstatus;
    return FALX_OK;
}
}  // namespace falx

extern "C" {

// Walk the gzip members of a bgzf stream (bgzf.rs:42-108): magic 1f 8b,
// CM 8, FEXTRA set, the BC subfield's BSIZE gives the member length; the
// payload is the member less its header, extra field and 8-byte trailer,
// whose last 4 bytes are ISIZE. Empty members (the EOF marker) are skipped.
int falx_bgzf_scan(const uint8_t *comp, uint64_t len, falx_gz_block *blocks, uint64_t cap, uint64_t *n_blocks,
                   uint64_t *out_len) {
    if (!n_blocks || !out_len || (len && !comp) || (cap && !blocks)) return FALX_ERR_INVALID;
    constexpr uint64_t kHeader = 12, kTrailer = 8;
    uint64_t pos = 0, n = 0, total = 0;
    while (pos < len) {
        if (len - pos < kHeader) return FALX_ERR_FORMAT;
        const uint8_t *h = comp + pos;
        if (h[0] != 0x1f || h[1] != 0x8b || h[2] != 8 || !(h[3] & 0x04)) return FALX_ERR_FORMAT;
        const uint64_t xlen = le16(h + 10);
        if (len - pos - kHeader < xlen) return FALX_ERR_FORMAT;
        const uint8_t *x = h + kHeader;
        int64_t bsize = -1;
        for (uint64_t i = 0; i + 4 <= xlen;) {
            const uint64_t slen = le16(x + i + 2);
            if (x[i] == 'B' && x[i + 1] == 'C' && slen == 2 && i + 6 <= xlen) {
                bsize = le16(x + i + 4);
                break;
            }
            i += 4 + slen;
        }
        if (bsize < 0) return FALX_ERR_FORMAT;
        const uint64_t block_len = (uint64_t)bsize + 1;
        if (block_len <= kHeader + xlen + kTrailer || block_len > len - pos) return FALX_ERR_FORMAT;
        const uint32_t isize = le32(h + block_len - 4);
        if (isize > 0) {
            if (n < cap) {
                blocks[n].in_off = pos + kHeader + xlen;
                blocks[n].in_len = (uint32_t)(block_len - kHeader - xlen - kTrailer);
                blocks[n].out_off = total;
                blocks[n].out_len = isize;
            }
            n++;
            total += isize;
        }
        pos += block_len;
    }
    *n_blocks = n;
    *out_len = total;
    return n > cap ? FALX_ERR_CAPACITY : FALX_OK;
}

int falx_bgzf_inflate(falx_ctx *c, const uint8_t *comp, uint64_t comp_len, const falx_gz_block *blocks,
                      uint64_t n_blocks, uint8_t *out, uint64_t out_cap, int32_t *block_status,
                      uint64_t *n_failed) {
    if (!c || (comp_len && !comp) || (n_blocks && !blocks) || (out_cap && !out) || n_blocks > 0xFFFFFFFFull)
        return FALX_ERR_INVALID;
    if (n_failed) *n_failed = 0;
    if (n_blocks == 0) return FALX_OK;
    FALX_CUDA(cudaSetDevice(c->device));
    unsigned long long *dcounters = nullptr;
    int32_t *dstatus = nullptr;
    const int rc = falx::gz_launch(c, comp, comp_len, blocks, n_blocks, out, out_cap, &dcounters, &dstatus);
    if (rc) return rc;
    unsigned long long failed = 0;
    FALX_CUDA(cudaMemcpyAsync(&failed, dcounters, sizeof failed, cudaMemcpyDeviceToHost, c->stream));
    if (block_status)
        FALX_CUDA(cudaMemcpyAsync(block_status, dstatus, n_blocks * 4, cudaMemcpyDeviceToHost, c->stream));
    FALX_CUDA(cudaStreamSynchronize(c->stream));
    if (n_failed) *n_failed = failed;
    return failed ? FALX_ERR_FORMAT : FALX_OK;
}

}  // extern "C"
