// Batched documents: one persistent launch over a device work queue.
//
// The reference parses a collection of files one call at a time (each call
// a parse_columns_par over its own threads, csv_geo.rs:1216-1284; the
// multi-file example drivers loop over files). On the GPU every document of
// a batch runs in one cooperative launch:
//
//  - A work item is either a whole document (at most `chunk_bytes`, run
//    tile after tile by one CTA, so each tile's look-back finds its own
//    predecessor's inclusive prefix at distance 1) or one 16 KiB tile of a
//    larger document (round-robin over CTAs, decoupled look-back bounded to
//    that document's tiles).
//  - CTAs claim items from an atomic ticket in queue order: large
//    documents' tiles first (in tile order), then whole documents largest
//    first. Every tile waits only on earlier tiles of its own document,
//    which are earlier items, so the oldest unfinished item can always
//    progress (all CTAs are resident: cooperative launch).
//  - Each CTA keeps `NB` tiles in flight (TMA bulk copies into NB shared
//    buffers), claiming the item of its next tile ahead of time.
//  - The dialect is per document (CSV, TSV or logfmt: the geo schemas'
//    formats), dispatched per tile.
//
// Per document: structural index and two f64 columns with validity (the
// lat / lon pair of the geo schemas), plus its counts in a device header.
// The whole launch sequence (status / header / ticket / validity resets, the
// kernel, the copy of the headers back) is captured once in a CUDA graph and
// replayed per batch. falx_batch_tune times candidate (chunk size, CTAs per
// SM, staging depth) configurations on the caller's batch and keeps the
// fastest in the context.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/falx_gpu.h"
#include "batch_kernel.cuh"
#include "context.h"

namespace falx {

// Clear the validity bitmaps of every document (rows are OR'ed in).
__global__ void batch_clear(uint64_t *const *ptrs, const uint64_t *words, uint32_t n) {
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        uint64_t *p = ptrs[k];
        for (uint64_t i = threadIdx.x; i < words[k]; i += blockDim.x) p[i] = 0;
    }
}

}  // namespace falx

using namespace falx;

struct falx_batch {
    falx_ctx *c = nullptr;
    uint32_t ndocs = 0, n_items = 0, total_tiles = 0;
    falx_batch_config cfg{};
    Params *d_params = nullptr;
    BatchItem *d_items = nullptr;
    uint32_t *d_ticket = nullptr;
    DevHeader *d_hdrs = nullptr;
    DevHeader *h_hdrs = nullptr;  // pinned
    TileStatus *d_status = nullptr;
    ArenaStatus *d_astatus = nullptr;
    uint64_t **d_clear_ptrs = nullptr;
    uint64_t *d_clear_words = nullptr;
    uint32_t n_clear = 0;
    int grid = 0;
    size_t smem = 0;
    bool use_graph = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> caps;  // per document: index capacity
    std::vector<uint64_t> rows_caps;
};

namespace {

int fail_cuda(cudaError_t e) {
    if (e == cudaSuccess) return FALX_OK;
    (void)cudaGetLastError();
    return FALX_ERR_CUDA;
}
#define BATCH_CUDA(x)                                 \
    do {                                              \
        cudaError_t e_ = (x);                         \
        if (e_ != cudaSuccess) return fail_cuda(e_);  \
    } while (0)

int batch_occupancy(uint32_t staging, int &nb, size_t &smem) {
    return staging == 3 ? batch_occupancy_nb3(nb, smem) : batch_occupancy_nb2(nb, smem);
}

bool doc_dialect_ok(int d) { return d == FALX_CSV || d == FALX_TSV || d == FALX_LOGFMT; }

void batch_free(falx_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    void *ps[] = {b->d_params, b->d_items, b->d_ticket, b->d_hdrs, b->d_status, b->d_astatus, b->d_clear_ptrs,
                  b->d_clear_words};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (b->h_hdrs) cudaFreeHost(b->h_hdrs);
}

int batch_launch_kernel(falx_batch *b, cudaStream_t st) {
    void *args[] = {(void *)&b->d_params, (void *)&b->d_items, (void *)&b->n_items, (void *)&b->d_ticket};
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.gridDim = dim3((unsigned)b->grid);
    lc.blockDim = dim3(kThreads);
    lc.stream = st;
    lc.attrs = attr;
    lc.numAttrs = 1;
    lc.dynamicSmemBytes = b->smem;
    return fail_cuda(b->cfg.staging == 3 ? batch_launch_nb3(lc, args) : batch_launch_nb2(lc, args));
}

// The launch sequence of one batch on stream `st`.
int batch_enqueue(falx_batch *b, cudaStream_t st) {
    BATCH_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(TileStatus) * (size_t)b->total_tiles, st));
    BATCH_CUDA(cudaMemsetAsync(b->d_hdrs, 0, sizeof(DevHeader) * (size_t)b->ndocs, st));
    BATCH_CUDA(cudaMemsetAsync(b->d_ticket, 0, 4, st));
    if (b->n_clear) {
        batch_clear<<<std::min<uint32_t>(b->n_clear, 4096), 256, 0, st>>>(b->d_clear_ptrs, b->d_clear_words,
                                                                           b->n_clear);
        BATCH_CUDA(cudaGetLastError());
    }
    int rc = batch_launch_kernel(b, st);
    if (rc) return rc;
    BATCH_CUDA(cudaMemcpyAsync(b->h_hdrs, b->d_hdrs, sizeof(DevHeader) * (size_t)b->ndocs, cudaMemcpyDeviceToHost,
                               st));
    return FALX_OK;
}

}  // namespace

extern "C" {

int falx_batch_plan(const uint64_t *lens, uint32_t ndocs, uint32_t chunk_bytes, uint32_t *items, uint32_t cap,
                    uint32_t *n_items) {
    if (!n_items || (ndocs && !lens)) return FALX_ERR_INVALID;
    // large documents' tiles in tile order, then whole documents largest first
    std::vector<uint32_t> whole;
    uint32_t k = 0;
    auto put = [&](uint32_t d, uint32_t lo, uint32_t hi) {
        if (items && k < cap) {
            items[3 * k] = d;
            items[3 * k + 1] = lo;
            items[3 * k + 2] = hi;
        }
        k++;
    };
    for (uint32_t d = 0; d < ndocs; d++) {
        // tiles as the kernel counts them, for 16-byte aligned document starts
        const uint64_t tiles = (lens[d] + kTile - 1) / kTile;
        if (tiles == 0) continue;
        if (lens[d] > chunk_bytes) {
            for (uint32_t t = 0; t < tiles; t++) put(d, t, t + 1);
        } else {
            whole.push_back(d);
        }
    }
    std::stable_sort(whole.begin(), whole.end(), [&](uint32_t a, uint32_t b) { return lens[a] > lens[b]; });
    for (uint32_t d : whole) put(d, 0, (uint32_t)((lens[d] + kTile - 1) / kTile));
    *n_items = k;
    return items && k > cap ? FALX_ERR_CAPACITY : FALX_OK;
}

int falx_batch_create(falx_ctx *c, const falx_doc *docs, uint32_t ndocs, const falx_batch_config *cfg,
                      falx_batch **out) {
    if (!c || !out || (ndocs && !docs)) return FALX_ERR_INVALID;
    *out = nullptr;
    falx_batch_config conf = {};
    if (cfg) {
        conf = *cfg;
    } else if (c->batch_tuned.valid) {
        conf.chunk_bytes = c->batch_tuned.chunk_bytes;
        conf.ctas_per_sm = c->batch_tuned.ctas_per_sm;
        conf.staging = c->batch_tuned.staging;
    }
    if (conf.chunk_bytes == 0) conf.chunk_bytes = 1u << 20;
    if (conf.staging == 0) conf.staging = 2;
    if (conf.staging != 2 && conf.staging != 3) return FALX_ERR_INVALID;
    std::vector<uint64_t> lens(ndocs);
    for (uint32_t d = 0; d < ndocs; d++) {
        const falx_doc &x = docs[d];
        if (!doc_dialect_ok(x.dialect) || (x.len && !x.data) || x.len >= (1ull << 32)) return FALX_ERR_INVALID;
        if ((uintptr_t)x.data & 15) return FALX_ERR_INVALID;  // documents start 16-byte aligned
        if ((x.index_cap && !x.index) ||
            (x.rows_cap && (!x.col0 || !x.col1 || !x.valid0 || !x.valid1)))
            return FALX_ERR_INVALID;
        lens[d] = x.len;
    }
    cudaSetDevice(c->device);
    falx_batch *b = new (std::nothrow) falx_batch;
    if (!b) return FALX_ERR_INVALID;
    b->c = c;
    b->ndocs = ndocs;
    b->cfg = conf;
    int rc = FALX_OK;
    uint32_t n_items = 0;
    falx_batch_plan(lens.data(), ndocs, conf.chunk_bytes, nullptr, 0, &n_items);
    std::vector<uint32_t> items(3 * (size_t)std::max<uint32_t>(n_items, 1));
    falx_batch_plan(lens.data(), ndocs, conf.chunk_bytes, items.data(), n_items, &n_items);
    b->n_items = n_items;
    // per-document parameters
    std::vector<Params> ps(std::max<uint32_t>(ndocs, 1));
    std::vector<uint64_t *> clear_ptrs;
    std::vector<uint64_t> clear_words;
    uint32_t first = 0;
    auto alloc = [&](void **p, size_t bytes) {
        if (!rc && cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) rc = FALX_ERR_CUDA;
    };
    for (uint32_t d = 0; d < ndocs; d++) first += (uint32_t)((lens[d] + kTile - 1) / kTile);
    b->total_tiles = first;
    alloc((void **)&b->d_status, sizeof(TileStatus) * (size_t)std::max<uint32_t>(first, 1));
    alloc((void **)&b->d_astatus, sizeof(ArenaStatus) * (size_t)std::max<uint32_t>(first, 1));
    alloc((void **)&b->d_hdrs, sizeof(DevHeader) * (size_t)std::max<uint32_t>(ndocs, 1));
    alloc((void **)&b->d_params, sizeof(Params) * (size_t)std::max<uint32_t>(ndocs, 1));
    alloc((void **)&b->d_items, sizeof(BatchItem) * (size_t)std::max<uint32_t>(n_items, 1));
    alloc((void **)&b->d_ticket, 4);
    if (!rc && cudaMallocHost(&b->h_hdrs, sizeof(DevHeader) * (size_t)std::max<uint32_t>(ndocs, 1)) != cudaSuccess)
        rc = FALX_ERR_CUDA;
    first = 0;
    for (uint32_t d = 0; d < ndocs && !rc; d++) {
        const falx_doc &x = docs[d];
        Params &P = ps[d];
        memset(&P, 0, sizeof P);
        const uint32_t tiles = (uint32_t)((x.len + kTile - 1) / kTile);
        P.data = x.data;
        P.abase = x.data;
        P.len = x.len;
        P.shift = 0;
        P.num_tiles = tiles;
        P.epoch = 1;
        P.halo = kHaloBytes;
        P.status = b->d_status + first;
        P.astatus = b->d_astatus + first;
        P.hdr = b->d_hdrs + d;
        P.index = x.index_cap ? x.index : nullptr;
        P.index_cap = x.index_cap;
        P.dialect = x.dialect;
        RowSpec &rs = P.rows;
        rs.rows_cap = x.rows_cap;
        rs.ncols = x.rows_cap ? 2 : 0;
        rs.nstr = 0;
        rs.max_field = 0;
        if (x.rows_cap) {
            rs.field[0] = x.field0;
            rs.field[1] = x.field1;
            rs.type[0] = rs.type[1] = FALX_F64;
            rs.str_slot[0] = rs.str_slot[1] = -1;
            rs.values[0] = x.col0;
            rs.values[1] = x.col1;
            rs.valid[0] = x.valid0;
            rs.valid[1] = x.valid1;
            rs.max_field = (x.field0 > x.field1 ? x.field0 : x.field1) + 1;
            const uint64_t words = (x.rows_cap + 63) / 64;
            clear_ptrs.push_back(x.valid0);
            clear_words.push_back(words);
            clear_ptrs.push_back(x.valid1);
            clear_words.push_back(words);
        }
        first += tiles;
    }
    b->n_clear = (uint32_t)clear_ptrs.size();
    if (b->n_clear) {
        alloc((void **)&b->d_clear_ptrs, sizeof(uint64_t *) * b->n_clear);
        alloc((void **)&b->d_clear_words, sizeof(uint64_t) * b->n_clear);
    }
    cudaStream_t st = c->stream;
    if (!rc && ndocs)
        rc = fail_cuda(cudaMemcpyAsync(b->d_params, ps.data(), sizeof(Params) * ndocs, cudaMemcpyHostToDevice, st));
    if (!rc && n_items)
        rc = fail_cuda(cudaMemcpyAsync(b->d_items, items.data(), sizeof(BatchItem) * n_items,
                                       cudaMemcpyHostToDevice, st));
    if (!rc && b->n_clear) {
        rc = fail_cuda(cudaMemcpyAsync(b->d_clear_ptrs, clear_ptrs.data(), sizeof(uint64_t *) * b->n_clear,
                                       cudaMemcpyHostToDevice, st));
        if (!rc)
            rc = fail_cuda(cudaMemcpyAsync(b->d_clear_words, clear_words.data(), sizeof(uint64_t) * b->n_clear,
                                           cudaMemcpyHostToDevice, st));
    }
    // grid: resident CTAs (cooperative), capped by the configuration
    int nb = 0;
    if (!rc) rc = batch_occupancy(conf.staging, nb, b->smem);
    if (!rc && nb <= 0) rc = FALX_ERR_CUDA;
    if (!rc) {
        if (conf.ctas_per_sm > 0 && (int)conf.ctas_per_sm < nb) nb = (int)conf.ctas_per_sm;
        b->cfg.ctas_per_sm = (uint32_t)nb;
        uint64_t grid = (uint64_t)c->sm_count * (uint64_t)nb;
        if (grid > n_items) grid = n_items;
        b->grid = grid ? (int)grid : 1;
    }
    if (!rc) rc = fail_cuda(cudaStreamSynchronize(st));
    // capture the launch sequence in a graph (a capture the driver refuses
    // leaves plain stream launches)
    if (!rc) {
        cudaStream_t cs;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess) {
            bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) ok = batch_enqueue(b, cs) == FALX_OK;
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(cs, &g);
            ok = ok && ce == cudaSuccess && g;
            if (ok && cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess) {
                b->graph = g;
                b->use_graph = true;
            } else if (g) {
                cudaGraphDestroy(g);
            }
            (void)cudaGetLastError();
            cudaStreamDestroy(cs);
        }
    }
    if (rc) {
        batch_free(b);
        delete b;
        return rc;
    }
    *out = b;
    return FALX_OK;
}

int falx_batch_run(falx_batch *b, falx_doc *docs) {
    if (!b) return FALX_ERR_INVALID;
    falx_ctx *c = b->c;
    if (b->use_graph) {
        BATCH_CUDA(cudaGraphLaunch(b->exec, c->stream));
    } else {
        const int rc = batch_enqueue(b, c->stream);
        if (rc) return rc;
    }
    BATCH_CUDA(cudaStreamSynchronize(c->stream));
    int rc = FALX_OK;
    for (uint32_t d = 0; d < b->ndocs; d++) {
        const DevHeader &h = b->h_hdrs[d];
        int r = FALX_OK;
        if (h.error & ERR_TIMEOUT) r = FALX_ERR_TIMEOUT;
        else if (h.error & ERR_TMA) r = FALX_ERR_TIMEOUT;
        else if (h.error & ERR_ARENA) r = FALX_ERR_OVERFLOW;
        if (docs) {
            falx_doc &x = docs[d];
            x.n_index = h.n_struct;
            x.rows = h.n_rows;
            if (!r && ((x.index_cap && h.n_struct > x.index_cap) || (x.rows_cap && h.n_rows > x.rows_cap)))
                r = FALX_ERR_CAPACITY;
            x.status = r;
        }
        if (r && !rc) rc = r;
    }
    return rc;
}

int falx_batch_info(const falx_batch *b, falx_batch_config *cfg, uint32_t *n_items, uint32_t *grid,
                    int *graph) {
    if (!b) return FALX_ERR_INVALID;
    if (cfg) *cfg = b->cfg;
    if (n_items) *n_items = b->n_items;
    if (grid) *grid = (uint32_t)b->grid;
    if (graph) *graph = b->use_graph ? 1 : 0;
    return FALX_OK;
}

void falx_batch_destroy(falx_batch *b) {
    if (!b) return;
    cudaSetDevice(b->c->device);
    batch_free(b);
    delete b;
}

int falx_batch_tune(falx_ctx *c, falx_doc *docs, uint32_t ndocs, falx_batch_config *best, float *best_ms) {
    if (!c || (ndocs && !docs)) return FALX_ERR_INVALID;
    static const uint32_t chunks[] = {64u << 10, 256u << 10, 1u << 20, 4u << 20};
    float best_t = 3.0e38f;
    falx_batch_config bc = {};
    cudaEvent_t e0, e1;
    BATCH_CUDA(cudaEventCreate(&e0));
    BATCH_CUDA(cudaEventCreate(&e1));
    int rc = FALX_OK;
    for (uint32_t staging = 2; staging <= 3 && !rc; staging++) {
        int nb = 0;
        size_t smem = 0;
        rc = batch_occupancy(staging, nb, smem);
        for (int ctas = 1; ctas <= nb && !rc; ctas++) {
            for (uint32_t chunk : chunks) {
                falx_batch_config cf = {chunk, (uint32_t)ctas, staging};
                falx_batch *b = nullptr;
                rc = falx_batch_create(c, docs, ndocs, &cf, &b);
                if (rc) break;
                float tmin = 3.0e38f;
                for (int rep = 0; rep < 3 && !rc; rep++) {
                    cudaEventRecord(e0, c->stream);
                    rc = falx_batch_run(b, nullptr);
                    cudaEventRecord(e1, c->stream);
                    cudaEventSynchronize(e1);
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0 && ms < tmin) tmin = ms;
                }
                falx_batch_destroy(b);
                if (!rc && tmin < best_t) {
                    best_t = tmin;
                    bc = cf;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    c->batch_tuned.valid = 1;
    c->batch_tuned.chunk_bytes = bc.chunk_bytes;
    c->batch_tuned.ctas_per_sm = bc.ctas_per_sm;
    c->batch_tuned.staging = bc.staging;
    if (best) *best = bc;
    if (best_ms) *best_ms = best_t;
    return FALX_OK;
}

}  // extern "C"
