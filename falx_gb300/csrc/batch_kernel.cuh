// Batched persistent kernel (see batch.cu): work items, per-CTA slots,
// the dialect dispatch and the kernel itself, instantiated per staging
// depth in its own translation unit (batch_nb2.cu, batch_nb3.cu) so they
// compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/falx_gpu.h"
#include "tile.cuh"

namespace falx {

struct BatchItem {
    uint32_t doc;
    uint32_t tile_lo, tile_hi;  // tiles [lo, hi) of the document, in order, on one CTA
};

template <int NB>
struct BatchSmem {
    Smem<true, NB> s;
    uint32_t slot_doc[NB], slot_tile[NB], slot_valid[NB];
};

// The CTA's next (document, tile): the next tile of its current item, or
// the first tile of a newly claimed item. Thread 0 only.
__device__ __forceinline__ bool batch_next(const BatchItem *items, uint32_t n_items, uint32_t *ticket,
                                           uint32_t &item, uint32_t &tile, bool &have) {
    if (have && tile + 1 < items[item].tile_hi) {
        tile++;
        return true;
    }
    const uint32_t k = atomicAdd(ticket, 1u);
    if (k >= n_items) {
        have = false;
        return false;
    }
    item = k;
    tile = items[k].tile_lo;
    have = true;
    return true;
}

// Dialects of batched documents: the geo schemas' CSV, TSV and logfmt.
template <int NB>
__device__ __forceinline__ void batch_tile(const Params &p, Smem<true, NB> &S, uint32_t tile, uint8_t *b) {
    switch (p.dialect) {
    case FALX_CSV: process_tile<D_CSV, true, NB>(p, S, tile, b); break;
    case FALX_TSV: process_tile<D_TSV, true, NB>(p, S, tile, b); break;
    default: process_tile<D_LOGFMT, true, NB>(p, S, tile, b); break;
    }
}

template <int NB>
__global__ void __launch_bounds__(kThreads, 3) batch_kernel(const Params *docs, const BatchItem *items,
                                                         uint32_t n_items, uint32_t *ticket) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    BatchSmem<NB> &B = *reinterpret_cast<BatchSmem<NB> *>(smem_raw);
    Smem<true, NB> &S = B.s;
    const int tid = threadIdx.x;
    uint32_t item = 0, tile = 0;  // thread 0's cursor
    bool have = false;
    if (tid == 0) {
        for (int s = 0; s < NB; s++) mbar_init(&S.bar[s], 1);
        fence_mbar_init();
        for (int s = 0; s < NB; s++) {
            const bool v = batch_next(items, n_items, ticket, item, tile, have);
            B.slot_valid[s] = v;
            if (v) {
                const uint32_t d = items[item].doc;
                B.slot_doc[s] = d;
                B.slot_tile[s] = tile;
                issue_tile<true>(docs[d], tile, S.buf[s], &S.bar[s]);
            }
        }
    }
    __syncthreads();
    uint32_t phase[NB];
#pragma unroll
    for (int s = 0; s < NB; s++) phase[s] = 0;
    for (int s = 0;; s = s + 1 == NB ? 0 : s + 1) {
        if (!B.slot_valid[s]) break;
        const uint32_t d = B.slot_doc[s], t = B.slot_tile[s];
        const Params &p = docs[d];
        const bool ok = mbar_wait(&S.bar[s], phase[s], kWaitNs);
        if (__syncthreads_or(!ok || (tid == 0 && aborted(p.hdr)))) {
            if (tid == 0) {
                if (!ok) fail(p.hdr, ERR_TMA);
                // never leave a bulk copy in flight into this CTA's shared memory
                for (int k = 1; k < NB; k++) {
                    const int s2 = (s + k) % NB;
                    if (B.slot_valid[s2]) mbar_wait(&S.bar[s2], phase[s2], kWaitNs);
                }
            }
            break;
        }
        phase[s] ^= 1;
        batch_tile<NB>(p, S, t, S.buf[s]);
        __syncthreads();  // every read of buf[s] and S.* for this tile is done
        if (tid == 0) {
            const bool v = batch_next(items, n_items, ticket, item, tile, have);
            B.slot_valid[s] = v;
            if (v) {
                const uint32_t d2 = items[item].doc;
                B.slot_doc[s] = d2;
                B.slot_tile[s] = tile;
                fence_proxy_async();
                issue_tile<true>(docs[d2], tile, S.buf[s], &S.bar[s]);
            }
        }
    }
}

// Host entry points of one staging depth (defined in batch_nb<NB>.cu).
int batch_occupancy_nb2(int &blocks, size_t &smem);
int batch_occupancy_nb3(int &blocks, size_t &smem);
cudaError_t batch_launch_nb2(const cudaLaunchConfig_t &lc, void **args);
cudaError_t batch_launch_nb3(const cudaLaunchConfig_t &lc, void **args);

}  // namespace falx
