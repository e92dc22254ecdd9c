// Engine context (falx_ctx of the C ABI): device, stream, look-back
// scratch and tuned launch parameters. Shared by the translation units of
// the engine library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "tile.cuh"

namespace falx {
struct NdjsonAcc;
}

// Autotuned configuration of batched launches (falx_batch_tune).
struct falx_batch_tuning {
    int valid = 0;
    uint32_t chunk_bytes = 0;  // documents up to this size run whole on one CTA
    uint32_t ctas_per_sm = 0;
    uint32_t staging = 0;      // tile buffers in flight per CTA
};

struct falx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    int blocks_per_sm[5][2] = {};
    int blocks_per_sm_spec[5] = {};
    int blocks_per_sm_pass[5] = {};  // index_pass_kernel
    int old_index = 0;               // FALX_INDEX_KERNEL=tile: plain scans use index_kernel instead
    int ctas_per_sm = 0;  // FALX_CTAS_PER_SM caps the persistent grid (tuning)
    falx::TileStatus *status = nullptr;
    falx::ArenaStatus *astatus = nullptr;
    uint32_t status_cap = 0;
    uint32_t epoch = 0;
    falx::DevHeader *hdr = nullptr;   // device
    falx::DevHeader *hhdr = nullptr;  // pinned host mirror
    // staging for the host-buffer entry points
    uint8_t *dev_in = nullptr;
    uint64_t dev_in_cap = 0;
    void *dev_out = nullptr;
    uint64_t dev_out_cap = 0;
    falx::NdjsonAcc *nd_acc = nullptr;   // device
    falx::NdjsonAcc *nd_host = nullptr;  // pinned
    // entry-region predictor: activations and classes for `mlp_cap` samples
    uint8_t *mlp_scratch = nullptr;
    uint64_t mlp_cap = 0;
    uint8_t *pred = nullptr;  // predicted entry state per tile
    uint64_t pred_cap = 0;
    falx_batch_tuning batch_tuned;  // last autotuned batched-launch configuration
    void *summary_dev = nullptr;    // shard summary result (device)
    // rows from the tape: scratch tape, per-record-block sums
    int rows_path = 0;              // 0: index + tape, then columns_kernel; 1: fused tile pass
    uint32_t *tape_seps = nullptr;
    uint64_t tape_seps_cap = 0;     // bytes
    uint64_t *tape_ends = nullptr;
    uint64_t tape_ends_cap = 0;     // bytes
    // host-buffer parse: the structural index is copied back on its own
    // stream while the columns kernel runs
    cudaStream_t copy_stream = nullptr;
    uint32_t *host_index = nullptr;
    uint64_t host_index_cap = 0;
    bool host_index_done = false;
    // host-buffer parse: the input is copied in chunks on copy_stream, each
    // followed by a flag write; the first index launch waits per tile for
    // its chunk instead of for the whole copy
    uint32_t *arrive = nullptr;      // device, kMaxArriveChunks flags
    uint32_t arrive_tag = 0;
    void *write_value = nullptr;     // cuStreamWriteValue32, from the driver
    int write_value_state = 0;       // 0 not looked up, 1 available, -1 not
    cudaEvent_t in_free = nullptr;   // earlier work on `stream` is done with the input buffer
    const uint32_t *pend_arrive = nullptr;
    uint32_t pend_tag = 0, pend_chunk_tiles = 0;
    void *rec_sums = nullptr;       // look-back records of the columns pass
    uint64_t rec_sums_cap = 0;      // bytes
    uint32_t col_epoch = 0;         // their tag
    uint64_t stall_test_ns = 0;     // falx_test_stalled_lookback
    int col_grid[5][2] = {};        // persistent columns grid per dialect, without / with the count-sum sink
    // pipelined host-buffer parse: input chunks copied in, parsed and their
    // outputs copied out while the next chunks are still on their way
    int pipeline = 1;               // FALX_OPT_PIPELINE
    const void *pipe = nullptr;     // the call's host buffers while one runs (falx_parse_host)
    bool pipe_done = false;         // the outputs were copied back chunk by chunk
    cudaStream_t out_stream = nullptr;
    uint32_t *pipe_dev = nullptr;   // seed records, tickets and per-chunk totals
    unsigned long long *pipe_host = nullptr;  // pinned copies of the seed records and per-chunk totals
    cudaEvent_t pipe_ev[32] = {};   // per chunk: input landed, results ready
    // bgzf inflate: block table, per-block status and failure count
    void *gz_scratch = nullptr;
    uint64_t gz_cap = 0;
    int gz_grid = 0;
    uint8_t *gz_comp = nullptr;     // falx_parse_gz_host: the compressed stream in device memory
    uint64_t gz_comp_cap = 0;
    unsigned long long *gz_host = nullptr;  // pinned: members that failed to inflate
    // per-launch timing of the last rows call (FALX_OPT_TIMING)
    int timing = 0;
    cudaEvent_t ev[5] = {};
    float last_ms[4] = {};
    int last_n = 0;
};

namespace falx {
// Inflate every member of a bgzf stream into `out` on the context's stream
// without waiting (inflate.cu). *counters (device): [0] members that
// failed, [1] the member ticket; *status (device): per member.
int gz_launch(falx_ctx *c, const uint8_t *comp, uint64_t comp_len, const falx_gz_block *blocks, uint64_t n_blocks,
              uint8_t *out, uint64_t out_cap, unsigned long long **counters, int32_t **status);
}  // namespace falx
