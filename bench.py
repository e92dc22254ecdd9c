"""Benchmark: device-resident parse throughput of the structural-index +
column-materialisation path on one GB300.

Workload (the csv-hash comment+quote dialect, 1 GiB, device-resident): one
step = one falx_parse call (two launches: the index + tape kernel, then the
record-parallel columns kernel) that produces the structural index
(byte-identical to the serial path), the field-byte totals and the typed
columns u32 id, City string arena, u32 population, f64 latitude and f64
longitude. Inputs are seeded synthetic documents with the workload's shapes
(falx_gb300/gen.py); 1 GiB is larger than L2, so no flush is needed.

--impl reference times the CPU port of the reference's parallel drivers
(oracle/, all host threads) on a bounded sample of the same workload.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GIB = float(1 << 30)
SCHEMA_COLS = [(0, 1), (1, 3), (3, 1), (4, 2), (5, 2)]  # u32 id, str City, u32 pop, f64 lat, f64 lon
METRIC = "device-resident parse GiB/s vs HBM peak; learned-speculative vs plain, bit-exact"
WORKLOAD = ("csv_hash 1 GiB: structural index + field bytes + typed columns "
            "(u32 id, str City, u32 population, f64 lat, f64 lon)")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Sample SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max((float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons}


STEP_KERNELS = ["index_kernel (index + tape)", "columns_kernel"]


def measured_traffic(n):
    """DRAM bytes of one step, per kernel and in total, scaled to n input
    bytes from the committed ncu capture (the traffic of every kernel grows
    in proportion to the input)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)["csv_hash_parse_step"]
        scale = n / t["input_bytes"]
        per = {k: int((v["dram_read"] + v["dram_write"]) * scale) for k, v in t["kernels"].items()}
        return sum(per.values()), per
    except Exception:
        return None, {}


def make_input(size):
    from falx_gb300 import gen

    return gen.generate(gen.CSV_HASH, size)


def cpu_sample(size):
    from falx_gb300 import gen

    return gen.generate(gen.CSV_HASH, size)


def run_cpu(data, threads):
    """One CPU step over `data`: the reference's parallel index, field bytes
    and columns drivers (port)."""
    import oracle

    oracle.index_par(data, oracle.CSV_HASH, threads)
    oracle.field_bytes(data, oracle.CSV_HASH, par_threads=threads)
    oracle.parse_columns(data, oracle.CSV_HASH, SCHEMA_COLS, par_threads=threads)


def cpu_baseline(sample_bytes, threads, budget_s=20.0):
    data = cpu_sample(sample_bytes)
    run_cpu(data, threads)  # warm-up
    t0 = time.perf_counter()
    reps = 0
    best = None
    while True:
        s = time.perf_counter()
        run_cpu(data, threads)
        dt = time.perf_counter() - s
        best = dt if best is None else min(best, dt)
        reps += 1
        if time.perf_counter() - t0 > budget_s or reps >= 5:
            break
    return data.size / GIB / best, data.size


def bench_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = args.cpu_sample
    t_total = []
    from falx_gb300 import gen

    data = gen.generate(gen.CSV_HASH, sample)
    for _ in range(args.warmup):
        run_cpu(data, threads)
    for _ in range(args.steps):
        s = time.perf_counter()
        run_cpu(data, threads)
        t_total.append(time.perf_counter() - s)
    sec = sum(t_total) / len(t_total)
    v = data.size / GIB / sec
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GiB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": WORKLOAD, "input": "host memory; each step a CPU sample of the workload",
                       "sample_bytes": int(data.size)},
            "cpu_baseline": {"value": round(v, 4), "unit": "GiB/s", "cores": threads, "kind": "port",
                             "sample": "%d-byte csv_hash document, full index + field bytes + columns" % data.size},
            "e2e": {"value": round(v, 4), "unit": "GiB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def bench_gpu(args):
    import ctypes

    import numpy as np
    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    host = make_input(args.size)
    n = int(host.size)
    pinned = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = host
    data = pinned.to("cuda", non_blocking=False)

    eng = fx.Engine(local)
    schema = fx.Schema(fx.CSV_HASH, SCHEMA_COLS)
    cs = schema.to_c()
    stream = torch.cuda.current_stream()
    eng.lib.falx_set_stream(eng.ctx, ctypes.c_void_p(stream.cuda_stream))
    eng.lib.falx_set_option(eng.ctx, _lib.OPT_TIMING, 1)  # CUDA events around each launch of a step
    kms = (ctypes.c_float * 4)()
    kernel_ms = [[] for _ in STEP_KERNELS]

    # Size outputs from a first pass.
    idx_cap = n // 4 + 1024
    rows_cap = n // 8 + 64
    str_cap = n
    index = torch.empty(idx_cap, dtype=torch.int32, device="cuda")
    bufs = eng.alloc_columns(schema, rows_cap, str_cap)
    cols = eng.columns_struct(schema, bufs, rows_cap, str_cap)
    fb = _lib.falx_field_byte_stats()
    out = _lib.falx_outputs()
    out.index = index.data_ptr()
    out.index_cap = idx_cap
    out.columns = ctypes.pointer(cols)
    out.field_bytes = ctypes.pointer(fb)

    def step():
        rc = eng.lib.falx_parse(eng.ctx, ctypes.byref(cs), ctypes.c_void_p(data.data_ptr()), n, ctypes.byref(out))
        _lib.check(rc, "falx_parse")

    step()
    n_struct, rows = out.n_index, cols.rows
    str_len = cols.cols[1].str_len
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    per = []
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            per.append(ev0.elapsed_time(ev1))
            if eng.lib.falx_last_timings(eng.ctx, kms, 4) == len(STEP_KERNELS):
                for k in range(len(STEP_KERNELS)):
                    kernel_ms[k].append(kms[k])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    ms = sum(per) / len(per)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = n * world / GIB / (ms / 1e3)

    # Algorithmic bytes per launch: input + index + columns + validity + string offsets/arena.
    words = (rows + 63) // 64
    algo = n + 4 * n_struct + rows * (4 + 4 + 8 + 8) + 5 * words * 8 + 4 * (rows + 1) + str_len
    peak, peak_kind = peaks()
    achieved = algo / (ms / 1e3) / 1e9
    traffic, traffic_per = measured_traffic(n)
    kernels = []
    for name, ts in zip(STEP_KERNELS, kernel_ms):
        if not ts:
            continue
        kt = sum(ts) / len(ts)
        ent = {"name": name, "ms": round(kt, 4), "share": round(kt / ms, 4)}
        if name in traffic_per:
            ent["dram_bytes"] = traffic_per[name]
            ent["dram_gbs"] = round(traffic_per[name] / (kt / 1e3) / 1e9, 1)
        kernels.append(ent)

    # End to end through the host-buffer C ABI entry point; input and output
    # buffers in pinned host memory.
    def pinned_np(count, dtype):
        t = torch.empty(count * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
        return t.numpy().view(dtype)

    h_index = pinned_np(idx_cap, np.uint32)
    h_vals = []
    hcols = _lib.falx_columns()
    hcols.rows_cap = rows_cap
    for k, (f, t) in enumerate(SCHEMA_COLS):
        if t == fx.STR:
            v = pinned_np(rows_cap + 1, np.int32)
            sd = pinned_np(str_cap, np.uint8)
            hcols.cols[k].str_data = sd.ctypes.data
            hcols.cols[k].str_cap = str_cap
        else:
            v = pinned_np(rows_cap, np.float64 if t == fx.F64 else np.uint32)
            sd = None
        valid = pinned_np((rows_cap + 63) // 64, np.uint64)
        hcols.cols[k].values = v.ctypes.data
        hcols.cols[k].valid = valid.ctypes.data
        h_vals.append((v, valid, sd))
    hfb = _lib.falx_field_byte_stats()
    hout = _lib.falx_outputs()
    hout.index = h_index.ctypes.data
    hout.index_cap = idx_cap
    hout.columns = ctypes.pointer(hcols)
    hout.field_bytes = ctypes.pointer(hfb)
    src = pinned.numpy()

    def e2e_step():
        rc = eng.lib.falx_parse_host(eng.ctx, ctypes.byref(cs), ctypes.c_void_p(src.ctypes.data), n,
                                     ctypes.byref(hout))
        _lib.check(rc, "falx_parse_host")

    e2e_step()
    # median of several calls: the host link and host memory are shared with
    # other jobs on the machine, so single calls can be slow
    e2e_t = []
    for _ in range(max(5, min(args.steps, 9))):
        s = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - s)
    e2e_s = float(np.median(e2e_t))
    d2h = 4 * n_struct + rows * (4 + 4 + 8 + 8) + 5 * words * 8 + 4 * (rows + 1) + str_len
    e2e = {"value": round(n / GIB / e2e_s, 4), "unit": "GiB/s", "h2d_bytes_per_step": n, "d2h_bytes_per_step": d2h,
           "ms_per_step": round(e2e_s * 1e3, 3), "ms_min_max": [round(min(e2e_t) * 1e3, 3), round(max(e2e_t) * 1e3, 3)],
           "calls": len(e2e_t)}

    spec = None if args.no_spec else bench_speculation(eng, args)
    batched = None if args.no_batch else bench_batch(eng, args)

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        v, sb = cpu_baseline(args.cpu_sample, threads)
        cpu = {"value": round(v, 4), "unit": "GiB/s", "cores": threads, "kind": "port",
               "sample": "%d-byte csv_hash document: parallel index + field bytes + columns" % sb}
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "GiB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "input": "device-resident (value); pinned host buffers (e2e)",
                   "bytes": n, "structurals": int(n_struct), "rows": int(rows), "tile_bytes": 16384,
                   "l2": "input 1 GiB > L2, no flush", "parallelism": "replicas" if world > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes": int(algo),
                     "scope": "the whole step (index + tape kernel, columns kernel): algorithmic bytes of the "
                              "path / step time; traffic = DRAM bytes of the step's kernels"},
        "kernels": kernels,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": args.steps * len(STEP_KERNELS),
        "clocks": clk.summary(),
        "field_bytes": {"fields": fb.fields, "bytes": fb.bytes},
        "learned_speculation": spec,
        "batched": batched,
        "wall_s": round(wall, 3),
    }
    print(json.dumps(line))
    eng.close()
    if dist:
        dist.destroy_process_group()


def bench_speculation(eng, args):
    """Learned speculation on the adversarial csv_hash workload (1 GiB,
    device-resident): the plain structural index against predict + the
    speculative index with a model trained here on separately seeded
    documents, the constant 'outside any region' guess beside them; outputs
    are compared for identity."""
    import ctypes

    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib, gen, speculation

    model, info = speculation.train_model(eng, train_bytes=512 << 20, epochs=3, stride=512)
    calib = gen.generate(gen.ADVERSARIAL, 128 << 20, seed=speculation.EVAL_SEED)
    conf = speculation.calibrate_confidence(eng, model, calib)
    host = gen.generate(gen.ADVERSARIAL, args.size)
    data = torch.from_numpy(host.copy()).cuda()
    n = data.numel()
    cap = n // 3
    idx = torch.empty(cap, dtype=torch.int32, device="cuda")
    idx2 = torch.empty(cap, dtype=torch.int32, device="cuda")
    cnt, cnt2 = ctypes.c_uint64(), ctypes.c_uint64()
    st = _lib.falx_spec_stats()
    ptr = ctypes.c_void_p(data.data_ptr())

    def plain():
        _lib.check(eng.lib.falx_index_structurals(eng.ctx, fx.CSV_HASH, ptr, n, ctypes.c_void_p(idx.data_ptr()), cap,
                                                  ctypes.byref(cnt)), "falx_index_structurals")

    def spec(m):
        _lib.check(eng.lib.falx_index_structurals_speculative(eng.ctx, m, fx.CSV_HASH, ptr, n,
                                                              ctypes.c_void_p(idx2.data_ptr()), cap,
                                                              ctypes.byref(cnt2), ctypes.byref(st)),
                   "falx_index_structurals_speculative")

    reps = max(3, min(args.steps, 10))
    t_plain = speculation.time_index(eng, plain, reps)
    t_const = speculation.time_index(eng, lambda: spec(None), reps)
    wrong_const = st.mispredicted
    t_spec = speculation.time_index(eng, lambda: spec(model.ptr), reps)
    wrong, tiles = st.mispredicted, st.tiles
    identical = cnt.value == cnt2.value and bool(torch.equal(idx[: cnt.value], idx2[: cnt2.value]))
    pred = model.predict_tiles(data)
    hedged = int((pred == 255).sum())
    t_pred = speculation.time_index(eng, lambda: model.predict_tiles(data), reps)
    gib = n / GIB
    return {
        "workload": "adversarial csv_hash 1 GiB device-resident (20% quoted cells up to 4 KiB with '#' and "
                    "newlines, 5% comment lines with '\"'): structural index",
        "plain": {"value": round(gib / (t_plain / 1e3), 3), "unit": "GiB/s", "ms": round(t_plain, 4)},
        "speculative": {"value": round(gib / (t_spec / 1e3), 3), "unit": "GiB/s", "ms": round(t_spec, 4),
                        "predict_ms": round(t_pred, 4)},
        "speedup_vs_plain": round(t_plain / t_spec, 4),
        "constant_guess": {"value": round(gib / (t_const / 1e3), 3), "unit": "GiB/s",
                           "mispredicted_tiles": int(wrong_const)},
        "tiles": int(tiles), "mispredicted_tiles": int(wrong), "misprediction_rate": round(wrong / max(tiles, 1), 6),
        "rerun_fraction": round(wrong / max(tiles, 1), 6), "hedged_tiles": hedged, "confidence": conf,
        "output_identical": identical, "training": info,
    }


def bench_batch(eng, args):
    """Batched documents: 4096 seeded documents (sizes log-uniform over
    4 KiB-64 MiB scaled to 6 GiB in total; 50% CSV, 25% TSV, 25% logfmt),
    one persistent launch per run from a CUDA graph with the autotuned
    configuration; outputs per document: structural index and lat / lon f64
    columns. Beside it: the same documents through one falx_parse call each."""
    import ctypes

    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib, batch, speculation

    ndocs, total = 4096, 6 << 30
    sizes = batch.mixed_sizes(ndocs, total)
    dialects = batch.mixed_dialects(ndocs)
    host, offs, lens = batch.generate(sizes, dialects)
    data = torch.from_numpy(host).cuda()
    del host
    b = batch.Batch(eng, data, offs, lens, dialects)
    tuned = batch.tune(eng, b)
    b.close()
    b = batch.Batch(eng, data, offs, lens, dialects)
    info = b.info()
    reps = max(3, min(args.steps, 10))
    t = speculation.time_index(eng, b.run, reps)
    n_in = int(lens.sum())
    n_index = sum(int(b.docs[k].n_index) for k in range(ndocs))
    rows = sum(int(b.docs[k].rows) for k in range(ndocs))
    algo = n_in + 4 * n_index + 16 * rows + 2 * sum((int(b.docs[k].rows) + 63) // 64 * 8 for k in range(ndocs))
    peak, peak_kind = peaks()
    schemas = {d: fx.Schema(d, [(f0, fx.F64), (f1, fx.F64)]).to_c() for d, (f0, f1) in batch.GEO_FIELDS.items()}

    def per_document():
        for k in range(ndocs):
            x = b.docs[k]
            if x.len == 0:
                continue
            cols = _lib.falx_columns()
            cols.rows_cap = x.rows_cap
            cols.cols[0].values, cols.cols[0].valid = x.col0, x.valid0
            cols.cols[1].values, cols.cols[1].valid = x.col1, x.valid1
            out = _lib.falx_outputs()
            out.index, out.index_cap = x.index, x.index_cap
            out.columns = ctypes.pointer(cols)
            _lib.check(eng.lib.falx_parse(eng.ctx, ctypes.byref(schemas[x.dialect]), ctypes.c_void_p(x.data), x.len,
                                          ctypes.byref(out)), "falx_parse")

    t_one = speculation.time_index(eng, per_document, 2)
    b.close()
    gib = n_in / GIB
    return {
        "workload": "4096 documents, 6 GiB (log-uniform sizes 4 KiB-64 MiB scaled to 6 GiB; 50% CSV, 25% TSV, "
                    "25% logfmt): per-document structural index + lat/lon f64 columns",
        "value": round(gib / (t / 1e3), 3), "unit": "GiB/s", "ms": round(t, 3), "bytes": n_in,
        "structurals": n_index, "rows": rows, "items": info["items"], "grid": info["grid"],
        "cuda_graph": info["graph"], "tuned": tuned,
        "roofline": {"bound": "hbm", "achieved": round(algo / (t / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(algo / (t / 1e3) / 1e9 / peak, 4), "algorithmic_bytes": algo,
                     "peak_kind": peak_kind},
        "per_document_calls": {"value": round(gib / (t_one / 1e3), 3), "unit": "GiB/s", "ms": round(t_one, 3)},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="falx_gb300")
    ap.add_argument("--size", type=int, default=1 << 30)
    ap.add_argument("--cpu-sample", type=int, default=64 << 20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-spec", action="store_true", help="skip the learned-speculation comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-documents run")
    args = ap.parse_args()
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_gpu(args)


if __name__ == "__main__":
    main()
