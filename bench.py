"""Benchmark: device-resident parse throughput of the structural-index +
column-materialisation path on one GB300.

Workload (the csv-hash comment+quote dialect, 1 GiB, device-resident): one
step = one falx_parse call (two launches: the index + tape kernel, then the
record-parallel columns kernel) that produces the structural index
(byte-identical to the serial path), the field-byte totals and the typed
columns u32 id, City string arena, u32 population, f64 latitude and f64
longitude. Inputs are seeded synthetic documents with the workload's shapes
(falx_gb300/gen.py); 1 GiB is larger than L2, so no flush is needed.

Beside the headline step the same JSON line carries the csv-geo config
(64 MiB, index + lat/lon columns + fused count/sum; L2 flushed between
steps), the NDJSON config (1 GiB, sum(id + nested.score)), learned
speculation and the batched documents. The CPU-baseline leg runs the CPU
port of the reference's parallel drivers (oracle/, all host threads) over
the same full inputs; its outputs are compared with the GPU's, and the
result is the line's `parity` object.

--impl reference times that CPU port on the headline workload, full size.
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


STEP_KERNELS = ["index_pass_kernel (index + tape)", "columns_kernel"]


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


def run_cpu(data, threads):
    """One CPU step over `data`: the port of the reference's parallel drivers
    (chunk transfer functions, serial composition, then one pass per chunk
    feeding the index, field-byte and column sinks). Returns the outputs."""
    import oracle

    return oracle.parse_par(data, oracle.CSV_HASH, SCHEMA_COLS, threads)


def cpu_isa():
    import platform

    m = platform.machine()
    return "aarch64 NEON + PMULL" if m == "aarch64" else "%s portable 64-bit SWAR" % m


def timed_best(fn, budget_s=20.0, max_reps=3):
    """Best wall time of fn() after one warm-up call, and the last result."""
    out = fn()
    t0 = time.perf_counter()
    best = None
    for _ in range(max_reps):
        s = time.perf_counter()
        out = fn()
        dt = time.perf_counter() - s
        best = dt if best is None else min(best, dt)
        if time.perf_counter() - t0 > budget_s:
            break
    return best, out


def compare_columns(got_cols, want_cols, schema_cols, rows_got, rows_want, mism):
    """Columns bit-for-bit (values, validity, offsets, arena)."""
    import numpy as np

    if rows_got != rows_want:
        mism.append("rows %d != %d" % (rows_got, rows_want))
        return
    for k, (f, t) in enumerate(schema_cols):
        g, w = got_cols[k], want_cols[k]
        if not np.array_equal(g["valid"], w["valid"]):
            mism.append("column %d validity" % k)
        if t == 3:
            if not np.array_equal(g["offsets"], w["offsets"]):
                mism.append("column %d offsets" % k)
            if g["data"] != w["data"]:
                mism.append("column %d arena" % k)
        elif not np.array_equal(g["values"].view(np.uint8), w["values"].view(np.uint8)):
            mism.append("column %d values" % k)


def host_columns(schema_cols, bufs, rows, str_lens):
    """The GPU's column buffers as NumPy (copied once, after timing)."""
    import numpy as np

    out = []
    words = (rows + 63) // 64
    for k, (f, t) in enumerate(schema_cols):
        v, valid, sd = bufs[k]
        c = {"valid": valid[:words].cpu().numpy().view(np.uint64)}
        if t == 3:
            c["offsets"] = v[: rows + 1].cpu().numpy().view(np.int32)
            c["data"] = sd[: str_lens[k]].cpu().numpy().tobytes()
        elif t == 1:
            c["values"] = v[:rows].cpu().numpy().view(np.uint32)
        else:
            c["values"] = v[:rows].cpu().numpy().view(np.uint64)
        out.append(c)
    return out


def bench_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t_total = []
    import oracle

    data = oracle.generate(oracle.GEN_CSV_HASH, args.size)
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
            "config": {"workload": WORKLOAD, "input": "host memory; each step the whole workload",
                       "bytes": int(data.size)},
            "cpu_baseline": {"value": round(v, 4), "unit": "GiB/s", "cores": threads, "kind": "port",
                             "isa": cpu_isa(), "same_config": True,
                             "sample": "the full %d-byte csv_hash document: index + field bytes + columns, one pass "
                                       "per chunk" % data.size},
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
    spread = [round(min(per), 4), round(sorted(per)[len(per) // 2], 4), round(max(per), 4)]
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
    # the same calls without the pipeline: one copy in, the parse, the copies back
    eng.lib.falx_set_option(eng.ctx, _lib.OPT_PIPELINE, 0)
    whole_t = []
    for _ in range(3):
        s = time.perf_counter()
        e2e_step()
        whole_t.append(time.perf_counter() - s)
    eng.lib.falx_set_option(eng.ctx, _lib.OPT_PIPELINE, 1)
    d2h = 4 * n_struct + rows * (4 + 4 + 8 + 8) + 5 * words * 8 + 4 * (rows + 1) + str_len
    e2e = {"value": round(n / GIB / e2e_s, 4), "unit": "GiB/s", "h2d_bytes_per_step": n, "d2h_bytes_per_step": d2h,
           "ms_per_step": round(e2e_s * 1e3, 3), "ms_min_max": [round(min(e2e_t) * 1e3, 3), round(max(e2e_t) * 1e3, 3)],
           "calls": len(e2e_t),
           "form": ("pipelined: input chunks of 16, 32, 64 MiB, then about 96 MiB, then 64, 32, 16 MiB, each "
                    "copied in, parsed and copied back while the others move"),
           "whole_input": {"value": round(n / GIB / float(np.median(whole_t)), 4), "unit": "GiB/s",
                           "ms_per_step": round(float(np.median(whole_t)) * 1e3, 3)}}

    # The step's outputs, copied back once after timing, for the parity check.
    gpu_out = None
    if not args.no_cpu and rank == 0:
        gpu_out = {"index": index[:n_struct].cpu().numpy().view(np.uint32), "field_bytes": (fb.fields, fb.bytes),
                   "rows": int(rows),
                   "columns": host_columns(SCHEMA_COLS, bufs, int(rows),
                                           [cols.cols[k].str_len for k in range(len(SCHEMA_COLS))])}
    del h_index, h_vals

    geo = None if args.no_configs else bench_geo(eng, args, rank)
    nd = None if args.no_configs else bench_ndjson(eng, args, rank)
    gz = None if args.no_configs else bench_gz(eng, args, rank)
    spec = None if args.no_spec else bench_speculation(eng, args)
    batched = None if args.no_batch else bench_batch(eng, args)

    if rank != 0:
        return
    cpu = None
    parity = {"status": "unchecked", "why": "--no-cpu"}
    if not args.no_cpu:
        # CPU baseline on the full workload; its outputs check the GPU's.
        threads = os.cpu_count() or 1
        best, ref = timed_best(lambda: run_cpu(host, threads))
        cpu = {"value": round(n / GIB / best, 4), "unit": "GiB/s", "cores": threads, "kind": "port",
               "isa": cpu_isa(), "same_config": True,
               "sample": "the full %d-byte csv_hash document: index + field bytes + columns, one pass per chunk" % n}
        mism = []
        if gpu_out["index"].size != ref["index"].size or not np.array_equal(gpu_out["index"], ref["index"]):
            mism.append("structural index (%d vs %d entries)" % (gpu_out["index"].size, ref["index"].size))
        if tuple(gpu_out["field_bytes"]) != tuple(ref["field_bytes"]):
            mism.append("field bytes %s != %s" % (gpu_out["field_bytes"], ref["field_bytes"]))
        compare_columns(gpu_out["columns"], ref["columns"], SCHEMA_COLS, gpu_out["rows"], ref["rows"], mism)
        parity = {"status": "ok" if not mism else "mismatch", "mismatches": mism,
                  "checked": "structural index, field bytes, rows, every column's values / validity / "
                             "offsets / arena, bit for bit against the CPU port on the same 1 GiB input"}
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "GiB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "input": "device-resident (value); pinned host buffers (e2e)",
                   "bytes": n, "structurals": int(n_struct), "rows": int(rows), "tile_bytes": 16384,
                   "l2": "input 1 GiB > L2, no flush", "parallelism": "replicas" if world > 1 else "single",
                   "step_ms_min_median_max": spread},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes": int(algo),
                     "scope": "the whole step (index + tape kernel, columns kernel): algorithmic bytes of the "
                              "path / step time; traffic = DRAM bytes of the step's kernels"},
        "kernels": kernels,
        "cpu_baseline": cpu,
        "parity": parity,
        "e2e": e2e,
        "gpu_launches": args.steps * len(STEP_KERNELS),
        "clocks": clk.summary(),
        "field_bytes": {"fields": fb.fields, "bytes": fb.bytes},
        "csv_geo": geo,
        "ndjson": nd,
        "bgzf": gz,
        "learned_speculation": spec,
        "batched": batched,
        "wall_s": round(wall, 3),
    }
    print(json.dumps(line))
    eng.close()
    if dist:
        dist.destroy_process_group()


def flush_l2(buf):
    """Write a buffer larger than L2 (129 MB) on the current stream."""
    buf.zero_()


def bench_geo(eng, args, rank):
    """csv-geo (CSV dialect, header row, 64 MiB, device-resident): one
    falx_parse per step giving the structural index, lat / lon f64 columns
    and the fused count / sum (csv_geo.rs:1513 parse_csv_geo_stats_par). The
    input fits L2, so L2 is flushed before every timed step. The CPU port
    runs the same work on the same input; outputs are compared."""
    import ctypes

    import numpy as np
    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib, gen

    size = 64 << 20
    host = gen.generate(gen.CSV_GEO, size)
    n = int(host.size)
    data = torch.from_numpy(host.copy()).cuda()
    cols_spec = [(4, fx.F64), (5, fx.F64)]
    schema = fx.Schema(fx.CSV, cols_spec)
    cs = schema.to_c()
    idx_cap, rows_cap = n // 4 + 1024, n // 8 + 64
    index = torch.empty(idx_cap, dtype=torch.int32, device="cuda")
    bufs = eng.alloc_columns(schema, rows_cap, 0)
    cols = eng.columns_struct(schema, bufs, rows_cap, 0)
    st = _lib.falx_geo_stats()
    out = _lib.falx_outputs()
    out.index, out.index_cap = index.data_ptr(), idx_cap
    out.columns = ctypes.pointer(cols)
    out.stats = ctypes.pointer(st)
    out.stats_fields[0], out.stats_fields[1] = 4, 5
    stream = torch.cuda.current_stream()
    eng.lib.falx_set_stream(eng.ctx, ctypes.c_void_p(stream.cuda_stream))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step():
        _lib.check(eng.lib.falx_parse(eng.ctx, ctypes.byref(cs), ctypes.c_void_p(data.data_ptr()), n,
                                      ctypes.byref(out)), "falx_parse")

    for _ in range(max(3, args.warmup)):
        step()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per = []
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            per.append(ev0.elapsed_time(ev1))
    ms = sum(per) / len(per)
    n_struct, rows = int(out.n_index), int(cols.rows)
    words = (rows + 63) // 64
    algo = n + 4 * n_struct + 16 * rows + 2 * 8 * words
    peak, peak_kind = peaks()
    res = {"workload": "csv-geo 64 MiB (CSV dialect, header row, 5% quoted City cells): structural index + "
                       "lat / lon f64 columns + fused count / sum",
           "value": round(n / GIB / (ms / 1e3), 3), "unit": "GiB/s", "ms": round(ms, 4), "bytes": n,
           "structurals": n_struct, "rows": rows, "l2": "flushed before every step (512 MiB write)",
           "roofline": {"bound": "hbm", "achieved": round(algo / (ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(algo / (ms / 1e3) / 1e9 / peak, 4), "algorithmic_bytes": algo,
                        "peak_kind": peak_kind},
           "stats": {"records": st.records, "values": list(st.values), "checksum": [hex(x) for x in st.checksum],
                     "sum_e6": list(st.sum_e6), "sum_f64": list(st.sum_f64)},
           "clocks": clk.summary()}
    if rank != 0 or args.no_cpu:
        return res
    import oracle

    g_idx = index[:n_struct].cpu().numpy().view(np.uint32)
    g_cols = host_columns(cols_spec, bufs, rows, [0, 0])
    threads = os.cpu_count() or 1

    def cpu_run():
        r = oracle.parse_par(host, oracle.CSV, cols_spec, threads, field_bytes=False, stats_fields=(4, 5))
        return r["index"], r["rows"], r["columns"], r["stats"]

    best, (w_idx, w_rows, w_cols, w_st) = timed_best(cpu_run)
    fold = oracle.geo_stats(host, oracle.CSV, 4, 5).fold  # the sequential fold, row order
    mism = []
    if not np.array_equal(g_idx, w_idx):
        mism.append("structural index")
    compare_columns(g_cols, w_cols, cols_spec, rows, w_rows, mism)
    if st.records != w_st.records or list(st.values) != list(w_st.values) or \
            list(st.checksum) != list(w_st.checksum) or list(st.sum_e6) != list(w_st.sum_e6):
        mism.append("count / sum stats")
    for k in range(2):
        if abs(st.sum_f64[k] - fold[k]) > 1e-12 * max(1.0, abs(fold[k])):
            mism.append("sum_f64[%d] beyond 1e-12 relative of the sequential fold" % k)
    res["parity"] = {"status": "ok" if not mism else "mismatch", "mismatches": mism,
                     "checked": "index, lat / lon values and validity bit for bit; records, values, bit checksums "
                                "and exact e6 sums equal; f64 sums within 1e-12 relative of the sequential fold"}
    res["cpu_baseline"] = {"value": round(n / GIB / best, 4), "unit": "GiB/s", "cores": threads, "kind": "port",
                           "isa": cpu_isa(), "sample": "the same 64 MiB input: index + lat / lon columns + count / "
                                                       "sum, one pass per chunk"}
    return res


def bench_ndjson(eng, args, rank):
    """NDJSON (1 GiB, device-resident): records and sum(id + nested.score)
    as exact fixed-point totals and an f64 total per step
    (ndjson.rs:726 parse_ndjson_id_score_par, JSON-aware). The CPU port's
    JSON-aware sink runs on the same input; totals are compared."""
    import torch

    from falx_gb300 import gen

    host = gen.generate(gen.NDJSON, args.size)
    n = int(host.size)
    data = torch.from_numpy(host.copy()).cuda()
    stream = torch.cuda.current_stream()
    eng._sync_stream()
    for _ in range(max(3, args.warmup)):
        r = eng.ndjson_id_score(data)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per = []
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            ev0.record(stream)
            r = eng.ndjson_id_score(data)
            ev1.record(stream)
            ev1.synchronize()
            per.append(ev0.elapsed_time(ev1))
    ms = sum(per) / len(per)
    peak, peak_kind = peaks()
    res = {"workload": "NDJSON 1 GiB (id int64 < 2^40, name with escapes, nested.score decimal with 1-6 "
                       "fraction digits, tags, active; 0-2 spaces around ':' and ','): records, sum(id + "
                       "nested.score) exact and f64",
           "value": round(n / GIB / (ms / 1e3), 3), "unit": "GiB/s", "ms": round(ms, 4), "bytes": n,
           "records": int(r.records), "total_f64": r.total_f64, "l2": "input 1 GiB > L2, no flush",
           "roofline": {"bound": "hbm", "achieved": round(n / (ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(n / (ms / 1e3) / 1e9 / peak, 4), "algorithmic_bytes": n,
                        "peak_kind": peak_kind},
           "clocks": clk.summary()}
    if rank != 0 or args.no_cpu:
        return res
    import oracle

    threads = os.cpu_count() or 1
    best, want = timed_best(lambda: oracle.ndjson_json(host, threads=threads))
    mism = []
    if want is None:
        mism.append("the CPU sink rejected the input")
    else:
        if r.records != want["records"] or r.sum_id != want["sum_id"] or r.sum_score_e6 != want["sum_score_e6"]:
            mism.append("records / sums")
        if r.total_e6 != want["total_e6"]:
            mism.append("exact total")
        if abs(r.total_f64 - want["total_f64"]) > 1e-12 * max(1.0, abs(want["total_f64"])):
            mism.append("f64 total beyond 1e-12 relative")
    res["parity"] = {"status": "ok" if not mism else "mismatch", "mismatches": mism,
                     "checked": "records, wrapping id and score sums, exact 128-bit total; f64 total within "
                                "1e-12 relative"}
    res["cpu_baseline"] = {"value": round(n / GIB / best, 4), "unit": "GiB/s", "cores": threads, "kind": "port",
                           "sample": "the same 1 GiB input, JSON-aware sink, lines split across the threads"}
    return res


def bench_gz(eng, args, rank):
    """bgzf input (bgzf.rs:538 parse_gz_par; examples/gpu_pipeline.rs): the
    1 GiB csv_hash document as a bgzf stream (zlib level 6, 65280-byte
    members). Device-resident compressed bytes: one step = the inflate
    kernel (every member at once) then falx_parse over the text in place
    (index + field bytes + columns). The inflate kernel is also timed alone.
    End to end: the compressed bytes from pinned host memory, the step, the
    columns and index back. The CPU port inflates the members on all host
    threads and parses the text; its output is compared with the GPU's."""
    import ctypes

    import numpy as np
    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib, bgzf

    host = make_input(args.size)
    n = int(host.size)
    t0 = time.perf_counter()
    comp = bgzf.compress(host.tobytes(), 6, threads=os.cpu_count() or 8)
    comp_s = time.perf_counter() - t0
    blocks, total = bgzf.scan(comp)
    assert total == n
    pinned = torch.empty(len(comp), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = np.frombuffer(comp, dtype=np.uint8)
    dcomp = pinned.to("cuda")
    text = torch.empty(n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    eng._sync_stream()
    schema = fx.Schema(fx.CSV_HASH, SCHEMA_COLS)
    bptr = blocks.ctypes.data_as(ctypes.c_void_p)
    failed = ctypes.c_uint64()

    def inflate():
        _lib.check(eng.lib.falx_bgzf_inflate(eng.ctx, ctypes.c_void_p(dcomp.data_ptr()), dcomp.numel(), bptr,
                                             len(blocks), ctypes.c_void_p(text.data_ptr()), n, None,
                                             ctypes.byref(failed)), "falx_bgzf_inflate")

    res_box = {}

    def step():
        inflate()
        res_box["r"] = eng.parse_all(text, schema, stats_fields=None)

    for _ in range(max(3, args.warmup)):
        step()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per, per_inf = [], []
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            ev0.record(stream)
            inflate()
            ev1.record(stream)
            ev1.synchronize()
            per_inf.append(ev0.elapsed_time(ev1))
        for _ in range(args.steps):
            ev0.record(stream)
            step()
            ev1.record(stream)
            ev1.synchronize()
            per.append(ev0.elapsed_time(ev1))
    ms, ms_inf = sum(per) / len(per), sum(per_inf) / len(per_inf)
    r = res_box["r"]
    # End to end through falx_parse_gz_host: the compressed stream from
    # pinned host memory, the index and the columns back into pinned host
    # buffers; the copies are inside the call (the outputs go back chunk by
    # chunk while the parse goes on).
    def pinned_np(count, dtype):
        t = torch.empty(max(count, 1) * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
        return t.numpy().view(dtype)

    cols = r["columns"]
    rows_cap, idx_cap = cols.rows + 64, r["index"].numel() + 64
    hcols = _lib.falx_columns()
    hcols.rows_cap = rows_cap
    keep = []
    for k, (f, t) in enumerate(SCHEMA_COLS):
        sd = None
        if t == fx.STR:
            str_cap = cols.column(k)["data"].numel() + 64
            v = pinned_np(rows_cap + 1, np.int32)
            sd = pinned_np(str_cap, np.uint8)
            hcols.cols[k].str_data = sd.ctypes.data
            hcols.cols[k].str_cap = str_cap
        else:
            v = pinned_np(rows_cap, np.float64 if t == fx.F64 else np.uint32)
        valid = pinned_np((rows_cap + 63) // 64, np.uint64)
        hcols.cols[k].values = v.ctypes.data
        hcols.cols[k].valid = valid.ctypes.data
        keep.append((v, valid, sd))
    h_index = pinned_np(idx_cap, np.uint32)
    hout = _lib.falx_outputs()
    hout.index = h_index.ctypes.data
    hout.index_cap = idx_cap
    hout.columns = ctypes.pointer(hcols)
    hfb = _lib.falx_field_byte_stats()
    hout.field_bytes = ctypes.pointer(hfb)
    cs = schema.to_c()
    src = pinned.numpy()

    def e2e_step():
        _lib.check(eng.lib.falx_parse_gz_host(eng.ctx, ctypes.byref(cs), ctypes.c_void_p(src.ctypes.data), len(comp),
                                              bptr, len(blocks), ctypes.byref(hout)), "falx_parse_gz_host")

    e2e_step()
    e2e_ok = (hcols.rows == cols.rows and hout.n_index == r["index"].numel() and
              np.array_equal(h_index[: hout.n_index], r["index"].cpu().numpy().view(np.uint32)))
    d2h = 4 * hout.n_index + sum(o.numel() * o.element_size() for k in range(len(SCHEMA_COLS))
                                 for o in cols.column(k).values())
    e2e_t = []
    for _ in range(max(3, min(args.steps, 7))):
        s0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - s0)
    e2e_s = float(np.median(e2e_t))
    peak, peak_kind = peaks()
    algo_inf = len(comp) + n
    res = {"workload": "csv_hash 1 GiB as bgzf (zlib level 6, %d members of up to 65280 bytes, %d compressed "
                       "bytes): inflate on the GPU, then index + field bytes + typed columns over the text in "
                       "place" % (len(blocks), len(comp)),
           "value": round(n / GIB / (ms / 1e3), 3), "unit": "GiB/s (uncompressed)", "ms": round(ms, 4),
           "inflate": {"value": round(n / GIB / (ms_inf / 1e3), 3), "unit": "GiB/s (uncompressed)",
                       "ms": round(ms_inf, 4),
                       "roofline": {"bound": "issue (serial Huffman decode per member)",
                                    "achieved": round(algo_inf / (ms_inf / 1e3) / 1e9, 1), "peak": peak,
                                    "unit": "GB/s", "frac": round(algo_inf / (ms_inf / 1e3) / 1e9 / peak, 4),
                                    "algorithmic_bytes": algo_inf, "peak_kind": peak_kind,
                                    "note": "compressed bytes read + text written, against the HBM copy peak"}},
           "ratio": round(n / len(comp), 3), "bytes": n, "compressed_bytes": len(comp),
           "e2e": {"value": round(n / GIB / e2e_s, 3), "unit": "GiB/s (uncompressed)",
                   "h2d_bytes_per_step": len(comp), "d2h_bytes_per_step": int(d2h),
                   "ms_per_step": round(e2e_s * 1e3, 3), "entry_point": "falx_parse_gz_host",
                   "outputs_equal_device_step": bool(e2e_ok)},
           "compress_s_host": round(comp_s, 2), "l2": "text 1 GiB > L2, no flush", "clocks": clk.summary()}
    if rank != 0 or args.no_cpu:
        return res
    import oracle

    threads = os.cpu_count() or 1

    def cpu():
        out, st = oracle.bgzf_inflate_par(comp, threads)
        return oracle.parse_par(out, oracle.CSV_HASH, SCHEMA_COLS, threads), int(st.sum())

    best, (ref, bad) = timed_best(cpu)
    t_inf, _ = timed_best(lambda: oracle.bgzf_inflate_par(comp, threads))

    def zlib_par():
        import zlib
        from concurrent.futures import ThreadPoolExecutor

        mv = memoryview(comp)
        with ThreadPoolExecutor(threads) as ex:
            return list(ex.map(lambda b: zlib.decompress(mv[int(b["in_off"]): int(b["in_off"]) + int(b["in_len"])],
                                                         -15), blocks))

    t_zlib, _ = timed_best(zlib_par)
    mism = []
    if bad:
        mism.append("CPU port failed %d members" % bad)
    if not np.array_equal(r["index"].cpu().numpy().view(np.uint32), ref["index"]):
        mism.append("structural index")
    if (r["field_bytes"].fields, r["field_bytes"].bytes) != tuple(ref["field_bytes"]):
        mism.append("field bytes")
    cols = r["columns"]
    compare_columns(host_columns(SCHEMA_COLS, cols._bufs, cols.rows, cols._str_lens), ref["columns"], SCHEMA_COLS,
                    cols.rows, ref["rows"], mism)
    res["parity"] = {"status": "ok" if not mism else "mismatch", "mismatches": mism,
                     "checked": "index, field bytes and every column of the text inflated on the GPU against "
                                "the CPU port's inflate + parse of the same stream"}
    res["cpu_baseline"] = {"value": round(n / GIB / best, 4), "unit": "GiB/s (uncompressed)", "cores": threads,
                           "kind": "port", "isa": cpu_isa(),
                           "sample": "the same bgzf stream: members inflated on all threads, then the parse",
                           "inflate_only": round(n / GIB / t_inf, 4),
                           "zlib_inflate_only": round(n / GIB / t_zlib, 4)}
    return res


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
        "speedup_vs_constant_guess": round(t_const / t_spec, 4),
        "plain_kernel": "index_pass_kernel (groups of two tiles); the speculative scan runs on the tile kernel",
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


def bench_sharded(args):
    """One file over N GPUs (torchrun, one rank per GPU): the file is N
    seeded csv_hash documents of --size bytes, cut a little way into each
    document so the seams fall inside records; rank r's shard runs from that
    point in document r to the same point in document r + 1 (about --size
    bytes: per-GPU work is fixed and the file grows with N). A step on every rank: shard summary,
    summary exchange, first record start, start exchange, one falx_parse
    over the rank's records (index + tape + field bytes + columns; the last
    record's bytes past the shard come from host memory), then the exchange
    of row and arena counts that places the part in the global table. Each
    exchange is one all-gather (NCCL; gloo when ranks share a GPU)."""
    import numpy as np
    import torch
    import torch.distributed as dist

    import falx_gb300 as fx
    import oracle
    from falx_gb300 import gen, shards

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ndev = torch.cuda.device_count()
    gpu_id = local % ndev
    torch.cuda.set_device(gpu_id)
    shared = world > ndev  # ranks sharing a GPU: exercises the path only, exchanges over gloo
    dist.init_process_group("gloo" if shared else "nccl")
    dev = torch.device("cuda", gpu_id)
    gdev = "cpu" if shared else dev

    def gather(o):
        return shards.fixed_all_gather(o, gdev)

    docs = {k: gen.generate(gen.CSV_HASH, args.size, seed=0x5EED0 + k) for k in (rank, rank + 1) if k < world}
    lens = gather(int(docs[rank].size))
    doc_at = [sum(lens[:k]) for k in range(world + 1)]
    file_len = doc_at[world]
    # seams a little way into documents 1 .. N-1, inside a record
    cut = [0] + [doc_at[k] + (64 << 10) + 977 * k for k in range(1, world)] + [file_len]
    lo, hi = cut[rank], cut[rank + 1]

    def read(a, b):
        parts = []
        for k, d in docs.items():
            s0, s1 = max(a, doc_at[k]), min(b, doc_at[k] + d.size)
            if s0 < s1:
                parts.append(d[s0 - doc_at[k]: s1 - doc_at[k]].tobytes())
        data = b"".join(parts)
        if len(data) != b - a:
            raise RuntimeError("bytes %d..%d are not held by rank %d" % (a, b, rank))
        return data

    host_shard = np.frombuffer(read(lo, hi), dtype=np.uint8)
    prev = read(lo - 1, lo)[0] if lo else -1
    pinned = torch.empty(host_shard.size, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = host_shard
    buf = torch.empty(host_shard.size + (1 << 20), dtype=torch.uint8, device=dev)  # room for the last record
    shard = buf[: host_shard.size]
    shard.copy_(pinned)
    eng = fx.Engine(gpu_id)
    eng._sync_stream()
    gpu = shards.GpuShards(eng, full=True)
    stream = torch.cuda.current_stream()

    def step():
        return shards.parse_columns_sharded(gpu, shard, fx.CSV_HASH, SCHEMA_COLS, rank, lo, prev, file_len, read,
                                            gather)

    def outputs():
        last = gpu.last
        outs = [last["index"], last["seps"], last["ends"]]
        for k in range(len(SCHEMA_COLS)):
            outs.extend(last["columns"].column(k).values())
        return [o.reshape(-1).view(torch.uint8) for o in outs]

    for _ in range(max(args.warmup, 3)):
        part = step()
    torch.cuda.synchronize()
    dist.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    per = []
    with Clocks(gpu_id) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            ev0.record(stream)
            part = step()
            ev1.record(stream)
            ev1.synchronize()
            per.append(ev0.elapsed_time(ev1))
        t_wall = time.perf_counter() - t_wall
    dist.barrier()
    t = torch.tensor([sum(per) / len(per)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    value = file_len / GIB / (ms / 1e3)

    # End to end: each step copies the shard in from pinned host memory and
    # the part's outputs back into pinned host buffers.
    h_outs = [torch.empty(max(o.numel(), 1), dtype=torch.uint8, pin_memory=True) for o in outputs()]
    d2h = sum(o.numel() for o in outputs())
    e2e_t = []
    for _ in range(max(3, min(args.steps, 7))):
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        shard.copy_(pinned, non_blocking=True)
        step()
        for h, o in zip(h_outs, outputs()):
            if o.numel():
                h[: o.numel()].copy_(o, non_blocking=True)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - s0)
    t = torch.tensor([float(np.median(e2e_t))], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_s = float(t.item())

    # Parity: every rank checks its part against the CPU port over the
    # part's bytes; rank 0 checks that the parts tile the file.
    mism = []
    if not args.no_cpu:
        a, b = part["bounds"]
        piece = np.frombuffer(read(a, b), dtype=np.uint8) if b > a else np.zeros(0, np.uint8)
        ref = run_cpu(piece, max(1, (os.cpu_count() or 1) // max(1, min(world, ndev))))
        last = gpu.last
        if not np.array_equal(last["index"].cpu().numpy().view(np.uint32), ref["index"]):
            mism.append("rank %d: structural index" % rank)
        if (last["field_bytes"].fields, last["field_bytes"].bytes) != tuple(ref["field_bytes"]):
            mism.append("rank %d: field bytes" % rank)
        cols = last["columns"]
        compare_columns(host_columns(SCHEMA_COLS, cols._bufs, cols.rows, cols._str_lens), ref["columns"],
                        SCHEMA_COLS, cols.rows, ref["rows"], mism)
    checks = gather((part["bounds"], part["rows"], part["row_at"], mism, d2h))
    if rank == 0:
        bounds = [c[0] for c in checks]
        tiled = bounds[0][0] == 0 and bounds[-1][1] == file_len and all(
            p[1] == q[0] for p, q in zip(bounds, bounds[1:]))
        placed = all(checks[r][2] == sum(c[1] for c in checks[:r]) for r in range(world))
        allm = [m for c in checks for m in c[3]] + ([] if tiled else ["parts do not tile the file"]) + \
            ([] if placed else ["row offsets"])
        parity = {"status": "unchecked", "why": "--no-cpu"} if args.no_cpu else \
            {"status": "ok" if not allm else "mismatch", "mismatches": allm,
             "checked": "every rank's index, field bytes and columns against the CPU port over its part's bytes; "
                        "parts tile the file; row offsets"}
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "GiB/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("1 GiB", "%d x %d-byte documents, one file" % (world, args.size)),
                       "input": "each rank's shard device-resident (value); pinned host memory (e2e)",
                       "bytes": int(file_len), "bytes_per_rank": [int(c[0][1] - c[0][0]) for c in checks],
                       "rows": int(sum(c[1] for c in checks)), "l2": "shards of 1 GiB > L2, no flush",
                       "parallelism": "shards of one file, %d ranks%s" % (world, " on shared GPUs" if shared else "")},
            "cpu_baseline": None,
            "parity": parity,
            "e2e": {"value": round(file_len / GIB / e2e_s, 4), "unit": "GiB/s",
                    "h2d_bytes_per_step": int(file_len), "d2h_bytes_per_step": int(sum(c[4] for c in checks)),
                    "ms_per_step": round(e2e_s * 1e3, 3)},
            # per rank and step: shard summary (2), first-record window (1; none on rank 0), falx_parse (2)
            "gpu_launches": args.steps * (5 * world - 1),
            "clocks": clk.summary(),
            "wall_s": round(t_wall, 3),
        }
        print(json.dumps(line))
    dist.barrier()
    eng.close()
    dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="falx_gb300")
    ap.add_argument("--size", type=int, default=1 << 30)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-spec", action="store_true", help="skip the learned-speculation comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-documents run")
    ap.add_argument("--no-configs", action="store_true", help="skip the csv-geo and NDJSON configs")
    args = ap.parse_args()
    if args.impl == "reference":
        bench_reference(args)
    elif int(os.environ.get("WORLD_SIZE", "1")) > 1:
        bench_sharded(args)
    else:
        bench_gpu(args)


if __name__ == "__main__":
    main()
