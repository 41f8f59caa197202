"""Benchmark: exact triangle counting throughput (oriented edges/s) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload rmat23_parts|rmat21|road|rmat16|rmat18|rmat23|rmat23_k8_batch|
                                batch256|serve|refstudy|io]

Default workload (rmat23_parts): the partitioned halo path on R-MAT scale 23,
edge factor 16, (a, b, c) = (0.57, 0.19, 0.19), seeded and vertex-permuted,
cleaned and degree-oriented on the device; k = 2, 4, 8 seeded random parts,
halo subgraphs extracted on the device.  One step = one count of all k = 8
parts in one batched persistent launch (CUDA-graph replay, counting halo:
TC_HALO_COUNT); beside it, per part: one launch per part with a host sync
after each (the reference's per-part loop, without_sorting_tc.cu:244-465) on
the reference's parts and on the counting parts, and the unpartitioned count.
Every result is checked: the parts sum to the whole graph's count.

Printed on rank 0 as ONE JSON line:
  value      whole-job oriented edges/s (|E+| of the graph / batched k = 8 time)
             with the parts resident in HBM, L2 flushed (512 MiB memset)
             before every timed step, CUDA events on the launching stream,
             max over ranks
  e2e        the same metric through the C ABI (tc_count_parts_csr_i32) from
             pinned host buffers of the k = 8 parts: upload + validation +
             batched count + result read-back
  roofline   of the dominant kernel (count_kernel of the batched launch):
             achieved = the bytes this design must read (each root list, each
             edge's row_ptr pair and the cheaper side's list) / its device time;
             the DRAM traffic of one launch (ncu) and the every-wedge byte
             model (every N+(v) read, the reference's probes) beside it
  cpu_baseline  the OpenMP merge-intersection oracle on the machine's host cores,
             one full count of the graph
  reference_gpu_kernel  the reference's own TC_128 kernel (built from its
             sources for sm_103a) on the unpartitioned graph, same GPU

--impl reference times the reference's CPU path on the host cores: the OpenMP
oracle restatement (the reference's counting code is CUDA only; its CPU
orientation tool has no counter), one bounded slice of roots per step; its
input comes from the oracle's own generators (no library code is loaded).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "oriented edges/s"
UNIT = "edges/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["rmat23_parts", "rmat21", "road", "rmat16", "rmat18", "rmat23",
                                           "rmat23_k8_batch", "batch256", "refstudy", "io", "serve"],
                    default="rmat23_parts")
    ap.add_argument("--scale", type=int, default=23,
                    help="rmat23_parts / rmat23_k8_batch: R-MAT scale (23 is the benchmark; smaller for tests)")
    ap.add_argument("--rates", default="50,200,1000,4000", help="serve: Poisson arrival rates (requests/s)")
    ap.add_argument("--requests", type=int, default=400, help="serve: requests per rate")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-ref-kernel", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default thresholds (no autotuning)")
    ap.add_argument("--tuning", default="", help='plain workloads: fixed thresholds as JSON (e.g. \'{"intersect": 2}\'), '
                                             'instead of autotuning')
    return ap.parse_args()


def workload_edges(name: str):
    from trianglecount_gb300 import generators as gen
    if name.startswith("rmat"):
        scale = int("".join(ch for ch in name[4:6] if ch.isdigit()))
        src, dst = gen.rmat(scale, 16)
        return src, dst, {"workload": f"rmat{scale}_ef16_plain", "generator": "R-MAT", "scale": scale,
                          "edge_factor": 16, "abc": [gen.RMAT_A, gen.RMAT_B, gen.RMAT_C],
                          "seed": gen.SEED.get(f"rmat{scale}", 0), "vertex_permutation": True}
    src, dst = gen.road()
    return src, dst, {"workload": "road_1448x1448_plain", "generator": "jittered grid",
                      "side": gen.ROAD_SIDE, "p_delete": gen.ROAD_P_DELETE, "diag_rate": gen.ROAD_DIAG_RATE,
                      "seed": gen.SEED["road"]}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(x: float, pg, device) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def parts_config(scale: int) -> dict:
    """The partitioned workload as both arms name it."""
    return {"workload": f"rmat{scale}_ef16_halo_parts", "generator": "R-MAT", "scale": scale, "edge_factor": 16,
            "abc": [0.57, 0.19, 0.19], "seed": 0x5EED0000 + scale if scale not in (16, 21, 23) else
            {16: 0x5EED0016, 21: 0x5EED0021, 23: 0x5EED0023}[scale], "vertex_permutation": True,
            "parts_k": [2, 4, 8], "partition": "seeded uniform random parts (seed 0x5EED9A27 + k)",
            "headline": "k = 8 parts (counting halo) in one batched persistent launch",
            "tie_break": "reference (deg u < deg w, or equal and w < u)", "index_type": "int32",
            "l2": "flushed before every timed step (512 MiB memset on the launching stream)"}


def run_reference(args, world, rank):
    """CPU path of the reference (OpenMP oracle restatement), rank 0 only.
    R-MAT inputs come from the oracle's own generators, so this arm loads no
    library code."""
    if rank != 0:
        return
    import oracle
    if args.workload in ("rmat23_parts", "rmat23_k8_batch"):
        cfg = parts_config(args.scale)
        src, dst = oracle.gen_rmat(args.scale)
    elif args.workload.startswith("rmat"):
        scale = int("".join(ch for ch in args.workload[4:6] if ch.isdigit()))
        src, dst = oracle.gen_rmat(scale)
        cfg = {"workload": f"rmat{scale}_ef16_plain", "generator": "R-MAT", "scale": scale, "edge_factor": 16,
               "abc": list(oracle.RMAT_ABC), "seed": oracle.SEED_RMAT.get(scale, 0x5EED0000 + scale),
               "vertex_permutation": True}
    else:
        src, dst, cfg = workload_edges(args.workload)
    rp, col = oracle.clean(src, dst)
    del src, dst
    orp, ocl = oracle.orient(rp, col)
    del rp, col
    orp, ocl = orp.astype(np.int32), ocl.astype(np.int32)
    V = len(orp) - 1
    n_samples = 8
    bounds = [V * i // n_samples for i in range(n_samples + 1)]
    times, edges = [], []
    for step in range(args.warmup + args.steps):
        i = step % n_samples
        r0, r1 = bounds[i], bounds[i + 1]
        t0 = time.perf_counter()
        oracle.count_range_i32(orp, ocl, r0, r1)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
            edges.append(int(orp[r1] - orp[r0]))
    value = sum(edges) / sum(times)
    cores = oracle.num_threads()
    cfg.update({"V": V, "oriented_edges": int(len(ocl))})
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "strong" if "halo_parts" in cfg["workload"] else "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"one 1/{n_samples} slice of the roots per step (permuted ids), "
                                   "OpenMP merge intersection, schedule(dynamic,64); the parts of the graph "
                                   "sum to its whole count, so the whole graph's roots are the sample space"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def load_traffic(workload: str):
    """DRAM traffic of one count_kernel launch from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"count_kernel_{workload}.traffic.txt")
    if not os.path.exists(p):
        return None
    out = {}
    for line in open(p):
        if "=" in line and not line.startswith("#"):
            k, v = (x.strip() for x in line.split("=", 1))
            out[k] = int(v) if v.isdigit() else v
    return out


def run_ours(args, world, rank, local, pg):
    import torch

    import trianglecount_gb300 as tc

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    ctx = tc.Context(local)
    ctx.set_stream(stream.cuda_stream)

    src, dst, cfg = workload_edges(args.workload)
    t0 = time.perf_counter()
    ug = ctx.ugraph_from_edges(src, dst)  # upload + clean-up (dedupe, symmetrise, drop isolated)
    clean_s = time.perf_counter() - t0
    # degree orientation on the device, timed with events (the last of 4 runs is kept)
    orient_ms = []
    for _ in range(4):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g = ctx.orient(ug)
        e1.record(stream)
        e1.synchronize()
        orient_ms.append(e0.elapsed_time(e1))
    prep_s = clean_s + orient_ms[-1] / 1000.0
    ug_rows, ug_nnz = ug.info()
    ug.free()
    tuning, tune_ms = ({}, None)
    if args.tuning:  # fixed thresholds (profiling an alternative strategy)
        ctx.set_tuning(**json.loads(args.tuning))
    elif not args.no_tune:  # per-graph strategy thresholds, picked on the device before timing
        t0 = time.perf_counter()
        tuning, tune_ms = ctx.autotune(g, max_trials=40)
        cfg["autotune_s"] = round(time.perf_counter() - t0, 3)
    cfg["tuning"] = tuning or ctx.get_tuning()
    rp, col = g.download()
    V, E = len(rp) - 1, len(col)
    dplus = np.diff(rp).astype(np.int64)
    W = int(dplus[col].sum())
    B_alg = 4 * (V + 1) + 12 * E + 4 * W + 8
    P_min = int(np.minimum(np.repeat(dplus, dplus), dplus[col]).sum())  # probes of the min-side rule

    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    d_out = torch.zeros(1, dtype=torch.int64, device=dev)
    lib = tc.lib()

    def one_step(e0, e1):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            st = lib.tc_count_async(ctx.handle, g.handle, d_out.data_ptr())
            e1.record(stream)
        if st != 0:
            raise tc.TCError(st, "tc_count_async", lib.tc_last_error().decode())

    for _ in range(args.warmup):
        one_step(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    torch.cuda.synchronize()
    count, st0 = ctx.count(g, stats=True)
    launches_per_count = int(st0["launches"])

    clocks = ClockSampler(local)
    clocks.start()
    barrier(pg)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    import ctypes as C
    kms, kernel_ms = C.c_float(), []
    for e0, e1 in evs:
        one_step(e0, e1)
        # the count kernel alone, from the library's events around its launch
        if lib.tc_ctx_last_count_kernel_ms(ctx.handle, C.byref(kms)) == 0:
            kernel_ms.append(kms.value)
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    ms = max_over_ranks(sum(step_ms) / len(step_ms), pg, dev)
    value = world * E / (ms / 1000.0)
    assert int(d_out.item()) == count

    # ---- end to end through the C ABI from pinned host memory ----
    rp_h = torch.from_numpy(rp).pin_memory()
    col_h = torch.from_numpy(col).pin_memory()
    out = np.zeros(1, np.uint64)
    import ctypes as C
    e2e_ms = []
    for step in range(args.warmup + args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
        st = lib.tc_count_csr_i32(ctx.handle, C.c_void_p(rp_h.data_ptr()), C.c_void_p(col_h.data_ptr()), V, E,
                                  out.ctypes.data_as(C.POINTER(C.c_uint64)))
        with torch.cuda.stream(stream):
            e1.record(stream)
        if st != 0:
            raise tc.TCError(st, "tc_count_csr_i32", lib.tc_last_error().decode())
        e1.synchronize()
        if step >= args.warmup:
            e2e_ms.append(e0.elapsed_time(e1))
        assert int(out[0]) == count
    e2e = max_over_ranks(sum(e2e_ms) / len(e2e_ms), pg, dev)

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    kernel_avg_ms = sum(kernel_ms) / len(kernel_ms) if kernel_ms else ms
    sec = kernel_avg_ms / 1000.0
    # a graph with no row longer than 8 is counted by one flat kernel that
    # intersects every oriented edge directly (W+ probes, exactly B_alg)
    flat = launches_per_count == 1
    probes = W if flat else P_min
    # the bytes this design must read: each root's row_ptr and list, each
    # oriented edge's row_ptr pair and the cheaper side's list (every N+(v)
    # for the flat kernel)
    B_min = 4 * (V + 1) + 12 * E + 4 * probes + 8
    tr = load_traffic(cfg["workload"])
    traffic = (tr or {}).get("traffic_bytes_per_launch")

    res = None
    if rank == 0:
        cfg.update({"V": V, "oriented_edges": E, "undirected_edges": E, "W_plus": W, "triangles": count,
                    "tie_break": "reference (deg u < deg w, or equal and w < u)", "index_type": "int32",
                    "l2": "flushed before every timed step (512 MiB memset on the launching stream)",
                    "device_preprocess_s": round(prep_s, 3), "parallelism": f"replicas x{world}"})
        # the orientation's own algorithmic bytes: row_ptr read and written, every
        # undirected entry and its endpoint's degree read, the kept half written
        B_orient = 8 * (ug_rows + 1) + 4 * ug_nnz + 4 * ug_nnz + 4 * E
        o_ms = min(orient_ms[1:])
        res = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded R-MAT / grid generators)",
            "config": cfg,
            "gpu_launches": launches_per_count * args.steps,
            "e2e": {"value": world * E / (e2e / 1000.0), "unit": UNIT, "ms_per_step": e2e,
                    "h2d_bytes_per_step": 4 * (V + 1) + 4 * E, "d2h_bytes_per_step": 8 + 8 + 24,
                    "path": "tc_count_csr_i32 (upload + validate + count + read-back)",
                    "gpu_launches": (launches_per_count + 2) * args.steps},
            "roofline": {"bound": "hbm", "achieved": B_min / sec / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": B_min / sec / 1e9 / peak, "peak_source": f"{peak_src} hbm_gbs (copy, burst)",
                         "kernel": (("flat4_kernel" if int(dplus.max(initial=0)) <= 4 else "flat_kernel") if flat
                                    else "count_kernel"), "kernel_ms": kernel_avg_ms,
                         "algorithmic_bytes_per_launch": B_min,
                         "algorithmic_bytes_definition": (
                             "4(V+1) + 12|E+| + 4 W+ + 8 (the flat kernel probes every wedge)" if flat else
                             "4(V+1) + 12|E+| + 4 sum_{u->v} min(d+(u), d+(v)) + 8: each root's row_ptr and list, "
                             "each oriented edge's row_ptr pair and the cheaper side's list -- the bytes this "
                             f"design must read ({P_min / max(W, 1):.2f} W+ probes on this graph)"),
                         "probes_done": probes,
                         "dram_achieved": traffic / sec / 1e9 if traffic else None,
                         "dram_frac": traffic / sec / 1e9 / peak if traffic else None,
                         "traffic": traffic,
                         "traffic_source": (tr or {}).get("source"),
                         "wedge_model_bytes": B_alg, "wedge_model_frac": B_alg / sec / 1e9 / peak,
                         "wedge_model_note": "4(V+1) + 12|E+| + 4 W+ + 8 (every N+(v) read, W+ = sum over oriented "
                                             "edges of d+(v)): work the min-side design does not do, so its "
                                             "fraction can exceed 1 and is not evidence"},
            "clocks": clk,
            "preprocess": {"clean_upload_s": round(clean_s, 4),
                           "clean_note": "host-timed: edge upload + device sort, dedupe, symmetrise, relabel",
                           "orient_ms": o_ms, "orient_algorithmic_bytes": B_orient,
                           "orient_bytes_definition": "8(V+1) + 4*2m (undirected col) + 4*2m (degree gathers) "
                                                      "+ 4m (oriented col written)",
                           "orient_achieved_gbs": B_orient / (o_ms / 1000.0) / 1e9,
                           "orient_frac": B_orient / (o_ms / 1000.0) / 1e9 / peak,
                           "orient_edges_per_s": E / (o_ms / 1000.0)},
        }
        # the CPU and reference-kernel baselines are taken at N = 1 only
        if not args.no_ref_kernel and world == 1:
            try:
                import oracle
                if oracle.ref_kernel_available():
                    pr, _ = oracle.ref_tc128(rp, col, runs=1)
                    ref_ms = []
                    for _ in range(3):
                        flush.zero_()
                        torch.cuda.synchronize()
                        pr, t_ms = oracle.ref_tc128(rp, col, runs=1)
                        ref_ms.append(t_ms)
                    ok = int(pr.sum()) == count
                    rms = statistics.median(ref_ms)
                    res["reference_gpu_kernel"] = {
                        "value": E / (rms / 1000.0), "unit": UNIT, "ms": rms, "count_matches": ok,
                        "source": "TC_128 Find_Triangle (ShareKernelTCV62_update_v1.cu) built from the reference "
                                  "sources for sm_103a, one 128-thread block per vertex, median of 3, L2 flushed",
                        "speedup_of_ours": rms / ms}
            except Exception as ex:  # reported, never fatal
                res["reference_gpu_kernel"] = {"unavailable": str(ex)[:200]}
        if not args.no_cpu and world == 1:
            import oracle
            t0 = time.perf_counter()
            ccount = oracle.count(rp, col)
            cdt = time.perf_counter() - t0
            res["cpu_baseline"] = {"value": E / cdt, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                                   "sample": "the whole graph, one full count (OpenMP merge intersection, "
                                             "schedule(dynamic,64), u64 reduction)",
                                   "seconds": cdt, "count_matches": ccount == count}
    barrier(pg)
    ctx.close()
    return res


def _timed(stream, flush, fn, steps, warmup, after=None):
    """Mean device time (CUDA events on `stream`) of fn over `steps` runs after
    `warmup`, L2 flushed before each; after() runs once each step has ended."""
    import torch
    ms = []
    for i in range(warmup + steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
        fn()
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        if after is not None:
            after()
        if i >= warmup:
            ms.append(e0.elapsed_time(e1))
    return sum(ms) / len(ms)


def run_refstudy(args, world, rank, local, pg):
    """The reference's design-space study re-run on this GPU: its Find_Triangle
    variants built from their own sources (src/WithoutPartition/:
    ShareKernelTCV62_update_v1.cu 128 threads, shareMemSize.cu 64 threads,
    With_Atomic_op.cu 256 threads with one atomic per probe,
    Without_ShareMemory_TC.cu 2 threads with a u64 binary search in global
    memory), each launched as its driver does, beside this library's count
    of the same graph.  R-MAT scale 16 (all variants) and 18 (the two
    shared-memory ones; the atomic variants serialise on one counter).  L2 is
    flushed before every launch."""
    import torch

    import oracle
    import trianglecount_gb300 as tc
    from trianglecount_gb300 import generators as gen
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    ctx = tc.Context(local)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    d_out = torch.zeros(1, dtype=torch.int64, device=dev)
    lib = tc.lib()
    graphs = {}
    for scale, variants in ((16, ("tc128", "smem64", "atomic256", "nosmem2")), (18, ("tc128", "smem64"))):
        src, dst = gen.rmat(scale, 16)
        g = ctx.graph_from_edges(src, dst)
        rp, col = g.download()
        want = ctx.count(g)
        ours = _timed(stream, flush, lambda: lib.tc_count_async(ctx.handle, g.handle, d_out.data_ptr()),
                      args.steps, args.warmup)
        assert int(d_out.item()) == want
        row = {"V": g.n_rows, "oriented_edges": g.nnz, "triangles": want, "ours_ms": ours}
        for v in variants:
            if not oracle.ref_variant_available(v):
                row[v] = "unavailable: cubin not built (needs the reference tree at build time)"
                continue
            total, ms = oracle.ref_variant(v, rp, col, runs=3 if v in ("tc128", "smem64") else 1)
            row[v] = {"ms": ms, "count_matches": total == want, "speedup_of_ours": ms / ours}
        graphs[f"rmat{scale}"] = row
    r16 = graphs["rmat16"]
    cfg = {"workload": "reference_design_space_study", "graphs": graphs,
           "variants": {k: {"cubin": c, "threads_per_block": t, "u64": bool(u), "one_atomic_per_probe": bool(a)}
                        for k, (c, _, t, u, a) in oracle.REF_VARIANTS.items()},
           "l2": "flushed before every launch (512 MiB memset)"}
    res = {"metric": METRIC, "value": world * r16["oriented_edges"] / (r16["ours_ms"] / 1000.0), "unit": UNIT,
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r16["ours_ms"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded R-MAT)", "config": cfg}
    ctx.close()
    return res


def _part_bytes(prp: np.ndarray, pcol: np.ndarray, n_roots: int) -> tuple[int, int, int]:
    """Bytes one count of a graph (roots [0, n_roots)) reads: (model, min-side, W+).
    model = 4(R+1) + 12 E_R + 4 W+ + 8: the roots' row_ptr and lists, each
    root edge u -> v's row_ptr pair and all of N+(v) (W+ = sum d+(v));
    min-side: the same with min(d+(u), d+(v)) entries per edge, the list of
    the cheaper side, which is what this design streams through a hash."""
    d = np.diff(prp).astype(np.int64)
    er = int(prp[n_roots])
    if er == 0:
        return 4 * (n_roots + 1) + 8, 4 * (n_roots + 1) + 8, 0
    du = np.repeat(d[:n_roots], d[:n_roots])
    dv = d[pcol[:er]]
    W = int(dv.sum())
    P = int(np.minimum(du, dv).sum())
    base = 4 * (n_roots + 1) + 12 * er + 8
    return base + 4 * W, base + 4 * P, W


def run_parts(args, world, rank, local, pg):
    """Partitioned halo path (the default workload): device clean-up,
    orientation and halo extraction of R-MAT scale 23 for k = 2, 4, 8 seeded
    random parts, in the reference's halo (round_clean_sg's parts) and the
    counting halo (TC_HALO_COUNT); per-part launches with a host sync after
    each (the reference's loop, without_sorting_tc.cu:244-465) versus one
    batched persistent launch; the unpartitioned count beside them.  With
    N > 1 ranks, the k = 8 counting parts are split over the ranks by work
    (largest first), each rank counts its parts in one batched launch, and the
    per-part counts are summed: a fixed total, so scaling is strong."""
    import ctypes as C

    import torch

    import trianglecount_gb300 as tc
    from trianglecount_gb300 import generators as gen
    from trianglecount_gb300 import shard

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    ctx = tc.Context(local)
    ctx.set_stream(stream.cuda_stream)
    lib = tc.lib()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    scale = args.scale
    cfg = parts_config(scale)
    detail: dict = {}

    t0 = time.perf_counter()
    src, dst = gen.rmat(scale, 16)
    detail["host_generate_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ug = ctx.ugraph_from_edges(src, dst)
    ctx.synchronize()
    detail["device_clean_s"] = time.perf_counter() - t0
    del src, dst
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    og = ctx.orient(ug)
    e1.record(stream)
    e1.synchronize()
    detail["device_orient_ms"] = e0.elapsed_time(e1)
    V, E = og.n_rows, og.nnz
    rp, col = og.download()
    cfg.update({"V": V, "oriented_edges": E})
    whole = ctx.count(og)
    detail["triangles"] = whole

    def timed(fn, after=None):
        ms, extra = [], []
        for i in range(args.warmup + args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.zero_()
                a.record(stream)
            fn()
            with torch.cuda.stream(stream):
                b.record(stream)
            b.synchronize()
            if i >= args.warmup:
                ms.append(a.elapsed_time(b))
                if after is not None:
                    extra.append(after())
        return ms, extra

    def mean(x):
        return sum(x) / len(x) if x else 0.0

    clocks = ClockSampler(local)
    per_k, head = {}, None
    if world == 1:
        clocks.start()
        d_out = torch.zeros(1, dtype=torch.int64, device=dev)
        kms = C.c_float()

        def kernel_ms():
            lib.tc_ctx_last_count_kernel_ms(ctx.handle, C.byref(kms))
            return kms.value

        w_ms, w_k = timed(lambda: lib.tc_count_async(ctx.handle, og.handle, d_out.data_ptr()), kernel_ms)
        assert int(d_out.item()) == whole
        detail["whole_graph_plain_ms"] = mean(w_ms)
        detail["whole_graph_count_kernel_ms"] = mean(w_k)
        for k in (2, 4, 8):
            part = gen.parts_random(V, k)
            row = {}
            for mode in ("reference", "count"):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                parts = ctx.halo_extract(ug, part, k, mode=mode)
                ctx.synchronize()
                ext_s = time.perf_counter() - t0
                pp_ms, _ = timed(lambda: ctx.count_each(parts))
                assert int(ctx.count_each(parts).sum()) == whole
                b = ctx.batch(parts)
                assert int(b.run().sum()) == whole
                b_ms, b_k = timed(lambda: b.run_async(), lambda: b.stats()["count_kernel_ms"])
                outs = b.results()
                assert int(outs.sum()) == whole, "the parts do not sum to the whole graph's count"
                row[mode] = {"halo_extract_s": ext_s, "per_part_launches_ms": mean(pp_ms),
                             "batched_ms": mean(b_ms), "batched_count_kernel_ms": mean(b_k),
                             "batched_vs_per_part": mean(pp_ms) / mean(b_ms),
                             "parts_nnz_total": int(sum(p.nnz for p in parts)),
                             "parts_nnz_over_graph": sum(p.nnz for p in parts) / E,
                             "parts_rows_total": int(sum(p.n_rows for p in parts)),
                             "per_part_counts": [int(x) for x in outs]}
                if k == 8 and mode == "count":
                    head = (parts, b, b_ms, b_k)
                else:
                    b.free()
                    del parts
            row["batched_count_halo_vs_per_part_reference_halo"] = (row["reference"]["per_part_launches_ms"] /
                                                                    row["count"]["batched_ms"])
            per_k[str(k)] = row
        detail["parts"] = per_k
        # the same graph on balanced label-propagation parts (the stand-in for
        # the reference's METIS assignment), k = 8, counting halo, batched
        t0 = time.perf_counter()
        lp_part = ctx.parts_lp(ug, 8)
        lp_s = time.perf_counter() - t0
        rp_u, col_u, _ = ug.download()
        rows_u = np.repeat(np.arange(len(rp_u) - 1, dtype=np.int64), np.diff(rp_u))
        cut = float((lp_part[rows_u] != lp_part[col_u]).mean())
        del rows_u, rp_u, col_u
        lp_parts = ctx.halo_extract(ug, lp_part, 8, mode="count")
        lb = ctx.batch(lp_parts)
        assert int(lb.run().sum()) == whole
        lp_ms, _ = timed(lambda: lb.run_async())
        assert int(lb.results().sum()) == whole
        detail["lp_parts_k8"] = {"partition_s": lp_s, "cut_fraction": cut,
                                 "max_part_over_mean": float(np.bincount(lp_part).max() * 8 / V),
                                 "parts_nnz_over_graph": sum(p.nnz for p in lp_parts) / E, "batched_ms": mean(lp_ms),
                                 "note": "balanced label propagation on the device (tc_gen_parts_lp), counting halo"}
        lb.free()
        del lp_parts
        parts, b, b_ms, b_k = head
        ms = mean(b_ms)
        launches = b.stats()["launches"]
    else:
        # sharded: the k = 8 counting parts, split over the ranks by work
        parts_all = ctx.halo_extract(ug, gen.parts_random(V, 8), 8, mode="count")
        work = [p.nnz for p in parts_all]
        mine = shard.assign_parts(work, world)[rank]
        parts = [parts_all[i] for i in mine]
        for i, p in enumerate(parts_all):
            if i not in mine:
                p.free()
        b = ctx.batch(parts) if parts else None
        clocks.start()
        barrier(pg)
        torch.cuda.synchronize()
        b_ms, b_k = timed((lambda: b.run_async()) if b else (lambda: None),
                          (lambda: b.stats()["count_kernel_ms"]) if b else None)
        torch.cuda.synchronize()
        barrier(pg)
        local_sum = int(b.results().sum()) if b else 0
        t = torch.tensor([local_sum], dtype=torch.int64, device=dev)
        pg.all_reduce(t)
        assert int(t.item()) == whole, "the ranks' parts do not sum to the whole graph's count"
        ms = mean(b_ms)
        launches = b.stats()["launches"] if b else 0
        detail["sharding"] = {"parts_per_rank": len(mine), "rank0_parts": mine,
                              "assignment": "largest first by nnz (trianglecount_gb300/shard.py)"}
    ms = max_over_ranks(ms, pg, dev)
    value = E / (ms / 1000.0)

    # ---- roofline of the batched count kernel (this rank's parts) ----
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    B_model = B_min = W_tot = 0
    host_parts = []
    for p in parts:
        prp, pcol = p.download()
        bm, bn, w = _part_bytes(prp, pcol, p.n_roots)
        B_model, B_min, W_tot = B_model + bm, B_min + bn, W_tot + w
        host_parts.append((prp, pcol, p.n_roots))
    k_ms = mean(b_k) if b_k else ms
    tr = load_traffic(f"rmat{scale}_parts_k8")
    traffic = (tr or {}).get("traffic_bytes_per_launch")
    sec = k_ms / 1000.0
    roofline = {"bound": "hbm", "achieved": B_min / sec / 1e9, "peak": peak, "unit": "GB/s",
                "frac": B_min / sec / 1e9 / peak, "traffic": traffic,
                "peak_source": f"{peak_src} hbm_gbs (copy, burst)", "kernel": "count_kernel, the batched k = 8 count's two phase kernels (heavy units, then light tasks)",
                "kernel_ms": k_ms, "algorithmic_bytes_per_launch": B_min,
                "algorithmic_bytes_definition": "sum over parts of 4(R+1) + 12 E_R + 4 sum_{u->v} min(d+(u), d+(v)) "
                                                "+ 8 (R roots, E_R root edges): each root's row_ptr and list, each "
                                                "root edge's row_ptr pair and the cheaper side's list -- the bytes "
                                                "this design must read",
                "dram_achieved": traffic / sec / 1e9 if traffic else None,
                "dram_frac": traffic / sec / 1e9 / peak if traffic else None,
                "traffic_source": (tr or {}).get("source"),
                "wedge_model_bytes": B_model, "wedge_model_frac": B_model / sec / 1e9 / peak,
                "wedge_model_note": "4(R+1) + 12 E_R + 4 W+ + 8 per part (every N+(v) read): work the min-side "
                                     "design does not do, so its fraction can exceed 1 and is not evidence",
                "W_plus": W_tot}

    # ---- end to end through the C ABI from pinned host memory (k = 8 parts) ----
    pinned = []
    for prp, pcol, nr in host_parts:
        a = torch.from_numpy(prp).pin_memory()
        c = torch.from_numpy(pcol).pin_memory()
        pinned.append((a.numpy(), c.numpy(), nr, a, c))
    want = [int(x) for x in b.results()] if b else []
    e2e_ms = []
    if pinned:
        def e2e_call():
            got = ctx.count_parts_csr([(q[0], q[1], q[2]) for q in pinned])
            assert [int(x) for x in got] == want
        e2e_ms, _ = timed(e2e_call)
    clk = clocks.stop()
    e2e = max_over_ranks(mean(e2e_ms), pg, dev)
    h2d = sum(4 * len(q[0]) + 4 * len(q[1]) for q in pinned)

    res = None
    if rank == 0:
        res = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "int32", "data": f"synthetic (seeded R-MAT scale {scale})",
            "config": cfg, "gpu_launches": launches * args.steps,
            "e2e": {"value": E / (e2e / 1000.0) if e2e else None, "unit": UNIT, "ms_per_step": e2e,
                    "ms_min": min(e2e_ms) if e2e_ms else None,
                    "ms_median": sorted(e2e_ms)[len(e2e_ms) // 2] if e2e_ms else None,
                    "ms_steps": [round(x, 2) for x in e2e_ms],
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 20 * len(pinned) + 48,
                    "path": "tc_count_parts_csr_i32: every part's upload issued at once; each part validated as "
                            "soon as it is in; the parts counted in groups of 1, 2, then the rest, one launch per "
                            "group, under the later uploads; read-back"},
            "roofline": roofline, "clocks": clk, "detail": detail,
        }
        if world == 1 and not args.no_ref_kernel:
            try:
                import oracle
                if oracle.ref_kernel_available():
                    oracle.ref_tc128(rp, col, runs=1)
                    ref_ms, ok = [], True
                    for _ in range(3):
                        flush.zero_()
                        torch.cuda.synchronize()
                        pr, t_ms = oracle.ref_tc128(rp, col, runs=1)
                        ref_ms.append(t_ms)
                        ok = ok and int(pr.sum()) == whole
                    rms = statistics.median(ref_ms)
                    res["reference_gpu_kernel"] = {
                        "value": E / (rms / 1000.0), "unit": UNIT, "ms": rms, "count_matches": ok,
                        "source": "TC_128 Find_Triangle (ShareKernelTCV62_update_v1.cu) built from the reference "
                                  "sources for sm_103a, on the unpartitioned graph, one 128-thread block per "
                                  "vertex, median of 3, L2 flushed",
                        "speedup_of_batched_parts": rms / ms,
                        "speedup_of_whole_plain": rms / detail["whole_graph_plain_ms"]}
            except Exception as ex:  # reported, never fatal
                res["reference_gpu_kernel"] = {"unavailable": str(ex)[:200]}
        if world == 1 and not args.no_cpu:
            import oracle
            t0 = time.perf_counter()
            ccount = oracle.count(rp, col)
            cdt = time.perf_counter() - t0
            res["cpu_baseline"] = {"value": E / cdt, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                                   "sample": f"the whole R-MAT {scale} graph, one full count (OpenMP merge "
                                             "intersection, schedule(dynamic,64), u64 reduction); the parts sum "
                                             "to this count",
                                   "seconds": cdt, "count_matches": ccount == whole}
    barrier(pg)
    if b:
        b.free()
    ctx.close()
    return res


def run_k8_batch(args, world, rank, local, pg):
    """Profiling case: only the batched count of R-MAT's k = 8 counting-halo
    parts, replayed warmup + steps times (the first count_kernel launch of the
    process is the first replay's)."""
    import torch

    import trianglecount_gb300 as tc
    from trianglecount_gb300 import generators as gen
    torch.cuda.set_device(local)
    ctx = tc.Context(local)
    src, dst = gen.rmat(args.scale, 16)
    ug = ctx.ugraph_from_edges(src, dst)
    del src, dst
    parts = ctx.halo_extract(ug, gen.parts_random(ug.info()[0], 8), 8, mode="count")
    ug.free()
    b = ctx.batch(parts)
    ms = []
    for _ in range(args.warmup + args.steps):
        b.run_async()
        b.results()
        ms.append(b.stats()["count_kernel_ms"])
    total = int(b.results().sum())
    b.free()
    ctx.close()
    return {"workload": f"rmat{args.scale}_parts_k8_batch", "triangles": total,
            "count_kernel_ms": ms[args.warmup:], "parts_nnz": [p.nnz for p in parts]}


def _peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_batch(args, world, rank, local, pg):
    """Uneven batch: 256 seeded ER / Chung-Lu / R-MAT graphs, one launch per
    graph (host sync after each) versus one persistent launch for all."""
    import torch

    import oracle
    import trianglecount_gb300 as tc
    from trianglecount_gb300 import generators as gen
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    ctx = tc.Context(local)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    specs = gen.batch_mix(256)
    graphs, gen_s, prep_s = [], 0.0, 0.0
    for sp in specs:
        t0 = time.perf_counter()
        src, dst = sp.edges()
        gen_s += time.perf_counter() - t0
        t0 = time.perf_counter()
        graphs.append(ctx.graph_from_edges(src, dst))
        prep_s += time.perf_counter() - t0
    E = sum(g.nnz for g in graphs)
    each = ctx.count_each(graphs)
    b = ctx.batch(graphs)
    outs = b.run()
    assert list(outs) == list(each)
    host = [g.download() for g in graphs]
    # oracle spot check on the smallest graphs
    small = sorted(range(len(specs)), key=lambda i: graphs[i].nnz)[:8]
    for i in small:
        assert oracle.count(*host[i]) == int(outs[i])
    clocks = ClockSampler(local)
    clocks.start()
    plain_ms = _timed(stream, flush, lambda: ctx.count_each(graphs), args.steps, args.warmup)
    kms = []
    batch_ms = _timed(stream, flush, lambda: b.run_async(), args.steps, args.warmup,
                      after=lambda: kms.append(b.stats()["count_kernel_ms"]))
    # end to end from pinned host memory: upload + validate all 256, one batched count
    pinned = [(torch.from_numpy(rp).pin_memory(), torch.from_numpy(cl).pin_memory()) for rp, cl in host]
    views = [(a.numpy(), c.numpy(), len(a) - 1) for a, c in pinned]

    def e2e_call():
        assert list(ctx.count_parts_csr(views)) == list(outs)

    e2e_ms = _timed(stream, flush, e2e_call, args.steps, args.warmup)
    clk = clocks.stop()
    B_min = B_model = 0
    for rp, cl in host:
        bm, bn, _ = _part_bytes(rp, cl, len(rp) - 1)
        B_model, B_min = B_model + bm, B_min + bn
    peak, peak_src = _peak()
    k_ms = sum(kms[args.warmup:]) / max(1, len(kms[args.warmup:]))
    t0 = time.perf_counter()
    cpu_total = sum(oracle.count(rp, cl) for rp, cl in host)
    cpu_s = time.perf_counter() - t0
    kinds = {k: sum(1 for s in specs if s.kind == k) for k in ("er", "chung_lu", "rmat")}
    cfg = {"workload": "uneven_batch_256", "graphs": len(graphs), "kinds": kinds, "oriented_edges": E,
           "l2": "flushed before every timed step (512 MiB memset on the launching stream)"}
    detail = {"triangles_total": int(outs.sum()), "plain_per_graph_ms": plain_ms, "batched_ms": batch_ms,
              "speedup": plain_ms / batch_ms, "host_generate_s": gen_s, "device_preprocess_s": prep_s,
              "largest_graph_edges": max(g.nnz for g in graphs), "smallest_graph_edges": min(g.nnz for g in graphs)}
    res = {"metric": METRIC, "value": world * E / (batch_ms / 1000.0), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": batch_ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded ER / Chung-Lu / R-MAT mix)", "config": cfg, "detail": detail,
           "gpu_launches": b.stats()["launches"] * args.steps, "clocks": clk,
           "e2e": {"value": E / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
                   "h2d_bytes_per_step": sum(4 * len(rp) + 4 * len(cl) for rp, cl in host),
                   "d2h_bytes_per_step": 20 * len(host) + 48,
                   "path": "tc_count_parts_csr_i32 with every row a root: upload + validate 256 graphs, one "
                           "batched count, read-back"},
           "roofline": {"bound": "hbm", "achieved": B_min / (k_ms / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": B_min / (k_ms / 1000.0) / 1e9 / peak, "traffic": None,
                        "peak_source": f"{peak_src} hbm_gbs (copy, burst)",
                        "kernel": "count_kernel (batched, 256 graphs)", "kernel_ms": k_ms,
                        "algorithmic_bytes_per_launch": B_min,
                        "algorithmic_bytes_definition": "sum over graphs of 4(V+1) + 12|E+| + 4 sum_{u->v} "
                                                        "min(d+(u), d+(v)) + 8",
                        "wedge_model_bytes": B_model,
                        "wedge_model_frac": B_model / (k_ms / 1000.0) / 1e9 / peak},
           "cpu_baseline": {"value": E / cpu_s, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                            "sample": "all 256 graphs, one OpenMP count each", "seconds": cpu_s,
                            "count_matches": cpu_total == int(outs.sum())}}
    b.free()
    ctx.close()
    return res


def serve_pool(n_graphs: int = 40, seed: int | None = None):
    """Seeded graphs with edge counts log-uniform in [1e3, 5e7], alternating
    R-MAT (edge factor 16) and Chung-Lu (gamma 2.1, mean degree 16)."""
    import math

    from trianglecount_gb300 import generators as gen
    r = gen.SplitMix64(gen.SEED["serve"] if seed is None else seed)
    pool = []
    for i in range(n_graphs):
        m = r.log_uniform(1e3, 5e7)
        gseed = r.next()
        if i % 2 == 0:
            scale = max(6, min(21, int(math.log2(m / 16))))
            pool.append(("rmat", {"scale": scale}, gen.rmat(scale, 16, seed=gseed)))
        else:
            n = max(64, int(m / 8))
            pool.append(("chung_lu", {"n": n, "avg_deg": 16.0}, gen.chung_lu(n, 16.0, gseed)))
    return pool


def run_serve(args, world, rank, local, pg):
    """Serving stream: Poisson arrivals of count requests over a pool of
    graphs; graphs are oriented on the device at admission and kept resident
    by key (LRU under an 80% HBM budget); latency is submit -> result.
    Requests of at most 2^20 edges take the small lane, the others the large
    one; latencies are reported for all requests and per lane."""
    import random

    import oracle
    import trianglecount_gb300 as tc
    ctx = tc.Context(local)
    t0 = time.perf_counter()
    pool = serve_pool()
    gen_s = time.perf_counter() - t0
    solo, nnz, host = [], [], []
    for kind, params, (src, dst) in pool:
        g = ctx.graph_from_edges(src, dst)
        solo.append(ctx.count(g))
        nnz.append(g.nnz)
        host.append(g.download())
        g.free()
    small_edges = 1 << 20
    is_small = [len(p[2][0]) <= small_edges for p in pool]
    rates = [float(x) for x in args.rates.split(",")]
    rng = random.Random(0x5EED5E7E)
    sweep = []

    def pct(v, q):
        return v[min(len(v) - 1, int(q * len(v)))] if v else None

    clocks = ClockSampler(local)
    clocks.start()
    srv = tc.Server(ctx, hbm_budget_frac=0.8, max_batch=256, small_edges=small_edges)
    h2d = 0
    for rate in rates:
        picks = [rng.randrange(len(pool)) for _ in range(args.requests)]
        gaps = [rng.expovariate(rate) for _ in range(args.requests)]
        ids = []
        start = time.perf_counter()
        t_next = start
        for k, gi in zip(picks, gaps):
            t_next += gi
            dt = t_next - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            src, dst = pool[k][2]
            ids.append(srv.submit(src, dst, key=k + 1))
            h2d += 16 * len(src)
        lat, lat_s, lat_l, edges = [], [], [], 0
        for rid, k in zip(ids, picks):
            c, ms = srv.wait(rid)
            assert c == solo[k], "serving result differs from the solo count"
            lat.append(ms)
            (lat_s if is_small[k] else lat_l).append(ms)
            edges += nnz[k]
        wall = time.perf_counter() - start
        lat.sort()
        lat_s.sort()
        lat_l.sort()
        st = srv.stats()
        sweep.append({"rate_rps": rate, "requests": len(ids), "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                      "max_ms": lat[-1], "small_p50_ms": pct(lat_s, 0.5), "small_p99_ms": pct(lat_s, 0.99),
                      "large_p50_ms": pct(lat_l, 0.5), "large_p99_ms": pct(lat_l, 0.99),
                      "small_requests": len(lat_s), "large_requests": len(lat_l),
                      "achieved_rps": len(ids) / wall, "aggregate_edges_per_s": edges / wall,
                      "batches_so_far": st["batches"], "small_batches_so_far": st["small_batches"],
                      "large_batches_so_far": st["large_batches"], "cache_hits_so_far": st["cache_hits"],
                      "evictions_so_far": st["evictions"], "max_batch_seen": st["max_batch_seen"]})
    srv.close()
    clk = clocks.stop()
    t0 = time.perf_counter()
    cpu_ok = all(oracle.count(rp, cl) == solo[i] for i, (rp, cl) in enumerate(host))
    cpu_s = time.perf_counter() - t0
    top = sweep[-1]
    low = sweep[0]
    cfg = {"workload": "serve_poisson", "pool_graphs": len(pool), "pool_oriented_edges": sum(nnz),
           "pool_edges_range": [min(nnz), max(nnz)], "rates_rps": rates, "requests_per_rate": args.requests,
           "hbm_budget": "80% of device memory", "small_lane": f"requests of at most {small_edges} edges",
           "exact": "every result equals the graph's solo count"}
    res = {"metric": "serve aggregate oriented edges/s", "value": top["aggregate_edges_per_s"], "unit": UNIT,
           "n_gpus": world, "steps": len(rates), "warmup": 0, "ms_per_step": None, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded R-MAT / Chung-Lu pool, Poisson arrivals)", "config": cfg,
           "detail": {"sweep": sweep, "host_generate_s": gen_s},
           "p50_ms": low["p50_ms"], "p99_ms": low["p99_ms"], "rate_rps": low["rate_rps"],
           "p50_p99_note": f"p50 / p99 at the lowest offered rate ({low['rate_rps']:g} req/s); every rate in "
                           "detail.sweep",
           "clocks": clk,
           "e2e": {"value": top["aggregate_edges_per_s"], "unit": UNIT,
                   "h2d_bytes_per_step": h2d // max(1, len(rates)), "d2h_bytes_per_step": 8 * args.requests,
                   "path": "tc_server_submit -> tc_server_wait: host edge lists in, counts out (the measurement "
                           "is end to end by construction)"},
           "roofline": None,
           "roofline_note": "a mixed stream of builds and batched counts: the count kernel's roofline is on the "
                            "rmat23_parts and batch256 lines",
           "cpu_baseline": {"value": sum(nnz) / cpu_s, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                            "sample": "every pool graph counted once by the OpenMP oracle", "seconds": cpu_s,
                            "count_matches": cpu_ok}}
    ctx.close()
    return res


def run_io(args, world, rank, local, pg):
    """The TC_128 driver's host path (its time goes to reading the .csr text):
    R-MAT 21's oriented CSR written as a .csr file, read by the reference's
    one-fscanf-per-integer loop (restated in the oracle, one thread) and by the
    library's parallel text parser, and written and read back as the binary
    .tcsr.  Host work only; rank 0 runs it."""
    import shutil
    import tempfile

    import oracle
    import trianglecount_gb300 as tc
    from trianglecount_gb300 import formats as F
    from trianglecount_gb300 import generators as gen
    if rank != 0:
        return None
    with tc.Context(local) as ctx:
        g = ctx.graph_from_edges(*gen.rmat(21, 16))
        rp, col = g.download()
        g.free()
    V, E = len(rp) - 1, len(col)
    d = tempfile.mkdtemp(prefix="tc_io_")
    try:
        text = os.path.join(d, "rmat21_output.csr")
        F.write_csr(text, V, 2 * E, rp, col)
        text_bytes = os.path.getsize(text)
        n_ints = 4 + (V + 1) + E
        t0 = time.perf_counter()
        hdr, r1, c1 = oracle.read_csr_fscanf(text)
        fscanf_s = time.perf_counter() - t0
        assert np.array_equal(r1, rp) and np.array_equal(c1, col)
        del r1, c1
        parse_s = []
        for _ in range(max(3, args.steps)):
            t0 = time.perf_counter()
            fast = F.read_csr(text)
            parse_s.append(time.perf_counter() - t0)
        assert np.array_equal(fast.row_ptr, rp) and np.array_equal(fast.col, col)
        del fast
        bin_path = os.path.join(d, "rmat21.tcsr")
        t0 = time.perf_counter()
        F.write_tcsr(bin_path, rp, col)
        tcsr_write_s = time.perf_counter() - t0
        tcsr_read_s = []
        for _ in range(max(3, args.steps)):
            t0 = time.perf_counter()
            r2, c2, _, _ = F.read_tcsr(bin_path)
            tcsr_read_s.append(time.perf_counter() - t0)
        assert np.array_equal(r2, rp) and np.array_equal(c2, col)
        tcsr_bytes = os.path.getsize(bin_path)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    parse = statistics.median(parse_s)
    cfg = {"workload": "rmat21_csr_text_io", "V": V, "oriented_edges": E, "text_bytes": text_bytes,
           "integers": n_ints, "fscanf_s": fscanf_s, "parallel_parse_s": parse,
           "parallel_parse_gbs": text_bytes / parse / 1e9, "speedup_vs_fscanf": fscanf_s / parse,
           "tcsr_bytes": tcsr_bytes, "tcsr_write_s": tcsr_write_s, "tcsr_read_s": statistics.median(tcsr_read_s),
           "host_threads": os.cpu_count(), "note": "host work; files on the local disk (page cache warm after the write)"}
    return {"metric": "integers parsed/s", "value": n_ints / parse, "unit": "integers/s", "n_gpus": world,
            "steps": max(3, args.steps), "warmup": 0, "ms_per_step": parse * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded R-MAT 21)",
            "config": cfg,
            "cpu_baseline": {"value": n_ints / fscanf_s, "unit": "integers/s", "cores": 1, "kind": "port",
                             "sample": "the whole file, the reference's fscanf loop (one thread)"}}


def main():
    args = parse()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        fn = {"rmat23_parts": run_parts, "rmat23_k8_batch": run_k8_batch, "batch256": run_batch,
              "serve": run_serve, "refstudy": run_refstudy, "io": run_io}.get(args.workload, run_ours)
        res = fn(args, world, rank, local, pg)
        if rank == 0 and res is not None:
            print(json.dumps(res), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
