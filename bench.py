#!/usr/bin/env python
"""Benchmark of the exact kNN self-join on GB300.

Workload (one "step"): the full self-join of the 25M-point 2-D float32
sky-like dataset at k=64, BETA=0.025 (the configuration the reference's
headline figure is quoted on, README.md:34-37, with a seeded synthetic
stand-in for the Gaia DR2 file) -- reorder, eps0, grid build, starting radii
and every search pass -- with the points resident in HBM and the N x (k+1)
result table left in HBM.  value = queries/s over all ranks with the learned
starting radius; the plain BETA schedule is timed on the same data beside it
(plain_beta, learned_over_plain) and its table compared bit for bit
(identical_to_plain).  e2e = the learned join through the host API
(knnsj_selfjoin) from pinned host memory, host->device input copy and
device->host result copy inside the timed region.

The reference arm (--impl reference) times the CPU restatement of the
reference's algorithm (oracle/) on the host cores, on a bounded sample.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "sky2d_25m"
METRIC = "exact KNN queries/s on 1 GB300: learned-radius vs plain BETA; HBM roofline %"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64, device="cuda" if self.pg.get_backend() == "nccl" else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return {"hbm_gbs": float(j["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(workload: str):
    """DRAM traffic per search launch from the committed ncu summary, scaled to
    this workload when the capture was a smaller case of the same kernel."""
    p = os.path.join(ROOT, "profiles", "search_kernel_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        j = json.load(f)
    return j.get(workload)


def cpu_baseline(x, k: int, beta: float, di: int, n_sample: int, seed: int = 0) -> dict:
    """The oracle (CPU restatement of the reference pipeline: its host grid
    construction with a parallel sort, a per-query ring scan with a bounded
    heap, the same retry schedule) on all host cores.  One run does the full
    preprocessing of all N points (reorder, eps0, grid and every rebuild) and
    the search passes of a seeded query subsample; the full join's time is
    that run with the search part scaled by N / sample."""
    import numpy as np

    import oracle
    n = x.shape[0]
    q = np.sort(np.random.default_rng(seed).choice(n, n_sample, replace=False)).astype(np.uint32)
    threads = oracle.max_threads()
    t0 = time.perf_counter()
    rc, _, _, st = oracle.join(x, k, di=di, beta=beta, queries=q)
    wall = time.perf_counter() - t0
    assert rc == 0, rc
    # preprocessing and the grid rebuilds of each radius growth cost the same
    # for any number of queries; only the search passes scale with them
    t_full = st.seconds_prep + st.seconds_regrid + st.seconds_search * n / n_sample
    return {"value": n / t_full, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": (f"oracle/ (CPU restatement of the reference pipeline, OpenMP, {threads} threads): "
                       f"reorder + eps0 + grid on all {n} points ({st.seconds_prep:.2f} s), "
                       f"{st.reindexes} grid rebuilds ({st.seconds_regrid:.2f} s) and the search passes of a "
                       f"seeded {n_sample}-query subsample = {100.0 * n_sample / n:.2f}% of the queries "
                       f"({st.seconds_search:.2f} s, {st.iterations} passes); value = N / (prep + rebuilds + "
                       f"search x N/{n_sample})"),
            "ms_per_join_extrapolated": t_full * 1e3, "ms_observed": wall * 1e3,
            "sample_queries": n_sample}


def make_workload():
    from hybrid_k_nearest_neighbor_self_join_gb300 import datasets
    gen, k, beta, di = datasets.CONFIGS[WORKLOAD]
    return gen(), k, beta, di


def workload_config(n: int, d: int, k: int, beta: float, di: int) -> dict:
    """The `config` of both arms' lines (identical by construction)."""
    return {"workload": WORKLOAD, "n_points": n, "d": d, "k": k, "beta": beta, "num_indexed_dims": di,
            "l2": "inputs (200 MB) and outputs (13 GB) exceed the 129 MB L2; no flush"}


def config_records(kj, torch, steps: int = 2) -> dict:
    """The other configurations, device-resident, learned and plain starting
    radius on the same data with their tables compared bit for bit: the
    uniform 100k-point 2-D set (k=8, BETA=0), the 10M-point 6-D float64
    mixture (k=16, BETA=0.05), the held-out 5M-point 4-D mixture (k=128), and
    the 512 uneven sets through the batched host API (learned radius)."""
    import numpy as np

    from hybrid_k_nearest_neighbor_self_join_gb300 import datasets
    out = {}
    fp64_peak = 1.25e12  # nominal GB300 FP64 FLOP/s
    for name in ("uniform2d_100k", "gmm6d_10m", "heldout4d_5m"):
        gen, k, beta, di = datasets.CONFIGS[name]
        x = gen()
        n, d = x.shape
        tx = torch.from_numpy(x).cuda()
        tids = torch.empty((n, k + 1), dtype=torch.int32, device="cuda")
        td = torch.empty((n, k + 1), dtype=tx.dtype, device="cuda")
        # joins of a millisecond or so are timed over 20 calls, the large ones
        # over `steps`
        reps = steps if n > 1_000_000 else 20
        rec = {"n_points": n, "d": d, "k": k, "beta": beta, "num_indexed_dims": di, "dtype": str(x.dtype),
               "joins_timed": reps}
        tables = {}
        for label, mode in (("learned", kj.RADIUS_LEARNED), ("plain", kj.RADIUS_PLAIN)):
            kj.selfjoin_device(tx.data_ptr(), x.dtype, n, d, k, tids.data_ptr(), td.data_ptr(),
                               num_indexed_dims=di, beta=beta, radius_mode=mode)  # warm-up
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            sts = [kj.selfjoin_device(tx.data_ptr(), x.dtype, n, d, k, tids.data_ptr(), td.data_ptr(),
                                      num_indexed_dims=di, beta=beta, radius_mode=mode) for _ in range(reps)]
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            st = sts[-1]
            r = {"ms_per_join": ms, "queries_per_s": n / (ms / 1e3), "iterations": st["iterations"],
                 "queries_run": st["queries_run"], "re_attempts": st["queries_run"] - n,
                 "candidates": st["candidates"], "ms_search_kernels": st["ms_search_kernels"],
                 "regrids": st["regrids"]}
            if x.dtype == np.float64:
                # FP64 arithmetic of the candidates a double join evaluates
                # (3d per candidate), against the nominal FP64 rate; the float
                # prefilter moves most of it to the FP32 pipe
                r["fp64_frac_of_nominal"] = st["search_alg_flops"] / (st["ms_search_kernels"] / 1e3) / fp64_peak
                r["hbm_gbs_alg"] = st["search_alg_bytes"] / (st["ms_search_kernels"] / 1e3) / 1e9
            rec[label] = r
            tables[label] = (tids.clone(), td.clone())
        a, b = tables["learned"], tables["plain"]
        bits = torch.int32 if x.dtype == np.float32 else torch.int64
        rec["identical_to_plain"] = bool(torch.equal(a[0], b[0]) and torch.equal(a[1].view(bits), b[1].view(bits)))
        rec["learned_over_plain"] = rec["plain"]["ms_per_join"] / rec["learned"]["ms_per_join"]
        out[name] = rec
        del tx, tids, td, tables, a, b
        torch.cuda.empty_cache()
    # 512 uneven sets, batched host API (host buffers: copies included)
    sets = list(datasets.batched_sets())
    xs = [x for x, _ in sets]
    ks = [k for _, k in sets]
    kj.selfjoin_batched(xs, ks, beta=0.05, radius_mode=kj.RADIUS_LEARNED)  # warm-up (and autotuning)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        kj.selfjoin_batched(xs, ks, beta=0.05, radius_mode=kj.RADIUS_LEARNED)
        times.append(time.perf_counter() - t0)
    npts = sum(x.shape[0] for x in xs)
    out["batched_512"] = {"sets": len(sets), "n_points": npts, "ms_per_call": 1e3 * statistics.median(times),
                          "queries_per_s": npts / statistics.median(times),
                          "note": "host buffers in and out (copies inside the timing), learned radius"}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    x, k, beta, di = make_workload()
    n, d = x.shape
    res = []
    # warm-up steps are shorter (they only warm the page cache and threads)
    for i in range(args.warmup):
        cpu_baseline(x, k, beta, di, max(1000, args.cpu_sample // 10), seed=1000 + i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        res.append(cpu_baseline(x, k, beta, di, args.cpu_sample, seed=i))
    wall_ms = (time.perf_counter() - t0) * 1e3
    vals = [r["value"] for r in res]
    v = statistics.median(vals)
    ms_extra = statistics.median([r["ms_per_join_extrapolated"] for r in res])
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(n, d, k, beta, di),
        "ms_per_join_extrapolated": ms_extra,
        "step_meaning": (f"one step = the oracle's full preprocessing of all {n} points plus the search of a "
                         f"seeded {args.cpu_sample}-query subsample ({100.0 * args.cpu_sample / n:.2f}%); "
                         "ms_per_step is that step's observed wall time, value the full join's queries/s "
                         "with the search scaled by N / sample (ms_per_join_extrapolated)"),
        "cpu_baseline": {"value": v, "unit": "queries/s", "cores": res[0]["cores"], "kind": "port",
                         "sample": res[0]["sample"]},
        "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import numpy as np
    import torch

    import hybrid_k_nearest_neighbor_self_join_gb300 as kj

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = Dist(world, "nccl")
    x, k, beta, di = make_workload()
    n, d = x.shape
    K = k + 1
    # ---- device-resident joins -------------------------------------------
    tx = torch.from_numpy(x).cuda()
    tids = torch.empty((n, K), dtype=torch.int32, device="cuda")
    td = torch.empty((n, K), dtype=torch.float32, device="cuda")

    def step(mode):
        return kj.selfjoin_device(tx.data_ptr(), np.float32, n, d, k, tids.data_ptr(), td.data_ptr(),
                                  num_indexed_dims=di, beta=beta, radius_mode=mode)

    def timed(mode, steps, warmup):
        for _ in range(warmup):
            step(mode)
        torch.cuda.synchronize()
        dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        sts = [step(mode) for _ in range(steps)]
        e1.record()
        torch.cuda.synchronize()
        dist.barrier()
        return dist.max(e0.elapsed_time(e1)), sts

    # the learned radius (the headline) first, then the plain BETA schedule
    # (the comparison); both must leave the same table, checked bit for bit
    clocks = ClockSampler(local)
    clocks.start()
    t_ms, sts = timed(kj.RADIUS_LEARNED, args.steps, args.warmup)
    clk = clocks.stop()
    ref_ids, ref_d = tids.clone(), td.clone()
    tids.fill_(-1)
    t_plain, st_plain = timed(kj.RADIUS_PLAIN, max(2, min(args.steps, 3)), 1)
    identical = bool(torch.equal(tids, ref_ids) and torch.equal(td.view(torch.int32), ref_d.view(torch.int32)))
    del ref_ids, ref_d
    st = sts[-1]
    ms_per_step = t_ms / args.steps
    value = n * world * args.steps / (t_ms / 1e3)
    plain_steps = len(st_plain)
    plain_value = n * world * plain_steps / (t_plain / 1e3)

    # ---- end to end through the host API, pinned buffers ------------------
    hx = torch.from_numpy(x).pin_memory()
    hids = torch.empty((n, K), dtype=torch.int32).pin_memory()
    hd = torch.empty((n, K), dtype=torch.float32).pin_memory()
    xs_np, ids_np, d_np = hx.numpy(), hids.numpy(), hd.numpy()

    def host_step():
        return kj.selfjoin(xs_np, k, num_indexed_dims=di, beta=beta, radius_mode=kj.RADIUS_LEARNED,
                           out_ids=ids_np, out_dists=d_np, return_stats=True)[2]

    host_step()
    torch.cuda.synchronize()
    dist.barrier()
    e2e_steps = max(1, args.steps)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(e2e_steps + 1)]
    marks[0].record()
    e2e_stats = []
    for i in range(e2e_steps):
        e2e_stats.append(host_step())
        marks[i + 1].record()
    torch.cuda.synchronize()
    t_e2e = dist.max(marks[0].elapsed_time(marks[-1]))
    e2e_value = n * world * e2e_steps / (t_e2e / 1e3)
    e2e_ms_steps = [round(marks[i].elapsed_time(marks[i + 1]), 2) for i in range(e2e_steps)]
    # rows reached the host during the join (written straight into the
    # pinned buffers) when no copy outlasted it: one copy of the 13 GB table
    # after the join takes tens of ms
    e2e_streamed = all(s_["ms_transfer"] < 0.5 * s_["ms_search"] for s_ in e2e_stats)

    # ---- roofline of the dominant kernel (the search) ----------------------
    pk = peaks()
    kms = statistics.median([s_["ms_search_kernels"] for s_ in sts])
    ab = statistics.median([s_["search_alg_bytes"] for s_ in sts])
    fl = statistics.median([s_["search_alg_flops"] for s_ in sts])
    achieved = ab / (kms / 1e3) / 1e9
    tr = ncu_traffic(WORKLOAD)
    # second roof: the FP32 pipe (152 SMs x 128 lanes x 2 flops x clock)
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_ach = fl / (kms / 1e3) / 1e12
    roofline = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": tr["dram_bytes_per_join"] if tr else None,
                "kernel": ("search kernels: tile_kernel<2,65,4> (first pass, query tiles) + search_kernel<float,2,2> "
                           "(retries and hand-overs)"), "kernel_ms_per_step": kms, "launches_per_step":
                st["iterations"], "alg_bytes_per_step": ab,
                "peak_source": f"{pk['source']} hbm_gbs (MEASURED_PEAKS.json): frac is of {pk['source']}",
                "fp32": {"achieved_tflops": fp32_ach, "peak_tflops": fp32_peak, "frac": fp32_ach / fp32_peak,
                         "alg_flops_per_step": fl, "peak_source": "nominal 152x128x2 x median SM clock"}}
    launches = sum(int(s_["kernel_launches"]) for s_ in sts)

    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(n, d, k, beta, di),
        "radius": "learned starting radius (built-in model)", "parallelism": f"replicas x{world}",
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(n * d * 4),
                "d2h_bytes_per_step": int(n * K * 8), "ms_per_step": e2e_ms_steps,
                "steps_detail": [{"ms_prep": round(s_["ms_prep"], 2), "ms_search": round(s_["ms_search"], 2),
                                  "ms_transfer": round(s_["ms_transfer"], 2), "iterations": s_["iterations"]}
                                 for s_ in e2e_stats],
                "rows_written_during_join": e2e_streamed},
        "gpu_launches": launches,
        "roofline": roofline,
        "clocks": clk,
        "plain_beta": {"value": plain_value, "ms_per_step": t_plain / plain_steps, "steps": plain_steps,
                       "iterations": st_plain[-1]["iterations"], "candidates": st_plain[-1]["candidates"],
                       "ms_search_kernels": st_plain[-1]["ms_search_kernels"]},
        "learned_over_plain": value / plain_value,
        "identical_to_plain": identical,
        "stats_last_step": {kk: st[kk] for kk in ("eps0", "iterations", "regrids", "candidates", "queries_run",
                                                  "ms_prep", "ms_search", "ms_search_kernels", "nonempty_cells")},
    }
    if rank == 0 and world == 1 and not args.no_configs:
        del tx, tids, td
        torch.cuda.empty_cache()
        line["configs"] = config_records(kj, torch)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(x, k, beta, di, args.cpu_sample)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def run_profile_case(which: str, mode: str):
    """One device-resident join for profiler captures.  'full' is the bench
    workload; 'slice' is its longitude slice x < 57.6 deg (about 4M points,
    the same densities), small enough for multi-pass ncu captures.  mode:
    'learned' (the bench headline) or 'plain'."""
    import numpy as np
    import torch

    import hybrid_k_nearest_neighbor_self_join_gb300 as kj
    x, k, beta, di = make_workload()
    if which == "slice":
        x = np.ascontiguousarray(x[x[:, 0] < 57.6])
    n, d = x.shape
    tx = torch.from_numpy(x).cuda()
    tids = torch.empty((n, k + 1), dtype=torch.int32, device="cuda")
    td = torch.empty((n, k + 1), dtype=torch.float32, device="cuda")
    st = kj.selfjoin_device(tx.data_ptr(), np.float32, n, d, k, tids.data_ptr(), td.data_ptr(),
                            num_indexed_dims=di, beta=beta,
                            radius_mode=kj.RADIUS_LEARNED if mode == "learned" else kj.RADIUS_PLAIN)
    torch.cuda.synchronize()
    print(json.dumps({"case": which, "mode": mode, "n": n, **{kk: st[kk] for kk in (
        "eps0", "iterations", "regrids", "candidates", "queries_run", "ms_prep", "ms_search", "ms_search_kernels",
        "search_alg_bytes", "kernel_launches")}}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=250_000,
                    help="queries the CPU baseline searches per step (1%% of the 25M-point workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations' records")
    ap.add_argument("--profile-case", choices=["full", "slice"], default=None,
                    help="run one join for a profiler capture and exit")
    ap.add_argument("--profile-mode", choices=["learned", "plain"], default="learned")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warning: fewer than 3 warm-up steps")
    if args.impl == "reference":
        return run_reference(args)
    import __graft_entry__
    __graft_entry__.build_library()
    if args.profile_case:
        return run_profile_case(args.profile_case, args.profile_mode)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
