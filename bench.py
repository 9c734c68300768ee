"""Benchmark of the GB300 TurtleSort path; prints one JSON line.

Default workload (the headline metric): n = 2^26 int32 keys, uniform over the
full int32 range, with an int32 index payload (= position); sorted keys/s.

  value   device-resident keys/s: inputs already in HBM, each step restores the
          unsorted input with a device copy (untimed) and times one
          turtle_sort_device call with CUDA events on the sorter's stream.
          The 512 MiB working set (keys + ids) is larger than L2 and the
          restore copy rewrites it, so every step starts from cold L2.
  e2e     the same sort through the reference-facing host API
          (turtle_start + turtle_sync: pinned host buffers, H2D copies,
          sort, D2H copies), wall clock per step.
  roofline  the dominant kernel of the form the tuned table picks: the radix
          form's digit-pass kernel (one read + one write of keys and ids per
          launch, 2 * n * 8 B) or the partition kernel (charged half of the
          two-pass bound), over its average launch time from CUDA events;
          sort_frac: the sort's two-pass bound 4 * n * (4 B key + 4 B id)
          over the step time.  All against the measured HBM copy bandwidth.
  cpu_baseline  the oracle port of the reference algorithm on all host cores,
          plus std::sort (1 thread) and __gnu_parallel::sort on a sample.

`--impl reference` times the reference algorithm's CPU restatement (the
oracle port: the reference has no CPU implementation of the path; its CUDA
code is built on the GPU host only to pin parity, by oracle/ref_build.sh) on
the same workload, and prints the same JSON shape with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "sorted keys/s (64M int32+idx, device-resident)"
UNIT = "keys/s"


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profile_traffic(n: int, kernel: str) -> tuple[float | None, str | None]:
    """DRAM bytes (read + write) per launch of `kernel` and the ncu summary
    they come from, for the workload size the figure was scaled to
    (profiles/traffic.json); (None, None) for other sizes."""
    p = ROOT / "profiles" / "traffic.json"
    try:
        e = json.loads(p.read_text())[kernel]
    except Exception:
        return None, None
    if int(e.get("bench_n", -1)) != n:
        return None, None
    return float(e["bytes_per_launch"]), e.get("summary")


class ClockSampler:
    """nvidia-smi clocks sampled every 200 ms while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, out: Path | None):
        self.out = out
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.out, "w") if self.out else subprocess.PIPE
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                out = None
            if self.out:
                self.f.close()
                out = self.out.read_text()
            self.text = out or ""

    def summary(self, device: int = 0) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.text or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or not f[0].isdigit() or int(f[0]) != device:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baselines(keys: np.ndarray, idx: np.ndarray, threads: int) -> dict:
    """The oracle port of the reference algorithm on all cores (full workload),
    std::sort on one core and __gnu_parallel::sort on all cores (samples)."""
    import oracle
    n = keys.size
    t0 = time.perf_counter()
    oracle.turtle_sort(keys, idx, leaf_max=8192, threads=threads)
    t_port = time.perf_counter() - t0
    ns = min(n, 1 << 23)
    k1, i1 = keys[:ns].copy(), idx[:ns].copy()
    t_std = oracle.cpu_sort_seconds(k1, i1, 0, 1)
    k2, i2 = keys.copy(), idx.copy()
    t_par = oracle.cpu_sort_seconds(k2, i2, 2, threads)
    k3, i3 = keys[:ns].copy(), idx[:ns].copy()
    t_pu = oracle.cpu_sort_seconds(k3, i3, 1, threads)
    return {
        "value": n / t_port, "unit": UNIT, "cores": threads, "kind": "port",
        "sample": f"oracle 3-pivot quicksort restatement on the full {n} int32+idx workload, "
                  f"{threads} OpenMP threads",
        "std_sort_1t_keys_per_s": ns / t_std,
        "std_sort_1t_sample": f"first {ns} elements",
        "gnu_parallel_sort_keys_per_s": n / t_par,
        "std_sort_par_unseq_keys_per_s": ns / t_pu,
        "par_unseq_note": "libstdc++ without TBB runs par_unseq serially",
        "host_threads": oracle.hardware_threads(),
    }


def max_over_ranks(x: float, dist, device) -> float:
    """The largest x over all ranks (the slowest rank's time), or x itself with
    one rank.  `device` is where the reduction tensor lives (cuda for NCCL,
    cpu for gloo)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, n: int, steps: int, slowest_total_s: float) -> float:
    """Whole-job throughput: the keys of every rank over the slowest rank's time."""
    return world * n * steps / slowest_total_s


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from turtlesort_gb300 import datagen as dg
    n = args.n
    keys, idx = dg.sweep_input("a", n)
    threads = os.cpu_count() or 1
    times = []
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.turtle_sort(keys, idx, leaf_max=8192, threads=threads)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    tot = sum(times)
    v = n * len(times) / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (splitmix64, seed 0x7475727432)",
        "config": {"workload": f"sort n={n} int32 keys uniform full range + int32 index"},
        "cpu_baseline": {
            "value": v, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the reference's 3-pivot quicksort restated in C++ (oracle), full workload "
                      "per step; the reference has no CPU sort and its CUDA sources are not "
                      "present on the GPU host"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args) -> None:
    import torch
    import turtlesort_gb300 as ts
    from turtlesort_gb300 import datagen as dg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_
        dist_.init_process_group("nccl")
        dist = dist_

    n = args.n
    keys, idx = dg.sweep_input("a", n)
    dev = torch.device("cuda", local)
    d_src_k = torch.from_numpy(keys).to(dev)
    d_src_i = torch.from_numpy(idx).to(dev)
    d_k = torch.empty_like(d_src_k)
    d_i = torch.empty_like(d_src_i)
    sorter = ts.TurtleSort(np.int32, n, compress=False, track_index=True, device=local)
    if args.form != "auto":
        sorter.set_pivot_rule(args.form)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def one_step(timed: bool):
        with torch.cuda.stream(stream):
            d_k.copy_(d_src_k)
            d_i.copy_(d_src_i)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sorter.sort_device(d_k.data_ptr(), d_i.data_ptr(), n, sh)
            e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        one_step(False)
    torch.cuda.synchronize()
    sorter.status(sh)
    # correctness spot check of the last warm-up result (cheap, untimed)
    out_k = d_k[: 1 << 16].cpu().numpy()
    if not np.all(out_k[:-1] <= out_k[1:]):
        raise RuntimeError("device sort produced unsorted output")

    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = sorter.launches
    sorter.time_kernels(True)
    clocks = ClockSampler(Path(args.clocks_csv) if args.clocks_csv else None)
    events = []
    with clocks:
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            events.append(one_step(True))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    sorter.status(sh)
    launches = sorter.launches - launches0
    nk, part_ms, leaf_ms = sorter.kernel_times(args.steps)
    _, setup_ms, pass_ms = sorter.pass_times(args.steps)
    sorter.time_kernels(False)
    part_ms /= max(nk, 1)
    leaf_ms /= max(nk, 1)
    setup_ms /= max(nk, 1)
    pass_ms /= max(nk, 1)
    form, levels = sorter.last_form, sorter.last_levels
    ms = [a.elapsed_time(b) for a, b in events]
    tot_ms = sum(ms)
    tot_ms = max_over_ranks(tot_ms, dist, dev)
    if dist is not None:
        dist.barrier()
    ms_step = tot_ms / args.steps
    value = job_rate(world, n, args.steps, tot_ms / 1e3)

    # the same steps under the compile-time default configuration (the table
    # disabled), for the tuned-against-default comparison
    sorter.set_tuning(False)
    ev_default = [one_step(True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    sorter.status(sh)
    sorter.set_tuning(True)
    default_ms = sum(a.elapsed_time(b) for a, b in ev_default) / args.steps

    # full check of the final result against the properties of a sort
    fk = d_k.cpu().numpy()
    fi = d_i.cpu().numpy()
    if not (np.all(fk[:-1] <= fk[1:]) and np.array_equal(keys[fi], fk)):
        raise RuntimeError("final device result is not a sorted permutation")

    # end to end through the reference-facing API with pinned host buffers
    h_k = torch.empty(n, dtype=torch.int32, pin_memory=True)
    h_i = torch.empty(n, dtype=torch.int32, pin_memory=True)
    hk, hi = h_k.numpy(), h_i.numpy()
    e2e_t = []
    e2e_launches = 0
    for s in range(args.warmup + args.steps):
        hk[:] = keys
        hi[:] = idx
        l0 = sorter.launches
        sorter.StartSorting(hk, hi)
        secs = sorter.Sync()
        if s >= args.warmup:
            e2e_t.append(secs)
            e2e_launches += sorter.launches - l0
    if not np.array_equal(hk, fk):
        raise RuntimeError("end-to-end result differs from the device result")
    e2e_value = job_rate(world, n, len(e2e_t), max_over_ranks(sum(e2e_t), dist, dev))

    if rank != 0:
        return
    peak, peak_kind = peaks()
    # two-pass bound of the sort: read + write keys and ids twice
    alg_bytes = 4.0 * n * (4 + 4)
    sort_achieved = alg_bytes / (ms_step / 1e3) / 1e9
    if form == "radix":
        # one launch per digit that moves keys; each reads and writes keys and ids once
        launch_bytes = 2.0 * n * (4 + 4)
        kernel_ms = pass_ms / max(levels, 1)
        kernel = f"radix_pass_kernel<uint32_t,true> ({levels} launches per sort, one per digit)"
        note = "one read + one write of keys and ids (2*n*8 B) per digit pass"
        traffic, traffic_src = profile_traffic(n, "radix_pass_kernel")
        split = {"kernel_ms": kernel_ms, "passes_ms": pass_ms,
                 "histogram_and_plan_ms": setup_ms, "finish_ms": leaf_ms}
        overlap = ("ids copy-in runs during the key passes (which carry element positions; "
                   "one gather then maps them to ids); the keys copy-out overlaps the gather")
    else:
        # the two kernels (partition, leaf) are charged one pass each
        launch_bytes = alg_bytes / 2
        kernel_ms = part_ms
        kernel = "persistent_sort_kernel<uint32_t,true> (one launch per sort)"
        note = "one read + one write of keys and ids (2*n*8 B), half of the sort's two-pass bound"
        traffic, traffic_src = profile_traffic(n, "persistent_sort_kernel")
        split = {"kernel_ms": kernel_ms, "leaf_kernel_ms": leaf_ms}
        overlap = ("leaf phase in position slices; each finished slice is copied to the "
                   "host while later slices sort")
    achieved = launch_bytes / (kernel_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (splitmix64 seed 0x7475727432; uniform full int32 range; index = position)",
        "config": {"workload": f"sort n={n} int32 keys + int32 index (64M, uniform)",
                   "n": n, "key": "int32", "payload": "int32", "l2": "inputs (512 MiB) larger "
                   "than L2; each step restores the input with a device copy (untimed)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": traffic_src,
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "kernel": kernel, "form": form,
                     "algorithmic_bytes_per_launch": launch_bytes,
                     "algorithmic_bytes_note": note, **split,
                     "sort_achieved": sort_achieved, "sort_frac": sort_achieved / peak},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 8,
                "path": "turtle_start/turtle_sync (StartSorting/Sync) with pinned host buffers",
                "ms_per_step": 1e3 * sum(e2e_t) / len(e2e_t),
                "ms_min_median_max": [1e3 * min(e2e_t), 1e3 * sorted(e2e_t)[len(e2e_t) // 2],
                                      1e3 * max(e2e_t)],
                "ms_steps": [round(1e3 * t, 3) for t in e2e_t],
                "gpu_launches_per_step": e2e_launches / len(e2e_t),
                "overlap": overlap},
        "tuning": {"table": ts.tuning_source(),
                   "config": ts.tuning_lookup(np.int32, True, n),
                   "tuned_ms_per_step": ms_step,
                   "default_config_ms_per_step": default_ms,
                   "speedup": default_ms / ms_step},
        "gpu_launches": int(launches),
        "wall_s_timed": t_wall,
        "levels": sorter.last_levels,
        "clocks": clocks.summary(local),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baselines(keys, idx, os.cpu_count() or 1)
    print(json.dumps(line), flush=True)
    sorter.close()
    if dist is not None:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", "--keys", dest="n", type=int, default=1 << 26,
                    help="keys per sort (--keys also works under torchrun)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--clocks-csv", default=None)
    ap.add_argument("--form", default="auto", choices=["auto", "radix", "two_level", "sampled"],
                    help="pass form of the sorts (auto: the tuned table's)")
    ap.add_argument("--workload", default="sort64m",
                    choices=["sort64m", "plain12m", "sweep", "multisort", "batched", "wide",
                             "floats", "serving"],
                    help="sort64m (default) is the headline line; the others print their own")
    ap.add_argument("--requests", type=int, default=20000, help="serving: requests in the stream")
    ap.add_argument("--rate", type=float, default=0.0,
                    help="serving: Poisson arrivals per second (0: 60%% of the saturated rate)")
    ap.add_argument("--arena-gb", type=int, default=12,
                    help="serving: pinned host arena that one wave of requests fills (GiB)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "gb300" and args.workload != "sort64m":
        import torch
        import bench_workloads
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        bench_workloads.WORKLOADS[args.workload](args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
