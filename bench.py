"""Benchmark of the GB300 correlator-node path.

Workload (the precision configuration the metric is quoted on): 16 stations x
8 subbands x 32 MHz, dual polarisation, 2-bit, 64 MS/s per subband, 4096
channels, one 2 s integration per step: 8 subband jobs of 32 streams each,
32.8 Gsamples per step.  Inputs are seeded synthetic data of that shape:
uniformly random 2-bit codes in input-node blocks of 2000 bytes per channel,
cubic delay models with |tau| <= 15 ms and |rate| <= 3e-6 s/s, and the
input-node protocol built by the library's own writer.  Inputs (8.2 GB of
protocol bytes per step) exceed the 129 MB L2, so no flush is needed.

value: device-resident throughput, Gsamples/s, from CUDA-event device times of
each job (the protocol bytes already in HBM).  e2e: the same work through the
C ABI with the protocol bytes in pinned host memory, host-to-device copies,
host planning, kernels and the device-to-host copy of the visibilities inside
the timed region (host wall clock around synchronous calls); the 8 subband
jobs run from one host thread each on their own contexts, each correlating
its integration `steps` times back to back, so the host side of one job
overlaps the kernels of the others.

--impl reference times the reference's correlator-node algorithm on the host
cores: the C restatement in oracle/ (the reference's own classes build only
where its checkout is present), one process per subband job in parallel, on a
bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sfxc-1_gb300"))

import numpy as np  # noqa: E402

METRIC = "input Gsamples/s per GB300, TC-FP16 vs FP32 X-step at <=1e-4 vis err vs FP64"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def workload(args, rank=0):
    """The 8 subband jobs of one timeslice; rank r correlates timeslice r (the
    jobs of different ranks are independent, as the manager deals them)."""
    from sfxc_gpu import scenario
    st = scenario.cubic_stations(args.stations, seed=4242, max_delay=15e-3, max_rate=3e-6)
    subs = []
    for sb in range(args.subbands):
        subs.append(scenario.Scenario(
            stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
            channel_freq=4_800_000_000 + sb * 32_000_000, nchan=args.nchan, integration_us=args.integration_us,
            n_integrations=1, sub_integration_us=125000, lead_us=16000 + rank * args.integration_us,
            seed=100 + sb + 1000 * rank, block_bytes=2000, frequency_nr=sb))
    return subs


def samples_per_step(subs):
    s = 0
    for sc in subs:
        s += len(sc.streams()) * sc.integration_us * sc.sample_rate // 1_000_000
    return s


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            v = [x.strip() for x in line.split(",")]
            if len(v) < 9:
                continue
            try:
                sm.append(float(v[1]))
                smax.append(float(v[2]))
            except ValueError:
                continue
            for n, x in zip(names, v[5:9]):
                if x.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_inputs(subs, log):
    """Per job: the job dict with its protocol bytes in pinned host memory."""
    import torch
    from sfxc_gpu import scenario
    jobs = []
    for i, sc in enumerate(subs):
        t = time.time()
        keep = []

        def alloc(n):
            buf = torch.empty(n, dtype=torch.uint8, pin_memory=True)
            keep.append(buf)
            return buf.numpy()

        job = scenario.build_job_bulk(sc, alloc=alloc)
        job["pinned"] = [p[0] for p in job["protocols"]]
        job["keep"] = keep
        jobs.append(job)
        log("built job %d in %.1f s" % (i, time.time() - t))
    return jobs


def scenario_job(sc):
    from sfxc_gpu import scenario
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    return job


def run_gpu(args):
    import torch
    import ctypes as C
    from sfxc_gpu import correlator, lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if rank == 0 else (lambda m: None)
    subs = workload(args, rank)
    total = samples_per_step(subs)
    jobs = build_inputs(subs, log)
    mode = lib.X_TC_HILO if args.x == "tc" else lib.X_FP32
    nodes = [correlator.CorrelatorNode(local, mode) for _ in jobs]
    for n, j in zip(nodes, jobs):
        n.set_parameters(j)

    host_ms = {"set_parameters": 0.0, "push_protocol": 0.0, "run_integration": 0.0}

    def node_step(n, j):
        """One job through the public API: parameters, input bytes, integration."""
        t0 = time.perf_counter()
        n.set_parameters(j)  # each step correlates the job's integration afresh
        t1 = time.perf_counter()
        for k, buf in enumerate(j["pinned"]):
            n._check(n._lib.sfxc_gpu_push_protocol(n._h, k, C.c_void_p(buf.ctypes.data), buf.size))
        t2 = time.perf_counter()
        o, _ = n.run_integration()
        t3 = time.perf_counter()
        return (t1 - t0, t2 - t1, t3 - t2), o

    def step_sequential(keep=None):
        """Jobs one after another: per-job CUDA-event device times are exact.
        keep: a list that receives each job's output bytes."""
        dev_ms, launches, out_bytes = 0.0, 0, 0
        for n, j in zip(nodes, jobs):
            (a, b, c), o = node_step(n, j)
            nb = len(o)
            if keep is not None:
                keep.append(bytes(o))
            host_ms["set_parameters"] += a * 1e3
            host_ms["push_protocol"] += b * 1e3
            host_ms["run_integration"] += c * 1e3
            out_bytes += nb
            t = n.timings()
            dev_ms += t["total_ms"]
            launches += t["launches"]
        return dev_ms, launches, out_bytes

    # One host thread per job context (each context owns its CUDA streams), each
    # correlating its job's integration `count` times back to back, as a
    # correlator node does with consecutive time slices: the host side of one
    # job (protocol copies, planning, output bytes) overlaps the kernels of
    # the others.
    pool = ThreadPoolExecutor(max_workers=len(nodes))

    def node_run(n, j, count):
        return sum(len(node_step(n, j)[1]) for _ in range(count))

    def run_concurrent(count):
        futs = [pool.submit(node_run, n, j, count) for n, j in zip(nodes, jobs)]
        return sum(f.result() for f in futs)

    clocks = ClockSampler()
    # ---- device-resident throughput: CUDA events around each job's kernels
    for _ in range(args.warmup):
        step_sequential()
    for k in host_ms:
        host_ms[k] = 0.0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_total, launches = 0.0, 0
    per_kernel = {}
    for _ in range(args.steps):
        d, l, _ob = step_sequential()
        dev_total += d
        launches += l
        for n in nodes:
            for k, v in n.timings().items():
                per_kernel[k] = per_kernel.get(k, 0.0) + v
    torch.cuda.synchronize()
    # ---- end to end: host buffers in, output bytes out, jobs concurrent
    run_concurrent(args.warmup)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out_bytes = run_concurrent(args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    pool.shutdown()
    # ---- the plain FP32 X-step on the same jobs (device time), for the
    # tensor-core form's speed-up over it
    host_ms_tc = dict(host_ms)  # the comparison below reuses the same step function
    compare = None
    if args.x == "tc" and not args.no_fp32_compare:
        tc_outs = []
        step_sequential(keep=tc_outs)  # untimed: the outputs for the agreement check
        for n in nodes:
            n.close()
        nodes = [correlator.CorrelatorNode(local, lib.X_FP32) for _ in jobs]
        f_outs = []
        step_sequential(keep=f_outs)
        f_total, f_kernel = 0.0, {}
        for _ in range(args.steps):
            f_total += step_sequential()[0]
            for n in nodes:
                for k, v in n.timings().items():
                    f_kernel[k] = f_kernel.get(k, 0.0) + v
        if world > 1:
            from sfxc_gpu import sharding
            f_total = sharding.max_over_ranks([f_total])[0]
        # full-size agreement of the two X-step forms on the same spectra: the
        # FP32 form is within ~1e-6 of the FP64 restatement (tests), so this
        # bounds the tensor-core form's error at the benchmark's own size
        worst = 0.0
        for a, b in zip(tc_outs, f_outs):
            _, va = correlator.split_output(a, args.nchan)
            _, vb = correlator.split_output(b, args.nchan)
            for x, y in zip(va, vb):
                ny = float(np.linalg.norm(y))
                worst = max(worst, float(np.linalg.norm(x - y)) / ny if ny else float(np.linalg.norm(x)))
        compare = (f_total, f_kernel, worst, sum(len(correlator.split_output(a, args.nchan)[1]) for a in tc_outs))
    if world > 1:
        from sfxc_gpu import sharding
        wall, dev_total = sharding.max_over_ranks([wall, dev_total])
    if rank != 0:
        return
    value = total * args.steps * world / (dev_total / 1e3) / 1e9
    e2e = total * args.steps * world / wall / 1e9
    in_bytes = sum(sum(b.size for b in j["pinned"]) for j in jobs)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Gsamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.x == "fp32" else "f16-hilo",
        "data": "synthetic (seeded uniform 2-bit codes, cubic delay models)",
        "config": {"workload": "%d stations x %d subbands x 32 MHz dual-pol 2-bit, %d channels, %.3g s integration"
                               % (args.stations, args.subbands, args.nchan, args.integration_us / 1e6),
                   "x_step": args.x, "streams_per_job": 2 * args.stations, "samples_per_step": total,
                   "l2": "inputs larger than L2 (no flush needed)"},
        "e2e": {"value": round(e2e, 3), "unit": "Gsamples/s", "h2d_bytes_per_step": in_bytes,
                "d2h_bytes_per_step": out_bytes // args.steps, "ms_per_step": round(wall * 1e3 / args.steps, 3)},
        "gpu_launches": launches,
        "clocks": clk,
        "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in per_kernel.items() if k != "launches"},
        "host_call_ms_per_step": {k: round(v / args.steps, 3) for k, v in host_ms_tc.items()},
        "e2e_jobs_concurrent": len(nodes),
        "real_time_factor": round(e2e / (total / (args.integration_us / 1e6) / 1e9), 2),
    }
    line["roofline"] = roofline(args, per_kernel, total)
    if compare is not None:
        f_total, f_kernel, worst, nvis = compare
        f_value = total * args.steps * world / (f_total / 1e3) / 1e9
        line["fp32_x_step"] = {
            "value": round(f_value, 3), "unit": "Gsamples/s", "ms_per_step": round(f_total / args.steps, 3),
            "xstep_ms": round(f_kernel.get("xstep_ms", 0.0) / args.steps, 3),
            "tc_over_fp32": round(value / f_value, 3),
            "tc_over_fp32_xstep": round(f_kernel.get("xstep_ms", 0.0) / max(per_kernel.get("xstep_ms", 0.0), 1e-9), 2),
            "tc_vs_fp32_max_rel_l2": float("%.3g" % worst), "visibility_vectors_compared": nvis}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, quick=True)
    print(json.dumps(line), flush=True)


def roofline(args, per_kernel, total):
    """Dominant kernel against the measured HBM copy bandwidth.  Algorithmic
    bytes per input sample: the X-step reads (M+1)/M spectrum values of 8 B
    (FP16 hi+lo or complex64) = 8.002 B; the windowed FFT reads 4 B
    (fringe-stopped series) and writes 8.002 B; the unpack+fringe stage reads
    0.25 B of 2-bit codes and writes 4 B."""
    try:
        peak = json.load(open(PEAKS))["hbm_gbs"]
        src = "measured"
    except Exception:
        peak, src = 6800.0, "fallback"
    M = args.nchan
    per_sample = {"xstep_ms": 8.0 * (M + 1) / M, "window_fft_ms": 4.0 + 8.0 * (M + 1) / M,
                  "unpack_fringe_ms": 0.25 + 4.0}
    k = max(per_sample, key=lambda n: per_kernel.get(n, 0.0))
    t = per_kernel[k] / args.steps / 1e3
    achieved = per_sample[k] * total / t / 1e9
    # DRAM bytes per input sample (dram__bytes_read + dram__bytes_write) that
    # ncu measured for the tensor-core path's kernels on the one-subband,
    # 4096-channel case; a launch covers one sub-integration chunk of one
    # subband job, so the per-launch traffic scales with the samples it covers
    measured = {"window_fft_ms": 11.87, "xstep_ms": 8.18, "unpack_fringe_ms": 4.27}
    traffic = None
    if args.x == "tc" and M == 4096 and k in measured:
        launches = args.subbands * -(-args.integration_us // 125000)
        traffic = round(measured[k] * total / launches / 1e9, 3)
    return {"kernel": k.replace("_ms", ""), "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_unit": "GB per launch",
            "peak_source": src, "algorithmic_bytes_per_sample": round(per_sample[k], 4)}


def cpu_baseline(args, quick):
    """The C restatement on the host cores: one process per subband job in
    parallel over a bounded sample (the same stations and rates, a shorter
    integration)."""
    from oracle import build_oracle, jobs as oj
    exe = build_oracle.build()
    us = 31250 if quick else 62500
    sub_args = argparse.Namespace(**vars(args))
    sub_args.integration_us = us
    subs = workload(sub_args)
    built = [scenario_job(sc) for sc in subs]
    ncores = min(len(built), os.cpu_count() or 1)
    t0 = time.perf_counter()
    errs = []

    def one(j):
        try:
            oj.correlate(j, impl="oracle")
        except Exception as e:  # pragma: no cover
            errs.append(str(e))

    threads = []
    for j in built:
        th = threading.Thread(target=one, args=(j,))
        th.start()
        threads.append(th)
    for th in threads:
        th.join()
    wall = time.perf_counter() - t0
    if errs:
        raise RuntimeError(errs[0])
    total = samples_per_step(subs)
    return {"value": round(total / wall / 1e9, 5), "unit": "Gsamples/s", "cores": ncores, "kind": "port",
            "sample": "%d subband jobs x %d streams x %.4g s (%.3g Gsamples), FP32 arithmetic, one process per job"
                      % (len(built), len(built[0]["streams"]), us / 1e6, total / 1e9)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import build_oracle
    build_oracle.build()
    vals = []
    base = None
    for _ in range(args.warmup):
        cpu_baseline(args, quick=True)
    for _ in range(args.steps):
        base = cpu_baseline(args, quick=True)
        vals.append(base["value"])
    v = float(np.mean(vals))
    subs = workload(args)
    line = {"metric": METRIC, "value": round(v, 5), "unit": "Gsamples/s", "n_gpus": int(os.environ.get(
        "WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
        "data": "synthetic (seeded uniform 2-bit codes, cubic delay models)",
        "config": {"workload": "%d stations x %d subbands x 32 MHz dual-pol 2-bit, %d channels, %.3g s integration"
                               % (args.stations, args.subbands, args.nchan, args.integration_us / 1e6)},
        "cpu_baseline": dict(base, value=round(v, 5)),
        "e2e": {"value": round(v, 5), "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--x", default="tc", choices=["fp32", "tc"])
    ap.add_argument("--no-fp32-compare", action="store_true",
                    help="skip the device-time run of the FP32 X-step beside the tensor-core one")
    ap.add_argument("--stations", type=int, default=16)
    ap.add_argument("--subbands", type=int, default=8)
    ap.add_argument("--nchan", type=int, default=4096)
    ap.add_argument("--integration-us", type=int, default=2_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    import __graft_entry__
    __graft_entry__.build()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
