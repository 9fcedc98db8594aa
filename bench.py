"""Benchmark of the GB300 correlator-node path.

Headline workload (the precision configuration the metric is quoted on): 16
stations x 8 subbands x 32 MHz, dual polarisation, 2-bit, 64 MS/s per subband,
4096 channels, one 2 s integration per step: 8 subband jobs of 32 streams,
32.8 Gsamples per step.  Inputs are seeded synthetic data of that shape and
signal model, generated on the GPU before timing: a common analytic sky
signal seen through each station's cubic delay model (|tau| <= 15 ms,
|rate| <= 3e-6 s/s) with its FP64 fringe phase, correlation coefficient 0.01,
station gains 0.5-2x and two RFI tones 30 dB over the per-channel noise at
channel centres, quantised to 2-bit codes at +-0.98 sigma; the input-node
protocol is built by the library's input-node writer.  Inputs (8.2 GB of
protocol bytes per step) exceed the 129 MB L2, so no flush is needed.

value: device-resident throughput, Gsamples/s, from CUDA-event device times of
each job (protocol bytes already in HBM).  e2e: the same work through the C
ABI with the protocol bytes in pinned host memory -- host-to-device copies,
host planning, kernels and the device-to-host copy of the visibilities inside
the timed region (host wall clock around synchronous calls); the subband jobs
run from one host thread each on their own contexts, each correlating its
integration `steps` times back to back.

Besides the headline line's fields, the default run also times the plain FP32
X-step on the same jobs, and two further configurations in device time: the
plain FP32 GPU path (8 stations x 8 subbands x 32 MHz dual-pol, 1 s) and
pulsar binning (10 stations x 4 subbands x 16 MHz dual-pol, 2048 channels,
256 bins plus the off-pulse bin, 1 s) on both X-step forms.

--impl reference times the reference's correlator-node algorithm on the host
cores without the GPU library: the C restatement in oracle/ (the reference's
own classes need its checkout, which this host may not have), one process per
(subband, time slice) job, as many jobs as host cores, over a bounded sample
of the same workload, with inputs built by the restatement's own input node.
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

# The configurations (stations, subbands, channels, integration, sampling).
CONFIGS = {
    "c1": dict(name="2 stations x 1 subband x 16 MHz single-pol 2-bit, 512 channels, 1 s integration",
               stations=2, subbands=1, pols=("R",), sample_rate=32_000_000, bandwidth=16_000_000, nchan=512,
               integration_us=1_000_000, f0=1_600_000_000, df=16_000_000, rho=0.01, gains=False, tones=False,
               pulsar=False),
    "c2": dict(name="8 stations x 8 subbands x 32 MHz dual-pol 2-bit, 4096 channels, 1 s integration",
               stations=8, subbands=8, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, nchan=4096,
               integration_us=1_000_000, f0=4_800_000_000, df=32_000_000, rho=0.01, gains=False, tones=False,
               pulsar=False),
    "c3": dict(name="16 stations x 8 subbands x 32 MHz dual-pol 2-bit, 4096 channels, 2 s integration",
               stations=16, subbands=8, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, nchan=4096,
               integration_us=2_000_000, f0=4_800_000_000, df=32_000_000, rho=0.01, gains=True, tones=True,
               pulsar=False),
    "c5": dict(name="10 stations x 4 subbands x 16 MHz dual-pol 2-bit, 2048 channels, 256+1 pulsar bins, 1 s "
                    "integration", stations=10, subbands=4, pols=("R", "L"), sample_rate=32_000_000,
               bandwidth=16_000_000, nchan=2048, integration_us=1_000_000, f0=1_400_000_000, df=16_000_000, rho=0.01,
               gains=False, tones=False, pulsar=True),
}


def config_of(args):
    cfg = dict(CONFIGS[args.config])
    for k in ("stations", "subbands", "nchan", "integration_us"):
        v = getattr(args, k)
        if v is not None:
            cfg[k] = v
    return cfg


def workload(cfg, rank=0, integration_us=None, lead_extra_us=0, seed_extra=0):
    """The subband jobs of one timeslice; rank r correlates timeslice r (the
    jobs of different ranks are independent, as the manager deals them).
    Returns [(scenario, extra job keys)]."""
    from sfxc_gpu import scenario
    gains = None
    if cfg["gains"]:
        rng = np.random.Generator(np.random.PCG64(4243))
        gains = list(rng.uniform(0.5, 2.0, size=cfg["stations"]))
    st = scenario.cubic_stations(cfg["stations"], seed=4242, max_delay=15e-3, max_rate=3e-6, gains=gains)
    iu = integration_us or cfg["integration_us"]
    out = []
    for sb in range(cfg["subbands"]):
        sc = scenario.Scenario(
            stations=st, pols=cfg["pols"], sample_rate=cfg["sample_rate"], bandwidth=cfg["bandwidth"], bits=2,
            channel_freq=cfg["f0"] + sb * cfg["df"], nchan=cfg["nchan"], integration_us=iu, n_integrations=1,
            sub_integration_us=125000, lead_us=16000 + rank * cfg["integration_us"] + lead_extra_us,
            seed=100 + sb + 1000 * rank + seed_extra, block_bytes=2000, frequency_nr=sb, rho=cfg["rho"])
        extra = scenario.pulsar_params(sc, nbins=256, gate=(0.0, 1.0)) if cfg["pulsar"] else {}
        out.append((sc, extra))
    return out


def samples_per_step(subs):
    return sum(len(sc.streams()) * sc.integration_us * sc.sample_rate // 1_000_000 for sc, _ in subs)


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


def model_source(sc, cfg, device):
    """codes(k, nbytes) for build_job_bulk: the signal model of one subband
    job, generated on the GPU (synth.model_codes_torch)."""
    from sfxc_gpu import scenario, synth
    M = cfg["nchan"]
    tones = []
    if cfg["tones"]:
        # two tones at channel centres, 30 dB over the per-channel power of
        # unit-variance white noise (1/M of the band)
        amp = float(np.sqrt(2 * 1000.0 / M))
        ch_w = sc.sample_rate / (2.0 * M)
        tones = [(round(0.234 * M) * ch_w + ch_w / 2, amp), (round(0.664 * M) * ch_w + ch_w / 2, amp)]
    pulse = None
    if cfg["pulsar"]:
        pulse = synth.PulseModel(t_ref=float(sc.sec0))
    nbytes = scenario.bulk_stream_bytes(sc)
    gen = synth.model_codes_torch(sc.stations, sc.pols, sc.sample_rate, float(sc.channel_freq), nbytes * 4,
                                  float(sc.sec0), sc.rho, sc.seed, tones=tones, pulse=pulse,
                                  band_centre_hz=sc.channel_freq + sc.bandwidth / 2, device=device)
    data = dict(gen)  # (station index, pol) -> packed codes
    keys = sc.streams()
    return lambda k, n: data[keys[k]]


def build_inputs(subs, cfg, signal, log, device="cuda:0"):
    """Per job: the job dict with its protocol bytes in pinned host memory."""
    import torch
    from sfxc_gpu import scenario
    jobs = []
    for i, (sc, extra) in enumerate(subs):
        t = time.time()
        keep = []

        def alloc(n):
            buf = torch.empty(n, dtype=torch.uint8, pin_memory=True)
            keep.append(buf)
            return buf.numpy()

        codes = model_source(sc, cfg, device) if signal == "model" else None
        job = scenario.build_job_bulk(sc, alloc=alloc, codes=codes)
        job.update(extra)
        job["pinned"] = [p[0] for p in job["protocols"]]
        job["keep"] = keep
        jobs.append(job)
        log("built job %d in %.1f s" % (i, time.time() - t))
    torch.cuda.empty_cache()
    return jobs


def measured_peaks():
    try:
        d = json.load(open(PEAKS))
        return d["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


def compute_peaks(lib_handle, device):
    """FP32 FMA and FP16 tensor peaks of this GPU, measured now with the
    library's own probe kernels (sfxc_gpu_measure_peaks)."""
    import ctypes as C
    out = (C.c_double * 4)()
    rc = lib_handle.sfxc_gpu_measure_peaks(device, out)
    if rc != 0:
        return None
    return {"fp32_tflops": round(out[0], 1), "f16_tensor_tflops": round(out[1], 1),
            "how": "own probe kernels: 16 independent FMA chains x 2048 threads per SM; tcgen05.mma kind::f16 "
                   "128x256x16 back to back, one CTA per SM; best of 3 CUDA-event timings"}


class Runner:
    """The jobs of one configuration on one set of contexts."""

    def __init__(self, jobs, device, mode):
        from sfxc_gpu import correlator
        self.jobs = jobs
        self.device = device
        self.nodes = [correlator.CorrelatorNode(device, mode) for _ in jobs]
        for n, j in zip(self.nodes, jobs):
            n.set_parameters(j)
        self.host_ms = {"set_parameters": 0.0, "push_protocol": 0.0, "run_integration": 0.0}

    def close(self):
        for n in self.nodes:
            n.close()

    def node_step(self, n, j):
        """One job through the public API: parameters, input bytes, integration."""
        import ctypes as C
        t0 = time.perf_counter()
        n.set_parameters(j)  # each step correlates the job's integration afresh
        t1 = time.perf_counter()
        for k, buf in enumerate(j["pinned"]):
            n._check(n._lib.sfxc_gpu_push_protocol(n._h, k, C.c_void_p(buf.ctypes.data), buf.size))
        t2 = time.perf_counter()
        o, _ = n.run_integration()
        t3 = time.perf_counter()
        return (t1 - t0, t2 - t1, t3 - t2), o

    def step_sequential(self, keep=None, per_kernel=None):
        """Jobs one after another: per-job CUDA-event device times are exact."""
        dev_ms, launches = 0.0, 0
        for n, j in zip(self.nodes, self.jobs):
            (a, b, c), o = self.node_step(n, j)
            if keep is not None:
                keep.append(bytes(o))
            self.host_ms["set_parameters"] += a * 1e3
            self.host_ms["push_protocol"] += b * 1e3
            self.host_ms["run_integration"] += c * 1e3
            t = n.timings()
            dev_ms += t["total_ms"]
            launches += t["launches"]
            if per_kernel is not None:
                for k, v in t.items():
                    per_kernel[k] = per_kernel.get(k, 0.0) + v
        return dev_ms, launches

    def run_concurrent(self, pool, count):
        """One host thread per job context, each correlating its job `count`
        times back to back: the host side of one job overlaps the kernels of
        the others.  Returns the output bytes."""
        def node_run(n, j):
            return sum(len(self.node_step(n, j)[1]) for _ in range(count))
        futs = [pool.submit(node_run, n, j) for n, j in zip(self.nodes, self.jobs)]
        return sum(f.result() for f in futs)


def worst_rel_l2(outs_a, outs_b, nchan):
    from sfxc_gpu import correlator
    worst, nvis = 0.0, 0
    for a, b in zip(outs_a, outs_b):
        _, va = correlator.split_output(a, nchan)
        _, vb = correlator.split_output(b, nchan)
        for x, y in zip(va, vb):
            ny = float(np.linalg.norm(y))
            worst = max(worst, float(np.linalg.norm(x - y)) / ny if ny else float(np.linalg.norm(x)))
            nvis += 1
    return worst, nvis


# Algorithmic work per input sample of each stage (M channels, 2-bit input):
# bytes read + written, FP32 flops in the 5 N log2 N (complex) / 2.5 N log2 N
# (real) FFT convention.
def stage_work(M, binned_rmw=0.0):
    lg = np.log2(2 * M)
    return {
        "unpack_fringe_ms": {"bytes": 0.25 + 4.0, "flops": 7.5 * 8 + 8.0},
        "window_fft_ms": {"bytes": 4.0 + 8.0 * (M + 1) / M, "flops": 5.0 * lg},
        "xstep_ms": {"bytes": 8.0 * (M + 1) / M + binned_rmw, "flops": None},
    }


def roofline(cfg, per_kernel, total, steps, peaks, x_mode, nbl_per_stream):
    """The dominant kernel against the measured HBM copy bandwidth (its
    traffic bound) and, for the F-step kernels, against the measured FP32
    peak; plus the path bound min(HBM / bytes, FP32 / flops, tensor / X
    flops) per input sample."""
    hbm, src = measured_peaks()
    M = cfg["nchan"]
    work = stage_work(M)
    k = max(work, key=lambda n: per_kernel.get(n, 0.0))
    t = per_kernel[k] / steps / 1e3
    achieved = work[k]["bytes"] * total / t / 1e9
    # DRAM bytes per input sample (dram__bytes_read + dram__bytes_write) that
    # ncu measured for the tensor-core path's kernels on the one-subband,
    # 4096-channel case; a launch covers one sub-integration chunk of one
    # subband job, so the per-launch traffic scales with the samples it covers
    measured = {"window_fft_ms": 11.87, "xstep_ms": 8.18, "unpack_fringe_ms": 4.27}
    traffic = None
    if x_mode == "tc" and M == 4096 and k in measured and not cfg["pulsar"]:
        launches = cfg["subbands"] * -(-cfg["integration_us"] // 125000)
        traffic = round(measured[k] * total / launches / 1e9, 3)
    out = {"kernel": k.replace("_ms", ""), "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
           "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": traffic, "traffic_unit": "GB per launch",
           "peak_source": src, "algorithmic_bytes_per_sample": round(work[k]["bytes"], 4)}
    kernels = {}
    for name, w in work.items():
        if name not in per_kernel:
            continue
        tt = per_kernel[name] / steps / 1e3
        e = {"ms_per_step": round(per_kernel[name] / steps, 3),
             "hbm_gbs": round(w["bytes"] * total / tt / 1e9, 1),
             "hbm_frac": round(w["bytes"] * total / tt / 1e9 / hbm, 4)}
        if w["flops"] and peaks:
            tf = w["flops"] * total / tt / 1e12
            e.update({"fp32_tflops": round(tf, 2), "fp32_frac": round(tf / peaks["fp32_tflops"], 4),
                      "flops_per_sample": round(w["flops"], 1)})
        kernels[name.replace("_ms", "")] = e
    out["kernels"] = kernels
    stages = sum(per_kernel.get(n, 0.0) for n in ("unpack_fringe_ms", "window_fft_ms", "xstep_ms", "normalise_ms",
                                                    "bitstat_ms"))
    if "total_ms" in per_kernel and stages > 1.02 * per_kernel["total_ms"]:
        # the X-step on the context's third stream beside the next chunk's
        # F-step: both kernels' times are their elapsed times while sharing SMs
        out["stages_overlap"] = ("each chunk's X-step runs beside the next chunk's F-step; stage times are elapsed "
                                 "times while they share the SMs (sum %.1f ms, step %.1f ms)"
                                 % (stages / steps, per_kernel["total_ms"] / steps))
    if peaks and work[k]["flops"]:
        tf = work[k]["flops"] * total / t / 1e12
        out["compute"] = {"bound": "fp32", "achieved": round(tf, 2), "peak": peaks["fp32_tflops"], "unit": "TFLOP/s",
                          "frac": round(tf / peaks["fp32_tflops"], 4), "peak_source": "measured by bench.py",
                          "flops_per_sample": round(work[k]["flops"], 1)}
    if peaks:
        fstep_flops = work["unpack_fringe_ms"]["flops"] + work["window_fft_ms"]["flops"]
        xflops = 8.0 * nbl_per_stream
        bounds = {"hbm_fused_gsps": hbm / 0.25, "fp32_fstep_gsps": peaks["fp32_tflops"] * 1e3 / fstep_flops,
                  "xstep_gsps": (peaks["f16_tensor_tflops"] if x_mode == "tc" else peaks["fp32_tflops"]) * 1e3 / xflops}
        pb = min(bounds.values())
        design = hbm / (work["unpack_fringe_ms"]["bytes"] + work["window_fft_ms"]["bytes"] +
                        work["xstep_ms"]["bytes"])
        out["path_bound"] = {"gsps": round(pb, 1), "terms": {k2: round(v, 1) for k2, v in bounds.items()},
                             "unfused_design_hbm_gsps": round(design, 1)}
    return out


def measure(cfg, args, x_mode, log, world=1, rank=0, local=0, e2e=True, compare_fp32=True, peaks=None):
    """Device-resident throughput of one configuration (and, with e2e, the end
    to end figure), its roofline, and the FP32 X-step on the same jobs."""
    import torch
    from sfxc_gpu import lib
    subs = workload(cfg, rank)
    total = samples_per_step(subs)
    jobs = build_inputs(subs, cfg, args.signal, log, device="cuda:%d" % local)
    mode = lib.X_TC_HILO if x_mode == "tc" else lib.X_FP32
    runner = Runner(jobs, local, mode)
    clocks = ClockSampler()
    for _ in range(args.warmup):
        runner.step_sequential()
    for k in runner.host_ms:
        runner.host_ms[k] = 0.0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_total, launches, per_kernel = 0.0, 0, {}
    for _ in range(args.steps):
        d, l = runner.step_sequential(per_kernel=per_kernel)
        dev_total += d
        launches += l
    torch.cuda.synchronize()
    res = {"total": total, "dev_total": dev_total, "launches": launches, "per_kernel": per_kernel,
           "host_ms": dict(runner.host_ms), "jobs": jobs, "subs": subs}
    if e2e:
        pool = ThreadPoolExecutor(max_workers=len(jobs))
        runner.run_concurrent(pool, args.warmup)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out_bytes = runner.run_concurrent(pool, args.steps)
        torch.cuda.synchronize()
        res["wall"] = time.perf_counter() - t0
        res["out_bytes"] = out_bytes
        pool.shutdown()
    res["clocks"] = clocks.stop()
    if x_mode == "tc" and compare_fp32:
        tc_outs = []
        runner.step_sequential(keep=tc_outs)
        runner.close()
        runner = Runner(jobs, local, lib.X_FP32)
        f_outs = []
        runner.step_sequential(keep=f_outs)
        f_total, f_kernel = 0.0, {}
        for _ in range(args.steps):
            f_total += runner.step_sequential(per_kernel=f_kernel)[0]
        worst, nvis = worst_rel_l2(tc_outs, f_outs, cfg["nchan"])
        res["fp32"] = (f_total, f_kernel, worst, nvis)
    runner.close()
    nstreams = len(subs[0][0].streams())
    nbl = len(subs[0][0].stations) * len(cfg["pols"])
    nbl = nbl + (nbl * (nbl - 1) // 2 - (len(subs[0][0].stations) if len(cfg["pols"]) > 1 else 0))
    res["roofline"] = roofline(cfg, per_kernel, total, args.steps, peaks, x_mode, nbl / nstreams)
    return res


C4_NAME = ("20 stations (12 x 32 MHz 2-bit at 64 MS/s, 6 x 64 MHz 2-bit at 128 MS/s, 2 x 16 MHz 1-bit at 32 MS/s); "
           "one 2 s timeslice of 8 jobs in one CUDA graph: 4 x 32 MHz subbands of 40 streams, 4096 channels, 2 s "
           "integration; 2 x 16384 channels (32768-sample FFTs) of 24 streams, 4 x 0.5 s; 2 x 16 MHz subbands of 16 "
           "streams at up to 4x the job rate, 256 channels, 8 x 0.25 s")


def measure_c4(args, log, x_mode="tc"):
    """The batched uneven configuration: every job of one 2 s timeslice, all
    their integrations in one CUDA graph per step (sfxc_gpu_batch_run_counts),
    inputs in pinned host memory pushed through the C ABI each step.  Device time:
    CUDA events around the graph launch, timeslices one after another; e2e:
    wall clock of consecutive timeslices with two in flight (two sets of
    contexts, each timeslice's set-up, pushes and outputs on the host beside
    the other's graph, as a correlator runs a stream of timeslices), and the
    one-at-a-time wall clock beside it."""
    from sfxc_gpu import correlator, lib, scenario
    import torch
    scs = scenario.c4_jobs(scale=1.0)
    jobs, keep = [], []

    def alloc(n):  # protocol bytes in pinned host memory, as the headline e2e
        buf = torch.empty(n, dtype=torch.uint8, pin_memory=True)
        keep.append(buf)
        return buf.numpy()

    for i, sc in enumerate(scs):
        t = time.time()
        j = scenario.build_job_bulk(sc, alloc=alloc)
        jobs.append(j)
        log("built C4 job %d (%d streams, %d channels, %d x %d us) in %.1f s"
            % (i, len(sc.streams()), sc.nchan, sc.n_integrations, sc.integration_us, time.time() - t))
    # input samples: every stream at its own rate over the timeslice
    total = sum(sum(sc.station_modes.get(sc.stations[si].number, (sc.sample_rate,))[0] for si, _ in sc.streams())
                * sc.n_integrations * sc.integration_us // 1_000_000 for sc in scs)
    mode = lib.X_TC_HILO if x_mode == "tc" else lib.X_FP32
    sets = [[correlator.CorrelatorNode(0, mode) for _ in jobs] for _ in range(2)]
    batches = [correlator.Batch(nodes) for nodes in sets]
    try:
        for _ in range(args.warmup):
            for b in batches:
                b.correlate(jobs)
        dev_ms, t0 = 0.0, time.perf_counter()
        split = {}
        for _ in range(args.steps):
            batches[0].correlate(jobs)
            dev_ms += batches[0].last_ms()
            for k, v in batches[0].last_host_ms().items():
                split[k] = split.get(k, 0.0) + v / args.steps
        wall_seq = time.perf_counter() - t0
        # consecutive timeslices, two in flight: timeslice i on context set
        # i % 2, set-ups one at a time (each beside the other set's graph)
        n_e2e = 4 * args.steps  # the pipeline's fill and drain spread over a stream of timeslices
        setup = threading.Lock()
        with ThreadPoolExecutor(max_workers=2) as ex:
            t0 = time.perf_counter()
            futs = []
            for i in range(n_e2e):
                if len(futs) == 2:
                    futs.pop(0).result()
                futs.append(ex.submit(batches[i % 2].correlate, jobs, None, setup))
            for f in futs:
                f.result()
            wall = time.perf_counter() - t0
    finally:
        for b in batches:
            b.close()
        for nodes in sets:
            for n in nodes:
                n.close()
    return {"workload": C4_NAME, "x_step": x_mode, "value": round(total * args.steps / (dev_ms / 1e3) / 1e9, 3),
            "unit": "Gsamples/s", "ms_per_step": round(dev_ms / args.steps, 3), "samples_per_step": total,
            "e2e": {"value": round(total * n_e2e / wall / 1e9, 3), "unit": "Gsamples/s",
                    "ms_per_step": round(wall * 1e3 / n_e2e, 3), "timeslices": n_e2e, "in_flight": 2,
                    "one_at_a_time": {"value": round(total * args.steps / wall_seq / 1e9, 3),
                                      "ms_per_step": round(wall_seq * 1e3 / args.steps, 3)},
                    "batch_call_split_ms": {k: round(v, 3) for k, v in split.items()}},
            "graph_launches_per_step": 1, "jobs": len(jobs),
            "data": "seeded uniform 2-bit/1-bit codes, cubic delay models"}


F1_NAME = ("station front end: VDIF recording, 16 channels x 2 bits x 32 Ms/s in 32-bit words, 8000-byte "
           "payloads, 4 s (515 MB); headers decoded, 16 channels extracted, each channel's protocol for three "
           "1 s slices assembled")
TRACKS16 = [[2 * c + 1, 2 * c] for c in range(16)]


def measure_frontend(args, log):
    """The input node's front end on the device (sfxc_gpu_recording_*): one
    station's VDIF recording read (frame headers decoded, blocks found), all
    16 channels extracted where the frames lie, and every channel's protocol
    for three 1 s slices (delays from a cubic delay model) assembled on the
    device.  value: recording bytes per second with the recording resident in
    HBM; e2e: the same from pinned host memory, its copy to the device inside
    the timed region.  Host wall clock around the synchronous calls (the
    header walk and the writer's records run on the host between kernels)."""
    import torch
    from sfxc_gpu import correlator, lib, scenario, synth, timebase
    seconds, sr, nch = 4, 32_000_000, 16
    st = scenario.cubic_stations(1, seed=5, max_delay=4e-3, max_rate=1e-6)
    sc = scenario.Scenario(stations=st, pols=("R",), sample_rate=sr, bandwidth=sr // 2, bits=2,
                           channel_freq=1_600_000_000, nchan=512, integration_us=1_000_000,
                           n_integrations=seconds - 1, sub_integration_us=1_000_000, lead_us=100_000, seed=3)
    rng = np.random.Generator(np.random.PCG64(11))
    words = np.frombuffer(rng.bytes(seconds * sr * nch * 2 // 8), dtype=np.uint32)
    t = time.time()
    rec = synth.vdif_file_bytes(words, payload_bytes=8000, sample_rate=sr, nchan=nch, bits=2, start_mjd=sc.mjd,
                                start_sec_of_day=sc.sec0)
    pinned = torch.empty(len(rec), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = np.frombuffer(rec, dtype=np.uint8)
    del rec
    log("built the front-end recording (%d bytes) in %.1f s" % (pinned.numel(), time.time() - t))
    dels = scenario.del_tables(sc)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    slices = [(start + k * tint, start + (k + 1) * tint, slice_samples,
               correlator.delay_list(dels[0], start + k * tint, start + (k + 1) * tint, sr, 2))
              for k in range(sc.n_integrations)]
    params = dict(ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0), track_bit_rate=sr, frame_size=8000,
                  n_tracks=32, bits=2, channel_tracks=TRACKS16)
    node = correlator.CorrelatorNode(0, lib.X_FP32)
    resident = pinned.cuda()
    nbytes = pinned.numel()

    def step(src, marks=None):
        t = [time.perf_counter()]
        r = correlator.DeviceRecording(node, src, "vdif", **params)
        t.append(time.perf_counter())
        r.extract(4, 2, TRACKS16)
        t.append(time.perf_counter())
        for c in range(nch):
            r.protocol(c, slices, sr, 2, sc.integration_us, copy=False)
        t.append(time.perf_counter())
        n = r.n_blocks()
        r.close()
        t.append(time.perf_counter())
        if marks is not None:
            marks.update({k: round((t[i + 1] - t[i]) * 1e3, 3) for i, k in enumerate(
                ("read_ms", "extract_ms", "protocol_ms", "release_ms"))})
        return n

    out = {}
    try:
        for name, src in (("value", resident), ("e2e", pinned.numpy())):
            for _ in range(args.warmup):
                nblocks = step(src)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                step(src)
            torch.cuda.synchronize()
            out[name] = (time.perf_counter() - t0) / args.steps
        stages = {}
        step(resident, stages)  # one more step, split by call (synchronous calls, host clock)
    finally:
        node.close()
    # algorithmic bytes: the recording read once, the channels written,
    # read back into the protocol, the protocol written (about the channel bytes)
    chan_bytes = nblocks * 32000
    algo = nbytes + 3 * chan_bytes
    hbm, hbm_src = measured_peaks()
    achieved = algo / out["value"] / 1e9
    return {"workload": F1_NAME, "value": round(nbytes / out["value"] / 1e9, 3), "unit": "GB/s of recording",
            "ms_per_step": round(out["value"] * 1e3, 3), "recording_bytes": nbytes, "reader_blocks": nblocks,
            "real_time_factor": round(seconds / out["value"], 1), "resident_step_split_ms": stages,
            "e2e": {"value": round(nbytes / out["e2e"] / 1e9, 3), "unit": "GB/s of recording",
                    "ms_per_step": round(out["e2e"] * 1e3, 3), "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": 0},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                         "frac": round(achieved / hbm, 3), "peak_source": hbm_src, "unit": "GB/s",
                         "algorithmic_bytes_per_step": algo,
                         "note": "whole front end (host walk and writer records included) against the copy peak"},
            "data": "seeded uniform random payload words, cubic delay model"}


DRIVER_NAME = ("sfxc <ctrl> <vex> on one GPU (sfxc_gpu.run): 8 stations, VDIF 16 channels x 2 bits x 64 MS/s, "
               "8 x 32 MHz dual pol cross-polarised, 4096 channels, one 2 s scan, 1 s integrations")


def measure_driver(args, log):
    """The single-GPU driver on a synthetic experiment written to files
    (tmpfs where the host has one): the control file and VEX schedule
    planned, each station's 768 MB VDIF recording read from its file into
    device memory, channelled and turned into protocol there, the 16 jobs
    (8 subbands x 2 integrations, 16 streams each) correlated and the .cor
    file written.  value: input samples correlated per second of the whole
    run (host wall clock from the files to the written output)."""
    import shutil
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import control_cases
    from sfxc_gpu import lib, run, synth
    names = ["Ef", "Wb", "On", "Mc", "Nt", "Tr", "Jb", "Hh"]
    mjd, sr, nch, t0, secs = 60409, 64_000_000, 16, 43199, 3
    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    d = tempfile.mkdtemp(dir=base)
    try:
        t = time.time()
        os.makedirs(os.path.join(d, "delays"))
        os.makedirs(os.path.join(d, "data"))
        mode = [("FREQ", "f32", names), ("IF", "ifs", names), ("BBC", "bbcs", names), ("THREADS", "t16", names)]
        thr = ("t16", [(0, 2048.0, 16, 2, 8000)], [("CH%02d" % (k + 1), 0, k) for k in range(16)])
        vex = control_cases._base([(n, "dbbc") for n in names], [("dbbc", "Mark5C", "DBBC")], mode,
                                  [control_cases._freq_def("f32", control_cases._chans_rl(8, 32.0), 64.0)],
                                  threads=[thr], nbbc=16,
                                  scans=[("No0001", "2024y100d12h00m00s", "sess", ["SRC1"], [(n, 0, 2) for n in names])])
        ctrl = {"stations": names, "start": "2024y100d12h00m00s", "stop": "2024y100d12h00m02s", "integr_time": 1.0,
                "number_channels": 4096, "cross_polarize": True, "output_file": "file://out/bench.cor",
                "delay_directory": "file://delays", "data_sources": {n: ["file://data/%s.vdif" % n] for n in names}}
        with open(os.path.join(d, "bench.vex"), "w") as f:
            f.write(vex)
        with open(os.path.join(d, "bench.ctrl"), "w") as f:
            json.dump(ctrl, f)
        for k, n in enumerate(names):
            poly = synth.DelayPoly(coeffs=(-1.0e-3 * (k + 1) / 8, 1.0e-6 * (k - 4) / 4, 1.0e-11), t0=43200.0)
            with open(os.path.join(d, "delays", "N24X1_%s.del" % n), "wb") as f:
                f.write(synth.del_file_bytes(n, [("SRC1", mjd, t0 - 4, secs + 8, poly)]))
            rng = np.random.Generator(np.random.PCG64(900 + k))
            words = np.frombuffer(rng.bytes(secs * sr * nch * 2 // 8), dtype=np.uint32)
            synth.vdif_frames_array(words, payload_bytes=8000, sample_rate=sr, nchan=nch, bits=2, start_mjd=mjd,
                                    start_sec_of_day=t0).tofile(os.path.join(d, "data", "%s.vdif" % n))
        log("wrote the driver experiment (%d stations) in %.1f s" % (len(names), time.time() - t))
        cwd = os.getcwd()
        os.chdir(d)
        try:
            x_mode = lib.X_TC_HILO if args.x == "tc" else lib.X_FP32
            for _ in range(max(1, min(args.warmup, 2))):
                run.correlate("bench.ctrl", "bench.vex", x_mode=x_mode)
            runs = []
            for _ in range(max(1, args.steps)):
                st = {}
                t1 = time.perf_counter()
                files = run.correlate("bench.ctrl", "bench.vex", x_mode=x_mode, stats=st)
                st["wall_s"] = time.perf_counter() - t1
                runs.append(st)
        finally:
            os.chdir(cwd)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    best = min(runs, key=lambda r: r["wall_s"])
    samples = best["samples"]
    return {"workload": DRIVER_NAME, "metric": "input Gsamples/s through sfxc <ctrl> <vex>",
            "value": round(samples / best["wall_s"] / 1e9, 3), "unit": "Gsamples/s",
            "ms_per_run": round(best["wall_s"] * 1e3, 1), "runs": len(runs), "samples_per_run": samples,
            "recording_bytes": best["recording_bytes"], "x_step": args.x,
            "real_time_factor": round(2.0 / best["wall_s"], 2),
            "phase_s": {k[:-2]: v for k, v in best.items() if k.endswith("_s") and k != "wall_s"},
            "output_bytes": sum(len(b) for b in files.values()),
            "data": "seeded uniform random VDIF payloads on tmpfs; cubic delay models; best of the timed runs"}


def summary(cfg, res, args, x_mode, world=1):
    value = res["total"] * args.steps * world / (res["dev_total"] / 1e3) / 1e9
    d = {"workload": cfg["name"], "value": round(value, 3), "unit": "Gsamples/s",
         "ms_per_step": round(res["dev_total"] / args.steps, 3), "x_step": x_mode,
         "samples_per_step": res["total"],
         "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in res["per_kernel"].items() if k != "launches"},
         "gpu_launches": res["launches"], "roofline": res["roofline"],
         "real_time_factor_device": round(value / (res["total"] / (cfg["integration_us"] / 1e6) / 1e9), 2)}
    if "fp32" in res:
        f_total, f_kernel, worst, nvis = res["fp32"]
        f_value = res["total"] * args.steps * world / (f_total / 1e3) / 1e9
        d["fp32_x_step"] = {
            "value": round(f_value, 3), "unit": "Gsamples/s", "ms_per_step": round(f_total / args.steps, 3),
            "xstep_ms": round(f_kernel.get("xstep_ms", 0.0) / args.steps, 3),
            "tc_over_fp32": round(value / f_value, 3),
            "tc_over_fp32_xstep": round(f_kernel.get("xstep_ms", 0.0) /
                                        max(res["per_kernel"].get("xstep_ms", 0.0), 1e-9), 2),
            "tc_vs_fp32_max_rel_l2": float("%.3g" % worst), "visibility_vectors_compared": nvis}
    return d


def run_gpu(args):
    import torch
    from sfxc_gpu import lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if rank == 0 else (lambda m: None)
    cfg = config_of(args)
    peaks = compute_peaks(lib.load(), local)
    log("compute peaks: %s" % peaks)
    res = measure(cfg, args, args.x, log, world, rank, local, e2e=True, compare_fp32=not args.no_fp32_compare,
                  peaks=peaks)
    wall, dev_total = res["wall"], res["dev_total"]
    if world > 1:
        from sfxc_gpu import sharding
        wall, dev_total = sharding.max_over_ranks([wall, dev_total])
        res["dev_total"] = dev_total
    extra = {}
    if not args.no_extra_configs and world == 1:
        for name in ("c2", "c5"):
            c = dict(CONFIGS[name])
            modes = ("fp32",) if name == "c2" else ("tc",)
            for m in modes:
                r = measure(c, args, m, log, e2e=False, compare_fp32=(m == "tc"), peaks=peaks)
                extra[name] = summary(c, r, args, m)
        extra["c4"] = measure_c4(args, log)
        extra["f1"] = measure_frontend(args, log)
    if rank != 0:
        return
    total = res["total"]
    value = total * args.steps * world / (dev_total / 1e3) / 1e9
    e2e = total * args.steps * world / wall / 1e9
    in_bytes = sum(sum(b.size for b in j["pinned"]) for j in res["jobs"])
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Gsamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.x == "fp32" else "f16-hilo",
        "data": "synthetic (%s)" % ("signal model generated on the GPU: delayed analytic sky signal with FP64 fringe "
                                    "phase, gains, RFI tones" if args.signal == "model" else "seeded uniform 2-bit codes"),
        "config": {"workload": cfg["name"], "x_step": args.x, "streams_per_job": len(res["subs"][0][0].streams()),
                   "samples_per_step": total, "l2": "inputs larger than L2 (no flush needed)"},
        "e2e": {"value": round(e2e, 3), "unit": "Gsamples/s", "h2d_bytes_per_step": in_bytes,
                "d2h_bytes_per_step": res["out_bytes"] // args.steps, "ms_per_step": round(wall * 1e3 / args.steps, 3)},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in res["per_kernel"].items() if k != "launches"},
        "host_call_ms_per_step": {k: round(v / args.steps, 3) for k, v in res["host_ms"].items()},
        "e2e_jobs_concurrent": len(res["jobs"]),
        "real_time_factor": round(e2e / (total / (cfg["integration_us"] / 1e6) / 1e9), 2),
        "compute_peaks": peaks,
        "roofline": res["roofline"],
    }
    s = summary(cfg, res, args, args.x, world)
    if "fp32_x_step" in s:
        line["fp32_x_step"] = s["fp32_x_step"]
    line.update(extra)
    if not args.no_cpu_baseline and world == 1:  # rank 0 at one GPU only
        line["cpu_baseline"] = cpu_baseline(cfg, args.cpu_sample_us)
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- CPU arm ---
def oracle_job(sc, extra):
    """A job for the C restatement with its inputs built by the restatement's
    own input node (delay lists and protocol bytes): no GPU library involved."""
    from oracle import jobs as oj
    from sfxc_gpu import scenario

    def delays(db, s0, s1, sr, bits):
        return oj.delays(db, s0, s1, sr, bits, impl="oracle")[0]

    def protocol(blocks, slices, sr, bits, integr_us):
        return oj.protocol(blocks, slices, sr, bits, integr_us, impl="oracle")

    job = scenario.build_job(sc, delays, protocol, fast_random=True)
    job.update(extra)
    return job


_CPU_JOBS = {}


def cpu_baseline(cfg, sample_us, log=lambda m: None):
    """The C restatement on the host cores: as many (subband, time slice) jobs
    as host cores -- one correlator-node process each, the reference's own
    decomposition -- each a bounded sample of `sample_us` of every stream of
    its subband, timed together."""
    from oracle import build_oracle, jobs as oj
    build_oracle.build()
    nproc = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    slices = max(1, nproc // cfg["subbands"])
    key = (cfg["name"], sample_us, slices)
    if key not in _CPU_JOBS:  # inputs built once per process, outside the timed region
        t0 = time.time()
        with ThreadPoolExecutor(max_workers=nproc) as ex:
            futs = []
            for s in range(slices):
                subs = workload(cfg, integration_us=sample_us, lead_extra_us=s * sample_us, seed_extra=7 * s)
                futs += [ex.submit(oracle_job, sc, extra) for sc, extra in subs]
            _CPU_JOBS[key] = [f.result() for f in futs]
        log("built %d CPU jobs in %.1f s" % (len(_CPU_JOBS[key]), time.time() - t0))
    built = _CPU_JOBS[key]
    errs = []

    def one(j):
        try:
            oj.correlate(j, impl="oracle")
        except Exception as e:  # pragma: no cover
            errs.append(str(e))

    t0 = time.perf_counter()
    threads = [threading.Thread(target=one, args=(j,)) for j in built]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    wall = time.perf_counter() - t0
    if errs:
        raise RuntimeError(errs[0])
    total = sum(len(j["streams"]) * sample_us * j["sample_rate"] // 1_000_000 for j in built)
    return {"value": round(total / wall / 1e9, 5), "unit": "Gsamples/s", "cores": min(nproc, len(built)),
            "nproc": nproc, "kind": "port",
            "sample": "%d jobs (%d subbands x %d time slices) x %d streams x %.4g s (%.3g Gsamples), one process per "
                      "job; the restatement computes its FFTs in double precision where the reference calls FFTW "
                      "single precision, so this is a lower bound on the reference's own CPU throughput"
                      % (len(built), cfg["subbands"], slices, len(built[0]["streams"]), sample_us / 1e6,
                         total / 1e9)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = config_of(args)
    vals, base = [], None
    for _ in range(args.warmup):
        cpu_baseline(cfg, args.cpu_sample_us)
    for _ in range(args.steps):
        base = cpu_baseline(cfg, args.cpu_sample_us)
        vals.append(base["value"])
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": round(v, 5), "unit": "Gsamples/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic (seeded uniform 2-bit codes, cubic delay models)",
            "config": {"workload": cfg["name"], "sample_us": args.cpu_sample_us},
            "cpu_baseline": dict(base, value=round(v, 5)),
            "e2e": {"value": round(v, 5), "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--config", default="c3", choices=sorted(CONFIGS))
    ap.add_argument("--x", default="tc", choices=["fp32", "tc"])
    ap.add_argument("--signal", default="model", choices=["model", "uniform"],
                    help="inputs: the signal model generated on the GPU, or uniform random 2-bit codes")
    ap.add_argument("--no-fp32-compare", action="store_true",
                    help="skip the device-time run of the FP32 X-step beside the tensor-core one")
    ap.add_argument("--no-extra-configs", action="store_true",
                    help="skip the plain FP32 and pulsar configurations after the headline one")
    ap.add_argument("--stations", type=int, default=None)
    ap.add_argument("--subbands", type=int, default=None)
    ap.add_argument("--nchan", type=int, default=None)
    ap.add_argument("--integration-us", type=int, default=None)
    ap.add_argument("--cpu-sample-us", type=int, default=31250,
                    help="integration of each CPU job (a bounded sample of the workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frontend-only", action="store_true",
                    help="time only the station front end (recording to protocol on the device)")
    ap.add_argument("--driver", action="store_true",
                    help="time only the single-GPU driver on a synthetic experiment written to files")
    args = ap.parse_args()
    if args.impl == "reference":
        # the CPU arm builds only the restatement: the GPU library is neither
        # built nor loaded in this process
        from oracle import build_oracle
        build_oracle.build()
        run_reference(args)
    elif args.driver:
        import __graft_entry__
        __graft_entry__.build()
        print(json.dumps(measure_driver(args, lambda m: print(m, file=sys.stderr, flush=True))), flush=True)
    elif args.frontend_only:
        import __graft_entry__
        __graft_entry__.build()
        print(json.dumps(measure_frontend(args, lambda m: print(m, file=sys.stderr, flush=True))), flush=True)
    else:
        import __graft_entry__
        __graft_entry__.build()
        run_gpu(args)


if __name__ == "__main__":
    main()
