"""Generate the golden fixtures in tests/golden/ from the reference's own classes.

Run here, where the reference checkout exists:  python tests/golden/make_golden.py
The reference correlator-node classes are compiled by oracle/build_ref.py and
driven by oracle/ref_harness.cc; inputs are seeded synthetic scenarios
(sfxc_gpu.scenario).  Each fixture stores the inputs the reference consumed
(delay tables, channel streams) and what it produced: integer delay lists,
digests of the input-node protocol bytes and of the unpacked samples, a sample of the delay-
corrected spectra, the correlator output bytes, statistics and tsys records.
"""
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "sfxc-1_gb300"))
sys.path.insert(0, ROOT)

from oracle import jobs  # noqa: E402
from sfxc_gpu import scenario, synth  # noqa: E402


def ref_delays(*a):
    return jobs.delays(*a)[0]


def scenarios():
    out = {}
    out["c1_plain"] = scenario.c1_plain(integration_us=15625, n_integrations=2, seed=1)
    # three stations x two polarisations, large delay rates (integer-delay changes inside
    # the integrations), one lower-sideband station (sideband flip), invalid runs
    st = scenario.cubic_stations(3, seed=11, max_delay=2e-3, max_rate=3e-5)
    out["multi"] = scenario.Scenario(
        stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
        channel_freq=4_800_000_000, station_sidebands={2: "L"}, nchan=256, integration_us=4000,
        n_integrations=3, sub_integration_us=1000, lead_us=3000, rho=0.05, seed=5, block_bytes=2000,
        invalid={(1, "R"): [(6, 100, 300)], (0, "L"): [(9, 0, 2000), (10, 0, 500)]})
    # 1-bit streams
    st1 = scenario.cubic_stations(2, seed=3, max_delay=1e-3, max_rate=1e-5)
    out["onebit"] = scenario.Scenario(
        stations=st1, sample_rate=32_000_000, bandwidth=16_000_000, bits=1, channel_freq=1_400_000_000,
        nchan=512, integration_us=8000, n_integrations=2, rho=0.1, seed=9, block_bytes=4000)
    # pulsar binning
    stp = scenario.cubic_stations(2, seed=21, max_delay=1e-4, max_rate=1e-6)
    out["pulsar"] = scenario.Scenario(
        stations=stp, sample_rate=32_000_000, bandwidth=16_000_000, bits=2, channel_freq=1_400_000_000,
        nchan=256, integration_us=8000, n_integrations=1, rho=0.05, seed=13, block_bytes=8000)
    # spectral reduction: 1024-point correlation FFTs reduced to 256 channels,
    # with the Hann lag window, and with a rectangular window plus a user mask,
    # lag window and normalisation (Mask_parameters)
    st2 = scenario.cubic_stations(2, seed=31, max_delay=1e-3, max_rate=1e-5)
    out["reduced"] = scenario.Scenario(
        stations=st2, pols=("R", "L"), sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
        channel_freq=1_600_000_000, nchan=1024, number_channels=256, integration_us=8000, n_integrations=2,
        rho=0.05, seed=17, block_bytes=8000)
    out["reduced_mask"] = scenario.Scenario(
        stations=st2, sample_rate=32_000_000, bandwidth=16_000_000, bits=2, channel_freq=1_600_000_000,
        nchan=512, number_channels=64, window=0, integration_us=8000, n_integrations=1, rho=0.05, seed=19,
        block_bytes=8000)
    # two extra phase centres (same scan, residual delays of up to a few samples
    # between stations), sub-integrations of 2 ms: uvshift at every dump
    st3 = scenario.cubic_stations(3, seed=41, max_delay=1e-3, max_rate=1e-5)
    out["phase_centers"] = scenario.Scenario(
        stations=st3, sample_rate=32_000_000, bandwidth=16_000_000, bits=2, channel_freq=1_600_000_000,
        nchan=1024, integration_us=8000, sub_integration_us=2000, n_integrations=2, rho=0.05, seed=23,
        block_bytes=8000, extra_centers=[("SRC2", (2.1e-8, -4.0e-8, 7.5e-8)), ("SRC3", (-1.3e-7, 0.6e-7, 0.0))])
    # phased-array core: 3 stations, sub-integrations of 2 ms (5 sums per 8 ms integration)
    st4 = scenario.cubic_stations(3, seed=51, max_delay=1e-3, max_rate=1e-5)
    out["phased"] = scenario.Scenario(
        stations=st4, sample_rate=32_000_000, bandwidth=16_000_000, bits=2, channel_freq=1_600_000_000,
        nchan=512, integration_us=8000, sub_integration_us=2000, n_integrations=2, rho=0.05, seed=29,
        block_bytes=8000)
    return out


def mask_params(name, job):
    """User Mask_parameters of the reduced_mask case: a mask with a notch and
    a taper, a Gaussian lag window, normalisation on."""
    if name != "reduced_mask":
        return
    M, n = job["fft_size_correlation"], job["number_channels"]
    k = np.arange(M + 1)
    mask = np.where((k > M // 3) & (k < M // 3 + 9), 0.0, 1.0) * (1.0 - 0.3 * k / M)
    q = np.arange(2 * n)
    lag = np.minimum(q, 2 * n - q)
    job["mask"] = mask.astype(np.float32)
    job["lag_window"] = np.exp(-0.5 * (lag / (0.4 * n)) ** 2).astype(np.float32)
    job["mask_normalize"] = 1


def uvw_values(name, job):
    """UVW header values (what the correlator node's UVW model would give at
    each integration's mid-time) for some cases: seeded values of baseline-
    like size, different for each stream, so that the header shows which
    stream of a station and which phase centre was taken."""
    if name not in ("multi", "phase_centers", "pulsar", "phased"):
        return
    rng = np.random.Generator(np.random.PCG64(len(name) * 1000 + 7))
    npc = max(1, int(job.get("n_phase_centers", 1)))
    job["uvw"] = rng.normal(0.0, 3.0e6, size=(int(job["n_integrations"]), len(job["streams"]), npc, 3))


# two polycos (the closer one is used), non-zero phase polynomial
PULSAR = dict(nbins=8, gate=(0.2, 0.9),
              polyco=[(60000.0 + 36000.0 / 86400 - 0.01, 56.8, 0.25, 1 / 0.0334, 1400.0,
                       0.013, 0.0021, 1.3e-5, -2.2e-7, 4e-9) + (0.0,) * 7,
                      (60000.0 + 36000.0 / 86400 + 0.2, 56.8, 0.5, 1 / 0.0334, 1400.0) + (0.0,) * 12])


def make(name, sc):
    dels = scenario.del_tables(sc)
    chans, _ = scenario.channel_streams(sc)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    rec = {"del_bytes": np.array([np.frombuffer(d, np.uint8) for d in dels], dtype=object)}
    job = scenario.build_job(sc, ref_delays, jobs.protocol)
    if name == "pulsar":
        job["pulsar"] = (PULSAR["nbins"],) + PULSAR["gate"]
        job["polyco"] = PULSAR["polyco"]
    mask_params(name, job)
    uvw_values(name, job)
    if name == "phased":
        job["phased_array"] = 1
    res = jobs.correlate(job, dump=True)
    keys = sc.streams()
    for k, key in enumerate(keys):
        si = key[0]
        rec["chan_%d" % k] = chans[key]
        for it in range(sc.n_integrations):
            s0 = start + it * tint
            dl = ref_delays(dels[si], s0, s0 + tint, sc.sample_rate, sc.bits)
            rec["delays_%d_%d" % (k, it)] = np.array(dl, dtype=np.int64)
            pb = job["protocols"][k][it]
            rec["proto_sha_%d_%d" % (k, it)] = np.frombuffer(hashlib.sha256(pb).digest(), np.uint8)
            rec["proto_len_%d_%d" % (k, it)] = np.array(len(pb))
            un = res["unpacked"][(it, k)]
            rec["unpacked_sha_%d_%d" % (k, it)] = np.frombuffer(hashlib.sha256(un.tobytes()).digest(), np.uint8)
            rec["unpacked_head_%d_%d" % (k, it)] = un[:4096]
            rows = res["rows"][(it, k)].reshape(-1, job["fft_size_correlation"] + 4)
            pick = sorted(set([0, 1, rows.shape[0] // 2, rows.shape[0] - 1]))
            rec["rows_idx_%d_%d" % (k, it)] = np.array(pick)
            rec["rows_%d_%d" % (k, it)] = rows[pick, :job["fft_size_correlation"] + 1]
    if "pulsar" in job:
        rec["bins"] = res["bins"].astype(np.int8)
    rec["cor"] = np.frombuffer(res["cor"], np.uint8)
    rec["tsys"] = np.frombuffer(res["tsys"], np.uint8)
    rec["stats"] = np.frombuffer(res["stats"].encode(), np.uint8)
    for key in ("mask", "lag_window"):
        if key in job:
            rec[key] = np.asarray(job[key], dtype=np.float32)
    if "uvw" in job:
        rec["uvw"] = np.asarray(job["uvw"], dtype=np.float64)
    meta = {k: v for k, v in job.items() if k not in ("del_bytes", "protocols", "mask", "lag_window", "uvw")}
    meta["block_bytes"] = sc.block_bytes
    meta["rec0"] = rec0
    meta["slice_samples"] = slice_samples
    meta["nblocks"] = [len(chans[key]) // sc.block_bytes for key in keys]
    meta["invalid"] = {"%d,%s" % k: v for k, v in sc.invalid.items()}
    rec["meta"] = np.array(repr(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print(name, "cor bytes", len(res["cor"]))


def make_extract():
    # 16 channels x 2 bits in 32-bit words (VDIF multi-channel layout), reference tracks
    rng = np.random.Generator(np.random.PCG64(77))
    words = rng.integers(0, 2**32, size=8000, dtype=np.uint64).astype(np.uint32)
    tracks = [[2 * c + 1, 2 * c] for c in range(16)]
    out16 = jobs.extract(words.tobytes(), 4, 2, words.size, tracks)
    # 8 channels x 2 bits with fan-out 4 (two samples per channel per 32-bit word)
    tracks8 = [[2 * c + 1, 2 * c, 2 * c + 17, 2 * c + 16] for c in range(8)]
    out8 = jobs.extract(words.tobytes(), 4, 2, words.size, tracks8)
    # 1-bit, 32 tracks in pairs of fan-out 2 (Mark5B-like bitstreams)
    tracks1 = [[c, c + 16] for c in range(16)]
    out1 = jobs.extract(words.tobytes(), 4, 1, words.size, tracks1)
    np.savez_compressed(os.path.join(HERE, "extract.npz"), words=words,
                        tracks16=np.array(tracks16 := tracks), out16=np.frombuffer(b"".join(out16), np.uint8),
                        tracks8=np.array(tracks8), out8=np.frombuffer(b"".join(out8), np.uint8),
                        tracks1=np.array(tracks1), out1=np.frombuffer(b"".join(out1), np.uint8))
    print("extract done")


def make_formats():
    """Blocks of the reference's VDIF / Mark5B readers for the recordings of
    tests/format_cases.py (regenerated from their seeds by the tests): per
    block the channel, start ticks, payload SHA-256 and invalid runs."""
    import hashlib
    import json
    sys.path.insert(0, os.path.dirname(HERE))
    import format_cases
    out = {}
    for name, c in format_cases.cases().items():
        blocks = jobs.reader(c["rec"], c["fmt"], **c["params"])
        out[name] = {"recording_sha256": hashlib.sha256(c["rec"]).hexdigest(),
                     "blocks": [{"channel": b["channel"], "start_ticks": b["start_ticks"], "size": len(b["data"]),
                                 "sha256": hashlib.sha256(b["data"]).hexdigest(),
                                 "invalid": [list(r) for r in b["invalid"]]} for b in blocks]}
    with open(os.path.join(HERE, "formats.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("formats done")


def make_schedule():
    """Blocks the reference's reader tasklet (Input_data_format_reader_tasklet)
    pushes for the recordings of tests/format_cases.py (cases() and
    schedule_recordings()) and the interval sets of schedule_cases(): per
    block the channel, start ticks, size, invalid runs and the SHA-256 of its
    bytes -- null for a wholly invalid block, whose bytes are not defined, and
    "shared" for a block pushed in the same data buffer as another block that
    is not wholly invalid: the tasklet reads the next interval's first block
    into the buffer of the last block it pushed, so that block's bytes depend
    on whether its consumer took it first; "stale" for a block whose buffer
    holds no block's bytes (the last read into it failed at the end of the
    data, or none was made)."""
    import json
    sys.path.insert(0, os.path.dirname(HERE))
    import format_cases
    recs = dict(format_cases.cases(), **format_cases.schedule_recordings())
    out = {}
    for name, c in sorted(recs.items()):
        first = jobs.reader(c["rec"], c["fmt"], max_blocks=1, **c["params"])
        if not first:
            continue
        for iname, ivs in format_cases.schedule_cases(first[0]["start_ticks"], format_cases.reader_tbh(c)).items():
            blocks = jobs.schedule(c["rec"], c["fmt"], intervals=ivs, **c["params"])
            # each buffer's last push: its last block and the blocks of the
            # other channels of that VDIF thread pushed right before it
            last_push = set()
            seen = set()
            for i in range(len(blocks) - 1, -1, -1):
                b = blocks[i]
                if b["data"] is None or b["buffer"] in seen:
                    continue
                seen.add(b["buffer"])
                k = i
                while k >= 0 and blocks[k]["buffer"] == b["buffer"] and blocks[k]["start_ticks"] == b["start_ticks"] \
                        and (k == i or blocks[k]["channel"] != blocks[k + 1]["channel"]):
                    last_push.add(k)
                    k -= 1

            def digest(i, b):
                if b["data"] is None:
                    return None
                if i not in last_push:
                    return "shared"  # pushed before its buffer was read into again
                return "stale" if b["stale"] else hashlib.sha256(b["data"]).hexdigest()
            out[name + "/" + iname] = {
                "recording_sha256": hashlib.sha256(c["rec"]).hexdigest(), "intervals": [list(v) for v in ivs],
                "blocks": [{"channel": b["channel"], "start_ticks": b["start_ticks"], "size": b["size"],
                            "sha256": digest(i, b), "invalid": [list(r) for r in b["invalid"]]}
                           for i, b in enumerate(blocks)]}
            print(name, iname, len(blocks), "blocks")
    with open(os.path.join(HERE, "schedule.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


def uvw_cases():
    """.del tables with u, v, w columns (a two-centre scan, then a later
    scan) and probes (phase centre, ticks) in order: fractional and whole
    seconds, the first and last seconds of a scan (clamped windows), a later
    scan, and a step back in time (the model keeps its spline)."""
    from sfxc_gpu import timebase
    mjd, sec0 = 60200, 43000
    poly = synth.DelayPoly(coeffs=(1e-3, 2e-7, 0.0, 0.0), t0=sec0, phase_coeffs=(0.0,), amp=1.0)
    tables = {}
    for name, (b, dec, h0) in {"near": ((1200.0, -800.0, 300.0), 0.6, 0.3),
                               "far": ((-5.1e6, 2.2e6, 3.3e6), -0.2, 1.1)}.items():
        scans = [("SRC1", mjd, sec0, 20, poly, synth.earth_rotation_uvw(b, dec, h0)),
                 ("SRC2", mjd, sec0, 20, poly, synth.earth_rotation_uvw(b, dec + 0.01, h0 - 0.02)),
                 ("SRC3", mjd, sec0 + 40, 15, poly, synth.earth_rotation_uvw(b, dec - 0.3, h0 + 0.5))]
        tables[name] = synth.del_file_bytes("Xx", scans)
    t = lambda s: timebase.ticks_from_mjd_sec(mjd, s)  # noqa: E731
    probes = [(0, t(sec0 + 0.25)), (1, t(sec0 + 0.25)), (0, t(sec0 + 1.0)), (0, t(sec0 + 1.5)),
              (1, t(sec0 + 7.125)), (0, t(sec0 + 7.875)), (0, t(sec0 + 7.5)), (0, t(sec0 + 12.0)),
              (1, t(sec0 + 18.5)), (0, t(sec0 + 19.0)), (0, t(sec0 + 41.75)), (0, t(sec0 + 47.0625)),
              (0, t(sec0 + 54.0))]
    return tables, probes


def make_uvw():
    """u, v, w of the reference's Uvw_model for uvw_cases()."""
    import json
    tables, probes = uvw_cases()
    out = {name: {"del_sha256": hashlib.sha256(db).hexdigest(), "probes": probes,
                  "uvw": [list(v) for v in jobs.uvw(db, probes)]} for name, db in tables.items()}
    with open(os.path.join(HERE, "uvw.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("uvw done")


def make_phasecal():
    """Phase-cal messages of the reference's Input_node_data_writer for
    phasecal_cases(): per case the SHA-256 of each message, in order."""
    import json
    sys.path.insert(0, os.path.dirname(HERE))
    from golden_io import Golden, phasecal_blocks, phasecal_cases
    out = {}
    for name, (fx, k, ticks, first, inject) in phasecal_cases().items():
        g = Golden(fx)
        m, s = g.meta, g.meta["streams"][k]
        _, raw = jobs.protocol(phasecal_blocks(g, k, first, inject), g.slices(k), s[2], s[7],
                               m["integration_time_us"], phasecal_ticks=ticks)
        P = int(s[2] / 10e3)
        n = 24 + 4 * P
        assert len(raw) % n == 0
        msgs = [raw[i:i + n] for i in range(0, len(raw), n)]
        out[name] = {"messages": [hashlib.sha256(x).hexdigest() for x in msgs], "message_bytes": n}
        print(name, len(msgs), "messages")
    with open(os.path.join(HERE, "phasecal.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


OUTPUT_HEADER_CASES = [
    dict(experiment="N24L1", start_year=2024, start_day=123, start_time=43200, number_channels=4096,
         integration_time_us=2000000, correlator_version=2048, polarisation_type=3, correlator_branch="trunk",
         job_nr=17, subjob_nr=2),
    dict(experiment="EXPERIMENT_NAME_OF_31_CHARACTERS", start_year=2026, start_day=366, start_time=86399,
         number_channels=64, integration_time_us=125000, correlator_version=0, polarisation_type=0,
         correlator_branch="a-branch-longer-than-15", job_nr=0, subjob_nr=0),
]


def make_output_header():
    """Output_header_global bytes from the reference's own struct
    (oracle/ref_output_header.cc) for OUTPUT_HEADER_CASES."""
    import json
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref
    exe = build_ref.build_output_header()
    out = []
    for c in OUTPUT_HEADER_CASES:
        args = [c["experiment"][:31], c["start_year"], c["start_day"], c["start_time"], c["number_channels"],
                c["integration_time_us"], c["correlator_version"], c["polarisation_type"], c["correlator_branch"],
                c["job_nr"], c["subjob_nr"]]
        r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, check=True)
        out.append(dict(c, experiment=c["experiment"][:31], header_hex=r.stdout.strip()))
    with open(os.path.join(HERE, "output_header.json"), "w") as f:
        json.dump(out, f, indent=1)


def make_control():
    """The reference's plans for control_cases() (control.json.gz): per case the plan
    (Control_parameters and the manager's dealing, oracle/ref_harness.cc
    mode `control`) with the case directory written as <dir>, or null for a
    set-up the reference refuses."""
    import json
    import tempfile
    sys.path.insert(0, os.path.dirname(HERE))
    import control_cases
    out = {}
    for name, case in control_cases.cases().items():
        with tempfile.TemporaryDirectory() as d:
            ctrl, vex = control_cases.write_case(case, d)
            plan = jobs.control(ctrl, vex, d, control_cases.station_times(case))
            out[name] = json.loads(json.dumps(plan).replace(d, "<dir>")) if plan else None
        print(name, "refused" if plan is None else "%d jobs" % len(plan["jobs"]))
    import gzip
    with gzip.open(os.path.join(HERE, "control.json.gz"), "wt") as f:
        json.dump(out, f, indent=None, sort_keys=True, separators=(",", ":"))


def make_driver(variant="plain"):
    """The reference's own stages over driver_cases' experiment (driver.npz,
    driver_<variant>.npz for the other variants):
    its plan (Control_parameters and the manager's dealing), for each station
    the reader tasklet's blocks over the scan intervals, Channel_extractor_5
    on them (a block whose buffer the tasklet reused for its next read keeps
    its own bytes, the reader's block of that time; invalid runs rescaled as
    Channel_extractor_tasklet::do_task does,
    sfxc/src/channel_extractor_tasklet.cc:173-194; VDIF with one
    channel per thread takes the blocks as they are), Input_node_tasklet's
    delays per scan interval and Input_node_data_writer's protocol per slice,
    then each job's Correlation_core(_pulsar) output (with its file index)
    and u, v, w: the pulsar core for the pulsar's scan and file index 1 for
    other sources of a pulsar run, the manager's source list for extra phase
    centres (the core gives each centre its source's file index).  The glue
    between the stages restates Input_node and Correlator_node."""
    import json
    import tempfile
    sys.path.insert(0, os.path.dirname(HERE))
    import driver_cases
    from sfxc_gpu import timebase
    with tempfile.TemporaryDirectory() as d:
        ctrl_path, vex_path = driver_cases.write_experiment(d, variant)
        ctrl = json.load(open(ctrl_path))
        plan0 = jobs.control(ctrl_path, vex_path, d)
        per = {}
        for sci, sc in enumerate(plan0["scans"]):
            for e in sc["stations"]:
                per.setdefault(e["station"], []).append((sci, e))
        recs, params = {}, {}
        start = plan0["jobs"][0]["experiment_start"]
        for s, scans in per.items():
            e = scans[0][1]
            ip = e["input"]
            rec = b"".join(open(os.path.join(d, u[7:]), "rb").read() for u in ctrl["data_sources"][e["name"]])
            chans = [c for c in ip["channels"] if not (ip["n_tracks"] == 0 and c["tracks"][0] < 0)]
            recs[s] = rec
            params[s] = dict(ref_ticks=start, offset_ticks=e["reader_offset"], track_bit_rate=ip["track_bit_rate"],
                             frame_size=ip["frame_size"] if ip["data_format"] == "VDIF" else 0,
                             n_tracks=ip["n_tracks"], bits=chans[0]["bits_per_sample"],
                             channel_tracks=[c["tracks"] for c in chans])
        fmt = {s: "vdif" if per[s][0][1]["input"]["data_format"] == "VDIF" else "mark5b" for s in per}
        # the input node's current time at its first scan: its reader's first block
        first = {s: jobs.reader(recs[s], fmt[s], max_blocks=1, **params[s])[0]["start_ticks"] for s in per}
        times = [(s, per[s][0][0], first[s]) for s in per]
        plan = jobs.control(ctrl_path, vex_path, d, times)
        per = {}
        for sci, sc in enumerate(plan["scans"]):
            for e in sc["stations"]:
                per.setdefault(e["station"], []).append((sci, e))
        dels = {s: open(os.path.join(d, per[s][0][1]["delay_file"]), "rb").read() for s in per}
        integr_us = int(round(ctrl["integr_time"] * 1e6))
        slice_bytes = {}  # (station, channel in scan) -> [protocol bytes per slice]
        pcal = {}  # (station, channel in scan) -> phase-cal message bytes
        n_st = len(ctrl["stations"])
        station_nr = {sp["station_stream"] % n_st: sp["station_number"] for j in plan["jobs"] for sp in j["stations"]}
        for s, scans in per.items():
            p = params[s]
            ip = scans[0][1]["input"]
            iv = [(plan["scans"][sci]["first_slice_start"], plan["scans"][sci]["stop"], e["stop_time"])
                  for sci, e in scans]
            blocks = jobs.schedule(recs[s], fmt[s], intervals=iv, **p)
            # A block whose data buffer the tasklet reused for a later read
            # (the next interval's first block) shows that read's bytes in the
            # dump; it carries its own, the reader's block of the same time
            thread_mode = ip["n_tracks"] == 0
            own = {(b["channel"] if thread_mode else 0, b["start_ticks"]): b["data"]
                   for b in jobs.reader(recs[s], fmt[s], **p)}
            last_of_buffer = {b["buffer"]: k for k, b in enumerate(blocks)}
            for k, b in enumerate(blocks):
                if b["data"] is not None and last_of_buffer[b["buffer"]] != k:
                    b["data"] = own[(b["channel"] if thread_mode else 0, b["start_ticks"])]
            nch = len(p["channel_tracks"])
            chan_params = [c for c in ip["channels"] if not (ip["n_tracks"] == 0 and c["tracks"][0] < 0)]
            chan_blocks = [[] for _ in range(nch)]
            if ip["n_tracks"] == 0:  # one channel per VDIF thread: the blocks as they are
                for b in blocks:
                    data = b["data"] if b["data"] is not None else bytes(b["size"])
                    chan_blocks[b["channel"]].append((b["start_ticks"], data, b["invalid"]))
            else:
                word = 4 if ip["n_tracks"] <= 32 else 8
                fan_out = len(p["channel_tracks"][0])
                words = b"".join(b["data"] if b["data"] is not None else bytes(b["size"]) for b in blocks)
                outs = jobs.extract(words, word, p["bits"], len(words) // word, p["channel_tracks"])
                pos = 0
                for b in blocks:
                    n = b["size"] * fan_out // (8 * word)
                    inv = [(bb * fan_out // (8 * word), nn * fan_out // (8 * word)) for bb, nn in b["invalid"]]
                    for c in range(nch):
                        chan_blocks[c].append((b["start_ticks"], outs[c][pos:pos + n], inv))
                    pos += n
            sr = ip["track_bit_rate"] * len(p["channel_tracks"][0]) // p["bits"]
            delays = {}
            for sci, e in scans:
                sc = plan["scans"][sci]
                delays[sci] = jobs.delays(dels[s], sc["first_slice_start"], sc["stop"], sr, p["bits"],
                                          clock=(e["clock_offset"], e["clock_rate"], e["clock_epoch"]))[0]
            fft = ip["fft_size"]
            size = timebase.nr_ffts_per_integration_slice(integr_us, sr, fft) * fft
            for c in range(nch):
                sl = [(j["start_time"], j["stop_time"], size, delays[j["scan"]]) for j in plan["jobs"]
                      if any(i["station"] == s and i["channel_in_scan"] == c for i in j["inputs"])]
                if sl:
                    slice_bytes[(s, c)], msgs = jobs.protocol(chan_blocks[c], sl, sr, p["bits"], integr_us,
                                                              station_number=station_nr[s],
                                                              phasecal_ticks=ip["phasecal_integr_time"],
                                                              channel=chan_params[c])
                    pcal[(s, c)] = msgs
            print("station", s, len(blocks), "blocks")
        outs, tsys, used = [], [], {}
        for j in plan["jobs"]:
            n_st = len(ctrl["stations"])
            tables, clocks, table_of, streams, protos, uvws = [], [], {}, [], [], []
            sc_st = {e["station"]: e for e in plan["scans"][j["scan"]]["stations"]}
            by_stream = {i["stream"]: i for i in j["inputs"]}
            tmid = j["start_time"] + j["integration_time"] // 2
            for sp in j["stations"]:
                s = sp["station_stream"] % n_st
                if s not in table_of:
                    table_of[s] = len(tables)
                    tables.append(dels[s])
                    e = sc_st[s]
                    clocks.append((e["clock_offset"], e["clock_rate"], e["clock_epoch"]))
                streams.append((sp["station_number"], sp["station_stream"], sp["sample_rate"], sp["channel_freq"],
                                sp["bandwidth"], sp["sideband"], sp["polarisation"], sp["bits_per_sample"],
                                sp["lo_offset"], sp["tsys_freq"], table_of[s]))
                i = by_stream[sp["station_stream"]]
                key = (i["station"], i["channel_in_scan"])
                k = used.get(key, 0)
                used[key] = k + 1
                protos.append([slice_bytes[key][k]])
                npc = max(1, j["n_phase_centers"])
                uvws.append(jobs.uvw(dels[s], [(pc, tmid) for pc in range(npc)]))
            job = dict(experiment_start_ticks=j["experiment_start"], start_ticks=j["start_time"],
                       integration_time_us=integr_us, sub_integration_time_us=int(round(j["sub_integration_time"] / 512)),
                       number_channels=j["number_channels"], fft_size_delaycor=j["fft_size_delaycor"],
                       fft_size_correlation=j["fft_size_correlation"], sample_rate=j["sample_rate"],
                       channel_freq=j["channel_freq"], bandwidth=j["bandwidth"], sideband=j["sideband"],
                       frequency_nr=j["frequency_nr"], polarisation=j["polarisation"],
                       cross_polarize=int(j["cross_polarize"]), reference_station=j["reference_station"],
                       window=j["window"], source=j["source"], integration_nr=j["integration_nr"], n_integrations=1,
                       streams=streams, del_bytes=tables, clocks=clocks, protocols=protos, uvw=[uvws])
            if ctrl.get("pulsar_binning"):
                ps = {x["name"]: x for x in plan["pulsars"]}
                if j["source"] in ps:
                    x = ps[j["source"]]
                    job["pulsar"] = (x["nbins"], x["gate_start"], x["gate_stop"])
                    job["polyco"] = [[c["tmid"], c["dm"], c["ref_phase"], c["ref_freq"], c["obs_freq"]] + c["coef"]
                                     for c in x["polyco"]]
                else:
                    job["pulsar_mode"] = 1
            if ctrl.get("phased_array"):
                job["phased_array"] = 1
            if plan["sources"]:
                job["source_list"] = plan["sources"]
                job["n_phase_centers"] = j["n_phase_centers"]
            res = jobs.correlate(job)
            outs.append(np.frombuffer(res["cor"], dtype=np.uint8))
            tsys.append(np.frombuffer(res["tsys"], dtype=np.uint8))
            print("job", j["slice_nr"], "integration", j["integration_nr"], len(outs[-1]), "bytes")
        header = plan["header"]
        plan["output_files"] = [f.replace(d, "<dir>") for f in plan["output_files"]]
    pc = {"pcal_%d_%d" % k: np.frombuffer(v, dtype=np.uint8) for k, v in pcal.items()}
    name = "driver.npz" if variant == "plain" else "driver_%s.npz" % variant
    np.savez_compressed(os.path.join(HERE, name), header=json.dumps(header), files=json.dumps(plan["output_files"]),
                        slices=np.array(len(outs)), **{"slice%d" % k: o for k, o in enumerate(outs)},
                        **{"tsys%d" % k: t for k, t in enumerate(tsys)}, **pc)


if __name__ == "__main__":
    make_control()
    for v in ("plain", "pulsar", "phase_centres", "phased", "scans"):
        make_driver(v)
    make_output_header()
    make_phasecal()
    make_formats()
    make_schedule()
    make_uvw()
    make_extract()
    for name, sc in scenarios().items():
        make(name, sc)
