"""Single-GPU correlation of a control file and a VEX file: what the
reference's `sfxc <ctrl> <vex>` does with its manager, input, correlator and
output nodes (sfxc/src/manager_node.cc, input_node*.cc, correlator_node.cc,
output_node.cc), in one process on one GPU.

  python -m sfxc_gpu.run <ctrl> <vex> [--tc] [--device N]

The library plans the correlation (sfxc_gpu_control_*: Control_parameters and
the manager's dealing of the jobs).  Each station's recording (its
data_sources, VDIF or Mark5B) is read into device memory once; the reader
tasklet's blocks for every scan the station takes part in (sfxc_gpu_recording_
schedule), its channels, and each channel's input-node protocol for every
time slice it feeds are made on the device (stations side by side, each on
its own library context and host thread); the jobs of a time slice run side
by side on correlator contexts of their own, their streams pushed device to
device; the output node writes them in slice order to the output file(s)
with the global header, and the tsys and phase-cal records to their files
when the control file names them.  Delay tables are the stations' .del files (the
manager's delay_directory); the delay model generator is not run.

Set-ups the reference correlates that this driver refuses: Mark4 and VLBA
recordings (no Mark5A reader) and a station whose reader parameters change
between scans.
"""
import argparse
import os
import struct
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import control, correlator, lib as L, timebase


class DriverError(RuntimeError):
    pass


def _path(url, ctrl_dir):
    """A data-source or output URL as a file path (Control_parameters::create_path:
    file:// paths that are not absolute are relative to the control file)."""
    if not url.startswith("file://"):
        raise DriverError("only file:// paths are read: " + url)
    p = url[7:]
    return p if os.path.isabs(p) else os.path.join(ctrl_dir, p)


def _del_scans(del_bytes):
    """(source, first row's second) of each scan of a .del file (layout of
    sfxc/utils/delay/generate_delay_model_calc.c:440-467): int32 header
    size, the header, then per scan an 81-byte source name, int32 MJD and
    rows of seven doubles ending with a row of zeros."""
    (hs,) = struct.unpack_from("<i", del_bytes, 0)
    p = 4 + hs
    out = []
    while p + 85 <= len(del_bytes):
        src = del_bytes[p:p + 81].split(b"\0")[0].decode(errors="replace").strip()
        p += 85
        first = None
        while p + 56 <= len(del_bytes):
            row = struct.unpack_from("<7d", del_bytes, p)
            p += 56
            if all(v == 0.0 for v in row):
                break
            if first is None:
                first = row[0]
        out.append((src, first))
    return out


_TICKS_PER_DAY = 86400 * 512_000_000


def _mjd_secs(ticks):
    """The uint32 MJD and seconds of day the output node writes for a time
    (Time::get_mjd and get_time truncated, sfxc/src/correlator_time.cc:50-66)."""
    return 51544 + ticks // _TICKS_PER_DAY, (ticks % _TICKS_PER_DAY) // 512_000_000


def tsys_record(msg):
    """The tsys file record of a correlator's tsys message (four uint8
    station, frequency number, sideband, polarisation; int64 start ticks; four
    int64 counts): the ids, uint32 MJD, uint32 seconds, the counts as uint64
    (Output_node_controller, sfxc/src/output_node_controller.cc:171-205)."""
    (t,) = struct.unpack_from("<q", msg, 4)
    return bytes(msg[:4]) + struct.pack("<II", *_mjd_secs(t)) + bytes(msg[12:44])


def phasecal_record(msg):
    """The phase-cal file record of an input node's phase-cal message (four
    uint8 ids; int64 start and length ticks; int32 bin count P; P int32 bins):
    the ids, uint32 MJD, uint32 seconds, uint32 length in seconds, uint32 P,
    the bins (sfxc/src/output_node_controller.cc:110-155)."""
    t, length = struct.unpack_from("<qq", msg, 4)
    (p,) = struct.unpack_from("<i", msg, 20)
    mjd, secs = _mjd_secs(t)
    return bytes(msg[:4]) + struct.pack("<IIII", mjd, secs, (length % _TICKS_PER_DAY) // 512_000_000, p) + \
        bytes(msg[24:24 + 4 * p])


class _Station:
    """One station's recording on the device and its per-scan set-up."""

    def __init__(self, node, index, name, scans, data_bytes, experiment_start):
        first = scans[0][1]
        ip = first["input"]
        fmt = {"VDIF": "vdif", "Mark5B": "mark5b"}.get(ip["data_format"])
        if fmt is None:
            raise DriverError("station %s: %s recordings are not read (no Mark5A reader)" % (name, ip["data_format"]))
        for _, st in scans[1:]:
            if st["input"] != ip or st["reader_offset"] != first["reader_offset"]:
                raise DriverError("station %s: reader parameters change between scans" % name)
        self.index, self.name, self.fmt, self.input = index, name, fmt, ip
        present = [c for c in ip["channels"] if not (ip["n_tracks"] == 0 and c["tracks"][0] < 0)]
        self.channels = present
        self.bits = present[0]["bits_per_sample"]
        self.thread_mode = ip["n_tracks"] == 0
        subsamples = len(present[0]["tracks"]) // self.bits
        self.sample_rate = ip["track_bit_rate"] * subsamples  # Input_node_parameters::sample_rate
        self.rec = correlator.DeviceRecording(
            node, np.frombuffer(data_bytes, dtype=np.uint8), fmt, ref_ticks=experiment_start,
            offset_ticks=first["reader_offset"], track_bit_rate=ip["track_bit_rate"],
            frame_size=max(0, ip["frame_size"]) if fmt == "vdif" else 0, n_tracks=ip["n_tracks"], bits=self.bits,
            channel_tracks=[c["tracks"] for c in present])
        self.slices = {}  # channel -> [(job index, slice)]

    def first_time(self):
        return self.rec.block_start(0) if self.rec.n_blocks() > 0 else None

    def read(self, intervals):
        self.rec.schedule(intervals)
        if self.thread_mode:
            self.rec.extract_threads(len(self.channels))
        else:
            word = 4 if self.input["n_tracks"] <= 32 else 8
            self.rec.extract(word, self.bits, [c["tracks"] for c in self.channels])


def correlate(ctrl_path, vex_path, device=0, x_mode=L.X_FP32, log=None, stats=None):
    """Runs the whole correlation; returns {path: bytes written} of the
    output file(s) and, when the control file names them, the tsys and
    phase-cal files.  stats (a dict), if given, receives the wall-clock
    seconds of each phase and the samples correlated."""
    import time
    log = log or (lambda *a: None)
    clock = [time.perf_counter()]

    def lap(name):
        if stats is not None:
            t = time.perf_counter()
            stats[name + "_s"] = round(t - clock[0], 4)
            clock[0] = t
    ctrl_path, vex_path = os.path.abspath(ctrl_path), os.path.abspath(vex_path)
    ctrl_dir = os.path.dirname(ctrl_path)
    plan = control.plan(ctrl_path, vex_path)
    ctrl = plan["ctrl"]
    if not plan["jobs"]:
        raise DriverError("nothing to correlate between the start and stop times")
    names = ctrl["stations"]
    n_st = len(names)
    experiment_start = plan["jobs"][0]["experiment_start"]
    per_station = {}
    for sci, sc in enumerate(plan["scans"]):
        for st in sc["stations"]:
            per_station.setdefault(st["station"], []).append((sci, st))
    for s, scans in per_station.items():
        fmt = scans[0][1]["input"]["data_format"]
        if fmt not in ("VDIF", "Mark5B"):
            raise DriverError("station %s: %s recordings are not read (no Mark5A reader)" % (names[s], fmt))

    # one library context per station (its input node) and per concurrent
    # job (a correlator node): the contexts are driven from their own threads
    station_nodes = {s: correlator.CorrelatorNode(device, x_mode) for s in sorted(per_station)}
    nodes = []
    try:
        return _run(plan, ctrl, ctrl_path, vex_path, ctrl_dir, names, n_st, experiment_start, per_station,
                    station_nodes, nodes, device, x_mode, log, stats, lap)
    finally:
        for n in nodes + list(station_nodes.values()):  # each closes its recordings first
            n.close()


def _run(plan, ctrl, ctrl_path, vex_path, ctrl_dir, names, n_st, experiment_start, per_station, station_nodes,
         nodes, device, x_mode, log, stats, lap):
    workers = max(1, min(16, os.cpu_count() or 4))
    lap("plan")

    def open_station(s):  # read the recording files, put them on the device
        parts = [np.fromfile(_path(u, ctrl_dir), dtype=np.uint8) for u in ctrl["data_sources"][names[s]]]
        data = parts[0] if len(parts) == 1 else np.concatenate(parts)
        return s, _Station(station_nodes[s], s, names[s], per_station[s], data, experiment_start), data.size

    stations = {}
    with ThreadPoolExecutor(workers) as ex:
        for s, st, n in ex.map(open_station, sorted(per_station)):
            stations[s] = st
            log("station %s: %d bytes of %s" % (names[s], n, st.fmt))
            if stats is not None:
                stats["recording_bytes"] = stats.get("recording_bytes", 0) + n
    lap("read")

    # the manager moves a scan's first slice to the latest input node time
    # (its reader's first frame, at the first scan a station is in)
    first_scan = {s: scans[0][0] for s, scans in per_station.items()}
    first_time = {s: st.first_time() for s, st in stations.items()}
    plan = control.plan(ctrl_path, vex_path, lambda s, sc: (first_time.get(s) or 0) if first_scan.get(s) == sc else 0)
    per_station = {}
    for sci, sc in enumerate(plan["scans"]):
        for st in sc["stations"]:
            per_station.setdefault(st["station"], []).append((sci, st))
    jobs = plan["jobs"]

    # delay tables (the manager's delay_directory) and UVW models
    del_bytes = {}
    for s in per_station:
        path = per_station[s][0][1]["delay_file"]
        path = path if os.path.isabs(path) else os.path.join(os.getcwd(), path)
        if not os.path.exists(path):
            raise DriverError("no delay table %s for station %s (the delay model generator is not run)"
                              % (path, names[s]))
        del_bytes[s] = open(path, "rb").read()
    uvw = {s: correlator.UvwModel(b) for s, b in del_bytes.items()}

    # the input nodes: reader blocks for each scan interval, channels, delays,
    # protocols, and the phase-cal of every channel the writers take up
    # (Input_node_data_writer::do_phasecal); each station on its own context
    integration_us = int(round(ctrl["integr_time"] * 1e6))
    station_number = {sp["station_stream"] % n_st: sp["station_number"] for j in jobs for sp in j["stations"]}
    for ji, j in enumerate(jobs):
        for inp in j["inputs"]:
            stations[inp["station"]].slices.setdefault(inp["channel_in_scan"], []).append((ji, j))

    def input_node(s):
        st, scans = stations[s], per_station[s]
        st.read([(plan["scans"][sci]["first_slice_start"], plan["scans"][sci]["stop"], e["stop_time"])
                 for sci, e in scans])
        delays = {}
        for sci, e in scans:
            sc = plan["scans"][sci]
            delays[sci] = correlator.delay_list(
                del_bytes[s], sc["first_slice_start"], sc["stop"], st.sample_rate, st.bits,
                clock=(e["clock_offset"], e["clock_rate"], e["clock_epoch"]))
        fft = st.input["fft_size"]
        size_slice = timebase.nr_ffts_per_integration_slice(integration_us, st.sample_rate, fft) * fft
        for c, sl in st.slices.items():
            if not 0 <= c < len(st.channels):
                raise DriverError("station %s: channel %d of the scan is not in its recording set-up" % (st.name, c))
            st.rec.protocol(c, [(j["start_time"], j["stop_time"], size_slice, delays[j["scan"]]) for _, j in sl],
                            st.sample_rate, st.bits, integration_us, copy=False)
        msgs = []
        ticks = st.input["phasecal_integr_time"]
        if ctrl.get("phasecal_file") and ticks > 0:
            for c in sorted(st.slices):
                ch = st.channels[c]
                pc = correlator.PhaseCal(station_nodes[s], st.sample_rate, st.bits, ticks, station_number.get(s, 0),
                                         ch["frequency_number"], 1 if ch["sideband"] == "U" else 0,
                                         1 if ch["polarisation"] == "L" else 0)
                msgs += pc.push(st.rec.channel(c))
                pc.close()
        return msgs

    with ThreadPoolExecutor(workers) as ex:
        pcal = [m for msgs in ex.map(input_node, sorted(per_station)) for m in msgs]
    log("input nodes: %d channel streams" % sum(len(st.slices) for st in stations.values()))
    lap("input_nodes")

    # the correlator nodes: the jobs of one time slice side by side, each on
    # its own context; the output node takes their slices in order
    pulsars = {p["name"]: p for p in plan.get("pulsars", [])}
    mask = plan.get("mask")
    sources = plan["sources"]
    phased = int(bool(ctrl.get("phased_array")))
    h = plan["header"]
    out = correlator.OutputFiles(len(plan["output_files"]), experiment=h["experiment"], start_year=h["start_year"],
                                 start_day=h["start_day"], start_time=h["start_time"],
                                 number_channels=h["number_channels"], integration_time_us=h["integration_time"],
                                 correlator_version=0, polarisation_type=h["polarisation_type"],
                                 correlator_branch="gb300", job_nr=h["job_nr"], subjob_nr=h["subjob_nr"])
    slice_of = {}  # job index -> the protocol slice of each of its streams
    used = {}
    for ji, j in enumerate(jobs):
        by_stream = {inp["stream"]: inp for inp in j["inputs"]}
        pushes = []
        for sp in j["stations"]:
            inp = by_stream[sp["station_stream"]]
            key = (inp["station"], inp["channel_in_scan"])
            pushes.append((inp["station"], inp["channel_in_scan"], used.get(key, 0)))
            used[key] = used.get(key, 0) + 1
        slice_of[ji] = pushes

    def job_of(j):
        sc = plan["scans"][j["scan"]]
        sc_station = {e["station"]: e for e in sc["stations"]}
        streams, tables, clocks, table_of = [], [], [], {}
        for sp in j["stations"]:
            s = sp["station_stream"] % n_st
            if s not in table_of:
                table_of[s] = len(tables)
                tables.append(del_bytes[s])
                e = sc_station[s]
                clocks.append((e["clock_offset"], e["clock_rate"], e["clock_epoch"]))
            streams.append((sp["station_number"], sp["station_stream"], sp["sample_rate"], sp["channel_freq"],
                            sp["bandwidth"], sp["sideband"], sp["polarisation"], sp["bits_per_sample"],
                            sp["lo_offset"], sp["tsys_freq"], table_of[s]))
        tint = j["integration_time"]
        job = dict(experiment_start_ticks=j["experiment_start"], start_ticks=j["start_time"],
                   integration_time_us=int(round(tint / 512.0)), sub_integration_time_us=int(round(
                       j["sub_integration_time"] / 512.0)), number_channels=j["number_channels"],
                   fft_size_delaycor=j["fft_size_delaycor"], fft_size_correlation=j["fft_size_correlation"],
                   sample_rate=j["sample_rate"], bandwidth=j["bandwidth"], frequency_nr=j["frequency_nr"],
                   channel_freq=j["channel_freq"], sideband=j["sideband"], polarisation=j["polarisation"],
                   cross_polarize=int(j["cross_polarize"]), reference_station=j["reference_station"],
                   window=j["window"], integration_nr=j["integration_nr"], streams=streams, del_bytes=tables,
                   clocks=clocks, n_integrations=1, phased_array=phased)
        n_bins = 1
        if j["pulsar_binning"]:
            p = pulsars.get(j["source"])
            if p is None:  # not a pulsar: the normal core, written as source 1 (0 is off-pulse data)
                job["pc_file_index"] = [1]
            else:
                job["pulsar"] = (p["nbins"], p["gate_start"], p["gate_stop"])
                job["polyco"] = [[pc["tmid"], pc["dm"], pc["ref_phase"], pc["ref_freq"], pc["obs_freq"]] + pc["coef"]
                                 for pc in p["polyco"]]
                n_bins = p["nbins"] + 1
        elif sources:  # multiple phase centres: every output carries its source's file index
            job["n_phase_centers"] = j["n_phase_centers"]
            job["pc_file_index"] = _phase_centre_files(_del_scans(tables[0]), j, sources)
            n_bins = j["n_phase_centers"]
        if mask is not None:
            if mask["mask"]:
                job["mask"] = np.asarray(mask["mask"], dtype=np.float32)
            if mask["window"]:
                job["lag_window"] = np.asarray(mask["window"], dtype=np.float32)
            job["mask_normalize"] = int(mask["normalize"])
        # u, v, w at the integration's mid-time (the models keep state: here, in job order)
        tmid = j["start_time"] + tint // 2
        npc = max(1, j["n_phase_centers"])
        job["uvw_now"] = [[uvw[sp["station_stream"] % n_st].get(pc, tmid) for pc in range(npc)]
                          for sp in j["stations"]]
        return job, n_bins

    def correlate_one(args):
        node, ji, job = args
        node.set_parameters(job)
        node.set_uvw(job["uvw_now"])
        for k, (s, c, i) in enumerate(slice_of[ji]):
            stations[s].rec.push(c, i, node, k)
        return node.run_integration()

    groups = []  # runs of jobs of one time slice
    for ji, j in enumerate(jobs):
        if groups and (jobs[groups[-1][0]]["scan"], jobs[groups[-1][0]]["integration_nr"]) == (j["scan"],
                                                                                               j["integration_nr"]):
            groups[-1].append(ji)
        else:
            groups.append([ji])
    n_nodes = min(max(len(g) for g in groups), workers)
    nodes += [correlator.CorrelatorNode(device, x_mode) for _ in range(n_nodes)]
    tsys_msgs = []
    with ThreadPoolExecutor(n_nodes) as ex:
        for g in groups:
            for k0 in range(0, len(g), n_nodes):
                part = g[k0:k0 + n_nodes]
                built = [job_of(jobs[ji]) for ji in part]
                results = list(ex.map(correlate_one, [(nodes[k], ji, built[k][0]) for k, ji in enumerate(part)]))
                for k, ji in enumerate(part):
                    j = jobs[ji]
                    data, tsys = results[k]
                    out.put_slice(j["slice_nr"], data, built[k][1])
                    tsys_msgs += tsys
                    if stats is not None:
                        n = sum(sp["sample_rate"] for sp in j["stations"]) * j["integration_time"] // 512_000_000
                        stats["samples"] = stats.get("samples", 0) + n
                    log("slice %d: %s channel %d integration %d" % (
                        j["slice_nr"], plan["scans"][j["scan"]]["name"], j["channel"], j["integration_nr"]))
    lap("correlate")
    files = out.finish()
    written = {}
    for url, b in zip(plan["output_files"], files):
        path = _path(url, ctrl_dir)
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        with open(path, "wb") as f:
            f.write(b)
        written[path] = b
    side = [("tsys_file", [tsys_record(m) for m in tsys_msgs]), ("phasecal_file", [phasecal_record(m) for m in pcal])]
    for key, records in side:
        if ctrl.get(key):
            path = _path(ctrl[key], ctrl_dir)
            os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
            b = b"".join(records)
            with open(path, "wb") as f:
                f.write(b)
            written[path] = b
    out.close()
    for n in nodes + list(station_nodes.values()):  # each closes its recordings first
        n.close()
    lap("output")
    return written


def _phase_centre_files(del_scans, job, sources):
    """File index of each phase centre: its source's place in the manager's
    source list (Correlation_core::do_task, sfxc/src/correlation_core.cc:
    55-58): the centres are the .del scans that start with the covering one."""
    t = job["start_time"]
    mjd = int(timebase.mjd_of(t))
    sec = (t - timebase.ticks_from_mjd_sec(mjd, 0.0)) / 512e6
    starts = [f for _, f in del_scans if f is not None and f <= sec]
    if not starts:
        raise DriverError("no delay-table scan covers the job at second %.1f" % sec)
    group = [s for s, f in del_scans if f == max(starts)]
    n = job["n_phase_centers"]
    if len(group) < n:
        raise DriverError("the delay table holds %d phase centres, the scan %d" % (len(group), n))
    return [sources.index(src) if src in sources else 0 for src in group[:n]]


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m sfxc_gpu.run", description=__doc__.split("\n\n")[0])
    ap.add_argument("ctrl")
    ap.add_argument("vex")
    ap.add_argument("--tc", action="store_true", help="tensor-core X-step (FP16 hi+lo products)")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("-q", "--quiet", action="store_true")
    a = ap.parse_args(argv)
    log = (lambda *x: None) if a.quiet else (lambda *x: print(*x, file=sys.stderr))
    files = correlate(a.ctrl, a.vex, a.device, L.X_TC_HILO if a.tc else L.X_FP32, log)
    for p, b in files.items():
        print("%s: %d bytes" % (p, len(b)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
