"""Job files for the checkers: the reference's own classes (oracle/_ref/ref_harness)
and the C restatement (oracle/_build/sfxc_oracle) take identical jobs and write
identical output files, so one job can be run through both and compared.

Test infrastructure only (tests/, golden-fixture generation, the CPU baseline).
The reference harness needs the reference checkout (oracle/build_ref.py) and so
runs only where that checkout exists; the restatement builds anywhere with gcc.
"""
import os
import subprocess
import tempfile

import numpy as np

from . import build_ref, build_oracle


def harness():
    exe = build_ref.build()
    if exe is None:
        raise RuntimeError("reference checkout not available; the reference harness cannot be built")
    return exe


def restatement():
    return build_oracle.build()


_EXE = {"reference": harness, "oracle": restatement}


def _write_job(path, lines):
    with open(path, "w") as f:
        for key, *vals in lines:
            f.write(key + " " + " ".join(str(v) for v in vals) + "\n")


def _run(mode, lines, out, workdir, impl, timeout=None):
    job = os.path.join(workdir, mode + ".job")
    _write_job(job, lines)
    r = subprocess.run([_EXE[impl](), mode, job, out], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("%s %s failed (%d): %s%s" % (impl, mode, r.returncode, r.stdout, r.stderr))


def delays(del_bytes, start_ticks, stop_ticks, sample_rate, bits, probes=(), clock=None, impl="reference"):
    """Input_node_tasklet delay list for one interval + spline probes.

    Returns (list of (ticks, bytes, remaining_samples), list of
    (ticks, delay, rate, phase, amplitude)).
    """
    with tempfile.TemporaryDirectory() as d:
        delf = os.path.join(d, "st.del")
        open(delf, "wb").write(del_bytes)
        lines = [("delfile", delf), ("start_ticks", start_ticks), ("stop_ticks", stop_ticks),
                 ("sample_rate", sample_rate), ("bits_per_sample", bits)]
        if clock is not None:
            lines.append(("clock",) + tuple(clock))
        lines += [("probe", p) for p in probes]
        out = os.path.join(d, "out.txt")
        _run("delays", lines, out, d, impl)
        dl, pr = [], []
        for line in open(out):
            v = line.split()
            if v[0] == "P":
                pr.append((int(v[1]),) + tuple(float(x) for x in v[2:]))
            else:
                dl.append((int(v[0]), int(v[1]), int(v[2])))
        return dl, pr


def protocol(blocks, slices, sample_rate, bits, integr_time_us, station_number=0, impl="reference",
             phasecal_ticks=None, channel=None):
    """Input_node_data_writer protocol bytes for each slice.

    blocks: list of (start_ticks, bytes, [(invalid_begin, nr_invalid), ...])
    slices: list of (start_ticks, stop_ticks, nr_samples, delay_list)
    phasecal_ticks: phase-cal integration time; when given, returns
    (protocols, phase-cal message bytes) (Input_node_data_writer::do_phasecal)
    channel: the channel's {sideband, polarisation, frequency_number} for
    those messages (default U, R, 0)
    """
    with tempfile.TemporaryDirectory() as d:
        blob = os.path.join(d, "blocks.bin")
        offs = []
        with open(blob, "wb") as f:
            pos = 0
            for st, data, inv in blocks:
                f.write(bytes(data))
                offs.append((st, pos, len(data), inv))
                pos += len(data)
        lines = [("sample_rate", sample_rate), ("bits_per_sample", bits),
                 ("integr_time_us", integr_time_us), ("station_number", station_number),
                 ("blockfile", blob)]
        if channel is not None:
            lines.append(("channel_params", channel["sideband"], channel["polarisation"],
                          channel["frequency_number"]))
        for st, pos, n, inv in offs:
            flat = [x for pair in inv for x in pair]
            lines.append(("block", st, pos, n, *flat))
        for k, (s0, s1, ns, dl) in enumerate(slices):
            dpath = os.path.join(d, "dl%d.txt" % k)
            with open(dpath, "w") as f:
                for t, b, r in dl:
                    f.write("%d %d %d\n" % (t, b, r))
            lines.append(("slice", s0, s1, ns))
            lines.append(("dlist", dpath))
        out = os.path.join(d, "proto.bin")
        pc_out = os.path.join(d, "pcal.bin")
        if phasecal_ticks is not None:
            lines += [("phasecal_ticks", phasecal_ticks), ("phasecal_out", pc_out)]
        _run("protocol", lines, out, d, impl)
        raw = open(out, "rb").read()
        res, p = [], 0
        while p < len(raw):
            n = int(np.frombuffer(raw[p:p + 8], dtype=np.uint64)[0])
            res.append(raw[p + 8:p + 8 + n])
            p += 8 + n
        if phasecal_ticks is not None:
            return res, open(pc_out, "rb").read()
        return res


def extract(words_bytes, word_bytes, bits, nsamples, tracks, impl="reference"):
    """Channel_extractor_5 output per subband (bytes)."""
    with tempfile.TemporaryDirectory() as d:
        inf = os.path.join(d, "in.bin")
        open(inf, "wb").write(bytes(words_bytes))
        lines = [("word_bytes", word_bytes), ("bits_per_sample", bits), ("nsamples", nsamples),
                 ("infile", inf)] + [("subband", *t) for t in tracks]
        out = os.path.join(d, "out.bin")
        _run("extract", lines, out, d, impl)
        raw = open(out, "rb").read()
        per = nsamples * len(tracks[0]) // 8
        return [raw[i * per:(i + 1) * per] for i in range(len(tracks))]


def reader(recording, fmt, *, ref_ticks, offset_ticks=0, track_bit_rate, frame_size=0, n_tracks, bits,
           channel_tracks, max_blocks=1000000, timeout=None):
    """Blocks of the reference's VDIF_reader / Mark5b_reader over a recording:
    dicts {channel, start_ticks, data, invalid [(begin, n)]}.  Only the
    reference's own classes implement this (there is no restatement).
    timeout (s): subprocess.TimeoutExpired when the reader runs longer."""
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "rec.bin")
        open(path, "wb").write(bytes(recording))
        lines = [("format", fmt), ("file", path), ("ref_ticks", ref_ticks), ("offset_ticks", offset_ticks),
                 ("track_bit_rate", track_bit_rate), ("frame_size", frame_size), ("n_tracks", n_tracks),
                 ("bits", bits), ("max_blocks", max_blocks)]
        lines += [("channel#%d" % c, *tr) for c, tr in enumerate(channel_tracks)]
        out = os.path.join(d, "out")
        os.makedirs(out)
        _run("reader", lines, out, d, "reference", timeout=timeout)
        raw = open(os.path.join(out, "data.bin"), "rb").read()
        blocks, pos = [], 0
        for line in open(os.path.join(out, "blocks.txt")):
            v = [int(x) for x in line.split()]
            ch, ticks, size, inv = v[0], v[1], v[2], v[3:]
            blocks.append({"channel": ch, "start_ticks": ticks, "data": raw[pos:pos + size],
                           "invalid": [(inv[k], inv[k + 1]) for k in range(0, len(inv), 2)]})
            pos += size
        return blocks


def schedule(recording, fmt, *, ref_ticks, offset_ticks=0, track_bit_rate, frame_size=0, n_tracks, bits,
             channel_tracks, intervals):
    """Blocks the reference's reader tasklet (Input_data_format_reader_tasklet)
    pushes for a recording and time intervals [(start, stop, leave) ticks]:
    dicts {channel, start_ticks, size, data (None for a wholly invalid block),
    invalid [(begin, n)], buffer (blocks with the same number were pushed in
    one data buffer and show its last bytes), stale (the buffer's bytes are
    not a block's: the last read into it failed, or none was made)}.  Only
    the reference's own classes implement this."""
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "rec.bin")
        open(path, "wb").write(bytes(recording))
        lines = [("format", fmt), ("file", path), ("ref_ticks", ref_ticks), ("offset_ticks", offset_ticks),
                 ("track_bit_rate", track_bit_rate), ("frame_size", frame_size), ("n_tracks", n_tracks),
                 ("bits", bits)]
        lines += [("channel#%d" % c, *tr) for c, tr in enumerate(channel_tracks)]
        lines += [("interval#%d" % k, *iv) for k, iv in enumerate(intervals)]
        out = os.path.join(d, "out")
        os.makedirs(out)
        _run("schedule", lines, out, d, "reference")
        raw = open(os.path.join(out, "data.bin"), "rb").read()
        blocks, pos = [], 0
        for line in open(os.path.join(out, "schedule.txt")):
            v = [int(x) for x in line.split()]
            ch, ticks, size, buf, stale, inv = v[0], v[1], v[2], v[3], v[4], v[5:]
            runs = [(inv[k], inv[k + 1]) for k in range(0, len(inv), 2)]
            whole = any(b == 0 and n >= size for b, n in runs)
            blocks.append({"channel": ch, "start_ticks": ticks, "size": size, "invalid": runs, "buffer": buf,
                           "stale": bool(stale), "data": None if whole else raw[pos:pos + size]})
            if not whole:
                pos += size
        return blocks


def uvw(del_bytes, probes):
    """The reference's Uvw_model over a .del file at probes [(phase centre,
    ticks)], in order: [(u, v, w)].  Only the reference's own class implements
    this (the library's restatement is what it pins)."""
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "st.del")
        open(p, "wb").write(del_bytes)
        lines = [("delfile", p)] + [("probe#%d" % k, pc, t) for k, (pc, t) in enumerate(probes)]
        out = os.path.join(d, "uvw.txt")
        _run("uvw", lines, out, d, "reference")
        return [tuple(float(x) for x in line.split()) for line in open(out)]


def control(ctrl_path, vex_path, workdir, station_times=()):
    """The reference's Control_parameters over a control file and a VEX file,
    with the manager's dealing of the jobs: the plan as a dict, or None when
    the reference refuses the set-up (returns false or aborts).  Runs in
    workdir, which relative paths of the control file are taken from, as the
    reference takes them from its working directory.  station_times:
    [(station, scan, ticks)]."""
    job = os.path.join(workdir, "control.job")
    _write_job(job, [("ctrl", ctrl_path), ("vex", vex_path)] +
               [("station_time", s, sc, t) for s, sc, t in station_times])
    out = os.path.join(workdir, "control.json")
    r = subprocess.run([harness(), "control", job, out], capture_output=True, text=True, cwd=workdir)
    if r.returncode != 0:
        return None
    import json
    plan = json.load(open(out))
    return None if "error" in plan else plan


def correlate_lines(job, d, dump=False, precision=32, dump_bins=False):
    """The job file lines of the 'correlate' mode for a job dict, with its
    delay tables, protocols and mask files written into directory d (read by
    the reference harness, the restatement and the adapter driver)."""
    lines = []
    for k, db in enumerate(job["del_bytes"]):
        p = os.path.join(d, "st%d.del" % k)
        open(p, "wb").write(db)
        lines.append(("delfile", p))
    if job.get("clocks") is not None:  # Delay_table::set_clock_offset per table: offset, rate, epoch ticks
        for c in job["clocks"]:
            lines.append(("clock",) + tuple(c if c is not None else (0.0, 0.0, 0)))
    for key in ["experiment_start_ticks", "start_ticks", "integration_time_us",
                "sub_integration_time_us", "number_channels", "fft_size_delaycor",
                "fft_size_correlation", "sample_rate", "channel_freq", "bandwidth", "sideband",
                "frequency_nr", "polarisation", "cross_polarize", "reference_station", "window",
                "source", "integration_nr", "n_integrations"]:
        lines.append((key, job[key]))
    for k, s in enumerate(job["streams"]):
        lines.append(("stream",) + tuple(s))
        p = os.path.join(d, "proto%d.bin" % k)
        with open(p, "wb") as f:
            for chunk in job["protocols"][k]:
                f.write(np.uint64(len(chunk)).tobytes())
                f.write(bytes(chunk))
        lines.append(("protocol", p))
    # Mask_parameters (spectral reduction): float32 files, and the flag
    for key in ("mask", "lag_window"):
        if job.get(key) is not None:
            p = os.path.join(d, key + ".f32")
            np.asarray(job[key], dtype=np.float32).tofile(p)
            lines.append((key, p))
    if job.get("mask_normalize"):
        lines.append(("mask_normalize", 1))
    # UVW for the timeslice headers: float64 [integration][stream][centre][3]
    if job.get("uvw") is not None:
        p = os.path.join(d, "uvw.f64")
        np.asarray(job["uvw"], dtype=np.float64).tofile(p)
        lines.append(("uvw", p))
    if job.get("phased_array"):
        lines.append(("phased_array", 1))
    if int(job.get("n_phase_centers", 1)) > 1:
        lines.append(("n_phase_centers", int(job["n_phase_centers"])))
        if job.get("pc_file_index") is not None:
            lines.append(("pc_file_index",) + tuple(int(x) for x in job["pc_file_index"]))
    if job.get("source_list"):
        lines.append(("source_list",) + tuple(job["source_list"]))
    if job.get("pulsar_mode"):
        lines.append(("pulsar_mode", 1))
    if "pulsar" in job:
        lines.append(("pulsar",) + tuple(job["pulsar"]))
        for pc in job["polyco"]:
            lines.append(("polyco",) + tuple(pc))
    if dump:
        lines.append(("dump", 1))
    if dump_bins:
        lines.append(("dump_bins", 1))
    if precision != 32:
        lines.append(("precision", precision))
    return lines


def correlate(job, dump=False, impl="reference", precision=32, dump_bins=False):
    """Run Bit2float_worker -> Delay_correction -> Correlation_core(_pulsar).

    job: dict with keys of the harness 'correlate' mode (see ref_harness.cc);
    'del_bytes' (list per station), 'protocols' (list per stream of a list of
    per-integration byte strings).  Returns dict with cor bytes, stats lines,
    tsys bytes and (dump=True) per-integration unpacked/rows arrays;
    dump_bins=True (restatement): only the pulsar bin table, res["bins"].
    """
    with tempfile.TemporaryDirectory() as d:
        lines = correlate_lines(job, d, dump=dump, precision=precision, dump_bins=dump_bins)
        outdir = os.path.join(d, "out")
        os.makedirs(outdir)
        _run("correlate", lines, outdir, d, impl)
        res = {"cor": open(os.path.join(outdir, "out.cor"), "rb").read(),
               "stats": open(os.path.join(outdir, "stats.txt")).read(),
               "tsys": open(os.path.join(outdir, "tsys.bin"), "rb").read()}
        p64 = os.path.join(outdir, "out64.bin")
        if os.path.exists(p64):
            res["vis64"] = np.fromfile(p64, dtype=np.complex128)
        bp = os.path.join(outdir, "bins_i0.i32")
        if dump_bins and "pulsar" in job and os.path.exists(bp):
            K = int(job["fft_size_correlation"]) + 1
            res["bins"] = np.concatenate([
                np.fromfile(os.path.join(outdir, "bins_i%d.i32" % it), dtype=np.int32).reshape(-1, K)
                for it in range(int(job["n_integrations"]))])
        if dump:
            un, rows = {}, {}
            for it in range(int(job["n_integrations"])):
                for k in range(len(job["streams"])):
                    un[(it, k)] = np.fromfile(os.path.join(outdir, "unpacked_i%d_s%d.f32" % (it, k)),
                                              dtype=np.float32)
                    rows[(it, k)] = np.fromfile(os.path.join(outdir, "rows_i%d_s%d.c64" % (it, k)),
                                                dtype=np.complex64)
            res["unpacked"] = un
            res["rows"] = rows
            bp = os.path.join(outdir, "bins_i0.i32")
            if "pulsar" in job and os.path.exists(bp):
                K = int(job["fft_size_correlation"]) + 1
                res["bins"] = np.concatenate([
                    np.fromfile(os.path.join(outdir, "bins_i%d.i32" % it), dtype=np.int32).reshape(-1, K)
                    for it in range(int(job["n_integrations"]))])
        return res
