"""Control files and VEX schedules for the correlation set-up parity tests.

Each case writes a VEX file, a control file and the files they name (empty
delay tables, polyco and mask files) into a directory; tests/golden/control.json.gz
holds the plan the reference's own Control_parameters (with its manager's
dealing restated, oracle/ref_harness.cc mode `control`) derives from them
(tests/golden/make_golden.py).  The VEX texts exercise the scanner's rules
(comments, literal blocks, quoted strings, '&' references, words of several
tokens, empty fields) and the set-ups the correlator takes: VDIF with many
channels per thread or one channel per thread, Mark5B with $BITSTREAMS,
with Mark5B $TRACKS and with the standard BBC mapping, Mark4 head-stack
tracks, cross polarisations, mixed bandwidths, extra phase centres, pulsar
binning, masks, clock breaks and rates, scans a station leaves out, and
stations whose data start late."""
import json
import os

# ---------------------------------------------------------------- VEX text


def _freq_def(name, chans, sample_rate_ms):
    """chans: (band, freq MHz, sideband, bw MHz, channel name, BBC name)"""
    lines = ["def %s;" % name]
    for band, f, sb, bw, ch, bbc in chans:
        lines.append("    chan_def = &%s : %.2f MHz : %s : %.2f MHz : &%s : &%s : &L_cal;" % (band, f, sb, bw, ch, bbc))
    lines.append("    sample_rate = %.3f Ms/sec;  * (complex)" % sample_rate_ms)
    lines.append("enddef;")
    return lines


def _vex(exper, stations, modes, freqs, ifs, bbcs, threads=(), bitstreams=(), tracks=(), scans=(), clocks=(),
         das=(), extra=()):
    out = ["VEX_rev = 1.5;", "*    synthetic schedule for the correlator set-up tests", "$GLOBAL;",
           "    ref $EXPER = %s;" % exper, "*" + "-" * 60, "$EXPER;", "def %s;" % exper,
           "    exper_name = %s;" % exper, '    exper_description = "synthetic: test & check";',
           "    PI_name = A. Tester;", "enddef;", "$MODE;"]
    for name, refs in modes:
        out.append("def %s;" % name)
        for sec, d, sts in refs:
            out.append("    ref $%s = %s%s;" % (sec, d, "".join(":" + s for s in sts)))
        out.append("enddef;")
    out.append("$STATION;")
    for st, das_name, clock in stations:
        out += ["def %s;" % st, "    ref $SITE = SITE_%s;" % st, "    ref $ANTENNA = ANT_%s;" % st,
                "    ref $DAS = %s;" % das_name, "    ref $CLOCK = %s;" % clock, "enddef;"]
    out.append("$DAS;")
    for name, transport, rack in das:
        out += ["def %s;" % name, "    record_transport_type = %s;" % transport,
                "    electronics_rack_type = %s;" % rack, "    number_drives = 2;", "enddef;"]
    out.append("$CLOCK;")
    for name, lines in clocks:
        out.append("def %s;" % name)
        out += ["    clock_early = %s;" % l for l in lines]
        out.append("enddef;")
    out.append("$FREQ;")
    for f in freqs:
        out += f
    out.append("$IF;")
    for name, defs in ifs:
        out.append("def %s;" % name)
        out += ["    if_def = &%s : %s : %s : %s MHz : U : 1 MHz : 0 Hz;" % d for d in defs]
        out.append("enddef;")
    out.append("$BBC;")
    for name, defs in bbcs:
        out.append("def %s;" % name)
        out += ["    BBC_assign = &%s : %d : &%s;" % d for d in defs]
        out.append("enddef;")
    if threads:
        out.append("$THREADS;")
        for name, thr, chans in threads:
            out.append("def %s;" % name)
            out.append("    format = VDIF : : 1024;")
            out += ["    thread = %d : 1 : 1 : %.1f Ms/sec : %d : %d : : : %d;" % t for t in thr]
            out += ["    channel = &%s : %d : %d;" % c for c in chans]
            out.append("enddef;")
    if bitstreams:
        out.append("$BITSTREAMS;")
        for name, defs in bitstreams:
            out.append("def %s;" % name)
            out += ["    stream_def = &%s : %s : %d : %d;" % d for d in defs]
            out.append("enddef;")
    if tracks:
        out.append("$TRACKS;")
        for name, fmt, defs, more in tracks:
            out.append("def %s;" % name)
            out.append("    track_frame_format = %s;" % fmt)
            out += ["    " + m for m in more]
            out += ["    fanout_def = %s: &%s : %s : %d : %s;" % (d[0], d[1], d[2], d[3], " : ".join(str(t) for t in d[4]))
                    for d in defs]
            out.append("enddef;")
    out += ["$SOURCE;"]
    srcs = sorted({s for sc in scans for s in sc[3]})
    for s in srcs:
        out += ["def %s;" % s, "    source_name = %s;" % s, "    ra = 12h30m49.4233820s;",
                "    dec =  12d23'28.043840\";", "    ref_coord_frame = J2000;", "enddef;"]
    out += list(extra)
    out.append("$SCHED;")
    for name, start, mode, sources, sts in scans:
        out += ["scan %s;" % name, "    start = %s;" % start, "    mode = %s;" % mode]
        out += ["    source = %s;" % s for s in sources]
        out += ["    station = %s : %d sec : %d sec : 0.000 GB :   : &ccw : 1;" % s for s in sts]
        out.append("endscan;")
    return "\n".join(out) + "\n"


def _ifs_rl(name="ifs"):
    return (name, [("IF_A1", "A1", "R", "4600.00"), ("IF_C1", "C1", "L", "4600.00")])


def _bbcs(n, name="bbcs"):
    # BBC0k: odd ones on the R IF, even ones on the L IF
    return (name, [("BBC%02d" % (k + 1), k + 1, "IF_A1" if k % 2 == 0 else "IF_C1") for k in range(n)])


def _chans_rl(n_freq, bw, f0=4974.49, sb="U", prefix="CH", bbc_base=0):
    """n_freq frequencies x (R, L): channel names CH01.. in frequency, R before L"""
    out = []
    for i in range(n_freq):
        for p in range(2):
            k = 2 * i + p
            out.append(("B", f0 + i * bw, sb, bw, "%s%02d" % (prefix, k + 1), "BBC%02d" % (bbc_base + k + 1)))
    return out


def _scan(name, start, mode, sources, stations, length=20):
    return (name, start, mode, sources, [(s, 0, length) for s in stations])


# ---------------------------------------------------------------- cases


def _base(stations, das, mode_refs, freqs, threads=(), bitstreams=(), tracks=(), scans=None, clocks=None, nbbc=16,
          exper="N24X1", extra=()):
    st = [(s, d, s) for s, d in stations]
    clocks = clocks or [(s, ["2024y100d00h00m00s : %.3f usec : 2024y100d00h00m00s : 0.00%d" % (1.5 + i, i + 1)])
                        for i, (s, _) in enumerate(stations)]
    scans = scans or [_scan("No0001", "2024y100d12h00m00s", "sess", ["SRC1"], [s for s, _ in stations]),
                      _scan("No0002", "2024y100d12h00m30s", "sess", ["SRC2"], [s for s, _ in stations])]
    return _vex(exper, st, [("sess", mode_refs)], freqs, [_ifs_rl()], [_bbcs(nbbc)], threads=threads,
                bitstreams=bitstreams, tracks=tracks, scans=scans, clocks=clocks, das=das, extra=extra)


def _ctrl(stations, **kw):
    c = {"exper_name": "N24X1", "stations": stations, "start": "2024y100d12h00m00s", "stop": "2024y100d12h00m50s",
         "integr_time": 2.0, "number_channels": 512, "output_file": "file://out/n24x1.cor",
         "delay_directory": "file://delays", "data_sources": {s: ["file://data/%s.vdif" % s] for s in stations}}
    c.update(kw)
    return c


def _vdif16_threads(name="thr16", chans=None):
    chans = chans or ["CH%02d" % (k + 1) for k in range(16)]
    return (name, [(0, 1024.0, 16, 2, 8000)], [(c, 0, k) for k, c in enumerate(chans)])


def cases():
    out = {}
    sts = ["Ef", "Wb", "On"]
    freqs = [_freq_def("f32", _chans_rl(8, 32.0), 64.0)]
    das = [("dbbc_mk5c", "Mark5C", "DBBC")]
    vdif_mode = [("FREQ", "f32", sts), ("IF", "ifs", sts), ("BBC", "bbcs", sts), ("THREADS", "thr16", sts)]
    out["vdif_multichannel"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()]),
        ctrl=_ctrl(sts, channels=["CH01", "CH02", "CH05", "CH06"]))

    # one channel per thread at one station, eight channels in one thread at another
    freqs8 = [_freq_def("f16", _chans_rl(4, 16.0), 32.0)]
    thr_each = ("thr_each", [(k, 32.0, 1, 2, 1000) for k in range(8)], [("CH%02d" % (k + 1), k, 0) for k in range(8)])
    thr_one = ("thr_one", [(0, 256.0, 8, 2, 8000)], [("CH%02d" % (k + 1), 0, k) for k in range(8)])
    mode = [("FREQ", "f16", ["Ef", "Wb"]), ("IF", "ifs", ["Ef", "Wb"]), ("BBC", "bbcs", ["Ef", "Wb"]),
            ("THREADS", "thr_each", ["Ef"]), ("THREADS", "thr_one", ["Wb"])]
    out["vdif_threads"] = dict(
        vex=_base([("Ef", "dbbc_mk5c"), ("Wb", "dbbc_mk5c")], das, mode, freqs8, threads=[thr_each, thr_one]),
        ctrl=_ctrl(["Wb", "Ef"], integr_time=1.0, sub_integr_time=250000, number_channels=1024,
                   fft_size_correlation=2048, window_function="hamming"))

    # Mark5B: $BITSTREAMS (32 bitstreams), $TRACKS with Mark5B frames, and the standard mapping
    das_b = [("mk5b", "Mark5B", "DBBC")]
    bs = ("bs16", [(c, sm, n, n) for k, c in enumerate(["CH%02d" % (i + 1) for i in range(16)])
                   for sm, n in (("sign", 2 * k), ("mag", 2 * k + 1))])
    trk = ("trk_mk5b", "Mark5B", [("", "CH%02d" % (k + 1), sm, 1, [2 + 2 * k + (sm == "mag")])
                                  for k in range(16) for sm in ("sign", "mag")], ["data_modulation = off;"])
    # the standard mapping needs a $TRACKS def (for the bits per sample) that is not in Mark5B frames
    trk_std = ("trk_std", "VLBA", [("", "CH01", "sign", 1, [2]), ("", "CH01", "mag", 1, [4])], [])
    mode = [("FREQ", "f32", sts), ("IF", "ifs", sts), ("BBC", "bbcs", sts), ("BITSTREAMS", "bs16", ["Ef"]),
            ("TRACKS", "trk_mk5b", ["Wb"]), ("TRACKS", "trk_std", ["On"])]
    out["mark5b"] = dict(
        vex=_base([(s, "mk5b") for s in sts], das_b, mode, freqs, bitstreams=[bs], tracks=[trk, trk_std]),
        ctrl=_ctrl(sts, number_channels=256, LO_offset={"Wb": 12.5}, tsys_freq={"On": 40}))

    # Mark4 head stacks (reader parameters only; no Mark4 reader is built)
    das4 = [("mk5a", "Mark5A", "VLBA4")]
    trk4 = ("trk_mk4", "Mark4", [("A", "CH%02d" % (k + 1), sm, 1 + (k >= 4), [2 + 4 * (k % 4) + 2 * (sm == "mag"),
                                                                            3 + 4 * (k % 4) + 2 * (sm == "mag")])
                                 for k in range(8) for sm in ("sign", "mag")], ["data_modulation = on;"])
    mode = [("FREQ", "f16", ["Ef", "Wb"]), ("IF", "ifs", ["Ef", "Wb"]), ("BBC", "bbcs", ["Ef", "Wb"]),
            ("TRACKS", "trk_mk4", ["Ef", "Wb"])]
    out["mark4_tracks"] = dict(vex=_base([("Ef", "mk5a"), ("Wb", "mk5a")], das4, mode, freqs8, tracks=[trk4]),
                               ctrl=_ctrl(["Ef", "Wb"]))

    # cross polarisations, a reference station, a setup station
    out["cross_pol"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()]),
        ctrl=_ctrl(sts, cross_polarize=True, channels=["CH01", "CH02", "CH03", "CH04"], reference_station="Wb",
                   setup_station="On", integr_time=1.0))

    # mixed bandwidths: Ef at 32 MHz, Wb at 16 MHz (inside), On at 64 MHz (around)
    f_ef = _freq_def("f32", _chans_rl(4, 32.0, f0=4800.0), 64.0)
    f_wb = _freq_def("f16", _chans_rl(4, 16.0, f0=4800.0, prefix="NB"), 32.0)
    f_on = _freq_def("f64", _chans_rl(2, 64.0, f0=4800.0, prefix="WB"), 128.0)
    thr_ef = _vdif16_threads("t_ef", ["CH%02d" % (k + 1) for k in range(8)])
    thr_wb = ("t_wb", [(0, 256.0, 8, 2, 8000)], [("NB%02d" % (k + 1), 0, k) for k in range(8)])
    thr_on = ("t_on", [(0, 512.0, 4, 2, 8000)], [("WB%02d" % (k + 1), 0, k) for k in range(4)])
    mode = [("FREQ", "f32", ["Ef"]), ("FREQ", "f16", ["Wb"]), ("FREQ", "f64", ["On"]), ("IF", "ifs", sts),
            ("BBC", "bbcs", sts), ("THREADS", "t_ef", ["Ef"]), ("THREADS", "t_wb", ["Wb"]), ("THREADS", "t_on", ["On"])]
    out["mixed_bandwidth"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, mode, [f_ef, f_wb, f_on], threads=[thr_ef, thr_wb, thr_on]),
        ctrl=_ctrl(sts, channels=["CH01", "CH02", "CH03", "CH04"]))

    # extra phase centres: scans with two sources
    scans = [_scan("No0001", "2024y100d12h00m00s", "sess", ["SRC1", "SRC3"], sts),
             _scan("No0002", "2024y100d12h00m30s", "sess", ["SRC2"], sts)]
    out["multi_phase_center"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()], scans=scans),
        ctrl=_ctrl(sts, channels=["CH01", "CH02"], integr_time=1.0))

    # pulsar binning with a polyco file, and a mask
    out["pulsar"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()]),
        ctrl=_ctrl(sts, channels=["CH01", "CH02"], pulsar_binning=True,
                   pulsars={"B0329+54": {"polyco_file": "file://polyco_b0329.dat", "nbins": 16,
                                         "interval": [0.25, 0.75]},
                            "J1234": {"polyco_file": "file://polyco_j1234.dat"}}),
        files={"polyco_b0329.dat": _polyco("0329+54", 60400.5, 26.8, 2), "polyco_j1234.dat": _polyco("1234", 60400.5, 8.1, 1)})
    out["mask"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()]),
        ctrl=_ctrl(sts, channels=["CH03"], number_channels=64, fft_size_correlation=512,
                   mask={"normalize": True, "mask": "file://mask.txt", "window": "file://window.txt"}),
        files={"mask.txt": "\n".join("%.3f" % (1.0 if 50 < k < 460 else 0.0) for k in range(513)) + "\n",
               "window.txt": " ".join("%.6f" % (0.5 - 0.5 * ((k % 7) / 7.0)) for k in range(128)) + "\n"})

    # clock breaks, rates with and without units, a large offset (reader seconds)
    clocks = [("Ef", ["2024y099d00h00m00s : 1.25 usec : 2024y099d00h00m00s : 0.5",
                      "2024y100d12h00m20s : 2.5 sec : 2024y100d12h00m20s : 1.0e-12 sec/sec"]),
              ("Wb", ["2024y100d00h00m00s : -0.75 sec", "2024y090d00h00m00s : 3.0 usec : 2024y090d00h00m00s : 0.1"]),
              ("On", ["2024y100d12h00m00s : 12.0 usec : 2024y100d06h00m00s : 2.0e-13"])]
    scans = [_scan("No0001", "2024y100d12h00m00s", "sess", ["SRC1"], sts),
             _scan("No0002", "2024y100d12h00m30s", "sess", ["SRC2"], sts)]
    out["clocks"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()], clocks=clocks,
                  scans=scans),
        ctrl=_ctrl(sts, channels=["CH01"]))

    # scan structure: a station leaves a scan, scans with gaps, start inside a
    # scan, stop inside a later one, late station data, a scan of another length
    scans = [("No0003", "2024y100d12h00m00s", "sess", ["SRC1"], [("Ef", 0, 20), ("Wb", 0, 20), ("On", 5, 17)]),
             ("No0004", "2024y100d12h00m25s", "sess", ["SRC2"], [("Ef", 0, 15), ("On", 0, 15)]),
             ("No0007", "2024y100d12h01m00s", "sess", ["SRC1"], [("Ef", 0, 30), ("Wb", 0, 30), ("On", 0, 30)])]
    out["scans"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()], scans=scans),
        ctrl=_ctrl(sts, channels=["CH01", "CH02"], start="2024y100d12h00m05s", stop="2024y100d12h01m11s",
                   integr_time=3.0),
        station_times=[(1, 0, "2024y100d12h00m11s"), (2, 2, "2024y100d12h01m04s")])

    # the scanner's rules: literal blocks, comments, quotes, default channels and scans
    extra = ["$TAPELOG_OBS;", "def Ef;", "start_literal( );", "  this = is : not ; parsed $ at all", "  * neither",
             "end_literal();", "  VSN = 1 : \"EVN+0001\" : 2024y100d11h00m00s : 2024y100d13h00m00s;", "enddef;",
             "* a comment with ; and = and $ in it"]
    out["vex_syntax"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()], extra=extra),
        ctrl=_ctrl(sts, stop="end", exper_name="N24X1", job=7, subjob=3, window_function="COSINE",
                   fft_size_delaycor=512, number_channels=256))

    # two modes: the second scan in another set-up (16 MHz channels, another
    # thread layout), which changes the reader parameters and the channels'
    # frequencies from one scan to the next
    sts2 = ["Ef", "Wb"]
    f16 = _freq_def("f16b", _chans_rl(4, 16.0, f0=4974.49), 32.0)
    thr8 = ("thr8", [(0, 256.0, 8, 2, 8000)], [("CH%02d" % (k + 1), 0, k) for k in range(8)])
    modes = [("wide", [("FREQ", "f32", sts2), ("IF", "ifs", sts2), ("BBC", "bbcs", sts2), ("THREADS", "thr16", sts2)]),
             ("narrow", [("FREQ", "f16b", sts2), ("IF", "ifs", sts2), ("BBC", "bbcs", sts2), ("THREADS", "thr8", sts2)])]
    scans = [("No0001", "2024y100d12h00m00s", "wide", ["SRC1"], [(x, 0, 20) for x in sts2]),
             ("No0002", "2024y100d12h00m30s", "narrow", ["SRC2"], [(x, 0, 20) for x in sts2])]
    out["two_modes"] = dict(
        vex=_vex("N24X1", [(x, "dbbc_mk5c", x) for x in sts2], modes, [_freq_def("f32", _chans_rl(8, 32.0), 64.0), f16],
                 [_ifs_rl()], [_bbcs(16)], threads=[_vdif16_threads(), thr8], scans=scans,
                 clocks=[(x, ["2024y100d00h00m00s : 1.0 usec"]) for x in sts2], das=das),
        ctrl=_ctrl(sts2, channels=["CH01", "CH02", "CH03", "CH04"], cross_polarize=True))

    # refused set-ups
    out["error_pulsar_multi_phase"] = dict(
        vex=_base([(s, "dbbc_mk5c") for s in sts], das, vdif_mode, freqs, threads=[_vdif16_threads()]),
        ctrl=_ctrl(sts, pulsar_binning=True, multi_phase_center=True,
                   pulsars={"P": {"polyco_file": "file://p.dat"}}),
        files={"p.dat": _polyco("P", 60400.5, 10.0, 1)})
    return out


def _polyco(name, tmid, dm, blocks):
    """A TEMPO polyco text: per block a header line, a line with the reference
    phase and frequency, then 12 coefficients three to a line."""
    lines = []
    for b in range(blocks):
        lines.append("%-10s %9s %11.2f %19.11f %21.6f %6.3f %7.3f" % (name, "10-Apr-24", 120000.00 + b * 100,
                                                                      tmid + b / 24.0, dm, 0.123, -5.456))
        lines.append("%20.6f %18.12f %4s %5d %5d %10.3f" % (1234567.123456 + b, 1.399538 + b * 1e-6, "ef", 60, 12,
                                                            1400.0))
        coef = [0.0, 1.5e-3 * (b + 1), -2.25e-7, 3.0e-9, -1.0e-11] + [0.0] * 7
        for k in range(0, 12, 3):
            lines.append(" ".join("%25.17e" % c for c in coef[k:k + 3]))
    return "\n".join(lines) + "\n"


def write_case(case, d):
    """Writes the case's files into directory d; returns (ctrl path, vex path)."""
    os.makedirs(d, exist_ok=True)
    os.makedirs(os.path.join(d, "delays"), exist_ok=True)
    vex_path = os.path.join(d, "exp.vex")
    with open(vex_path, "w") as f:
        f.write(case["vex"])
    ctrl_path = os.path.join(d, "exp.ctrl")
    with open(ctrl_path, "w") as f:
        json.dump(case["ctrl"], f, indent=2)
    for name, text in case.get("files", {}).items():
        with open(os.path.join(d, name), "w") as f:
            f.write(text)
    for s in case["ctrl"]["stations"]:  # the delay tables the set-up names must exist
        open(os.path.join(d, "delays", "N24X1_%s.del" % s), "a").close()
    return ctrl_path, vex_path


def vex_time_ticks(text):
    """Clock ticks (512 MHz since MJD 51544) of a VEX time "YYYYyDDDdHHhMMmSSs"."""
    import datetime
    import re
    y, d, h, m, sec = map(int, re.match(r"(\d+)y(\d+)d(\d+)h(\d+)m(\d+)s", text).groups())
    mjd = (datetime.date(y, 1, 1) - datetime.date(1858, 11, 17)).days + d - 1
    return ((mjd - 51544) * 86400 + h * 3600 + m * 60 + sec) * 512000000


def station_times(case):
    """[(station, scan, ticks)] of a case's late station data."""
    return [(s, sc, vex_time_ticks(t)) for s, sc, t in case.get("station_times", [])]
