"""A small synthetic experiment for the single-GPU driver (sfxc_gpu.run): a VEX
schedule, a control file, the stations' delay tables and their recordings,
written into a directory.

Three stations record 2 frequencies x R/L at 4 MS/s, 2 bits, each in its own
format: Ef VDIF with four channels in one thread, Wb VDIF with one channel per
thread (and a clock more than a second off, so that its reader time is
shifted by whole seconds), On Mark5B with eight bitstreams.  Two scans with a
gap between them; the recordings run from before the first to after the
last.  Cross-polarised correlation of the first frequency, 1 s integrations.
Three variants take two of the stations for pulsar binning, extra phase
centres and the phased array; a fourth has a station leave a scan and
another start recording late.  tests/golden/driver*.npz hold what the reference's own classes make of them,
stage by stage (tests/golden/make_golden.py: its plan, reader tasklet,
channel extractor, delays, input-node writer and correlation core)."""
import json
import os

import numpy as np

import control_cases
from sfxc_gpu import synth

MJD = 60409  # 2024y100d
SR = 4_000_000
T0 = 43198            # recordings start at 11:59:58
T1 = 43211            # and end at 12:00:11
STATIONS = ["Ef", "Wb", "On"]
WB_CLOCK = 1.0000021  # seconds: the reader takes 1 s of it


VARIANTS = ("plain", "pulsar", "phase_centres", "phased", "scans")
PULSAR = "B0329+54"


def _stations(variant):
    return {"plain": STATIONS, "pulsar": ["Ef", "On"], "phase_centres": ["Ef", "Wb"], "phased": ["Ef", "On"],
            "scans": STATIONS}[variant]


def _scan_sources(variant):
    return {"plain": (["SRC1"], ["SRC2"]), "pulsar": ([PULSAR], ["SRC2"]),
            "phase_centres": (["SRC1", "SRC3"], ["SRC2"]), "phased": (["SRC1"], ["SRC2"]),
            "scans": (["SRC1"], ["SRC2"])}[variant]


def vex_text(variant="plain"):
    freqs = [control_cases._freq_def("f4", control_cases._chans_rl(2, 2.0, f0=4974.49), 4.0)]
    das = [("vdif_dbbc", "Mark5C", "DBBC"), ("mk5b", "Mark5B", "DBBC")]
    thr_ef = ("t_ef", [(0, 32.0, 4, 2, 8000)], [("CH%02d" % (k + 1), 0, k) for k in range(4)])
    thr_wb = ("t_wb", [(k, 8.0, 1, 2, 8000) for k in range(4)], [("CH%02d" % (k + 1), k, 0) for k in range(4)])
    bs_on = ("bs_on", [("CH%02d" % (k + 1), sm, 2 * k + (sm == "mag"), 2 * k + (sm == "mag"))
                       for k in range(4) for sm in ("sign", "mag")])
    mode = [("FREQ", "f4", STATIONS), ("IF", "ifs", STATIONS), ("BBC", "bbcs", STATIONS),
            ("THREADS", "t_ef", ["Ef"]), ("THREADS", "t_wb", ["Wb"]), ("BITSTREAMS", "bs_on", ["On"])]
    clocks = [("Ef", ["2024y099d00h00m00s : 0.85 usec : 2024y100d12h00m00s : 1.0e-6"]),
              ("Wb", ["2024y099d00h00m00s : %.7f sec : 2024y100d12h00m00s : 0.0" % WB_CLOCK]),
              ("On", ["2024y099d00h00m00s : -1.25 usec"])]
    src1, src2 = _scan_sources(variant)
    sts = _stations(variant)
    sts2 = [s for s in sts if not (variant == "scans" and s == "Wb")]  # Wb leaves the second scan
    scans = [("No0001", "2024y100d12h00m00s", "sess", src1, [(s, 0, 4) for s in sts]),
             ("No0002", "2024y100d12h00m06s", "sess", src2, [(s, 0, 3) for s in sts2])]
    return control_cases._base([("Ef", "vdif_dbbc"), ("Wb", "vdif_dbbc"), ("On", "mk5b")], das, mode, freqs,
                               threads=[thr_ef, thr_wb], bitstreams=[bs_on], scans=scans, clocks=clocks, nbbc=4)


def ctrl_dict(variant="plain"):
    """plain: three stations cross-polarised, with the tsys and phase-cal
    files; pulsar: Ef and On, R only, the first scan on a pulsar (4 bins
    between pulse phases 0.1 and 0.9), the second on an ordinary source;
    phase_centres: Ef and Wb, R only, the first scan with two sources;
    phased: Ef and On summed as a phased array, R and L; scans: all three,
    R only, Wb not in the second scan and Ef's recording starting a second
    into the first (the manager starts that scan's correlation later)."""
    sts = _stations(variant)
    c = {"exper_name": "N24X1", "stations": sts, "start": "2024y100d12h00m00s",
         "stop": "2024y100d12h00m09s", "integr_time": 1.0, "number_channels": 256,
         "output_file": "file://out/n24x1.cor", "delay_directory": "file://delays",
         "data_sources": {k: v for k, v in {"Ef": ["file://data/ef.vdif"],
                                            "Wb": ["file://data/wb_a.vdif", "file://data/wb_b.vdif"],
                                            "On": ["file://data/on.m5b"]}.items() if k in sts}}
    if variant == "plain":
        c.update(cross_polarize=True, channels=["CH01", "CH02"], tsys_file="file://out/n24x1.tsys",
                 phasecal_file="file://out/n24x1.pcal", phasecal_integr_time=1)
    elif variant == "pulsar":
        c.update(channels=["CH01"], pulsar_binning=True,
                 pulsars={PULSAR: {"polyco_file": "file://b0329.polyco", "nbins": 4, "interval": [0.1, 0.9]}})
    elif variant == "phase_centres":
        c.update(channels=["CH01"], fft_size_correlation=256)
    elif variant == "scans":
        c.update(channels=["CH01"])
    else:
        c.update(channels=["CH01", "CH02"], phased_array=True)
    return c


def del_bytes(station, variant="plain"):
    """Delay table of a station: one .del scan per VEX scan (the first from
    5 s before its scan to just before the second, the second to 5 s after
    it: the delay model's scans do not overlap); a smooth delay and u, v, w.  The delays (clock
    included) stay negative: a slice of 1 s at 4 MS/s is exactly its 15625
    FFTs of 256 samples, and the reader tasklet reads up to its interval's
    stop time, so with a positive delay the last slice of a scan would lack
    its last samples (the reference's input-node writer then waits for data
    that never comes)."""
    k = STATIONS.index(station)
    poly = synth.DelayPoly(coeffs=(-2.0e-5 * (k + 1), 2.0e-7 * (1 + k), -1.0e-11), t0=43200.0)
    uvw = synth.earth_rotation_uvw((4.0e5 * (k - 1), 2.5e5 * k, 1.0e5), 0.6, 0.3)
    src1, src2 = _scan_sources(variant)
    scans = [(src1[0], MJD, 43195, 11, poly, uvw)]
    for extra in src1[1:]:  # another phase centre: a scan with the same start, a slightly other delay
        p2 = synth.DelayPoly(coeffs=(poly.coeffs[0] + 3.0e-7 * (k + 1), poly.coeffs[1] - 1.0e-9, poly.coeffs[2]),
                             t0=poly.t0)
        u2 = synth.earth_rotation_uvw((4.0e5 * (k - 1), 2.5e5 * k, 1.0e5), 0.61, 0.31)
        scans.append((extra, MJD, 43195, 11, p2, u2))
    scans.append((src2[0], MJD, 43206, 8, poly, uvw))
    return synth.del_file_bytes(station, scans)


def recordings(variant="plain"):
    """name -> bytes of each data file."""
    n = T1 - T0
    late = 3 if variant == "scans" else 0  # Ef's data from 12:00:01
    ef = synth.vdif_recording((n - late) * 500, payload_bytes=8000, frames_per_second=500, start_mjd=MJD,
                              start_sec_of_day=T0 + late, log2_nchan=2, bits=2, invalid=(1711,), seed=701)
    # Wb: one thread per channel, 125 frames/s each, its time stamps 1 s late (the clock);
    # two files, the second starting where the first ends, one frame lost
    wb = synth.vdif_recording(n * 500, payload_bytes=8000, frames_per_second=125, start_mjd=MJD,
                              start_sec_of_day=T0 + 1, log2_nchan=0, bits=2, threads=(0, 1, 2, 3),
                              drop=(2222,), seed=702)
    cut = 8032 * 1000
    on = synth.mark5b_recording(n * 400, mjd=MJD, sec_of_day=T0, frames_per_second=400, seed=703)
    return {"data/ef.vdif": ef, "data/wb_a.vdif": wb[:cut], "data/wb_b.vdif": wb[cut:], "data/on.m5b": on}


def write_experiment(d, variant="plain"):
    """Writes the experiment into directory d; returns (ctrl path, vex path)."""
    os.makedirs(os.path.join(d, "delays"), exist_ok=True)
    os.makedirs(os.path.join(d, "data"), exist_ok=True)
    vex = os.path.join(d, "n24x1.vex")
    with open(vex, "w") as f:
        f.write(vex_text(variant))
    ctrl = os.path.join(d, "n24x1.ctrl")
    c = ctrl_dict(variant)
    with open(ctrl, "w") as f:
        json.dump(c, f, indent=2)
    for s in c["stations"]:
        with open(os.path.join(d, "delays", "N24X1_%s.del" % s), "wb") as f:
            f.write(del_bytes(s, variant))
    files = {u[7:] for s in c["stations"] for u in c["data_sources"][s]}
    for name, b in recordings(variant).items():
        if name in files:
            with open(os.path.join(d, name), "wb") as f:
                f.write(b)
    if variant == "pulsar":
        with open(os.path.join(d, "b0329.polyco"), "w") as f:
            f.write(control_cases._polyco(PULSAR[1:], 60409.5, 26.8, 1))
    return ctrl, vex


def split_slices(cor, nchan):
    """A .cor file (global header, then slices) as (global header, [slice
    header bytes], [complex64 visibilities per baseline of each slice])."""
    from sfxc_gpu import correlator
    (hs,) = np.frombuffer(cor[:4], dtype=np.int32)
    g, p, hdrs, vis = cor[:hs], int(hs), [], []
    while p < len(cor):  # the output node writes each slice without its file index
        nbl, nuvw, nstat = np.frombuffer(cor[p + 4:p + 16], dtype=np.int32)
        n = 16 + int(nuvw) * 32 + int(nstat) * 24 + int(nbl) * (8 + (nchan + 1) * 8)
        h, v = correlator.split_output(b"\0\0\0\0" + cor[p:p + n], nchan)
        hdrs.append(h[4:])
        vis.append(v)
        p += n
    return g, hdrs, vis


def output_parts(data, nchan):
    """A correlator output (Correlation_core::integration_write, each part
    with its int32 file index) as [(file index, part bytes without it)]."""
    parts, p = [], 0
    while p < len(data):
        fi, _, nbl, nuvw, nstat = np.frombuffer(data[p:p + 20], dtype=np.int32)
        n = 20 + int(nuvw) * 32 + int(nstat) * 24 + int(nbl) * (8 + (nchan + 1) * 8)
        parts.append((int(fi), bytes(data[p + 4:p + n])))
        p += n
    return parts
