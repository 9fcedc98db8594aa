"""The single-GPU driver (sfxc_gpu.run: control file + VEX file -> .cor file)
on a small experiment of three stations in three recording formats
(tests/driver_cases.py), against the reference's own classes stage by stage
(tests/golden/driver.npz: its plan, reader tasklet, channel extractor, delays,
input-node writer and correlation core, composed as its nodes compose them):
the global header's fields, every slice's headers byte for byte, the
visibilities within the FP32 tolerance (1e-5 relative L2 per baseline; 1e-4
for the tensor-core X-step), and the tsys and phase-cal files made of the
reference's own messages."""
import json
import os

import numpy as np
import pytest

import driver_cases
from sfxc_gpu import lib as L

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "driver.npz")
NCHAN = 256


def _correlate(d, x_mode, variant="plain"):
    from sfxc_gpu import run
    ctrl, vex = driver_cases.write_experiment(d, variant)
    old = os.getcwd()
    os.chdir(d)  # the delay directory of the control file is relative to the working directory
    try:
        return run.correlate(ctrl, vex, x_mode=x_mode)
    finally:
        os.chdir(old)


def _run(tmp_path, x_mode):
    d = str(tmp_path)
    files = _correlate(d, x_mode)
    out = os.path.join(d, "out", "n24x1")
    assert sorted(files) == [out + ".cor", out + ".pcal", out + ".tsys"]
    return files[out + ".cor"], files[out + ".tsys"], files[out + ".pcal"]


def _global_fields(g):
    (size,) = np.frombuffer(g[:4], dtype=np.int32)
    year, day = np.frombuffer(g[36:40], dtype=np.int16)
    start, nchan, tint, fmt_version, version = np.frombuffer(g[40:60], dtype=np.int32)
    pol = g[60]
    job, subjob = np.frombuffer(g[76:84], dtype=np.int32)
    return dict(header_size=int(size), experiment=g[4:36].split(b"\0")[0].decode(), start_year=int(year),
                start_day=int(day), start_time=int(start), number_channels=int(nchan), integration_time=int(tint),
                polarisation_type=int(pol), job_nr=int(job), subjob_nr=int(subjob))


@pytest.mark.gpu
@pytest.mark.parametrize("x_mode,tol", [(L.X_FP32, 1e-5), (L.X_TC_HILO, 1e-4)])
def test_driver_matches_reference_stages(tmp_path, x_mode, tol):
    from sfxc_gpu import correlator, run
    cor, tsys, pcal = _run(tmp_path, x_mode)
    g = np.load(GOLDEN)
    want = json.loads(str(g["header"]))
    head, hdrs, vis = driver_cases.split_slices(cor, NCHAN)
    fields = _global_fields(head)
    assert fields["header_size"] == 84
    for k in ("experiment", "start_year", "start_day", "start_time", "number_channels", "integration_time",
              "polarisation_type", "job_nr", "subjob_nr"):
        assert fields[k] == want[k], k
    n = int(g["slices"])
    assert len(hdrs) == n == 7  # 4 + 3 one-second slices of the two scans
    for k in range(n):
        rh, rv = correlator.split_output(g["slice%d" % k].tobytes(), NCHAN)
        assert rh[:4] == b"\0\0\0\0"  # file index 0: the output node strips it
        assert hdrs[k] == rh[4:], "slice %d headers" % k
        assert len(vis[k]) == len(rv) == 18  # 6 streams: 6 autos + 12 crosses between stations
        for b, (x, y) in enumerate(zip(vis[k], rv)):
            err = np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-30)
            assert err <= tol, "slice %d baseline %d: %.3g" % (k, b, err)
    # side files: the correlation core's tsys messages of every job, the input
    # nodes' phase-cal messages of every station channel, as the output node
    # writes them
    msgs = [g["tsys%d" % k].tobytes() for k in range(n)]
    assert tsys == b"".join(run.tsys_record(m[i:i + 44]) for m in msgs for i in range(0, len(m), 44))
    want = b""
    for key in sorted(k for k in g.files if k.startswith("pcal_")):
        m = g[key].tobytes()
        p = 24 + 4 * 400
        assert len(m) % p == 0 and len(m) // p == 6  # seven seconds of data, the last integration unfinished
        want += b"".join(run.phasecal_record(m[i:i + p]) for i in range(0, len(m), p))
    assert pcal == want


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["pulsar", "phase_centres", "phased", "scans"])
@pytest.mark.parametrize("x_mode,tol", [(L.X_FP32, 1e-5), (L.X_TC_HILO, 1e-4)])
def test_driver_variants_match_reference_stages(tmp_path, variant, x_mode, tol):
    """Pulsar binning (the pulsar's scan in 4 + 1 bins, one file per bin;
    the other scan's source as file 1), extra phase centres (the first
    scan's two sources, one file per source), the phased array (one summed
    spectrum per sub-integration), and a station leaving a scan while another
    starts late: every output file's slices against the reference's core
    outputs routed by their file index."""
    from sfxc_gpu import correlator
    d = str(tmp_path)
    files = _correlate(d, x_mode, variant)
    g = np.load(os.path.join(HERE, "golden", "driver_%s.npz" % variant))
    names = [f.replace("<dir>", d)[7:] for f in json.loads(str(g["files"]))]
    assert sorted(files) == sorted(names)
    want = {k: [] for k in range(len(names))}
    for k in range(int(g["slices"])):
        for fi, part in driver_cases.output_parts(g["slice%d" % k].tobytes(), NCHAN):
            want[fi].append(part)
    assert all(want.values())  # every file has slices
    for fi, name in enumerate(names):
        head, hdrs, vis = driver_cases.split_slices(files[name], NCHAN)
        assert _global_fields(head)["header_size"] == 84
        assert len(hdrs) == len(want[fi]), name
        for k, part in enumerate(want[fi]):
            rh, rv = correlator.split_output(b"\0\0\0\0" + part, NCHAN)
            assert hdrs[k] == rh[4:], "%s slice %d headers" % (name, k)
            for b, (x, y) in enumerate(zip(vis[k], rv)):
                err = np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-30)
                assert err <= tol, "%s slice %d baseline %d: %.3g" % (name, k, b, err)


def test_driver_refuses_what_it_does_not_run(tmp_path, sfxc_lib):
    """Mark4 recordings (no Mark5A reader) stop the driver before it takes a
    GPU."""
    import control_cases
    from sfxc_gpu import run
    case = control_cases.cases()["mark4_tracks"]
    ctrl, vex = control_cases.write_case(case, str(tmp_path / "mk4"))
    with pytest.raises(run.DriverError, match="Mark4 recordings are not read"):
        run.correlate(ctrl, vex)


def test_driver_plan_of_the_experiment(tmp_path, sfxc_lib):
    """The experiment's plan: seven jobs, cross-polarised, Wb's reader one
    second off, each station in its own format."""
    from sfxc_gpu import control
    d = str(tmp_path)
    ctrl, vex = driver_cases.write_experiment(d)
    p = control.plan(ctrl, vex)
    assert [j["integration_nr"] for j in p["jobs"]] == [0, 1, 2, 3, 6, 7, 8]
    assert all(j["cross_polarize"] and len(j["stations"]) == 6 for j in p["jobs"])
    st = {e["name"]: e for e in p["scans"][0]["stations"]}
    assert st["Wb"]["reader_offset"] == 512_000_000 and st["Ef"]["reader_offset"] == 0
    assert {n: (e["input"]["data_format"], e["input"]["n_tracks"]) for n, e in st.items()} == \
        {"Ef": ("VDIF", 8), "Wb": ("VDIF", 0), "On": ("Mark5B", 8)}


def test_side_file_records():
    """The output node's tsys and phase-cal records of known messages."""
    import struct
    from sfxc_gpu import run
    t = ((60409 - 51544) * 86400 + 43201) * 512_000_000 + 12345  # 2024y100d12h00m01s and a bit
    msg = bytes([2, 1, 1, 0]) + struct.pack("<q4q", t, 10, 20, 30, 40)
    assert run.tsys_record(msg) == bytes([2, 1, 1, 0]) + struct.pack("<II4Q", 60409, 43201, 10, 20, 30, 40)
    msg = bytes([0, 3, 0, 1]) + struct.pack("<qqi", t, 2 * 512_000_000, 3) + struct.pack("<3i", -5, 0, 7)
    assert run.phasecal_record(msg) == bytes([0, 3, 0, 1]) + struct.pack("<IIII3i", 60409, 43201, 2, 3, -5, 0, 7)
