"""Correlation set-up from a control file and a VEX file (sfxc_gpu_control_*)
against the reference's own Control_parameters and its manager's dealing of
the jobs (tests/golden/control.json.gz, from oracle/ref_harness.cc mode
`control`): the global header, output files, per scan the stations' delay
tables, clock models and reader parameters (track lists), the channel
numbering, and every job's Correlation_parameters in output slice order.
Host only."""
import gzip
import json
import os

import pytest

import control_cases
from sfxc_gpu import control, lib as L

pytestmark = pytest.mark.usefixtures("sfxc_lib")

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "control.json.gz")


def _golden():
    with gzip.open(GOLDEN, "rt") as f:
        return json.load(f)


def _plan(case, d):
    ctrl, vex = control_cases.write_case(case, d)
    times = {(s, sc): t for s, sc, t in control_cases.station_times(case)}
    old = os.getcwd()
    os.chdir(d)  # relative paths of the control file are taken from the working directory, as the reference does
    try:
        p = control.plan(ctrl, vex, (lambda s, sc: times.get((s, sc), 0)) if times else None)
    finally:
        os.chdir(old)
    return p


CASES = control_cases.cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_plan_matches_reference(name, tmp_path):
    want = _golden()[name]
    d = str(tmp_path / name)
    if want is None:
        with pytest.raises(L.SfxcError):
            _plan(CASES[name], d)
        return
    got = _plan(CASES[name], d)
    ctrl = got.pop("ctrl")
    got = json.loads(json.dumps(got).replace(d, "<dir>"))
    assert set(got) == set(want)
    assert got["header"] == want["header"]
    assert got["output_files"] == want["output_files"] and got["sources"] == want["sources"]
    assert got["scans"] == want["scans"]
    assert len(got["jobs"]) == len(want["jobs"])
    for k, (g, w) in enumerate(zip(got["jobs"], want["jobs"])):
        assert g == w, "job %d" % k
    assert got.get("pulsars") == want.get("pulsars")
    assert got.get("mask") == want.get("mask")
    assert ctrl["stations"] == CASES[name]["ctrl"]["stations"]


def test_plan_covers_the_set_ups():
    """The fixture exercises what it claims: every reader format, thread
    layouts, cross polarisations, late data, clock rates, phase centres."""
    g = _golden()
    fmts = {s["input"]["data_format"] for p in g.values() if p for sc in p["scans"] for s in sc["stations"]}
    assert fmts == {"VDIF", "Mark5B", "Mark4"}
    thr = g["vdif_threads"]["scans"][0]["stations"]
    assert {s["name"]: s["input"]["n_tracks"] for s in thr} == {"Ef": 0, "Wb": 16}
    assert any(j["cross_channel"] >= 0 for j in g["cross_pol"]["jobs"])
    assert any(s["station_stream"] >= 3 for j in g["cross_pol"]["jobs"] for s in j["stations"])
    assert g["multi_phase_center"]["sources"] == ["SRC1", "SRC2", "SRC3"]
    assert g["pulsar"]["output_files"][-1].endswith(".bin16")
    rates = {s["clock_rate"] for sc in g["clocks"]["scans"] for s in sc["stations"]}
    assert len(rates) >= 3 and any(s["reader_offset"] != 0 for sc in g["clocks"]["scans"] for s in sc["stations"])
    sc = g["scans"]["scans"]
    assert [s["name"] for s in sc] == ["No0003", "No0004", "No0007"]
    assert sc[0]["first_slice_start"] > g["scans"]["start"]


def test_refused_and_malformed(tmp_path):
    case = dict(CASES["vdif_multichannel"])
    d = str(tmp_path / "bad")
    ctrl, vex = control_cases.write_case(case, d)
    with open(vex, "a") as f:
        f.write("$BROKEN;\ndef x;\n  a = b\nenddef;\n")  # a statement without its ';'
    with pytest.raises(L.SfxcError, match="vex: syntax error"):
        control.plan(ctrl, vex)
    with open(ctrl, "w") as f:
        f.write('{"stations": ["Ef",]')
    with pytest.raises(L.SfxcError, match="ctrl file"):
        control.plan(ctrl, vex)
    with pytest.raises(L.SfxcError, match="could not open"):
        control.plan(os.path.join(d, "missing.ctrl"), vex)


REF = os.environ.get("REF_ROOT") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
REF_VEX = [("sfxc/lib/vex_parser/vex_parser/test/n06c2.vex", "N06C2", ["Ef", "Wb", "Jb", "On", "Mc", "Tr"],
            "2006y168d06h30m00s", "2006y168d06h31m10s"),
           ("sfxc/lib/vex_parser/vex_parser/test/n07c2.vex", "N07C2", ["Wb", "Jb", "On", "Mc"],
            "2007y152d10h44m00s", "2007y152d10h46m00s"),
           ("sfxc/webservices/vex2ccf_web_service/f07c2.vex", "F07C2", ["Cm", "Wb", "Mc", "On"],
            "2007y151d11h00m00s", "2007y151d11h00m40s")]


@pytest.mark.parametrize("vex,exper,stations,start,stop", REF_VEX)
@pytest.mark.parametrize("cross", [False, True])
def test_reference_vex_files(vex, exper, stations, start, stop, cross, tmp_path):
    """The VEX files the reference ships (Mark4 schedules of EVN
    experiments), read by both sides when the reference checkout is here."""
    path = os.path.join(REF, vex)
    if not os.path.exists(path):
        pytest.skip("reference checkout not available")
    from oracle import jobs
    d = str(tmp_path)
    os.makedirs(os.path.join(d, "delays"))
    for s in stations:
        open(os.path.join(d, "delays", "%s_%s.del" % (exper, s)), "w").close()
    ctrl = os.path.join(d, "c.ctrl")
    json.dump({"stations": stations, "start": start, "stop": stop, "integr_time": 4.0, "number_channels": 256,
               "output_file": "file://x.cor", "delay_directory": "file://delays", "cross_polarize": cross,
               "data_sources": {s: ["file://a"] for s in stations}}, open(ctrl, "w"))
    want = jobs.control(ctrl, path, d)
    assert want is not None
    old = os.getcwd()
    os.chdir(d)
    try:
        got = control.plan(ctrl, path)
    finally:
        os.chdir(old)
    got.pop("ctrl")
    assert got == want
