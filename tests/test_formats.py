"""VDIF and Mark5B readers (the library's host-side restatement of the
reference's VDIF_reader / Mark5b_reader) against the blocks the reference's
own readers produce: channel, start time, payload bytes and invalid runs of
every block, on recordings with misaligned first frames, invalid and fill
frames, gaps, unknown threads, legacy headers, CRC failures, lost sync,
garbage, fill-pattern runs, day roll-over, VLBA time stamps and truncation.
No GPU needed (the readers are host code behind the C ABI)."""
import hashlib
import json
import os
import subprocess

import pytest

import format_cases

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "sfxc-1_gb300", "csrc")
GOLDEN = json.load(open(os.path.join(HERE, "golden", "formats.json")))
CASES = format_cases.cases()


def _summary(blocks):
    return [{"channel": b["channel"], "start_ticks": b["start_ticks"], "size": len(b["data"]),
             "sha256": hashlib.sha256(b["data"]).hexdigest(), "invalid": [list(r) for r in b["invalid"]]}
            for b in blocks]


@pytest.mark.parametrize("name", sorted(CASES))
def test_reader_matches_reference_blocks(name, sfxc_lib):
    from sfxc_gpu import correlator
    c = CASES[name]
    g = GOLDEN[name]
    assert hashlib.sha256(c["rec"]).hexdigest() == g["recording_sha256"], "recording generator changed"
    got = correlator.read_recording(c["rec"], c["fmt"], **c["params"])
    assert _summary(got) == g["blocks"]


def test_fixtures_exercise_every_rule():
    """The fixtures cover invalid frames, fill runs, several VDIF channels and
    VLBA-time-stamp fallback (times not on the frame-number grid)."""
    inv = {n: sum(len(b["invalid"]) for b in g["blocks"]) for n, g in GOLDEN.items()}
    assert inv["vdif_multichannel"] >= 2 and inv["vdif_threads"] >= 2 and inv["mark5b_zero_crc_fill"] >= 3
    assert len({b["channel"] for b in GOLDEN["vdif_threads"]["blocks"]}) == 4
    assert all(len(g["blocks"]) > 0 for g in GOLDEN.values())


def test_reader_live_against_reference(sfxc_lib):
    """Where the reference checkout is present, its readers run on the same
    recordings in this process's host (the fixtures pin the rest)."""
    from oracle import build_ref, jobs
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")
    from sfxc_gpu import correlator
    for name, c in CASES.items():
        ref = jobs.reader(c["rec"], c["fmt"], **c["params"])
        got = correlator.read_recording(c["rec"], c["fmt"], **c["params"])
        assert got == ref, name


def test_reader_rejects_bad_parameters(sfxc_lib):
    from sfxc_gpu import correlator, lib
    c = CASES["vdif_legacy"]
    bad = dict(c["params"], bits=3)
    with pytest.raises(lib.SfxcError):
        correlator.read_recording(c["rec"], "vdif", **bad)
    bad = dict(c["params"], frame_size=0)
    with pytest.raises(lib.SfxcError):
        correlator.read_recording(c["rec"], "vdif", **bad)
    mk = dict(CASES["mark5b_day_rollover"]["params"], track_bit_rate=32_500_000)
    with pytest.raises(lib.SfxcError):
        correlator.read_recording(CASES["mark5b_day_rollover"]["rec"], "mark5b", **mk)
    assert correlator.read_recording(b"", "vdif", **c["params"]) == []


@pytest.fixture(scope="module")
def walk_driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("walk") / "walk_driver")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + CSRC, os.path.join(HERE, "walk_driver.cc"),
                    os.path.join(CSRC, "formats.cpp"), "-o", exe], check=True)
    return exe


def walk_blocks(exe, tmp_path, c, intervals=()):
    """Blocks of the frame walker (walk_frames over headers decoded by the
    device decode's functions, bytes assembled from the frame offsets), or
    with time intervals the blocks the reader tasklet pushes (data None for a
    wholly invalid block)."""
    rec = tmp_path / "rec"
    rec.write_bytes(bytes(c["rec"]))
    pr = c["params"]
    ct = pr["channel_tracks"]
    args = [exe, str(rec), str(tmp_path / "out"), "0" if c["fmt"] == "vdif" else "1", str(pr["ref_ticks"]),
            str(pr.get("offset_ticks", 0)), str(pr["track_bit_rate"]), str(pr.get("frame_size", 0)),
            str(pr["n_tracks"]), str(pr["bits"]), str(len(ct[0])), str(len(intervals))]
    args += [str(v) for iv in intervals for v in iv] + [str(t[0]) for t in ct]
    lines = subprocess.run(args, capture_output=True, text=True, check=True).stdout.split("\n")
    data = (tmp_path / "out").read_bytes()
    blocks, off = [], 0
    for line in filter(None, lines):
        v = list(map(int, line.split()))
        ch, start, size, nr = v[:4]
        inv = [(v[4 + 2 * i], v[5 + 2 * i]) for i in range(nr)]
        whole = bool(intervals) and any(b == 0 and n >= size for b, n in inv)
        blocks.append({"channel": ch, "start_ticks": start, "size": size, "invalid": inv,
                       "data": None if whole else data[off:off + size]})
        if not whole:
            off += size
    return blocks


@pytest.mark.parametrize("name", sorted(CASES))
def test_frame_walk_matches_reference_blocks(name, walk_driver, tmp_path):
    """The readers restated on decoded frame headers (the block decisions of
    the device-resident recording path) give the reference readers' blocks."""
    c = CASES[name]
    assert _summary(walk_blocks(walk_driver, tmp_path, c)) == GOLDEN[name]["blocks"]


SCHEDULE = json.load(open(os.path.join(HERE, "golden", "schedule.json")))
SCHED_RECS = dict(CASES, **format_cases.schedule_recordings())


def _sched_summary(blocks):
    return [{"channel": b["channel"], "start_ticks": b["start_ticks"], "size": b["size"],
             "sha256": None if b["data"] is None else hashlib.sha256(b["data"]).hexdigest(),
             "invalid": [list(r) for r in b["invalid"]]} for b in blocks]


@pytest.mark.parametrize("key", sorted(SCHEDULE))
def test_reader_tasklet_matches_reference(key, walk_driver, tmp_path):
    """The reader tasklet's time-interval scheduling over the walk (missing
    frames, data ending or starting inside an interval, skipping ahead, leave
    times, a read failing without the data ending, skewed and shared VDIF
    threads) pushes the blocks the reference's tasklet pushes, wholly invalid
    blocks where it fills in."""
    name = key.split("/")[0]
    c = SCHED_RECS[name]
    g = SCHEDULE[key]
    assert hashlib.sha256(c["rec"]).hexdigest() == g["recording_sha256"], "recording generator changed"
    got = _sched_summary(walk_blocks(walk_driver, tmp_path, c, [tuple(v) for v in g["intervals"]]))
    # the reference's bytes of a block pushed in a data buffer that a later
    # block reuses depend on whether its consumer took it first: every field
    # but those bytes is compared there.  A block whose buffer holds no
    # block's bytes (a read that failed at the end of the data left part of a
    # frame over older bytes) goes out wholly invalid here: its channel, time
    # and size are compared.
    size = g["blocks"][0]["size"] if g["blocks"] else 0
    want = []
    for i, b in enumerate(g["blocks"]):
        if b["sha256"] == "shared":
            b = dict(b, sha256=got[i]["sha256"] if i < len(got) and got[i]["sha256"] is not None else "own")
        elif b["sha256"] == "stale":
            b = dict(b, sha256=None, invalid=[[0, size]])
        want.append(b)
    assert got == want
