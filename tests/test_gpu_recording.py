"""The input-node front end on station recordings: VDIF (16 channels x 2 bits
per 32-bit word, one thread) and Mark5B (32 bitstreams) recordings of a job's
stations go through the reader, the channel extractor (GPU) and the
input-node writer.  The channel blocks, the protocol bytes and the correlator
output must equal those of the same job built from the channel streams
directly (Input_data_format_reader_tasklet -> Channel_extractor_tasklet ->
Input_node_data_writer, sfxc/src/input_data_format_reader_tasklet.cc:93-160,
sfxc/src/channel_extractor_tasklet.cc:120-220,
sfxc/src/input_node_data_writer.cc:107-229).  A VDIF frame marked invalid
becomes the same invalid run in both paths."""
import hashlib
import json
import os

import numpy as np
import pytest

import format_cases

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "formats.json")))

TRACKS16 = [[2 * c + 1, 2 * c] for c in range(16)]


def _job_and_streams(invalid):
    from sfxc_gpu import correlator, scenario
    st = scenario.cubic_stations(3, seed=91, max_delay=4e-3, max_rate=1e-6)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
                           channel_freq=1_600_000_000, nchan=512, integration_us=31250, n_integrations=1,
                           sub_integration_us=31250, lead_us=8000, seed=21, block_bytes=invalid["block_bytes"],
                           invalid=invalid["runs"](st))
    job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol, fast_random=True)
    chans, nsamp = scenario.channel_streams(sc, fast_random=True)
    return sc, job, chans, nsamp


def _words(chans, si, nsamp, seed):
    """16-channel words of station si: channels 0/1 its R/L streams, the rest noise."""
    from sfxc_gpu import synth
    rng = np.random.Generator(np.random.PCG64(seed))
    codes = [synth.unpack_codes(chans[(si, "R")], 2), synth.unpack_codes(chans[(si, "L")], 2)]
    codes += [rng.integers(0, 4, nsamp, dtype=np.uint8) for _ in range(14)]
    return synth.vdif_words_from_codes(codes, 2)


def _protocols_from_recordings(gpu_node, sc, recs, fmt, reader_params):
    from sfxc_gpu import correlator, scenario, timebase
    dels = scenario.del_tables(sc)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    protos = []
    for si in range(len(sc.stations)):
        blocks = correlator.read_recording(recs[si], fmt, ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0),
                                           channel_tracks=TRACKS16, **reader_params)
        per_pol = {"R": [], "L": []}
        for b in blocks:
            (r, l), inv = gpu_node.extract_block(b, 4, 2, [TRACKS16[0], TRACKS16[1]])
            per_pol["R"].append((b["start_ticks"], r, inv))
            per_pol["L"].append((b["start_ticks"], l, inv))
        slices = [(start, start + tint, slice_samples, correlator.delay_list(dels[si], start, start + tint,
                                                                              sc.sample_rate, sc.bits))]
        for pol in sc.pols:
            # the direct path's blocks, for the block-level comparison
            direct = scenario.blocks_of(sc, scenario.channel_streams(sc, fast_random=True)[0][(si, pol)], (si, pol))
            got = per_pol[pol][:len(direct)]
            assert [(t, d, list(map(tuple, inv))) for t, d, inv in got] == \
                [(t, d, list(map(tuple, inv))) for t, d, inv in direct], (si, pol)
            protos.append(correlator.write_protocol(per_pol[pol], slices, sc.sample_rate, sc.bits,
                                                    sc.integration_us))
    return protos


def test_vdif_recording_path(gpu_node):
    from sfxc_gpu import synth
    # frame 5 of station 1 invalid: block 1 (frames 4-7), frame 1 of it ->
    # channel bytes [500, 1000) of that block
    sc, job, chans, nsamp = _job_and_streams(dict(
        block_bytes=2000, runs=lambda st: {(st[1].number, "R"): [(1, 500, 500)], (st[1].number, "L"): [(1, 500, 500)]}))
    recs = [synth.vdif_file_bytes(_words(chans, si, nsamp, 300 + si), payload_bytes=8000, sample_rate=sc.sample_rate,
                                  nchan=16, bits=2, start_mjd=sc.mjd, start_sec_of_day=sc.sec0,
                                  invalid_frames=(5,) if si == 1 else ())
            for si in range(len(sc.stations))]
    protos = _protocols_from_recordings(gpu_node, sc, recs, "vdif",
                                        dict(track_bit_rate=sc.sample_rate, frame_size=8000, n_tracks=32, bits=2))
    assert protos == job["protocols"]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_rec, tsys_rec = gpu_node.correlate(dict(job, protocols=protos))
    assert cor_rec == cor_direct and tsys_rec == tsys_direct


def test_mark5b_recording_path(gpu_node):
    from sfxc_gpu import synth
    sc, job, chans, nsamp = _job_and_streams(dict(block_bytes=5000, runs=lambda st: {}))
    fps = sc.sample_rate * 32 // 80000  # one sample of every channel per 32-bit word
    recs = []
    for si in range(len(sc.stations)):
        w = _words(chans, si, nsamp, 400 + si)
        recs.append(synth.mark5b_recording(w.size // 2500, mjd=sc.mjd, sec_of_day=sc.sec0, frames_per_second=fps,
                                           crc="valid", payload_words=w))
    protos = _protocols_from_recordings(gpu_node, sc, recs, "mark5b",
                                        dict(track_bit_rate=sc.sample_rate, n_tracks=32, bits=2))
    assert protos == job["protocols"]


def test_vdif_thread_per_channel_path(gpu_node):
    """VDIF with one thread per channel (threads 0 and 1: a station's R and L
    streams, frames interleaved): the reader's blocks, one frame each in this
    mode (VDIF_reader::set_parameters, sfxc/src/vdif_reader.cc:211-218), go to
    their channels unextracted (Channel_extractor_tasklet_VDIF), and the
    protocol bytes and correlation equal the direct job's.  Frame 5 of thread 1
    of station 1 is invalid: the whole of block 5 of its L stream."""
    from sfxc_gpu import correlator, scenario, synth, timebase
    sc, job, chans, nsamp = _job_and_streams(dict(
        block_bytes=8000, runs=lambda st: {(st[1].number, "L"): [(5, 0, 8000)]}))
    dels = scenario.del_tables(sc)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    frame = 32 + 8000
    protos = []
    for si in range(len(sc.stations)):
        per_thread = []
        for th, pol in enumerate(("R", "L")):
            words = np.frombuffer(bytes(chans[(si, pol)]), dtype=np.uint32)
            per_thread.append(synth.vdif_file_bytes(words, payload_bytes=8000, sample_rate=sc.sample_rate, nchan=1,
                                                    bits=2, start_mjd=sc.mjd, start_sec_of_day=sc.sec0,
                                                    thread_id=th,
                                                    invalid_frames=(5,) if (si == 1 and pol == "L") else ()))
        nf = min(len(t) for t in per_thread) // frame
        rec = b"".join(per_thread[th][f * frame:(f + 1) * frame] for f in range(nf) for th in range(2))
        blocks = correlator.read_recording(rec, "vdif", ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0),
                                           track_bit_rate=sc.sample_rate, frame_size=8000, n_tracks=0, bits=2,
                                           channel_tracks=[[0, 1], [1, 0]])
        per_chan = correlator.thread_channel_blocks(blocks, 2)
        slices = [(start, start + tint, slice_samples, correlator.delay_list(dels[si], start, start + tint,
                                                                              sc.sample_rate, sc.bits))]
        for c, pol in enumerate(sc.pols):
            direct = scenario.blocks_of(sc, chans[(si, pol)], (si, pol))
            got = per_chan[c][:len(direct)]
            assert [(t, bytes(d), list(map(tuple, inv))) for t, d, inv in got] == \
                [(t, bytes(d), list(map(tuple, inv))) for t, d, inv in direct], (si, pol)
            protos.append(correlator.write_protocol(per_chan[c], slices, sc.sample_rate, sc.bits, sc.integration_us))
    assert protos == job["protocols"]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_rec, tsys_rec = gpu_node.correlate(dict(job, protocols=protos))
    assert cor_rec == cor_direct and tsys_rec == tsys_direct


# ---- the same paths with the recording kept on the device
# (sfxc_gpu_recording_*: headers decoded, fill runs found, channels
# extracted and protocol bytes assembled by kernels)

def _summary(blocks):
    return [{"channel": b["channel"], "start_ticks": b["start_ticks"], "size": len(b["data"]),
             "sha256": hashlib.sha256(b["data"]).hexdigest(), "invalid": [list(r) for r in b["invalid"]]}
            for b in blocks]


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_device_reader_matches_reference_blocks(name, gpu_node):
    """Every block of the reference readers on the format fixtures (misaligned
    first frames, invalid and fill frames, gaps, unknown threads, legacy
    headers, CRC failures, lost sync, garbage, fill runs, day roll-over, VLBA
    time stamps, truncation), from the device-resident recording."""
    from sfxc_gpu import correlator
    c = format_cases.cases()[name]
    rec = correlator.DeviceRecording(gpu_node, c["rec"], c["fmt"], **c["params"])
    assert _summary(rec.blocks()) == GOLDEN[name]["blocks"]
    rec.close()


def test_device_reader_in_place(gpu_node):
    """A recording already in device memory is read where it lies."""
    import torch
    from sfxc_gpu import correlator
    c = format_cases.cases()["mark5b_zero_crc_fill"]
    t = torch.frombuffer(bytearray(c["rec"]), dtype=torch.uint8).cuda()
    rec = correlator.DeviceRecording(gpu_node, t, c["fmt"], **c["params"])
    assert _summary(rec.blocks()) == GOLDEN["mark5b_zero_crc_fill"]["blocks"]
    rec.close()


@pytest.mark.parametrize("bits,tracks", [
    (2, TRACKS16),                                            # 16 subbands of 2 tracks (sign, magnitude)
    (1, [[k] for k in range(32)]),                            # 32 one-bit subbands
    (2, [[4 * c + 1, 4 * c, 4 * c + 3, 4 * c + 2] for c in range(8)]),  # fan-out 4
    (1, [[8 * c + t for t in range(8)] for c in range(4)]),   # fan-out 8
    (2, [[2 * c, 2 * c + 1] for c in range(16)]),             # pairs in the other order (no bit field)
    (2, [[c, c + 16] for c in range(16)]),                    # scattered tracks
])
@pytest.mark.parametrize("case", ["vdif_multichannel", "mark5b_zero_crc_fill"])
def test_device_extraction_matches_block_extractor(gpu_node, bits, tracks, case):
    """Every subband of every block, extracted where the frames lie (bit-field
    layouts and any other), equals the block extractor's output on the
    reader's blocks (invalid runs included); Mark5B frames are not a multiple
    of four output bytes, and with fan-out 1 an output byte spans two frames."""
    from sfxc_gpu import correlator
    c = format_cases.cases()[case]
    host_blocks = correlator.read_recording(c["rec"], c["fmt"], **c["params"])
    per_block = [gpu_node.extract_block(b, 4, bits, tracks) for b in host_blocks]
    r = correlator.DeviceRecording(gpu_node, c["rec"], c["fmt"], **c["params"])
    r.extract(4, bits, tracks)
    for sb in range(len(tracks)):
        assert r.channel(sb) == [(b["start_ticks"], outs[sb], inv) for b, (outs, inv) in zip(host_blocks, per_block)]
    r.close()


def _device_protocols(gpu_node, sc, recs, fmt, reader_params, chans=None):
    """Per station: the device recording, its subbands R/L (channels 0, 1 of
    the 16-channel words) compared block by block with the direct path, and
    their protocols for the job's slice."""
    from sfxc_gpu import correlator, scenario, timebase
    dels = scenario.del_tables(sc)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    protos, objs = [], []
    for si in range(len(sc.stations)):
        r = correlator.DeviceRecording(gpu_node, recs[si], fmt, ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0),
                                       channel_tracks=TRACKS16, **reader_params)
        r.extract(4, 2, [TRACKS16[0], TRACKS16[1]])
        slices = [(start, start + tint, slice_samples, correlator.delay_list(dels[si], start, start + tint,
                                                                              sc.sample_rate, sc.bits))]
        for c, pol in enumerate(sc.pols):
            direct = scenario.blocks_of(sc, scenario.channel_streams(sc, fast_random=True)[0][(si, pol)], (si, pol))
            got = r.channel(c)[:len(direct)]
            assert [(t, bytes(d), list(map(tuple, inv))) for t, d, inv in got] == \
                [(t, bytes(d), list(map(tuple, inv))) for t, d, inv in direct], (si, pol)
            protos.append(r.protocol(c, slices, sc.sample_rate, sc.bits, sc.integration_us))
        objs.append(r)
    return protos, objs


def _correlate_pushed(node, job, objs, per_station):
    """The job's single integration with every stream pushed device to device."""
    node.set_parameters(job)
    for k in range(len(job["streams"])):
        objs[k // per_station].push(k % per_station, 0, node, k)
    o, t = node.run_integration()
    return bytes(o), b"".join(t)


def test_vdif_recording_device_path(gpu_node):
    from sfxc_gpu import synth
    sc, job, chans, nsamp = _job_and_streams(dict(
        block_bytes=2000, runs=lambda st: {(st[1].number, "R"): [(1, 500, 500)], (st[1].number, "L"): [(1, 500, 500)]}))
    recs = [synth.vdif_file_bytes(_words(chans, si, nsamp, 300 + si), payload_bytes=8000, sample_rate=sc.sample_rate,
                                  nchan=16, bits=2, start_mjd=sc.mjd, start_sec_of_day=sc.sec0,
                                  invalid_frames=(5,) if si == 1 else ())
            for si in range(len(sc.stations))]
    protos, objs = _device_protocols(gpu_node, sc, recs, "vdif",
                                     dict(track_bit_rate=sc.sample_rate, frame_size=8000, n_tracks=32, bits=2))
    # the same bytes as the input-node writer's (SHA-equal per slice)
    assert [[hashlib.sha256(x).hexdigest() for x in p] for p in protos] == \
        [[hashlib.sha256(bytes(x)).hexdigest() for x in p] for p in job["protocols"]]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_dev, tsys_dev = _correlate_pushed(gpu_node, job, objs, len(sc.pols))
    assert cor_dev == cor_direct and tsys_dev == tsys_direct


def test_mark5b_recording_device_path(gpu_node):
    from sfxc_gpu import synth
    sc, job, chans, nsamp = _job_and_streams(dict(block_bytes=5000, runs=lambda st: {}))
    fps = sc.sample_rate * 32 // 80000
    recs = []
    for si in range(len(sc.stations)):
        w = _words(chans, si, nsamp, 400 + si)
        recs.append(synth.mark5b_recording(w.size // 2500, mjd=sc.mjd, sec_of_day=sc.sec0, frames_per_second=fps,
                                           crc="valid", payload_words=w))
    protos, objs = _device_protocols(gpu_node, sc, recs, "mark5b", dict(track_bit_rate=sc.sample_rate, n_tracks=32,
                                                                         bits=2))
    assert protos == [[bytes(x) for x in p] for p in job["protocols"]]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_dev, tsys_dev = _correlate_pushed(gpu_node, job, objs, len(sc.pols))
    assert cor_dev == cor_direct and tsys_dev == tsys_direct


def test_vdif_thread_per_channel_device_path(gpu_node):
    from sfxc_gpu import correlator, scenario, synth, timebase
    sc, job, chans, nsamp = _job_and_streams(dict(
        block_bytes=8000, runs=lambda st: {(st[1].number, "L"): [(5, 0, 8000)]}))
    dels = scenario.del_tables(sc)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    frame = 32 + 8000
    protos, objs = [], []
    for si in range(len(sc.stations)):
        per_thread = []
        for th, pol in enumerate(("R", "L")):
            words = np.frombuffer(bytes(chans[(si, pol)]), dtype=np.uint32)
            per_thread.append(synth.vdif_file_bytes(words, payload_bytes=8000, sample_rate=sc.sample_rate, nchan=1,
                                                    bits=2, start_mjd=sc.mjd, start_sec_of_day=sc.sec0,
                                                    thread_id=th,
                                                    invalid_frames=(5,) if (si == 1 and pol == "L") else ()))
        nf = min(len(t) for t in per_thread) // frame
        rec = b"".join(per_thread[th][f * frame:(f + 1) * frame] for f in range(nf) for th in range(2))
        r = correlator.DeviceRecording(gpu_node, rec, "vdif", ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0),
                                       track_bit_rate=sc.sample_rate, frame_size=8000, n_tracks=0, bits=2,
                                       channel_tracks=[[0, 1], [1, 0]])
        r.extract_threads(2)
        slices = [(start, start + tint, slice_samples, correlator.delay_list(dels[si], start, start + tint,
                                                                              sc.sample_rate, sc.bits))]
        for c, pol in enumerate(sc.pols):
            direct = scenario.blocks_of(sc, chans[(si, pol)], (si, pol))
            got = r.channel(c)[:len(direct)]
            assert [(t, bytes(d), list(map(tuple, inv))) for t, d, inv in got] == \
                [(t, bytes(d), list(map(tuple, inv))) for t, d, inv in direct], (si, pol)
            protos.append(r.protocol(c, slices, sc.sample_rate, sc.bits, sc.integration_us))
        objs.append(r)
    assert protos == [[bytes(x) for x in p] for p in job["protocols"]]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_dev, tsys_dev = _correlate_pushed(gpu_node, job, objs, len(sc.pols))
    assert cor_dev == cor_direct and tsys_dev == tsys_direct


def test_device_recording_errors(gpu_node):
    """Bad parameters and calls out of order fail with a status, no device work."""
    from sfxc_gpu import correlator, lib
    c = format_cases.cases()["vdif_legacy"]
    with pytest.raises(lib.SfxcError):
        correlator.DeviceRecording(gpu_node, c["rec"], "vdif", **dict(c["params"], frame_size=0))
    r = correlator.DeviceRecording(gpu_node, c["rec"], "vdif", **c["params"])
    with pytest.raises(lib.SfxcError):  # no channels extracted yet
        r.channel(0)
    with pytest.raises(lib.SfxcError):  # 8000-byte frames are not whole 3-byte words
        r.extract(3, 2, [[1, 0]])
    r.close()


# ---- the reader tasklet's scheduling (gap filling) on the device recording
SCHEDULE = json.load(open(os.path.join(HERE, "golden", "schedule.json")))


@pytest.mark.parametrize("key", sorted(SCHEDULE))
def test_device_schedule_matches_reference_tasklet(key, gpu_node):
    """The blocks the reference's reader tasklet pushes for the fixture
    recordings and time intervals (filled-in blocks for missing frames, data
    ending or starting inside an interval, skips, leave times, failed reads,
    skewed and shared VDIF threads), from the device recording.  Bytes the
    reference's run leaves to its consumer's timing ("shared") or to a failed
    read ("stale": wholly invalid here) are compared as the CPU test does."""
    from sfxc_gpu import correlator
    name = key.split("/")[0]
    c = dict(format_cases.cases(), **format_cases.schedule_recordings())[name]
    g = SCHEDULE[key]
    r = correlator.DeviceRecording(gpu_node, c["rec"], c["fmt"], **c["params"])
    r.schedule([tuple(v) for v in g["intervals"]])
    got = []
    for b in r.blocks():
        whole = any(x == 0 and n >= len(b["data"]) for x, n in b["invalid"])
        got.append({"channel": b["channel"], "start_ticks": b["start_ticks"], "size": len(b["data"]),
                    "sha256": None if whole else hashlib.sha256(b["data"]).hexdigest(),
                    "invalid": [list(x) for x in b["invalid"]]})
    r.close()
    size = g["blocks"][0]["size"] if g["blocks"] else 0
    want = []
    for i, b in enumerate(g["blocks"]):
        if b["sha256"] == "shared":
            b = dict(b, sha256=got[i]["sha256"] if i < len(got) and got[i]["sha256"] is not None else "own")
        elif b["sha256"] == "stale":
            b = dict(b, sha256=None, invalid=[[0, size]])
        want.append(b)
    assert got == want


def test_vdif_dropped_block_filled_on_device(gpu_node):
    """Station 1's recording loses a whole block of frames (block 2, frames
    8-11): the device front end's reader tasklet fills it in, and the
    protocols and correlation equal the job whose block 2 of station 1 is
    invalid."""
    from sfxc_gpu import correlator, scenario, synth, timebase
    runs = lambda st: {(st[1].number, "R"): [(2, 0, 2000)], (st[1].number, "L"): [(2, 0, 2000)]}  # noqa: E731
    sc, job, chans, nsamp = _job_and_streams(dict(block_bytes=2000, runs=runs))
    frame = 32 + 8000
    recs = []
    for si in range(len(sc.stations)):
        rec = synth.vdif_file_bytes(_words(chans, si, nsamp, 300 + si), payload_bytes=8000, sample_rate=sc.sample_rate,
                                    nchan=16, bits=2, start_mjd=sc.mjd, start_sec_of_day=sc.sec0)
        if si == 1:
            rec = rec[:8 * frame] + rec[12 * frame:]
        recs.append(rec)
    nblocks = len(recs[0]) // frame // 4
    rec0 = timebase.ticks_from_mjd_sec(sc.mjd, sc.sec0)
    tbh = 128000  # 4 frames of 2000 samples per channel at 32 Ms/s
    dels = scenario.del_tables(sc)
    _, start, tint, slice_samples = scenario.job_timing(sc)
    protos, objs = [], []
    for si in range(len(sc.stations)):
        r = correlator.DeviceRecording(gpu_node, recs[si], "vdif", ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0),
                                       track_bit_rate=sc.sample_rate, frame_size=8000, n_tracks=32, bits=2,
                                       channel_tracks=TRACKS16)
        r.schedule([(rec0, rec0 + nblocks * tbh, rec0 + nblocks * tbh)])
        assert r.n_blocks() == nblocks
        r.extract(4, 2, [TRACKS16[0], TRACKS16[1]])
        slices = [(start, start + tint, slice_samples, correlator.delay_list(dels[si], start, start + tint,
                                                                              sc.sample_rate, sc.bits))]
        for c, pol in enumerate(sc.pols):
            protos.append(r.protocol(c, slices, sc.sample_rate, sc.bits, sc.integration_us))
        objs.append(r)
    assert protos == [[bytes(x) for x in p] for p in job["protocols"]]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_dev, tsys_dev = _correlate_pushed(gpu_node, job, objs, len(sc.pols))
    assert cor_dev == cor_direct and tsys_dev == tsys_direct


def test_mark5b_dropped_block_filled_on_device(gpu_node):
    """Station 2's Mark5B recording loses block 1 (frames 8-15): the device
    front end's reader tasklet fills it in, and the protocols and correlation
    equal the job whose block 1 of station 2 is invalid."""
    from sfxc_gpu import correlator, scenario, synth, timebase
    runs = lambda st: {(st[2].number, "R"): [(1, 0, 5000)], (st[2].number, "L"): [(1, 0, 5000)]}  # noqa: E731
    sc, job, chans, nsamp = _job_and_streams(dict(block_bytes=5000, runs=runs))
    fps = sc.sample_rate * 32 // 80000
    frame = 16 + 10000
    recs = []
    for si in range(len(sc.stations)):
        w = _words(chans, si, nsamp, 400 + si)
        rec = synth.mark5b_recording(w.size // 2500, mjd=sc.mjd, sec_of_day=sc.sec0, frames_per_second=fps,
                                     crc="valid", payload_words=w)
        if si == 2:
            rec = rec[:8 * frame] + rec[16 * frame:]
        recs.append(rec)
    nblocks = len(recs[0]) // frame // 8
    rec0 = timebase.ticks_from_mjd_sec(sc.mjd, sc.sec0)
    tbh = 320000  # 8 frames of 10000 bytes at 32 bitstreams x 32 Mb/s: 625 us
    dels = scenario.del_tables(sc)
    _, start, tint, slice_samples = scenario.job_timing(sc)
    protos, objs = [], []
    for si in range(len(sc.stations)):
        r = correlator.DeviceRecording(gpu_node, recs[si], "mark5b", ref_ticks=timebase.ticks_from_mjd_sec(sc.mjd, 0.0),
                                       track_bit_rate=sc.sample_rate, n_tracks=32, bits=2, channel_tracks=TRACKS16)
        r.schedule([(rec0, rec0 + nblocks * tbh, rec0 + nblocks * tbh)])
        assert r.n_blocks() == nblocks
        r.extract(4, 2, [TRACKS16[0], TRACKS16[1]])
        slices = [(start, start + tint, slice_samples, correlator.delay_list(dels[si], start, start + tint,
                                                                              sc.sample_rate, sc.bits))]
        for c, pol in enumerate(sc.pols):
            protos.append(r.protocol(c, slices, sc.sample_rate, sc.bits, sc.integration_us))
        objs.append(r)
    assert protos == [[bytes(x) for x in p] for p in job["protocols"]]
    cor_direct, tsys_direct = gpu_node.correlate(job)
    cor_dev, tsys_dev = _correlate_pushed(gpu_node, job, objs, len(sc.pols))
    assert cor_dev == cor_direct and tsys_dev == tsys_direct
