"""Recordings for the format-reader parity tests: seeded VDIF and Mark5B
streams with the irregularities the reference's readers handle (misaligned
first frames, invalid and fill-pattern frames, gaps, unknown VDIF threads,
legacy headers, Mark5B CRC failures, lost sync, garbage between frames,
fill-pattern runs, day roll-over, frame numbers beyond one second, a
truncated file).  Each case gives the recording bytes and the reader
parameters; tests/golden/formats.json holds the blocks the reference's own
readers produce for them (tests/golden/make_golden.py)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "sfxc-1_gb300"))

from sfxc_gpu import synth, timebase  # noqa: E402

MJD = 60123


def _ref_ticks(mjd=MJD):
    return timebase.ticks_from_mjd_sec(mjd, 0.0)


def _vdif_tracks(nchan, bits, n_tracks):
    return [[c * bits + 1, c * bits] if bits == 2 else [c] for c in range(nchan)]


def cases():
    out = {}
    # 16 channels x 2 bits in 32-bit words, 8000-byte payloads, 4 frames per
    # block (32128 // 8000); 64 MS/s per channel
    fps = 64_000_000 * 2 * 16 // (8000 * 8)
    out["vdif_multichannel"] = dict(
        fmt="vdif",
        rec=synth.vdif_recording(44, payload_bytes=8000, frames_per_second=fps, start_mjd=MJD,
                                 start_sec_of_day=3600, log2_nchan=4, bits=2, first_frame=2,
                                 invalid=(6, 11), fill=(17,), drop=(25, 26), seed=1),
        params=dict(ref_ticks=_ref_ticks(), track_bit_rate=64_000_000, frame_size=8000, n_tracks=32, bits=2,
                    channel_tracks=_vdif_tracks(16, 2, 32)))
    fps1 = 32_000_000 * 2 // (8000 * 8)
    out["vdif_legacy"] = dict(
        fmt="vdif",
        rec=synth.vdif_recording(20, payload_bytes=8000, frames_per_second=fps1, start_mjd=MJD,
                                 start_sec_of_day=7200, log2_nchan=0, bits=2, legacy=True, invalid=(9,), seed=2),
        params=dict(ref_ticks=_ref_ticks(), offset_ticks=512 * 1000, track_bit_rate=32_000_000, frame_size=8000,
                    n_tracks=2, bits=2, channel_tracks=[[1, 0]]))
    # one channel per thread: threads 3, 5, 7, 9 -> channels 0..3; thread 11
    # is not in the list (its frames restart the read)
    fpst = 16_000_000 * 2 // (1000 * 8)
    out["vdif_threads"] = dict(
        fmt="vdif",
        rec=synth.vdif_recording(30, payload_bytes=1000, frames_per_second=fpst, start_mjd=MJD,
                                 start_sec_of_day=100, log2_nchan=0, bits=2, threads=(3, 5, 11, 7, 9),
                                 invalid=(4, 12), seed=3),
        params=dict(ref_ticks=_ref_ticks(), track_bit_rate=16_000_000, frame_size=1000, n_tracks=0, bits=2,
                    channel_tracks=[[3, 2], [5, 4], [7, 6], [9, 8]]))
    rec = synth.vdif_recording(12, payload_bytes=8000, frames_per_second=fps, start_mjd=MJD, start_sec_of_day=50,
                               log2_nchan=4, bits=2, fill=(0,), seed=4)
    out["vdif_fill_first_truncated"] = dict(
        fmt="vdif", rec=rec[:len(rec) - 3000],
        params=dict(ref_ticks=_ref_ticks(), track_bit_rate=64_000_000, frame_size=8000, n_tracks=32, bits=2,
                    channel_tracks=_vdif_tracks(16, 2, 32)))
    # Mark5B: 32 bitstreams at 32 Mb/s (12 800 frames/s); 8 frames per block
    mk = dict(track_bit_rate=32_000_000, n_tracks=32, bits=2,
              channel_tracks=[[2 * c + 1, 2 * c] for c in range(16)])
    fpm = 32_000_000 * 32 // (10000 * 8)
    out["mark5b_zero_crc_fill"] = dict(
        fmt="mark5b",
        rec=synth.mark5b_recording(40, mjd=MJD, sec_of_day=1000, frames_per_second=fpm, seed=5,
                                   fill_runs=[(9, 100, 300), (9, 2499, 1), (10, 0, 2500), (11, 0, 50),
                                              (14, 1200, 1300), (15, 0, 2500),   # to the end of block 1
                                              (16, 0, 2500), (17, 0, 1000),      # from the start of block 2
                                              (30, 7, 1), (31, 0, 2500)]),
        params=dict(ref_ticks=_ref_ticks(), **mk))
    out["mark5b_valid_crc_resync"] = dict(
        fmt="mark5b",
        rec=synth.mark5b_recording(56, mjd=MJD, sec_of_day=2000, frames_per_second=fpm, seed=6, crc="valid",
                                   first_frame=3, bad_crc=(13,), bad_sync=(29,), garbage={41: 1234}),
        params=dict(ref_ticks=_ref_ticks(), offset_ticks=-512 * 250, **mk))
    out["mark5b_day_rollover"] = dict(
        fmt="mark5b",
        rec=synth.mark5b_recording(48, mjd=MJD, sec_of_day=86399, frames_per_second=fpm, seed=7,
                                   first_frame=fpm - 16),
        params=dict(ref_ticks=_ref_ticks(), **mk))
    # frame numbers beyond one second at the declared rate: the reader falls
    # back to the header's sub-second field (VLBA time stamps)
    out["mark5b_vlba_time"] = dict(
        fmt="mark5b",
        rec=synth.mark5b_recording(32, mjd=MJD, sec_of_day=500, frames_per_second=4 * fpm, seed=8,
                                   first_frame=3 * fpm),
        params=dict(ref_ticks=_ref_ticks(), **mk))
    return out


def schedule_recordings():
    """Recordings for the reader-tasklet tests besides cases(): a VDIF stream
    with more than 256 fill frames in a row (a read that fails without the
    data ending), and one thread per channel with two channels on one thread
    and a thread that loses frames (skew)."""
    out = {}
    fps = 64_000_000 * 2 * 16 // (8000 * 8)
    out["vdif_long_fill"] = dict(
        fmt="vdif",
        rec=synth.vdif_recording(300, payload_bytes=8000, frames_per_second=fps, start_mjd=MJD, start_sec_of_day=10,
                                 log2_nchan=4, bits=2, fill=tuple(range(8, 8 + 270)), seed=9),
        params=dict(ref_ticks=_ref_ticks(), track_bit_rate=64_000_000, frame_size=8000, n_tracks=32, bits=2,
                    channel_tracks=_vdif_tracks(16, 2, 32)))
    fpst = 16_000_000 * 2 // (1000 * 8)
    out["vdif_threads_skew"] = dict(
        fmt="vdif",
        rec=synth.vdif_recording(60, payload_bytes=1000, frames_per_second=fpst, start_mjd=MJD, start_sec_of_day=200,
                                 log2_nchan=0, bits=2, threads=(1, 2), drop=tuple(range(21, 41, 2)), seed=10),
        params=dict(ref_ticks=_ref_ticks(), track_bit_rate=16_000_000, frame_size=1000, n_tracks=0, bits=2,
                    channel_tracks=[[1, 0], [2, 0], [1, 0]]))
    return out


def schedule_cases(first_ticks, tbh):
    """Time-interval sets (start, stop, leave ticks) of the reader-tasklet
    tests, relative to a recording's first block time and frame spacing:
    data starting inside the interval, a later interval (the reader skips
    ahead), a leave time before the stop, intervals after the data ended and
    before it started."""
    t0, T = first_ticks, tbh
    return {
        "covering": [(t0 - 3 * T, t0 + 40 * T, t0 + 40 * T)],
        "skip_ahead": [(t0 + 2 * T, t0 + 6 * T, t0 + 6 * T), (t0 + 9 * T, t0 + 14 * T, t0 + 14 * T)],
        "leave_early": [(t0, t0 + 12 * T, t0 + 4 * T)],
        "before_and_after": [(t0 - 20 * T, t0 - 16 * T, t0 - 16 * T), (t0 + 1 * T, t0 + 5 * T, t0 + 5 * T),
                             (t0 + 400 * T, t0 + 404 * T, t0 + 404 * T)],
    }


def reader_tbh(c):
    """The reader's time between block headers in ticks (VDIF_reader /
    Mark5b_reader::set_parameters, as Time(usec) rounds it)."""
    p = c["params"]
    sr = p["track_bit_rate"] * (len(p["channel_tracks"][0]) // p["bits"])
    if c["fmt"] == "vdif":
        fs = p["frame_size"]
        us = fs * 8e6 / (sr * p["bits"]) if p["n_tracks"] == 0 else \
            max(1, 32128 // fs) * fs * 8e6 / (sr * p["n_tracks"])
    else:
        us = 80000 / ((4 if p["n_tracks"] <= 32 else 8) * p["track_bit_rate"] // 1000000)
    return round(us * 512)
