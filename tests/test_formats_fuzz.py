"""Corrupted recordings: the library's VDIF and Mark5B readers, and the frame
walk of the device-resident path, against the reference's own readers
(VDIF_reader, sfxc/src/vdif_reader.cc:77-190; Mark5b_reader,
sfxc/src/mark5b_reader.cc:111-252; the fill-pattern search,
sfxc/src/input_data_format_reader.cc:20-72) on seeded random damage to the
eight reader fixtures: header bytes changed, bytes dropped or inserted
(misaligned frames, garbage), frames overwritten with the fill pattern, the
file cut short.  Every block -- channel, start time, bytes and invalid runs
-- must be equal; the one difference allowed is the frame walk's at the end
of a Mark5B file cut inside a resync, where the reference's reader returns
one more block whose tail is left over from its previous block.

Needs the reference checkout (its readers are compiled here); a mutation on
which the reference's reader itself fails or runs past a time limit is not
compared, and at least 90 % of them must be."""
import os
import struct

import numpy as np
import pytest

import format_cases
from test_formats import walk_blocks, walk_driver  # noqa: F401  (fixture)

CASES = format_cases.cases()
PER_CASE = 25
FILL = struct.pack("<I", 0x11223344)


def _frame_size(c):
    return c["params"]["frame_size"] + 32 if c["fmt"] == "vdif" else 10016


def _mutate(c, rng):
    """One random kind of damage to the recording."""
    rec = bytearray(c["rec"])
    fs = _frame_size(c)
    nf = max(1, len(rec) // fs)
    kind = int(rng.integers(0, 5))
    if kind == 0:  # a few header bytes of a few frames
        for _ in range(int(rng.integers(1, 4))):
            f = int(rng.integers(0, nf))
            for _ in range(int(rng.integers(1, 3))):
                pos = f * fs + int(rng.integers(0, 16))
                if pos < len(rec):
                    rec[pos] ^= 1 << int(rng.integers(0, 8))
    elif kind == 1:  # bytes dropped
        pos = int(rng.integers(0, len(rec)))
        del rec[pos:pos + int(rng.integers(1, fs))]
    elif kind == 2:  # garbage inserted
        pos = int(rng.integers(0, len(rec)))
        rec[pos:pos] = rng.integers(0, 256, size=int(rng.integers(1, fs)), dtype=np.uint8).tobytes()
    elif kind == 3:  # whole frames overwritten with the fill pattern
        f = int(rng.integers(0, nf))
        n = int(rng.integers(1, 3))
        rec[f * fs:(f + n) * fs] = FILL * (len(rec[f * fs:(f + n) * fs]) // 4)
    else:  # the file cut short
        del rec[int(rng.integers(len(rec) // 2, len(rec))):]
    return bytes(rec), kind


def _mutations():
    rng = np.random.Generator(np.random.PCG64(20261204))
    out = []
    for name in sorted(CASES):
        for k in range(PER_CASE):
            rec, kind = _mutate(CASES[name], rng)
            out.append((name, k, kind, rec))
    return out


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


def test_readers_match_reference_on_damaged_recordings(reference_available, sfxc_lib, walk_driver, tmp_path):
    import subprocess

    from oracle import jobs
    from sfxc_gpu import correlator
    compared, stale, refused = 0, 0, []
    for name, k, kind, rec in _mutations():
        c = CASES[name]
        try:
            ref = jobs.reader(rec, c["fmt"], timeout=60, **c["params"])
        except (RuntimeError, subprocess.TimeoutExpired) as e:
            refused.append((name, k, kind, str(e)[:200]))
            continue
        got = correlator.read_recording(rec, c["fmt"], **c["params"])
        assert got == ref, (name, k, kind)
        walked = [{kk: b[kk] for kk in ("channel", "start_ticks", "data", "invalid")}
                  for b in walk_blocks(walk_driver, tmp_path, dict(c, rec=rec))]
        want = [dict(b, invalid=list(b["invalid"])) for b in ref]
        if c["fmt"] == "mark5b" and len(want) >= 2 and walked == want[:-1]:
            # a Mark5B file that ends inside a resync: the reference's reader
            # returns one more block, whose tail is still its previous
            # block's bytes (the walk ends before it)
            a, b = want[-2]["data"], want[-1]["data"]
            assert len(a) == len(b) and a[-16:] == b[-16:], (name, k, kind)
            stale += 1
        else:
            assert walked == want, (name, k, kind)
        compared += 1
    total = compared + len(refused)
    assert compared >= 0.9 * total, refused
    print("%d damaged recordings compared (%d ending inside a Mark5B resync), %d refused by the reference"
          % (compared, stale, len(refused)))
