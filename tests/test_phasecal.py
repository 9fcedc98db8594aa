"""Phase-cal extraction (Input_node_data_writer::do_phasecal,
sfxc/src/input_node_data_writer.cc:230-312): the oracle's fold against the
messages the reference wrote (tests/golden/phasecal.json), and the GPU fold
against both.  Integer sums: bit-exact."""
import hashlib
import json
import os
import struct

import pytest

from golden_io import GOLDEN, Golden, phasecal_blocks, phasecal_cases
from oracle import jobs

FIXTURE = json.load(open(os.path.join(GOLDEN, "phasecal.json")))
CASES = sorted(phasecal_cases())


def _case(name):
    fx, k, ticks, first, inject = phasecal_cases()[name]
    g = Golden(fx)
    s = g.meta["streams"][k]
    return g, k, s, ticks, phasecal_blocks(g, k, first, inject)


def _split(raw, n):
    assert len(raw) % n == 0
    return [raw[i:i + n] for i in range(0, len(raw), n)]


@pytest.mark.parametrize("case", CASES)
def test_oracle_phasecal_messages(case, oracle_exe):
    g, k, s, ticks, blocks = _case(case)
    want = FIXTURE[case]
    _, raw = jobs.protocol(blocks, g.slices(k), s[2], s[7], g.meta["integration_time_us"], impl="oracle",
                           phasecal_ticks=ticks)
    msgs = _split(raw, want["message_bytes"])
    assert [hashlib.sha256(m).hexdigest() for m in msgs] == want["messages"]


def test_oracle_phasecal_leaves_protocol_alone(oracle_exe):
    """With phase-cal extraction on, the writer's protocol bytes are those of the fixture."""
    g = Golden("c1_plain")
    s = g.meta["streams"][0]
    pr, raw = jobs.protocol(g.blocks(0), g.slices(0), s[2], s[7], g.meta["integration_time_us"], impl="oracle",
                            phasecal_ticks=2048000)
    assert len(raw) > 0
    for it in range(g.nint):
        assert g.protocol_ok(0, it, pr[it])


def _boundaries(blocks, ticks):
    return sum(1 for st, _, _ in blocks if st % ticks == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_phasecal_messages(case, gpu_node, oracle_exe):
    from sfxc_gpu import correlator
    g, k, s, ticks, blocks = _case(case)
    want = FIXTURE[case]
    pc = correlator.PhaseCal(gpu_node, s[2], s[7], ticks, station=0, frequency_number=0, sideband=1,
                             polarisation=0)
    try:
        # uneven pushes (and an empty one): the running integration carries over
        cut1, cut2 = len(blocks) // 3, len(blocks) // 3 + 2
        msgs = pc.push(blocks[:cut1]) + pc.push([]) + pc.push(blocks[cut1:cut2]) + pc.push(blocks[cut2:])
    finally:
        pc.close()
    # the reference's writer stops at its last slice; the GPU folds every block pushed
    assert len(msgs) == max(0, _boundaries(blocks, ticks) - 1)
    assert len(msgs) >= len(want["messages"])
    assert [hashlib.sha256(m).hexdigest() for m in msgs[:len(want["messages"])]] == want["messages"]
    for m in msgs:
        assert len(m) == want["message_bytes"]
        station, freq, sb, pol, t0, dt, n = struct.unpack_from("<4Bqqi", m)
        assert (station, freq, sb, pol, n) == (0, 0, 1, 0, int(s[2] / 10e3))
        assert t0 % ticks == 0 and dt % ticks == 0 and dt > 0


@pytest.mark.gpu
def test_gpu_phasecal_header_fields(gpu_node):
    """Station, frequency, sideband and polarisation bytes as set_parameters packs them."""
    from sfxc_gpu import correlator
    g, k, s, ticks, blocks = _case("c1_every_block")
    pc = correlator.PhaseCal(gpu_node, s[2], s[7], ticks, station=5, frequency_number=3, sideband=0,
                             polarisation=1)
    try:
        msgs = pc.push(blocks[:4])
    finally:
        pc.close()
    assert len(msgs) == 3
    for m in msgs:
        assert m[:4] == bytes([5, 3, 0, 1])


@pytest.mark.gpu
def test_gpu_phasecal_parameters_are_checked(gpu_node):
    from sfxc_gpu import correlator, lib
    for sr, bits, ticks in ((32000000, 3, 1000), (32000000, 2, 0), (5000, 2, 1000), (30000, 2, 1000)):
        with pytest.raises(lib.SfxcError):
            correlator.PhaseCal(gpu_node, sr, bits, ticks)
    pc = correlator.PhaseCal(gpu_node, 32000000, 2, 2048000)
    try:
        with pytest.raises(lib.SfxcError, match="invalid"):
            pc.push([(0, b"\0" * 64, [(-1, 4)])])
    finally:
        pc.close()
