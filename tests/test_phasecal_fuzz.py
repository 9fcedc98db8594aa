"""Phase-cal extraction on seeded random set-ups (Input_node_data_writer::
do_phasecal, sfxc/src/input_node_data_writer.cc:230-312): the channel blocks,
delays and invalid runs of the random input-node set-ups
(test_input_node_fuzz.random_scenario: 1- and 2-bit, 16-64 MS/s, whole-block,
edge and paired invalid runs), with a phase-cal integration of one, two or
four blocks.

CPU: the restatement's messages against the reference writer's, byte for byte.
GPU: the library's fold (sfxc_gpu_phasecal_*) over the same blocks; the
reference's messages are the first of the GPU's (the writer stops at its last
slice, the fold takes every block pushed)."""
import hashlib

import pytest

from test_input_node_fuzz import random_scenario

SEEDS = range(12)


def phasecal_case(seed, delay_fn):
    """(blocks, slices, sample rate, bits, integration us, phase-cal ticks) of
    the first stream of a random set-up."""
    from sfxc_gpu import scenario, timebase
    sc = random_scenario(seed)
    chans, _ = scenario.channel_streams(sc, fast_random=True)
    key = sc.streams()[0]
    blocks = scenario.blocks_of(sc, chans[key], key)
    rec0, start, tint, slice_samples = scenario.job_timing(sc)
    dels = scenario.del_tables(sc)
    slices = [(start + it * tint, start + (it + 1) * tint, slice_samples,
               delay_fn(dels[key[0]], start + it * tint, start + (it + 1) * tint, sc.sample_rate, sc.bits))
              for it in range(sc.n_integrations)]
    block_ticks = blocks[1][0] - blocks[0][0]
    ticks = block_ticks * (1, 2, 4)[seed % 3]
    assert rec0 % ticks == 0 and block_ticks == sc.block_bytes * 8 // sc.bits * timebase.ticks_per_sample(
        sc.sample_rate)
    return blocks, slices, sc.sample_rate, sc.bits, sc.integration_us, ticks


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


@pytest.mark.parametrize("seed", SEEDS)
def test_restatement_matches_reference(seed, reference_available):
    from oracle import jobs
    blocks, slices, sr, bits, iu, ticks = phasecal_case(seed, lambda *a: jobs.delays(*a)[0])
    ref_p, ref_m = jobs.protocol(blocks, slices, sr, bits, iu, phasecal_ticks=ticks)
    mine_p, mine_m = jobs.protocol(blocks, slices, sr, bits, iu, impl="oracle", phasecal_ticks=ticks)
    assert len(ref_m) > 0
    assert mine_m == ref_m and mine_p == ref_p


@pytest.mark.gpu
def test_gpu_fold_matches_restatement(gpu_node, oracle_exe):
    from oracle import jobs
    from sfxc_gpu import correlator
    for seed in SEEDS:
        blocks, slices, sr, bits, iu, ticks = phasecal_case(seed, correlator.delay_list)
        _, want = jobs.protocol(blocks, slices, sr, bits, iu, impl="oracle", phasecal_ticks=ticks)
        n = 8 + 8 + 4 + 4 + 4 * int(sr / 10e3)  # fields, then one int32 per bin
        pc = correlator.PhaseCal(gpu_node, sr, bits, ticks, station=0, frequency_number=0, sideband=1,
                                 polarisation=0)
        try:
            got = pc.push(blocks)
        finally:
            pc.close()
        want_msgs = [want[i:i + n] for i in range(0, len(want), n)]
        assert len(want) % n == 0 and len(got) >= len(want_msgs), seed
        assert [hashlib.sha256(m).digest() for m in got[:len(want_msgs)]] == \
            [hashlib.sha256(m).digest() for m in want_msgs], seed
