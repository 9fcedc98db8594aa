"""Streams at sample rates other than the job's (the reference's
mixed-bandwidth correlation: per-stream windowed-FFT length 2M sr_st/sr and
channel offsets, sfxc/src/delay_correction.cc:187-259).

CPU: the C restatement against the reference's own classes.  For streams at
or below the job rate they agree throughout.  For a stream faster than the
job, the reference's Delay_correction ring (time_buffer, sized for input
blocks of CORRELATOR_BUFFER_SIZE samples, delay_correction.cc:200-203) is
smaller than one Bit2float block (nfft_max * sr_st / sr blocks,
bit2float_worker.cc:237-276) plus the half window still to be read, so the
first window after every input block reads samples already overwritten; the
restatement (and the GPU path) use the recorded samples there.  The test pins
that every other spectrum row is identical.

GPU: mixed-rate jobs through the library against the restatement, FP32 and
tensor-core X-steps."""
import numpy as np
import pytest

from golden_io import compare_cor

M = 1024


def mixed_job(modes, pols=("R",)):
    from sfxc_gpu import scenario
    st = scenario.cubic_stations(4, seed=5, max_delay=3e-3, max_rate=1e-6)
    sc = scenario.Scenario(stations=st, pols=pols, sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
                           channel_freq=1_400_000_000, nchan=M, integration_us=32768, n_integrations=1,
                           sub_integration_us=32768, lead_us=8000, seed=9, block_bytes=4000,
                           station_modes={st[i].number: v for i, v in modes.items()})
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    return job


# station index -> (sample rate, bits, band start minus the job's channel frequency)
SLOWER = {1: (16_000_000, 2, 0), 2: (16_000_000, 1, 4_000_000), 3: (32_000_000, 1, 0)}
FASTER = {1: (64_000_000, 2, 0), 2: (64_000_000, 2, -8_000_000)}


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


def test_restatement_matches_reference_at_or_below_job_rate(reference_available):
    from oracle import jobs
    job = mixed_job(SLOWER)
    ref = jobs.correlate(job, impl="reference")
    ora = jobs.correlate(job, impl="oracle")
    assert ref["tsys"] == ora["tsys"]
    compare_cor(ora["cor"], ref["cor"], M, 1e-5)


def test_faster_stream_differs_only_in_overwritten_windows(reference_available):
    from oracle import jobs
    job = mixed_job({1: FASTER[1]})
    ref = jobs.correlate(job, impl="reference", dump=True)
    ora = jobs.correlate(job, impl="oracle", dump=True)
    for k in range(len(job["streams"])):
        a = ref["rows"][(0, k)].reshape(-1, M + 4)
        b = ora["rows"][(0, k)].reshape(-1, M + 4)
        bad = [r for r in range(a.shape[0]) if not np.array_equal(a[r], b[r])]
        if k != 1:
            assert bad == [], k
        else:
            # input blocks of 64 x 256 samples at 64 MS/s = 8 hops of 2048:
            # the first window after each block boundary
            assert bad and all(r % 8 == 7 for r in bad) and len(bad) >= a.shape[0] // 8 - 1


@pytest.mark.gpu
@pytest.mark.parametrize("modes", [SLOWER, FASTER], ids=["slower", "faster"])
def test_mixed_rates_gpu_vs_restatement(gpu_node, modes):
    from oracle import jobs
    job = mixed_job(modes)
    cor, tsys = gpu_node.correlate(job)
    ref = jobs.correlate(job, impl="oracle")
    assert tsys == ref["tsys"]
    compare_cor(cor, ref["cor"], M, 1e-5)


@pytest.mark.gpu
def test_mixed_rates_tensor_core_vs_restatement():
    from oracle import jobs
    from sfxc_gpu import correlator, lib
    job = mixed_job({**SLOWER, 0: (64_000_000, 2, -8_000_000)}, pols=("R", "L"))
    node = correlator.CorrelatorNode(0, lib.X_TC_HILO)
    try:
        cor, tsys = node.correlate(job)
    finally:
        node.close()
    ref = jobs.correlate(job, impl="oracle")
    assert tsys == ref["tsys"]
    compare_cor(cor, ref["cor"], M, 1e-4)
