"""Whole correlator-node jobs on seeded random set-ups.

CPU: the C restatement against the reference's own classes (Bit2float_worker
-> Delay_correction -> Correlation_core, run as Correlator_node runs them),
which pins the restatement beyond the fixed fixtures.
GPU: both X-step forms of the library through the C ABI against the
restatement on the same set-ups.

Each set-up draws the stations (2 to 4), one or two polarisations (cross
products), sample rate and bit depth, the correlation FFT length (256 to
2048 channels), the window (none, rectangular, cosine, Hamming, Hann), a
lower-sideband station, an LO offset, the integration and sub-integration
lengths, a reference station, and invalid runs.  Bars: output headers and
tsys records byte-exact, visibilities within 1e-6 (restatement vs
reference) and 1e-5 (GPU vs restatement) relative L2 per baseline."""
import numpy as np
import pytest

from golden_io import compare_cor

N_SETUPS = 10


def random_job(seed, delay_fn, protocol_fn):
    from sfxc_gpu import scenario
    rng = np.random.Generator(np.random.PCG64(5000 + seed))
    n_st = int(rng.integers(2, 5))
    pols = ("R", "L") if rng.random() < 0.5 else ("R",)
    sr, bits = [(16_000_000, 2), (32_000_000, 2), (32_000_000, 1), (64_000_000, 2)][int(rng.integers(0, 4))]
    nchan = int(rng.choice([256, 512, 1024, 2048]))
    st = scenario.cubic_stations(n_st, seed=seed + 77, max_delay=float(rng.uniform(1e-4, 3e-3)),
                                 max_rate=float(rng.uniform(1e-7, 2e-5)))
    integration_us = int(rng.choice([4000, 8000]))
    sub = integration_us // int(rng.choice([1, 2, 4]))
    block_bytes = int(rng.choice([2000, 4000, 8000]))
    invalid = {}
    if rng.random() < 0.6:
        s = st[int(rng.integers(0, n_st))]
        b = int(rng.integers(2, 12))
        invalid[(s.number, pols[-1])] = [(b, int(rng.integers(0, block_bytes // 2)), int(rng.integers(1, block_bytes // 2)))]
    sc = scenario.Scenario(
        stations=st, pols=pols, sample_rate=sr, bandwidth=sr // 2, bits=bits,
        channel_freq=int(rng.choice([1_400_000_000, 4_800_000_000])), nchan=nchan,
        window=int(rng.integers(0, 5)), integration_us=integration_us, sub_integration_us=sub, n_integrations=2,
        lead_us=3500, rho=0.05, seed=seed + 3, block_bytes=block_bytes, invalid=invalid,
        station_sidebands={st[-1].number: "L"} if rng.random() < 0.4 else {},
        lo_offset=float(rng.choice([0.0, 0.0, 12.5, -3.75])),
        reference_station=int(st[0].number) if rng.random() < 0.2 else -1)
    return scenario.build_job(sc, delay_fn, protocol_fn, fast_random=True)


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


@pytest.mark.parametrize("seed", range(N_SETUPS))
def test_restatement_matches_reference(seed, reference_available):
    from oracle import jobs
    job = random_job(seed, lambda *a: jobs.delays(*a)[0], jobs.protocol)
    ref = jobs.correlate(job, impl="reference")
    mine = jobs.correlate(job, impl="oracle")
    assert mine["tsys"] == ref["tsys"]
    assert mine["stats"] == ref["stats"]
    compare_cor(mine["cor"], ref["cor"], job["number_channels"], 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp32", "tc"])
def test_gpu_matches_restatement(mode, sfxc_lib):
    from oracle import jobs
    from sfxc_gpu import correlator, lib
    node = correlator.CorrelatorNode(0, lib.X_FP32 if mode == "fp32" else lib.X_TC_HILO)
    try:
        for seed in range(N_SETUPS):
            job = random_job(seed, correlator.delay_list, correlator.write_protocol)
            ref = jobs.correlate(job, impl="oracle")
            cor, tsys = node.correlate(job)
            assert tsys == ref["tsys"], seed
            compare_cor(cor, ref["cor"], job["number_channels"], 1e-5)
    finally:
        node.close()
