"""Jobs of more than 32 streams (the reference's create_baselines takes any
number, sfxc/src/correlation_core.cc:134-171): 20 stations dual-pol = 40
streams, 800 baselines, on both X-step forms -- the FP32 X-step with its
stream-pair tiles split over work items, the tensor-core X-step with 64 stream
slots and two 128-component row blocks of the Gram.

Bars: output headers byte-exact; FP32 visibilities within relative L2 1e-5
per baseline of the FP32 restatement; both forms within 1e-4 of the FP64
restatement."""
import pytest

from golden_io import compare_cor, parse_cor, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wide_case(oracle_exe):
    from oracle import jobs
    from sfxc_gpu import scenario
    st = scenario.cubic_stations(20, seed=2020, max_delay=1e-2, max_rate=3e-6)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                           channel_freq=4_800_000_000, nchan=4096, integration_us=20000, n_integrations=1,
                           sub_integration_us=10000, lead_us=12000, seed=40, block_bytes=2000)
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    return job, jobs.correlate(job, impl="oracle"), jobs.correlate(job, impl="oracle", precision=64)


@pytest.mark.parametrize("mode", ["fp32", "tc"])
def test_forty_streams(mode, wide_case, sfxc_lib):
    from sfxc_gpu import correlator, lib
    job, ref32, ref64 = wide_case
    node = correlator.CorrelatorNode(0, lib.X_FP32 if mode == "fp32" else lib.X_TC_HILO)
    try:
        cor, tsys = node.correlate(job)
    finally:
        node.close()
    assert tsys == ref32["tsys"]
    M = job["fft_size_correlation"]
    _, vg = parse_cor(cor, M)
    assert len(vg) == 40 + 40 * 39 // 2 - 20
    e32 = compare_cor(cor, ref32["cor"], M, 1e-5 if mode == "fp32" else 1e-4)
    vis64 = ref64["vis64"].reshape(len(vg), M + 1)
    e64 = max(rel_err(a, b) for a, b in zip(vg, vis64))
    print("40 streams, %s X-step: worst vs FP32 restatement %.3g, vs FP64 %.3g" % (mode, e32, e64))
    assert e64 <= 1e-4
