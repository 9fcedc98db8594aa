"""Tensor-core X-step (FP16 hi+lo products on tcgen05, FP32 accumulation).

Bars: output headers byte-exact; visibilities within 1e-5 relative L2 per
baseline of the reference's FP32 output on the golden fixtures; and within
1e-4 per baseline of the FP64 restatement on the precision configuration's
shape (32 inputs, 4096 channels, gain scatter 0.5-2x, an RFI tone 30 dB over
the per-channel noise)."""
import numpy as np
import pytest

from golden_io import Golden, compare_cor, parse_cor, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tc_node(sfxc_lib):
    from sfxc_gpu import correlator, lib
    node = correlator.CorrelatorNode(0, lib.X_TC_HILO)
    yield node
    node.close()


@pytest.mark.parametrize("case", ["c1_plain", "multi", "onebit", "pulsar", "reduced", "reduced_mask", "phase_centers", "phased"])
def test_tc_golden(case, tc_node):
    from sfxc_gpu import correlator
    g = Golden(case)
    job = g.job(correlator.write_protocol)
    cor, tsys = tc_node.correlate(job)
    assert tsys == g.tsys
    worst = compare_cor(cor, g.cor, job["number_channels"], 1e-5)
    print("%s TC worst error vs reference %.3g" % (case, worst))


def test_tc_matches_fp32_path(tc_node, gpu_node):
    from sfxc_gpu import correlator, scenario
    st = scenario.cubic_stations(16, seed=77, max_delay=1e-2, max_rate=3e-6)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                           channel_freq=4_800_000_000, nchan=4096, integration_us=20000, n_integrations=1,
                           sub_integration_us=10000, lead_us=12000, seed=8, block_bytes=2000)
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    a, _ = tc_node.correlate(job)
    b, _ = gpu_node.correlate(job)
    compare_cor(a, b, 4096, 1e-5)


def test_tc_precision_vs_fp64(tc_node, gpu_node):
    """The precision statement: TC and FP32 paths against the FP64 restatement."""
    from oracle import jobs
    from sfxc_gpu import correlator, scenario, synth
    rng = np.random.Generator(np.random.PCG64(31))
    gains = list(rng.uniform(0.5, 2.0, size=16))
    st = scenario.cubic_stations(16, seed=3131, max_delay=1e-2, max_rate=3e-6, gains=gains)
    # RFI: a tone common to all stations, 30 dB over the per-channel noise power
    # (per-channel noise power of unit-variance white noise ~ 1/M of the band)
    M = 4096
    amp = np.sqrt(2 * 1000.0 / M)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                           channel_freq=4_800_000_000, nchan=M, integration_us=12000, n_integrations=1,
                           sub_integration_us=10000, lead_us=11000, seed=17, block_bytes=2000, rho=0.01,
                           tones=[(7.5e6 + 3906.25, amp), (21.25e6 + 3906.25, amp)])
    job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol)
    tc, _ = tc_node.correlate(job)
    f32, _ = gpu_node.correlate(job)
    ref = jobs.correlate(job, impl="oracle", precision=64)
    _, v64 = parse_cor(ref["cor"], M)
    vis64 = ref["vis64"].reshape(len(v64), M + 1)
    _, vtc = parse_cor(tc, M)
    _, vf = parse_cor(f32, M)
    e_tc = max(rel_err(a, b) for a, b in zip(vtc, vis64))
    e_f32 = max(rel_err(a, b) for a, b in zip(vf, vis64))
    print("precision: TC hi+lo %.3g, FP32 %.3g (worst baseline, relative L2 vs FP64)" % (e_tc, e_f32))
    assert e_tc <= 1e-4
    assert e_f32 <= 1e-4
