"""Pulsar binning on the GPU (Correlation_core_pulsar, sfxc/src/correlation_core_pulsar.cc:
13-146,188-238) on both X-step forms: CUDA cores in row order, and tensor
cores over each channel's rows sorted by bin.

Bars: the bin of every (FFT row, channel) bit-exact against the reference's
own bin table (golden fixture) and the restatement's (pulsar configuration's
shape); output headers byte-exact; FP32 visibilities within relative L2 1e-5
per (bin, baseline) of the reference's output (fixture) and of the
restatement's FP32 output; tensor-core visibilities within 1e-5 of the
reference's output on the fixture and within 1e-4 of the FP64 restatement on
the pulsar configuration's shape (10 stations dual-pol, 2048 channels, 256
on-pulse bins plus the off-pulse bin)."""
import numpy as np
import pytest

from golden_io import Golden, compare_cor, parse_cor, rel_err

pytestmark = pytest.mark.gpu

MODES = ["fp32", "tc"]


def _node(mode):
    from sfxc_gpu import correlator, lib
    return correlator.CorrelatorNode(0, lib.X_FP32 if mode == "fp32" else lib.X_TC_HILO)


def _nffts(job):
    from sfxc_gpu import timebase
    M = job["fft_size_correlation"]
    return timebase.nr_ffts_per_integration_slice(job["integration_time_us"], job["sample_rate"], M) - (
        1 if job["window"] != 0 else 0)


@pytest.mark.parametrize("mode", MODES)
def test_golden_bins_and_visibilities(mode, sfxc_lib):
    from sfxc_gpu import correlator
    g = Golden("pulsar")
    job = g.job(correlator.write_protocol)
    node = _node(mode)
    try:
        cor, tsys = node.correlate(job)
        bins = node.pulsar_bins(_nffts(job), job["fft_size_correlation"])
    finally:
        node.close()
    assert np.array_equal(bins, np.asarray(g.z["bins"], dtype=np.int32))
    assert tsys == g.tsys
    worst = compare_cor(cor, g.cor, job["number_channels"], 1e-5)
    print("pulsar fixture, %s X-step: worst visibility error vs reference %.3g" % (mode, worst))


def _c5_job(gate, integration_us):
    from sfxc_gpu import scenario
    sc = scenario.c5_pulsar(integration_us=integration_us)
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    job.update(scenario.pulsar_params(sc, nbins=256, gate=gate))
    return job


@pytest.fixture(scope="module", params=[(0.0, 1.0), (0.45, 0.55)], ids=["gate_full", "gate_onpulse"])
def c5_case(request, oracle_exe):
    from oracle import jobs
    # 64 ms: 999 FFTs of 2048 channels, about two pulse periods
    job = _c5_job(request.param, 64000)
    ref32 = jobs.correlate(job, impl="oracle", precision=32, dump_bins=True)
    ref64 = jobs.correlate(job, impl="oracle", precision=64)
    return job, ref32, ref64


@pytest.mark.parametrize("mode", MODES)
def test_c5_shape(mode, c5_case, sfxc_lib):
    job, ref32, ref64 = c5_case
    M = job["fft_size_correlation"]
    node = _node(mode)
    try:
        cor, tsys = node.correlate(job)
        bins = node.pulsar_bins(_nffts(job), M)
    finally:
        node.close()
    assert np.array_equal(bins, ref32["bins"])
    assert tsys == ref32["tsys"]
    hg, vg = parse_cor(cor, M)
    h32, v32 = parse_cor(ref32["cor"], M)
    assert hg == h32
    assert len(vg) == 257 * 200
    vis64 = ref64["vis64"].reshape(len(vg), M + 1)
    e64 = max(rel_err(a, b) for a, b in zip(vg, vis64))
    e32 = max(rel_err(a, b) for a, b in zip(vg, v32))
    print("C5 shape, %s X-step: worst vs FP32 restatement %.3g, vs FP64 %.3g" % (mode, e32, e64))
    if mode == "fp32":
        assert e32 <= 1e-5
    assert e64 <= 1e-4
