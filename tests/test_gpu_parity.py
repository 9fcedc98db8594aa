"""GPU parity: the CUDA path through the C ABI against the reference's golden
outputs and the C restatement.

Bars: unpacked samples, pulsar bins, statistics, tsys records and every
output header byte-exact; channel extraction bit-exact; FP32 visibilities
within relative L2 1e-5 per baseline (the tolerance the FP32 path is held to);
delay-corrected spectra within 1e-5 per row."""
import hashlib
import os

import numpy as np
import pytest

from golden_io import CASES, Golden, compare_cor, parse_cor, rel_err

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def run_golden(node, case):
    from sfxc_gpu import correlator
    g = Golden(case)
    from sfxc_gpu import timebase
    job = g.job(correlator.write_protocol)
    node.set_parameters(job)
    M = job["fft_size_correlation"]
    nffts = timebase.nr_ffts_per_integration_slice(job["integration_time_us"], job["sample_rate"], M) - (
        1 if job["window"] != 0 else 0)
    cor, tsys = [], []
    for it in range(g.nint):
        if job.get("uvw") is not None:
            node.set_uvw(job["uvw"][it])
        for k in range(g.nstreams):
            node.push_protocol(k, job["protocols"][k][it])
        o, t = node.run_integration()
        cor.append(o)
        tsys += t
        for k in range(g.nstreams):
            nb = g.meta["slice_samples"] // 256
            un = node.unpacked(k, nb * 256)
            assert hashlib.sha256(un.tobytes()).digest() == g.unpacked_sha(k, it), (case, k, it)
            rows = node.spectra(k, nffts, M)
            for r, w in zip(np.asarray(g.z["rows_idx_%d_%d" % (k, it)]), np.asarray(g.z["rows_%d_%d" % (k, it)])):
                assert rel_err(rows[r], w) < FP32_TOL, (case, k, it, r, rel_err(rows[r], w))
    return g, job, b"".join(cor), b"".join(tsys)


@pytest.mark.parametrize("case", CASES)
def test_golden_fp32(case, gpu_node):
    g, job, cor, tsys = run_golden(gpu_node, case)
    assert tsys == g.tsys
    worst = compare_cor(cor, g.cor, job["number_channels"], FP32_TOL)
    print("%s worst visibility error %.3g" % (case, worst))


def test_channel_extraction(gpu_node):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "extract.npz"))
    words = z["words"].tobytes()
    for key, bits in (("16", 2), ("8", 2), ("1", 1)):
        out = gpu_node.extract_channels(words, 4, bits, z["tracks" + key].tolist())
        assert b"".join(out) == z["out" + key].tobytes(), key


def test_fringe_at_injected_delay(gpu_node):
    """Synthetic-signal sanity: correlation 0.3 and a 37.25-sample delay with a
    1e-7 rate come out as a stationary fringe at zero lag with the 2-bit
    quantisation efficiency (~0.88) times the injected correlation."""
    from sfxc_gpu import correlator, scenario
    sc = scenario.c1_plain(integration_us=15625, n_integrations=1, seed=4)
    sc.rho = 0.3
    job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol)
    cor, _ = gpu_node.correlate(job)
    _, vis = parse_cor(cor, 512)
    cross = vis[2]
    lag = np.fft.irfft(cross)
    assert int(np.argmax(np.abs(lag))) == 0
    amp = np.abs(cross[32:480]).mean()
    assert 0.22 < amp < 0.30, amp
    ph = np.angle(cross[32:480].mean())
    assert abs(ph) < 0.1, ph


def test_larger_job_vs_oracle(gpu_node):
    """Eight stations x two polarisations, 4096 channels, 64 MS/s, cubic delays
    with |rate| up to 3e-6, against the C restatement."""
    from oracle import jobs
    from sfxc_gpu import correlator, scenario
    st = scenario.cubic_stations(8, seed=2024, max_delay=15e-3, max_rate=3e-6)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                           channel_freq=4_800_000_000, nchan=4096, integration_us=40000, n_integrations=1,
                           sub_integration_us=10000, lead_us=16000, seed=3, block_bytes=2000)
    job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol, fast_random=True)
    cor, tsys = gpu_node.correlate(job)
    ref = jobs.correlate(job, impl="oracle")
    assert tsys == ref["tsys"]
    compare_cor(cor, ref["cor"], 4096, FP32_TOL)


@pytest.mark.parametrize("nchan", [256, 16384])
def test_fft_length_extremes_vs_oracle(gpu_node, nchan):
    """The smallest (512-sample) and largest (32768-sample) windowed FFTs,
    three stations x two polarisations, against the C restatement."""
    from oracle import jobs
    from sfxc_gpu import correlator, scenario
    st = scenario.cubic_stations(3, seed=77, max_delay=5e-3, max_rate=2e-6)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
                           channel_freq=1_400_000_000, nchan=nchan, integration_us=65536, n_integrations=1,
                           sub_integration_us=32768, lead_us=8000, seed=11, block_bytes=4000)
    job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol, fast_random=True)
    cor, tsys = gpu_node.correlate(job)
    ref = jobs.correlate(job, impl="oracle")
    assert tsys == ref["tsys"]
    compare_cor(cor, ref["cor"], nchan, FP32_TOL)


def record_boundaries(data):
    """Offsets at which the correlator-node protocol records end."""
    out, p = [], 0
    while p < len(data):
        h = data[p]
        if h == 0:
            p += 3 + (data[p + 1] | data[p + 2] << 8)
        elif h == 1:
            p += 3
        elif h == 2:
            p += 2
        else:
            p += 1
        out.append(p)
    return out


def test_errors_leave_context_usable(gpu_node):
    from sfxc_gpu import correlator, lib
    g = Golden("c1_plain")
    job = g.job(correlator.write_protocol)
    proto = job["protocols"][0][0]
    gpu_node.set_parameters(job)
    # a record cut in the middle is malformed input
    with pytest.raises(lib.SfxcError) as e:
        gpu_node.push_protocol(0, proto[:1000])
    assert e.value.code == lib.EPROTO
    # whole records that end before the integration is complete: input ended early
    gpu_node.set_parameters(job)
    cut = [b for b in record_boundaries(proto) if b < len(proto) // 2][-1]
    gpu_node.push_protocol(0, proto[:cut])
    gpu_node.push_protocol(1, job["protocols"][1][0])
    with pytest.raises(lib.SfxcError) as e:
        gpu_node.run_integration()
    assert e.value.code == lib.ESTREAM
    with pytest.raises(lib.SfxcError) as e:
        gpu_node.push_protocol(7, proto)
    assert e.value.code == lib.EINVAL
    cor, _ = gpu_node.correlate(job)  # a fresh job on the same context works
    compare_cor(cor, g.cor, 512, FP32_TOL)


@pytest.mark.gpu
def test_uvw_header_values(gpu_node):
    """UVW values reach the timeslice header for the first stream of each
    station; a wrong count is refused; a new job starts from zeros."""
    import struct
    from sfxc_gpu import correlator, lib
    g = Golden("multi")
    job = g.job(correlator.write_protocol)
    gpu_node.set_parameters(job)
    with pytest.raises(lib.SfxcError) as e:
        gpu_node.set_uvw(job["uvw"][0][:2])
    assert e.value.code == lib.EINVAL
    cor, _ = gpu_node.correlate(job)
    hdr = struct.unpack_from("<i4i", cor, 0)
    nuvw = hdr[3]
    streams = job["streams"]
    first = {}
    for i, s in enumerate(streams):
        first.setdefault(s[0], i)
    for k in range(nuvw):
        station, _, u, v, w = struct.unpack_from("<2i3d", cor, 20 + 32 * k)
        assert (u, v, w) == tuple(job["uvw"][0][first[station]][0])
    cor0, _ = gpu_node.correlate(dict(job, uvw=None))
    for k in range(nuvw):
        assert struct.unpack_from("<3d", cor0, 28 + 32 * k) == (0.0, 0.0, 0.0)
