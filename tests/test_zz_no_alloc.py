"""The allocation-free spectra entry point (sfxc_gpu_copy_spectra_noalloc).

It serves callers that cannot allocate device memory when they inspect a
stream -- real-time loops with no time for the allocator (which may wait for
the whole device), or hosts that hand out GPU memory once at start-up -- by
keeping its scratch in a fixed static device array.  Through the C ABI it must give
the same delay-corrected spectra as sfxc_gpu_copy_spectra, on two calls in a
row (the array keeps the previous call's contents), and reject requests larger
than its array.  Collected last so that a stop-at-first-failure run has run
everything else before it."""
import numpy as np
import pytest

from golden_io import Golden, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the FP32 spectra tolerance of the parity tests


def test_noalloc_matches_allocating_entry_point(sfxc_lib):
    from sfxc_gpu import correlator, lib, timebase
    g = Golden("multi")
    job = g.job(correlator.write_protocol)
    node = correlator.CorrelatorNode(0, lib.X_FP32)
    try:
        node.correlate(job)
        M = job["fft_size_correlation"]
        nffts = timebase.nr_ffts_per_integration_slice(job["integration_time_us"], job["sample_rate"], M) - 1
        for stream in (4, 1):  # two calls in a row; the second overwrites the first's scratch
            want = node.spectra(stream, nffts, M)
            got = node.spectra_noalloc(stream, nffts, M)
            assert got.shape == want.shape
            worst = max(rel_err(a, b) for a, b in zip(got, want))
            assert worst <= TOL, (stream, worst)
    finally:
        node.close()


def test_noalloc_rejects_oversized_requests(sfxc_lib):
    from sfxc_gpu import correlator, lib, scenario
    sc = scenario.c1_plain(integration_us=125000, n_integrations=1, seed=2)  # 15625 blocks > 8192
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    node = correlator.CorrelatorNode(0, lib.X_FP32)
    try:
        node.correlate(job)
        with pytest.raises(lib.SfxcError) as e:
            node.spectra_noalloc(0, 7811, 512)
        assert e.value.code == lib.EINVAL
        assert "static scratch" in str(e.value)
    finally:
        node.close()
