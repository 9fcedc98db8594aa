"""The C restatement (oracle/sfxc_oracle.c) against the golden fixtures made by
the reference's own classes: integer delays, protocol bytes and unpacked
samples bit-exact; statistics, tsys records and output headers byte-exact;
visibilities within 1e-6 relative L2 (FFT rounding only)."""
import hashlib
import os

import numpy as np
import pytest

from golden_io import CASES, Golden, compare_cor
from oracle import jobs


def oracle_delays(*a):
    return jobs.delays(*a, impl="oracle")[0]


def oracle_protocol(*a):
    return jobs.protocol(*a, impl="oracle")


@pytest.mark.parametrize("case", CASES)
def test_delay_lists(case, oracle_exe):
    g = Golden(case)
    for k in range(g.nstreams):
        s = g.meta["streams"][k]
        for it, (s0, s1, _, dl) in enumerate(g.slices(k)):
            assert oracle_delays(g.dels[s[10]], s0, s1, s[2], s[7]) == dl


@pytest.mark.parametrize("case", CASES)
def test_protocol_and_correlation(case, oracle_exe):
    g = Golden(case)
    job = g.job(oracle_protocol)  # asserts protocol digests
    res = jobs.correlate(job, dump=True, impl="oracle")
    for k in range(g.nstreams):
        for it in range(g.nint):
            un = res["unpacked"][(it, k)]
            assert hashlib.sha256(un.tobytes()).digest() == g.unpacked_sha(k, it)
            M = job["fft_size_correlation"]
            rows = res["rows"][(it, k)].reshape(-1, M + 4)[:, :M + 1]
            idx = np.asarray(g.z["rows_idx_%d_%d" % (k, it)])
            want = np.asarray(g.z["rows_%d_%d" % (k, it)])
            for r, w in zip(idx, want):
                e = np.linalg.norm(rows[r] - w) / max(np.linalg.norm(w), 1e-30)
                assert e < 1e-6, (k, it, r, e)
    assert res["stats"] == g.stats
    assert res["tsys"] == g.tsys
    compare_cor(res["cor"], g.cor, job["number_channels"], 1e-6)


def test_channel_extraction(oracle_exe):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "extract.npz"))
    words = z["words"].tobytes()
    for key, bits in (("16", 2), ("8", 2), ("1", 1)):
        tracks = z["tracks" + key].tolist()
        out = jobs.extract(words, 4, bits, z["words"].size, tracks, impl="oracle")
        assert b"".join(out) == z["out" + key].tobytes()


def test_fp64_mode_close_to_fp32(oracle_exe):
    """precision 64 runs the same algorithm in double; it must agree with the
    float pipeline to float rounding."""
    g = Golden("c1_plain")
    job = g.job(oracle_protocol)
    r32 = jobs.correlate(job, impl="oracle")
    r64 = jobs.correlate(job, impl="oracle", precision=64)
    compare_cor(r64["cor"], r32["cor"], job["number_channels"], 5e-6)
    assert r64["stats"] == r32["stats"]


def test_short_protocol_is_rejected(oracle_exe):
    g = Golden("c1_plain")
    job = g.job(oracle_protocol)
    job["protocols"] = [[p[0][: len(p[0]) // 2], p[1]] for p in job["protocols"]]
    with pytest.raises(RuntimeError, match="protocol ended|data block"):
        jobs.correlate(job, impl="oracle")


def test_pulsar_bins_bit_exact(oracle_exe):
    g = Golden("pulsar")
    job = g.job(oracle_protocol)
    res = jobs.correlate(job, dump=True, impl="oracle")
    assert np.array_equal(res["bins"], np.asarray(g.z["bins"], dtype=np.int32))
