"""The library's host-side unpack plan (replica of the reference's bit-to-float
state machine, csrc/host.cpp) checked on the CPU: the samples it maps out of
the protocol reproduce the reference's unpacked-sample digests, and the
counted bytes reproduce the reference's level and tsys statistics, across
integration boundaries (state carried from one integration to the next),
delay changes, invalid runs and 1-bit data."""
import hashlib
import os
import subprocess
import tempfile

import numpy as np
import pytest

from golden_io import CASES, Golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sfxc-1_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("plan") / "plan_driver")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
                    os.path.join(ROOT, "tests", "plan_driver.cc"), os.path.join(CSRC, "host.cpp"), "-o", exe],
                   check=True)
    return exe


def levels_from_hist(h, bits, n_invalid):
    st5 = [0] * 5
    for i in range(256):
        c = h[i] + h[256 + i]
        if bits == 2:
            for k in range(4):
                st5[(i >> (2 * k)) & 3] += c
        else:
            for k in range(8):
                st5[(i >> k) & 1] += c
    st5[4] += n_invalid
    return st5


@pytest.mark.parametrize("case", CASES)
def test_plan_matches_reference(case, driver, sfxc_lib):
    from sfxc_gpu import correlator, scenario, synth, timebase
    g = Golden(case)
    job = g.job(correlator.write_protocol)
    M = job["fft_size_correlation"]
    nr = timebase.nr_ffts_per_integration_slice(job["integration_time_us"], job["sample_rate"], M)
    n_blocks = (M // 256) * nr
    nfft_max = max(8192 // 256, M // 256)
    stats_lines = [l.split() for l in g.stats.splitlines() if not l.startswith("I")]
    with tempfile.TemporaryDirectory() as d:
        for k in range(g.nstreams):
            s = job["streams"][k]
            path = os.path.join(d, "p%d.bin" % k)
            with open(path, "wb") as f:
                for it in range(g.nint):
                    f.write(np.uint64(len(job["protocols"][k][it])).tobytes())
                    f.write(job["protocols"][k][it])
            delays_at_start = []
            for (s0, s1, _, _) in g.slices(k):
                # delay at the slice start, evaluated by the library's spline via a one-entry list
                delays_at_start.append(_delay_seconds(g.dels[s[10]], s0, s1))
            subprocess.run([driver, path, str(g.nint), str(n_blocks), str(nfft_max), str(s[7]), str(s[2]),
                            str(s[9])] + ["%.17g" % v for v in delays_at_start] + [os.path.join(d, "o%d" % k)],
                           check=True)
            for it in range(g.nint):
                un = np.fromfile(os.path.join(d, "o%d_u%d.f32" % (k, it)), dtype=np.float32)
                assert hashlib.sha256(un.tobytes()).digest() == g.unpacked_sha(k, it), (k, it)
                lines = open(os.path.join(d, "o%d_h%d.txt" % (k, it))).read().split("\n")
                h = [int(x) for x in lines[:512]]
                n_invalid = int(lines[512])
                lv = levels_from_hist(h, s[7], n_invalid)
                want = stats_lines[it * g.nstreams + k]
                assert [int(x) for x in want[1:6]] == lv, (k, it)
                on = [0, 0, 0, 0]
                off = [0, 0, 0, 0]
                if s[7] == 2:
                    for i in range(256):
                        for q in range(4):
                            on[(i >> (2 * q)) & 3] += h[i]
                            off[(i >> (2 * q)) & 3] += h[256 + i]
                    tsys = [on[1] + on[2], on[0] + on[3], off[1] + off[2], off[0] + off[3]]
                    assert [int(x) for x in want[6:10]] == tsys, (k, it)


def _delay_seconds(del_bytes, s0, s1):
    """delay(s0) of the slice spline, through the C restatement's probe output."""
    from oracle import jobs
    _, probes = jobs.delays(del_bytes, s0, s1, 32_000_000, 2, probes=[s0], impl="oracle")
    return probes[0][1]
