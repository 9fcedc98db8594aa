"""The C-ABI library without a GPU: it loads, exports every function that
include/sfxc_gpu.h declares, and its host-side input-node functions (integer
delay lists, byte protocol) reproduce the reference's golden outputs bit for
bit.  No kernel runs here."""
import os
import re

import numpy as np
import pytest

from golden_io import CASES, Golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sfxc_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(sfxc_gpu_\w+)\s*\(", text))
    return sorted(n for n in names if not n.startswith("sfxc_gpu_ctx"))


def test_exports_every_declared_symbol(sfxc_lib):
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(sfxc_lib, n), n
    from sfxc_gpu import lib
    assert sorted(lib.EXPORTS) == names


@pytest.mark.parametrize("case", CASES)
def test_delay_lists(case, sfxc_lib):
    from sfxc_gpu import correlator
    g = Golden(case)
    for k in range(g.nstreams):
        s = g.meta["streams"][k]
        for s0, s1, _, dl in g.slices(k):
            assert correlator.delay_list(g.dels[s[10]], s0, s1, s[2], s[7]) == dl


@pytest.mark.parametrize("case", CASES)
def test_protocol_bytes(case, sfxc_lib):
    from sfxc_gpu import correlator
    g = Golden(case)
    g.job(correlator.write_protocol)  # asserts the digest of every slice


def test_delay_list_errors(sfxc_lib):
    from sfxc_gpu import correlator, lib
    g = Golden("c1_plain")
    s0, s1, _, _ = g.slices(0)[0]
    with pytest.raises(lib.SfxcError) as e:
        correlator.delay_list(g.dels[0], s1, s0, 32_000_000, 2)
    assert e.value.code == lib.EINVAL
    with pytest.raises(lib.SfxcError) as e:
        correlator.delay_list(g.dels[0], s0, s1, 32_000_000, 3)
    assert e.value.code == lib.EINVAL
    far = s0 + 3600 * 512_000_000
    with pytest.raises(lib.SfxcError) as e:
        correlator.delay_list(g.dels[0], far, far + 512_000_000, 32_000_000, 2)
    assert e.value.code == lib.EDELAY
    with pytest.raises(lib.SfxcError) as e:
        correlator.delay_list(b"\x03\x00\x00\x00ab\x00", s0, s1, 32_000_000, 2)
    assert e.value.code == lib.EDELTAB


def test_no_cpu_fallback(sfxc_lib):
    """Without a usable GPU the library refuses to create a context."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sfxc_gpu import correlator, lib
    with pytest.raises(lib.SfxcError):
        correlator.CorrelatorNode(0)


@pytest.mark.gpu
def test_reduction_parameters_are_checked(sfxc_lib):
    """number_channels must be a power of two no larger than the correlation
    FFT size (spectral reduction); a bad value fails before any device work."""
    from sfxc_gpu import correlator, lib, scenario
    sc = scenario.c1_plain(integration_us=15625, n_integrations=1, seed=1)
    job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol, fast_random=True)
    for bad in (3, 0, 1024):
        j = dict(job, number_channels=bad)
        node = correlator.CorrelatorNode(0, lib.X_FP32)
        with pytest.raises(lib.SfxcError, match="number_channels"):
            node.set_parameters(j)
        node.close()


@pytest.mark.parametrize("case", CASES)
def test_split_output(case):
    """The package's reader of the output layout agrees with the fixtures' parser."""
    from golden_io import parse_cor
    from sfxc_gpu import correlator
    g = Golden(case)
    nchan = int(g.meta.get("number_channels") or g.meta["fft_size_correlation"])
    h1, v1 = parse_cor(g.cor, nchan)
    h2, v2 = correlator.split_output(g.cor, nchan)
    assert h1 == h2 and len(v1) == len(v2)
    assert all(np.array_equal(a, b) for a, b in zip(v1, v2))


def test_uvw_model_matches_reference(sfxc_lib):
    """The library's UVW model (Akima splines of the .del file's u, v, w
    columns per phase centre, rebuilt per second as the reference's
    Uvw_model::get_uvw does) gives the reference's values bit for bit: two
    phase centres, whole and fractional seconds, clamped windows at a scan's
    ends, a later scan, and a step back in time (tests/golden/uvw.json, from
    the reference's own class)."""
    import hashlib
    import json
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    from sfxc_gpu import correlator
    tables, probes = make_golden.uvw_cases()
    golden = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "uvw.json")))
    for name, db in tables.items():
        g = golden[name]
        assert hashlib.sha256(db).hexdigest() == g["del_sha256"]
        m = correlator.UvwModel(db)
        got = [list(m.get(pc, t)) for pc, t in probes]
        assert got == g["uvw"], name
        m.close()


def test_uvw_model_errors(sfxc_lib):
    from sfxc_gpu import correlator, lib
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    tables, probes = make_golden.uvw_cases()
    m = correlator.UvwModel(tables["near"])
    with pytest.raises(lib.SfxcError):
        m.get(2, probes[0][1])  # two phase centres in the first scan
    with pytest.raises(lib.SfxcError):
        m.get(0, probes[-1][1] + 512_000_000 * 100)  # past the table
    with pytest.raises(lib.SfxcError):
        correlator.UvwModel(b"\x04\x00")
