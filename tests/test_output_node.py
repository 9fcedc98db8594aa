"""The output node (Output_node, sfxc/src/output_node.cc:68-214): the global
header against the reference's own struct (tests/golden/output_header.json,
made by oracle/ref_output_header.cc), slices written in slice order whatever
order they arrive in, and each bin's output routed by its file index.  Host
only (no GPU)."""
import json
import os

import numpy as np
import pytest

from golden_io import GOLDEN, Golden

HEADERS = json.load(open(os.path.join(GOLDEN, "output_header.json")))


def _fields(case):
    return {k: v for k, v in case.items() if k != "header_hex"}


@pytest.mark.parametrize("i", range(len(HEADERS)))
def test_global_header_bytes(sfxc_lib, i):
    from sfxc_gpu import correlator
    out = correlator.OutputFiles(2, **_fields(HEADERS[i]))
    files = out.finish()
    out.close()
    want = bytes.fromhex(HEADERS[i]["header_hex"])
    assert len(want) == 84
    assert files == [want, want]


def _integration_slices(cor, n):
    """A correlator output of n integrations of equal size, split per integration."""
    assert len(cor) % n == 0
    per = len(cor) // n
    return [cor[k * per:(k + 1) * per] for k in range(n)]


def test_slices_in_order(sfxc_lib):
    from sfxc_gpu import correlator
    g = Golden("multi")
    slices = _integration_slices(g.cor, g.nint)
    out = correlator.OutputFiles(1, **_fields(HEADERS[0]))
    for k in (2, 0, 1):  # arrival order
        out.put_slice(k, slices[k])
    files = out.finish()
    out.close()
    header = bytes.fromhex(HEADERS[0]["header_hex"])
    assert files[0] == header + b"".join(s[4:] for s in slices)


def test_bins_to_their_files(sfxc_lib):
    """Pulsar binning: one integration of nbins + 1 outputs, file index = bin."""
    from sfxc_gpu import correlator
    g = Golden("pulsar")
    nbins = int(g.meta["pulsar"][0]) + 1
    cor = g.cor
    per = len(cor) // nbins
    idx = [int(np.frombuffer(cor[b * per:b * per + 4], dtype=np.int32)[0]) for b in range(nbins)]
    assert idx == list(range(nbins))
    out = correlator.OutputFiles(nbins, **_fields(HEADERS[0]))
    out.put_slice(0, cor, nbins)
    files = out.finish()
    out.close()
    header = bytes.fromhex(HEADERS[0]["header_hex"])
    for b in range(nbins):
        assert files[b] == header + cor[b * per + 4:(b + 1) * per]


def test_errors(sfxc_lib):
    from sfxc_gpu import correlator, lib
    g = Golden("multi")
    slices = _integration_slices(g.cor, g.nint)
    out = correlator.OutputFiles(1, **_fields(HEADERS[0]))
    out.put_slice(1, slices[1])
    with pytest.raises(lib.SfxcError) as e:
        out.finish()  # slice 0 missing
    assert e.value.code == lib.ESTATE
    with pytest.raises(lib.SfxcError):
        out.put_slice(1, slices[1])  # given twice
    out.put_slice(0, slices[0])
    with pytest.raises(lib.SfxcError):
        out.put_slice(0, slices[0])  # already written
    with pytest.raises(lib.SfxcError):
        out.put_slice(2, slices[2], 3)  # not three equal parts with file indices 0
    out.close()
    bad = bytearray(slices[2])
    bad[:4] = np.int32(5).tobytes()  # file 5 of 1
    out = correlator.OutputFiles(1, **_fields(HEADERS[0]))
    with pytest.raises(lib.SfxcError):
        out.put_slice(0, bytes(bad))
    out.close()


def test_sink_refusal_fails_the_output(sfxc_lib):
    """A sink that refuses one bin's file stops the slice part way: the files
    before it already hold their part, so the slice is not written again and
    every later call fails instead of duplicating those bytes."""
    from sfxc_gpu import correlator, lib
    g = Golden("pulsar")
    nbins = int(g.meta["pulsar"][0]) + 1
    per = len(g.cor) // nbins
    out = correlator.OutputFiles(nbins, refuse_files=(3,), **_fields(HEADERS[0]))
    with pytest.raises(lib.SfxcError):
        out.put_slice(0, g.cor, nbins)
    with pytest.raises(lib.SfxcError) as e:
        out.put_slice(1, g.cor, nbins)
    assert e.value.code == lib.ESTATE
    with pytest.raises(lib.SfxcError) as e:
        out.finish()
    assert e.value.code == lib.ESTATE
    header = bytes.fromhex(HEADERS[0]["header_hex"])
    for b in range(nbins):
        want = header + (g.cor[b * per + 4:(b + 1) * per] if b < 3 else b"")
        assert bytes(out.files[b]) == want, b
    out.close()
