"""The Correlator_node adapter a maintainer adds to the reference
(sfxc-1_gb300/adapter/correlator_node_gpu.h) compiled against the reference's
own headers with its own flags, linked with the reference's compiled classes
and libsfxc_gpu.so (oracle/build_adapter.py), and driven by tests/adapter_main.cc
with the reference's Correlation_parameters filled as a correlator node
receives them.

Bars: it builds and links; the sfxc_correlation_params it hands the library
equal, field by field, those the library's own binding builds from the same
job (streams, delay tables, pulsar gate and polycos, mask, phase centres);
without a GPU the library refuses to create a context and the adapter stops
through the reference's sfxc_abort, as the reference does on errors.  Needs
the reference checkout (skipped without it); no GPU."""
import os
import subprocess
import tempfile

import pytest

from golden_io import Golden


def _expected(job):
    from sfxc_gpu import correlator
    p, _keep = correlator.correlation_params(job)
    exp = {
        "experiment_start_ticks": [p.experiment_start_ticks], "start_ticks": [p.start_ticks],
        "integration_time_us": [p.integration_time_us], "sub_integration_time_us": [p.sub_integration_time_us],
        "number_channels": [p.number_channels], "fft_size_delaycor": [p.fft_size_delaycor],
        "fft_size_correlation": [p.fft_size_correlation], "sample_rate": [p.sample_rate],
        "bandwidth": [p.bandwidth], "frequency_nr": [p.frequency_nr], "channel_freq": [p.channel_freq],
        "sideband": [p.sideband[0]], "polarisation": [p.polarisation[0]], "cross_polarize": [p.cross_polarize],
        "reference_station": [p.reference_station], "window": [p.window], "integration_nr": [p.integration_nr],
        "n_streams": [p.n_streams], "n_delay_tables": [p.n_delay_tables], "pulsar_nbins": [p.pulsar_nbins],
        "gate": [p.gate_start, p.gate_stop] if p.pulsar_nbins else [0.0, 0.0], "n_polyco": [p.n_polyco],
        "n_phase_centers": [p.n_phase_centers], "phased_array": [p.phased_array]}
    streams = []
    for i in range(p.n_streams):
        s = p.streams[i]
        streams.append([s.station_number, s.station_stream, s.sample_rate, s.bandwidth, s.bits_per_sample,
                        s.tsys_freq, s.channel_freq, s.sideband[0], s.polarisation[0], s.delay_table, s.lo_offset])
    tables = [[i, p.delay_tables[i].del_size] for i in range(p.n_delay_tables)]
    polyco = []
    for i in range(p.n_polyco):
        q = p.polyco[i]
        polyco.append([q.tmid, q.dm, q.ref_phase, q.ref_freq, q.obs_freq, q.n_coef] +
                      [q.coef[e] for e in range(q.n_coef)])
    M, n = job["fft_size_correlation"], job["number_channels"]
    mask = [M + 1 if job.get("mask") is not None and n < M else 0,
            2 * n if job.get("lag_window") is not None and n < M else 0, p.mask_normalize]
    return exp, streams, tables, polyco, mask


def _parse(path):
    out, streams, tables, polyco, mask = {}, [], [], [], None
    for line in open(path):
        v = line.split()
        if v[0] == "mask":
            mask = [int(v[1]), int(v[3]), int(v[5])]
            continue
        num = [float(x) if any(c in x for c in ".en") else int(x) for x in v[1:]]
        if v[0] == "stream":
            streams.append(num)
        elif v[0] == "delay_table":
            tables.append(num)
        elif v[0] == "polyco":
            polyco.append(num)
        else:
            out[v[0]] = num
    return out, streams, tables, polyco, mask


@pytest.fixture(scope="module")
def adapter_exe(sfxc_lib):
    from oracle import build_adapter
    exe = build_adapter.build()
    if exe is None:
        pytest.skip("reference checkout not available")
    return exe


@pytest.mark.parametrize("case", ["multi", "pulsar", "reduced_mask", "phase_centers"])
def test_adapter_flattens_like_the_binding(case, adapter_exe):
    from oracle import jobs
    from sfxc_gpu import correlator
    g = Golden(case)
    job = g.job(correlator.write_protocol)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "adapter.job")
        with open(path, "w") as f:
            for key, *vals in jobs.correlate_lines(job, d):
                f.write(key + " " + " ".join(str(v) for v in vals) + "\n")
        out = os.path.join(d, "out")
        os.makedirs(out)
        r = subprocess.run([adapter_exe, path, out, "1"], capture_output=True, text=True, timeout=120)
        got = _parse(os.path.join(out, "params.txt"))
    exp, streams, tables, polyco, mask = _expected(job)
    for k, v in exp.items():
        assert got[0][k] == pytest.approx(v, rel=0, abs=0), k
    assert got[1] == streams
    assert got[2] == tables
    assert got[3] == polyco
    assert got[4] == mask
    # no GPU here: the library refuses the context and the adapter aborts
    # through the reference's sfxc_abort, with the library's message
    assert r.returncode != 0
    assert "reference abort:" in r.stderr and "CUDA" in r.stderr, r.stderr
