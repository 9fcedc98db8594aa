"""Stations whose data are missing: one whose every input-node block is
invalid, one that drops out half-way through the first of two integrations.

The input-node writer then sends HEADER_INVALID records
(sfxc/src/input_node_data_writer.cc:436-462), the correlator node zero-fills
those samples (sfxc/src/bit2float_worker.cc:327-425) and the core meets zero
power and zero weights: autocorrelation norms max(1, mean power) and cross
norms of 1 where the flagged fractions leave less than 1 %
(Correlation_core::integration_normalize, sfxc/src/correlation_core.cc:275-314),
baseline weights from the merged invalid lists (find_invalid, 599-665).

The reference is pinned on what it defines.  Its Bit2float_worker never
initialises `bytes_left` (the constructor, bit2float_worker.cc:11-21, and
set_parameters, 280-313, leave it and `state` as they are), and only a
HEADER_DATA record sets it (61-62).  A stream whose first integration holds
no data record reaches the end-of-integration purge (152-176) with an
indeterminate `bytes_left`, which then swallows the next integration's bytes
and spins with nothing left to read.  So the wholly erased station is compared
with the reference over one integration, the drop-out over two; the library
and the restatement purge up to the end-of-stream record in either case.

CPU: the C restatement against the reference's own classes.
GPU: both X-step forms through the C ABI against the restatement.
"""
import numpy as np
import pytest

from golden_io import compare_cor, parse_cor

NCHAN = 512
BLOCK_BYTES = 4000  # 16,000 2-bit samples: 0.5 ms at 32 MS/s


def erased_scenario(n_integrations=2, whole=True, dropout=True):
    from sfxc_gpu import scenario
    st = scenario.cubic_stations(3, seed=61, max_delay=2e-3, max_rate=1e-5)
    invalid = {}
    if whole:  # station 1's R stream: no data at all
        invalid[(st[1].number, "R")] = [(b, 0, BLOCK_BYTES) for b in range(200)]
    if dropout:
        # the job starts 3 ms (block 6) into the recording; 8 ms integrations
        # are 16 blocks: from block 14 on, station 2's L stream has no data
        invalid[(st[2].number, "L")] = [(b, 0, BLOCK_BYTES) for b in range(14, 200)]
    return scenario.Scenario(
        stations=st, pols=("R", "L"), sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
        channel_freq=1_600_000_000, nchan=NCHAN, integration_us=8000, n_integrations=n_integrations,
        sub_integration_us=2000, lead_us=3000, rho=0.05, seed=37, block_bytes=BLOCK_BYTES, invalid=invalid)


def _check_structure(cor, zero_vectors):
    """No NaN or infinity anywhere, and exactly the visibility vectors of
    streams without data in an integration all zero: per such stream its
    autocorrelation and its four cross baselines (six streams, cross
    polarisations, none within a station)."""
    _, vis = parse_cor(cor, NCHAN)
    assert all(np.isfinite(v).all() for v in vis)
    assert sum(1 for v in vis if not v.any()) == zero_vectors


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


@pytest.mark.parametrize("variant,zeros", [(dict(n_integrations=1), 5), (dict(n_integrations=2, whole=False), 5)],
                         ids=["erased-one-integration", "dropout-two-integrations"])
def test_restatement_matches_reference(reference_available, variant, zeros):
    from oracle import jobs
    from sfxc_gpu import scenario

    def delays(*a):
        return jobs.delays(*a)[0]

    job = scenario.build_job(erased_scenario(**variant), delays, jobs.protocol)
    ref = jobs.correlate(job, impl="reference")
    mine = jobs.correlate(job, impl="oracle")
    assert mine["tsys"] == ref["tsys"]
    assert mine["stats"] == ref["stats"]
    compare_cor(mine["cor"], ref["cor"], NCHAN, 1e-6)
    _check_structure(ref["cor"], zeros)


def test_restatement_two_integrations_of_an_erased_station(oracle_exe):
    """Where the reference's behaviour is undefined, the restatement carries
    on: the erased station's vectors are zero in both integrations, and in
    the second those of the stream that dropped out too (5 + 9, the baseline
    of the two counted once)."""
    from oracle import jobs
    from sfxc_gpu import correlator, scenario
    job = scenario.build_job(erased_scenario(), correlator.delay_list, correlator.write_protocol)
    res = jobs.correlate(job, impl="oracle")
    _check_structure(res["cor"], 14)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp32", "tc"])
def test_gpu_matches_restatement(mode, sfxc_lib):
    from oracle import jobs
    from sfxc_gpu import correlator, lib, scenario
    job = scenario.build_job(erased_scenario(), correlator.delay_list, correlator.write_protocol)
    ref = jobs.correlate(job, impl="oracle")
    node = correlator.CorrelatorNode(0, lib.X_FP32 if mode == "fp32" else lib.X_TC_HILO)
    try:
        cor, tsys = node.correlate(job)
    finally:
        node.close()
    assert tsys == ref["tsys"]
    compare_cor(cor, ref["cor"], NCHAN, 1e-5)
    _check_structure(cor, 14)
