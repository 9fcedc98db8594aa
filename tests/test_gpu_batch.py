"""Batches: the jobs of a timeslice -- uneven in stream count, sample rate, bit
depth, FFT length and integration time -- correlated together, their device
work one CUDA graph per run (sfxc_gpu_batch_*), and the autotuner.

Bars: a batch gives byte-identical output to the same jobs run one by one
through sfxc_gpu_run_integration, on both X-step forms, also with several
integrations of one job in one graph, and with timeslices in flight on
two batches from two host threads; on the batched uneven configuration's
shape (20 stations: 32 MHz 2-bit, 64 MHz 2-bit at twice the job rate, 16 MHz
1-bit at half of it; 4096-, 16384- and 256-channel jobs with integration
times in the ratio 8:2:1) every job's visibilities are within relative L2
1e-5 of the FP32 restatement (FP32 X-step) and within 1e-4 of the FP64
restatement (both forms), headers and tsys records exact; autotuning leaves
every output byte unchanged."""
import pytest

from golden_io import compare_cor, parse_cor, rel_err

pytestmark = pytest.mark.gpu

MODES = ["fp32", "tc"]


def _mode(m):
    from sfxc_gpu import lib
    return lib.X_FP32 if m == "fp32" else lib.X_TC_HILO


def _job(sc):
    from sfxc_gpu import scenario
    job = scenario.build_job_bulk(sc)
    job["protocols"] = [[bytes(p) for p in prs] for prs in job["protocols"]]
    return job


@pytest.fixture(scope="module")
def c4_case(oracle_exe):
    """The uneven configuration at 1/250 scale: an 8 ms timeslice of one
    4096-channel job (1 integration), one 16384-channel job (4 of 2 ms) and
    one 256-channel job (8 of 1 ms)."""
    from oracle import jobs
    from sfxc_gpu import scenario
    scs = scenario.c4_jobs(scale=1 / 250, subbands=(1,), fine_subbands=(0,), narrow_subbands=(1,))
    built = [_job(sc) for sc in scs]
    refs = [(jobs.correlate(j, impl="oracle"), jobs.correlate(j, impl="oracle", precision=64)) for j in built]
    return built, refs


@pytest.mark.parametrize("mode", MODES)
def test_c4_batch_vs_restatement(mode, c4_case, sfxc_lib):
    from sfxc_gpu import correlator
    built, refs = c4_case
    nodes = [correlator.CorrelatorNode(0, _mode(mode)) for _ in built]
    batch = correlator.Batch(nodes)
    try:
        outs = batch.correlate(built)  # every job's whole timeslice in one graph
    finally:
        batch.close()
        for n in nodes:
            n.close()
    for job, (cor, tsys), (r32, r64) in zip(built, outs, refs):
        M = job["fft_size_correlation"]
        assert tsys == r32["tsys"]
        e32 = compare_cor(cor, r32["cor"], M, 1e-5 if mode == "fp32" else 1e-4)
        _, vg = parse_cor(cor, M)
        vis64 = r64["vis64"].reshape(len(vg), M + 1)
        e64 = max(rel_err(a, b) for a, b in zip(vg, vis64))
        print("C4 job M=%d, %d streams, %d integrations, %s: vs FP32 %.3g, vs FP64 %.3g"
              % (M, len(job["streams"]), job["n_integrations"], mode, e32, e64))
        assert e64 <= 1e-4


@pytest.mark.parametrize("mode", MODES)
def test_batch_equals_single_runs(mode, c4_case, sfxc_lib):
    """Batch output byte for byte equal to the jobs run one by one, in one
    integration per graph and all integrations in one graph."""
    from sfxc_gpu import correlator
    built, _ = c4_case
    single = []
    for job in built:
        node = correlator.CorrelatorNode(0, _mode(mode))
        try:
            single.append(node.correlate(job))
        finally:
            node.close()
    for per_run in ([1] * len(built), None):
        nodes = [correlator.CorrelatorNode(0, _mode(mode)) for _ in built]
        batch = correlator.Batch(nodes)
        try:
            outs = batch.correlate(built, per_run=per_run)
            outs2 = batch.correlate(built, per_run=per_run)  # the executable graph reused
        finally:
            batch.close()
            for n in nodes:
                n.close()
        assert outs == single
        assert outs2 == single


@pytest.mark.parametrize("mode", MODES)
def test_batches_in_flight_equal_single_runs(mode, c4_case, sfxc_lib):
    """Consecutive timeslices on two batches from two host threads (set-ups
    one at a time under a shared lock, each graph captured and run beside the
    other batch's): every timeslice byte for byte equal to the jobs run one
    by one."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    from sfxc_gpu import correlator
    built, _ = c4_case
    single = []
    for job in built:
        node = correlator.CorrelatorNode(0, _mode(mode))
        try:
            single.append(node.correlate(job))
        finally:
            node.close()
    sets = [[correlator.CorrelatorNode(0, _mode(mode)) for _ in built] for _ in range(2)]
    batches = [correlator.Batch(nodes) for nodes in sets]
    lock = threading.Lock()
    try:
        with ThreadPoolExecutor(max_workers=2) as ex:
            futs, outs = [], []
            for i in range(6):  # timeslice i on batch i % 2, once timeslice i - 2 is done
                if len(futs) == 2:
                    outs.append(futs.pop(0).result())
                futs.append(ex.submit(batches[i % 2].correlate, built, [1] * len(built) if i % 3 == 2 else None,
                                      lock))
            outs += [f.result() for f in futs]
    finally:
        for b in batches:
            b.close()
        for nodes in sets:
            for n in nodes:
                n.close()
    for i, o in enumerate(outs):
        assert o == single, "timeslice %d" % i


def test_autotune_keeps_every_byte(sfxc_lib):
    from sfxc_gpu import correlator, lib, scenario
    st = scenario.cubic_stations(6, seed=61, max_delay=1e-3, max_rate=1e-6)
    sc = scenario.Scenario(stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                           channel_freq=4_800_000_000, nchan=4096, integration_us=20000, n_integrations=1,
                           sub_integration_us=10000, lead_us=12000, seed=62, block_bytes=2000)
    job = _job(sc)
    for mode in (lib.X_FP32, lib.X_TC_HILO):
        node = correlator.CorrelatorNode(0, mode)
        try:
            before = node.correlate(job)
            assert node.autotune(2) >= 2  # the block stage and one windowed-FFT length
            after = node.correlate(job)
        finally:
            node.close()
        assert after == before
    kinds = {e[0] for e in correlator.plan_cache()}
    assert kinds == {0, 1}
