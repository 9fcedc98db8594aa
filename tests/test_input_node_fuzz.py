"""The input node's integer delays and protocol bytes on seeded random set-ups,
against the reference's own classes: Input_node_tasklet::get_delays
(sfxc/src/input_node_tasklet.cc:235-282) and Input_node_data_writer::do_task
(sfxc/src/input_node_data_writer.cc:107-229), the library's
sfxc_gpu_delay_list and sfxc_gpu_write_protocol, and the restatement's input
node (which feeds the CPU baseline).

Each set-up draws a sample rate and bit depth, block size, delay polynomials
with rates up to 5e-5 (many integer-delay changes per slice, both signs),
the integration length and invalid runs in random blocks (whole blocks,
runs at either edge, several runs in one block).  Delay lists must be equal
entry for entry and every slice's protocol byte for byte.  Needs the
reference checkout."""
import numpy as np
import pytest

N_SETUPS = 24


def random_scenario(seed):
    from sfxc_gpu import scenario
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    sr, bits = [(16_000_000, 2), (32_000_000, 2), (64_000_000, 2), (32_000_000, 1), (64_000_000, 1)][
        int(rng.integers(0, 5))]
    max_delay = float(rng.uniform(1e-4, 8e-3))
    st = scenario.cubic_stations(3, seed=seed, max_delay=max_delay, max_rate=float(rng.uniform(1e-7, 5e-5)))
    block_bytes = int(rng.choice([1000, 2000, 4000, 8000]))
    nblocks_guess = 400
    invalid = {}
    for s in st:
        runs = []
        for b in rng.choice(nblocks_guess, size=int(rng.integers(0, 12)), replace=False):
            kind = int(rng.integers(0, 4))
            if kind == 0:
                runs.append((int(b), 0, block_bytes))
            elif kind == 1:
                runs.append((int(b), 0, int(rng.integers(1, block_bytes))))
            elif kind == 2:
                n = int(rng.integers(1, block_bytes))
                runs.append((int(b), block_bytes - n, n))
            else:
                a = int(rng.integers(0, block_bytes // 2))
                runs.append((int(b), a, int(rng.integers(1, block_bytes // 4))))
                c = int(rng.integers(block_bytes // 2 + 1, block_bytes))
                runs.append((int(b), c, int(rng.integers(1, block_bytes - c + 1))))
        invalid[(s.number, "R")] = sorted(runs)
    integration_us = int(rng.choice([4000, 8000, 15625]))
    return scenario.Scenario(
        stations=st, sample_rate=sr, bandwidth=sr // 2, bits=bits, channel_freq=1_600_000_000, nchan=512,
        integration_us=integration_us, n_integrations=2, sub_integration_us=integration_us,
        lead_us=int(max_delay * 1e6) + int(rng.integers(1000, 4000)), seed=seed, block_bytes=block_bytes,
        invalid=invalid)


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


def _parts(seed, delay_fn, protocol_fn):
    """Every stream's delay list and protocol bytes of each slice."""
    from sfxc_gpu import scenario
    sc = random_scenario(seed)
    lists = []

    def delays(*a):
        dl = delay_fn(*a)
        lists.append(dl)
        return dl

    job = scenario.build_job(sc, delays, protocol_fn, fast_random=True)
    return lists, job["protocols"]


@pytest.mark.parametrize("seed", range(N_SETUPS))
def test_delays_and_protocol_match_reference(seed, reference_available, sfxc_lib):
    from oracle import jobs
    from sfxc_gpu import correlator

    ref = _parts(seed, lambda *a: jobs.delays(*a)[0], jobs.protocol)
    lib = _parts(seed, correlator.delay_list, correlator.write_protocol)
    port = _parts(seed, lambda *a: jobs.delays(*a, impl="oracle")[0],
                  lambda *a: jobs.protocol(*a, impl="oracle"))
    assert sum(len(d) for d in ref[0]) > len(ref[0])  # delay changes inside the slices
    assert lib[0] == ref[0] and port[0] == ref[0]
    assert lib[1] == ref[1]
    assert port[1] == ref[1]
