"""The UVW model on seeded random tables and probes, against the reference's
own Uvw_model (sfxc/src/uvw_model.cc:79-330) run live: baselines from a few
metres to continental, declinations and hour angles across the sky, two or
three scans (two phase centres sharing a start, a later scan; 6 to 30 rows
each), and probe sequences that walk forward through fractional and whole
seconds, land on scan edges, jump between scans and step back -- past the
start of the spline's window too, where GSL 1.9's evaluation extends the
first interval's cubic.  The library's sfxc_gpu_uvw_get must give the
reference's u, v, w bit for bit.  Host code only; needs the reference
checkout."""
import numpy as np
import pytest

N_TABLES = 30


def random_case(seed):
    from sfxc_gpu import synth, timebase
    rng = np.random.Generator(np.random.PCG64(9000 + seed))
    mjd, sec0 = 60200 + int(rng.integers(0, 300)), int(rng.integers(100, 80000))
    poly = synth.DelayPoly(coeffs=(float(rng.uniform(-5e-3, 5e-3)), float(rng.uniform(-3e-6, 3e-6)), 0.0, 0.0),
                           t0=sec0, phase_coeffs=(0.0,), amp=1.0)
    scale = float(10 ** rng.uniform(0, 6.8))
    b = tuple(float(x) for x in rng.uniform(-1, 1, size=3) * scale)
    dec, h0 = float(rng.uniform(-1.4, 1.4)), float(rng.uniform(-3, 3))
    n1 = int(rng.integers(6, 31))  # at least the five rows of a spline window
    scans = [("SRC1", mjd, sec0, n1, poly, synth.earth_rotation_uvw(b, dec, h0))]
    centres = 1
    if rng.random() < 0.6:
        scans.append(("SRC2", mjd, sec0, n1, poly, synth.earth_rotation_uvw(b, dec + 0.02, h0 - 0.01)))
        centres = 2
    gap = int(rng.integers(1, 20))
    n2 = int(rng.integers(6, 31))
    scans.append(("SRC3", mjd, sec0 + n1 + gap, n2, poly, synth.earth_rotation_uvw(b, dec - 0.2, h0 + 0.3)))
    del_bytes = synth.del_file_bytes("Xx", scans)
    probes = []
    latest = t = float(sec0) + float(rng.uniform(0, 1))
    for _ in range(40):
        r = rng.random()
        if r < 0.55:
            t += float(rng.choice([0.125, 0.25, 0.5, 1.0, 0.0625]))
        elif r < 0.7:
            t = float(np.floor(t)) + 1.0  # a whole second
        elif r < 0.8:
            t = float(sec0 + n1 + gap + rng.integers(0, n2))  # into the later scan
        elif r < 0.9:
            t -= float(rng.uniform(0, 3))  # a step back
        else:
            t = float(sec0 + n1) - 0.03125  # the end of the first scan
        t = min(max(t, float(sec0)), float(sec0 + n1 + gap + n2 - 1))  # the last row of the last scan
        latest = max(latest, t)
        # the second centre only while the model is still on the first scan
        # (it is rebuilt only for later times; asking a scan of one centre
        # for a second one is an error)
        pc = int(rng.integers(0, centres)) if latest < sec0 + n1 - 1 else 0
        probes.append((pc, timebase.ticks_from_mjd_sec(mjd, t)))
    return del_bytes, probes


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


@pytest.mark.parametrize("seed", range(N_TABLES))
def test_uvw_model_matches_reference(seed, reference_available, sfxc_lib):
    from oracle import jobs
    from sfxc_gpu import correlator
    del_bytes, probes = random_case(seed)
    want = jobs.uvw(del_bytes, probes)
    m = correlator.UvwModel(del_bytes)
    try:
        got = [tuple(m.get(pc, t)) for pc, t in probes]
    finally:
        m.close()
    assert got == want
