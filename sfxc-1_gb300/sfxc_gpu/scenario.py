"""Seeded synthetic correlator jobs: delay tables, channel streams and input-node
protocols for a set of station streams, packaged as the job dicts consumed by
CorrelatorNode.correlate (and by the checkers in oracle/, which take the same
dicts).

A scenario describes one subband job: stations with delay polynomials and
gains, the streams (station x polarisation) with their sampling, and the
correlation setup.  Channel data are generated per polarisation with a common
sky signal (synth.generate_station_samples), quantised, packed LSB-first and
cut into input-node blocks; optional invalid runs mark blocks like invalid
VDIF frames.  The integer delays and the byte protocol come from pluggable
functions so the same scenario can be run through the reference's own input
node (oracle/jobs.py), the C restatement or this library.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import synth, timebase


@dataclass
class Station:
    name: str
    number: int
    poly: synth.DelayPoly
    gain: float = 1.0


@dataclass
class Scenario:
    stations: list
    pols: tuple = ("R",)
    sample_rate: int = 32_000_000
    bandwidth: int = 16_000_000
    bits: int = 2
    channel_freq: int = 1_600_000_000
    sideband: str = "U"
    station_sidebands: dict = field(default_factory=dict)  # station number -> sideband
    nchan: int = 512
    number_channels: int = 0            # output channels (spectral reduction); 0: nchan
    # extra phase centres: per centre, (source name, per-station delay offsets in seconds)
    extra_centers: list = field(default_factory=list)
    window: int = 4
    integration_us: int = 15625
    sub_integration_us: int = 125000
    n_integrations: int = 2
    lead_us: int = 4000                 # recording start -> first integration
    rho: float = 0.05
    seed: int = 1
    tones: list = field(default_factory=list)
    block_bytes: int = 32000            # channel bytes per input-node block
    invalid: dict = field(default_factory=dict)  # (station number, pol) -> [(block, begin, n)]
    mjd: int = 60000
    sec0: int = 36000                   # recording start, seconds of day
    lo_offset: float = 0.0
    tsys_freq: int = 80
    reference_station: int = -1
    frequency_nr: int = 0
    # station number -> (sample rate, bits, start of the station's band minus
    # the job's channel frequency in Hz); stations not listed record the
    # job's band at the job's rate (build_job_bulk only)
    station_modes: dict = field(default_factory=dict)

    def streams(self):
        """(station index, pol) in correlator order: stations outer, pols inner."""
        return [(si, pol) for si in range(len(self.stations)) for pol in self.pols]


def del_tables(sc: Scenario):
    """One .del per station: the scan of the pointing centre, then one scan
    per extra phase centre with the same start (its delays offset)."""
    out = []
    for si, st in enumerate(sc.stations):
        scans = [("SRC", sc.mjd, sc.sec0 - 20, 140, st.poly)]
        for name, offsets in sc.extra_centers:
            c = list(st.poly.coeffs)
            c[0] += offsets[si]
            poly = synth.DelayPoly(coeffs=tuple(c), t0=st.poly.t0, phase_coeffs=st.poly.phase_coeffs,
                                   amp=st.poly.amp)
            scans.append((name, sc.mjd, sc.sec0 - 20, 140, poly))
        out.append(synth.del_file_bytes(st.name[:2], scans))
    return out


def channel_streams(sc: Scenario, fast_random=False):
    """Packed channel bytes per stream, covering the job plus delay margins."""
    sr, bits = sc.sample_rate, sc.bits
    int_samples = sc.integration_us * sr // 1_000_000
    span = sc.lead_us * sr // 1_000_000 + sc.n_integrations * int_samples
    max_tau = max(abs(float(st.poly.delay(sc.sec0 + sc.lead_us * 1e-6))) for st in sc.stations)
    tail = int(max_tau * sr) + 4 * (sc.block_bytes * 8 // bits)
    nsamp = span + tail
    spb_block = sc.block_bytes * 8 // bits
    nsamp = (nsamp + spb_block - 1) // spb_block * spb_block
    out = {}
    for pi, pol in enumerate(sc.pols):
        if fast_random:
            rng = np.random.Generator(np.random.PCG64(sc.seed * 7919 + pi))
            for si in range(len(sc.stations)):
                out[(si, pol)] = rng.integers(0, 256, size=nsamp * bits // 8, dtype=np.uint8)
            continue
        sub = synth.SubbandSignal(sample_rate=sr, f_lo=float(sc.channel_freq), rho=sc.rho,
                                  seed=sc.seed * 100 + pi, tones=list(sc.tones))
        sigs = [synth.StationSignal(st.poly, st.gain) for st in sc.stations]
        xs = synth.generate_station_samples(sub, sigs, float(sc.sec0), nsamp)
        for si, x in enumerate(xs):
            out[(si, pol)] = synth.pack_codes(synth.quantise(x, bits), bits)
    return out, nsamp


def blocks_of(sc: Scenario, stream_bytes, key):
    """Input-node blocks of one channel stream: (start ticks, bytes, invalid runs)."""
    rec0 = timebase.ticks_from_mjd_sec(sc.mjd, sc.sec0)
    tps = timebase.ticks_per_sample(sc.sample_rate)
    spb_block = sc.block_bytes * 8 // sc.bits
    nb = len(stream_bytes) // sc.block_bytes
    inv = {}
    for (b, begin, n) in sc.invalid.get((sc.stations[key[0]].number, key[1]), []):
        inv.setdefault(b, []).append((begin, n))
    return [(rec0 + b * spb_block * tps, bytes(stream_bytes[b * sc.block_bytes:(b + 1) * sc.block_bytes]),
             inv.get(b, [])) for b in range(nb)]


def job_timing(sc: Scenario):
    rec0 = timebase.ticks_from_mjd_sec(sc.mjd, sc.sec0)
    start = rec0 + timebase.ticks_from_usec(sc.lead_us)
    tint = timebase.ticks_from_usec(sc.integration_us)
    nr = timebase.nr_ffts_per_integration_slice(sc.integration_us, sc.sample_rate, max(256, sc.nchan))
    slice_samples = nr * max(256, sc.nchan)
    return rec0, start, tint, slice_samples


def build_job(sc: Scenario, delay_fn, protocol_fn, fast_random=False):
    """Complete job dict.  delay_fn(del_bytes, s0, s1, sample_rate, bits) -> delay list;
    protocol_fn(blocks, slices, sample_rate, bits, integration_us) -> [bytes per slice]."""
    dels = del_tables(sc)
    chans, _ = channel_streams(sc, fast_random=fast_random)
    rec0, start, tint, slice_samples = job_timing(sc)
    streams, protos = [], []
    for k, (si, pol) in enumerate(sc.streams()):
        st = sc.stations[si]
        slices = []
        for it in range(sc.n_integrations):
            s0 = start + it * tint
            s1 = s0 + tint
            slices.append((s0, s1, slice_samples, delay_fn(dels[si], s0, s1, sc.sample_rate, sc.bits)))
        blocks = blocks_of(sc, chans[(si, pol)], (si, pol))
        protos.append(protocol_fn(blocks, slices, sc.sample_rate, sc.bits, sc.integration_us))
        sb = sc.station_sidebands.get(st.number, sc.sideband)
        # A station recording the job's sky band in the other sideband has its LO
        # at the opposite band edge (Delay_correction::set_parameters then finds
        # a zero channel offset, sfxc/src/delay_correction.cc:226-241).
        cf = sc.channel_freq
        if sb != sc.sideband:
            cf += sc.bandwidth if sc.sideband == "U" else -sc.bandwidth
        streams.append((st.number, k, sc.sample_rate, cf, sc.bandwidth, sb, pol, sc.bits,
                        sc.lo_offset, sc.tsys_freq, si))
    return dict(del_bytes=dels, experiment_start_ticks=rec0, start_ticks=start,
                integration_time_us=sc.integration_us, sub_integration_time_us=sc.sub_integration_us,
                number_channels=sc.number_channels or sc.nchan, fft_size_delaycor=256, fft_size_correlation=max(256, sc.nchan),
                sample_rate=sc.sample_rate, channel_freq=sc.channel_freq, bandwidth=sc.bandwidth,
                sideband=sc.sideband, frequency_nr=sc.frequency_nr, polarisation=sc.pols[0],
                cross_polarize=1 if len(sc.pols) > 1 else 0, reference_station=sc.reference_station,
                window=sc.window, source="SRC", integration_nr=0, n_integrations=sc.n_integrations,
                n_phase_centers=1 + len(sc.extra_centers), streams=streams, protocols=protos)


def bulk_stream_bytes(sc: Scenario, k=0):
    """Channel bytes build_job_bulk records for stream k (whole input-node
    blocks covering the lead, the integrations and the largest delay)."""
    si, _ = sc.streams()[k]
    sr_k, bits_k, _ = sc.station_modes.get(sc.stations[si].number, (sc.sample_rate, sc.bits, 0))
    max_tau = max(abs(float(st.poly.delay(sc.sec0 + sc.lead_us * 1e-6))) for st in sc.stations)
    spb_block = sc.block_bytes * 8 // bits_k
    span = sc.lead_us * sr_k // 1_000_000 + sc.n_integrations * (sc.integration_us * sr_k // 1_000_000)
    nsamp = span + int(max_tau * sr_k) + 4 * spb_block
    return (nsamp + spb_block - 1) // spb_block * sc.block_bytes


def build_job_bulk(sc: Scenario, alloc=None, codes=None):
    """Large jobs: uniformly random 2-bit/1-bit codes generated per stream and
    turned straight into protocol bytes by the library's input-node writer
    (no per-block Python objects).  alloc(n) may supply the protocol buffers
    (pinned host memory for end-to-end timing); codes(k, nbytes), if given,
    supplies stream k's channel bytes instead of the uniform codes (at least
    nbytes; e.g. the signal model of synth.model_codes_torch).  No invalid
    runs."""
    from . import correlator
    dels = del_tables(sc)
    rec0, start, tint, slice_samples = job_timing(sc)
    sr, bits = sc.sample_rate, sc.bits
    max_tau = max(abs(float(st.poly.delay(sc.sec0 + sc.lead_us * 1e-6))) for st in sc.stations)
    streams, protos = [], []
    for k, (si, pol) in enumerate(sc.streams()):
        st = sc.stations[si]
        sr_k, bits_k, off_k = sc.station_modes.get(st.number, (sr, bits, 0))
        bw_k = sc.bandwidth * sr_k // sr
        tps = timebase.ticks_per_sample(sr_k)
        spb_block = sc.block_bytes * 8 // bits_k
        span = sc.lead_us * sr_k // 1_000_000 + sc.n_integrations * (sc.integration_us * sr_k // 1_000_000)
        nsamp = span + int(max_tau * sr_k) + 4 * spb_block
        nblocks = (nsamp + spb_block - 1) // spb_block
        starts = rec0 + np.arange(nblocks, dtype=np.int64) * spb_block * tps
        if codes is not None:
            data = np.ascontiguousarray(codes(k, nblocks * sc.block_bytes)[:nblocks * sc.block_bytes])
        else:
            rng = np.random.Generator(np.random.PCG64(sc.seed * 7919 + k))
            data = rng.integers(0, 256, size=nblocks * sc.block_bytes, dtype=np.uint8)
        slices = []
        for it in range(sc.n_integrations):
            s0 = start + it * tint
            slices.append((s0, s0 + tint, slice_samples * sr_k // sr,
                           correlator.delay_list(dels[si], s0, s0 + tint, sr_k, bits_k)))
        protos.append(correlator.write_protocol_stream(data, sc.block_bytes, starts, slices, sr_k, bits_k,
                                                       sc.integration_us, alloc=alloc))
        streams.append((st.number, k, sr_k, sc.channel_freq + off_k, bw_k, sc.sideband, pol, bits_k, sc.lo_offset,
                        sc.tsys_freq, si))
    return dict(del_bytes=dels, experiment_start_ticks=rec0, start_ticks=start,
                integration_time_us=sc.integration_us, sub_integration_time_us=sc.sub_integration_us,
                number_channels=sc.number_channels or sc.nchan, fft_size_delaycor=256, fft_size_correlation=max(256, sc.nchan),
                sample_rate=sr, channel_freq=sc.channel_freq, bandwidth=sc.bandwidth, sideband=sc.sideband,
                frequency_nr=sc.frequency_nr, polarisation=sc.pols[0], cross_polarize=1 if len(sc.pols) > 1 else 0,
                reference_station=sc.reference_station, window=sc.window, source="SRC", integration_nr=0,
                n_integrations=sc.n_integrations, n_phase_centers=1 + len(sc.extra_centers), streams=streams,
                protocols=protos)


def c1_plain(integration_us=15625, n_integrations=2, seed=1):
    """The plain CPU-runnable configuration, shortened: 2 stations, 1 subband of
    16 MHz at 32 MS/s, 2-bit, single pol; station 2 delayed by 37.25 samples
    with a rate of 1e-7 s/s; sky frequency 1.6 GHz; 512 channels."""
    sr = 32_000_000
    st = [Station("Aa", 0, synth.DelayPoly(coeffs=(0.0,), t0=36000.0)),
          Station("Bb", 1, synth.DelayPoly(coeffs=(37.25 / sr, 1e-7), t0=36000.0))]
    return Scenario(stations=st, sample_rate=sr, bandwidth=16_000_000, bits=2, channel_freq=1_600_000_000,
                    nchan=512, integration_us=integration_us, n_integrations=n_integrations, rho=0.01,
                    seed=seed)


def cubic_stations(n, seed, max_delay=15e-3, max_rate=3e-6, t0=36000.0, gains=None):
    """n stations with seeded cubic delay polynomials (|tau| <= max_delay, |rate| <= max_rate)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        c0 = rng.uniform(-max_delay, max_delay)
        c1 = rng.uniform(-max_rate, max_rate)
        c2 = rng.uniform(-1e-9, 1e-9)
        c3 = rng.uniform(-1e-13, 1e-13)
        g = 1.0 if gains is None else gains[i]
        out.append(Station("S%d" % i, i, synth.DelayPoly(coeffs=(c0, c1, c2, c3), t0=t0), g))
    return out


def pulsar_params(sc: Scenario, nbins=256, gate=(0.0, 1.0), period=0.0334, dm=56.8, obs_freq=1400.0, n_coef=12):
    """Pulsar binning of a job (the ctrl file's pulsar block and one polyco):
    `nbins` on-pulse bins over `gate` plus the off-pulse bin, and one polyco
    of n_coef coefficients, all zero -- a constant spin frequency 1/period --
    with its midpoint at the job's first integration.  Returned as the job
    keys "pulsar" and "polyco"."""
    tmid = sc.mjd + (sc.sec0 + sc.lead_us * 1e-6) / 86400.0
    polyco = (tmid, dm, 0.0, 1.0 / period, obs_freq) + (0.0,) * n_coef
    return {"pulsar": (nbins,) + tuple(gate), "polyco": [polyco]}


def c5_pulsar(n_stations=10, integration_us=1_000_000, subband=0, seed=5, n_integrations=1):
    """The pulsar configuration's subband job: n_stations dual-pol stations at
    16 MHz (32 MS/s), 2-bit, 2048 channels, sky frequency 1.4 GHz + 16 MHz per
    subband, cubic delay models."""
    st = cubic_stations(n_stations, seed=500 + seed, max_delay=1e-2, max_rate=3e-6)
    return Scenario(stations=st, pols=("R", "L"), sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
                    channel_freq=1_400_000_000 + subband * 16_000_000, nchan=2048, integration_us=integration_us,
                    n_integrations=n_integrations, sub_integration_us=125000, lead_us=12000, seed=seed + subband,
                    block_bytes=2000, frequency_nr=subband)


def c4_jobs(scale=1.0, seed=11, subbands=(0, 1, 2, 3), fine_subbands=(0, 1), narrow_subbands=(0, 1)):
    """The batched uneven configuration's jobs of one timeslice (2 s x scale),
    on 20 stations with cubic delay models: 12 record 32 MHz at 64 MS/s
    2-bit, 6 record 64 MHz at 128 MS/s 2-bit, 2 record 16 MHz at 32 MS/s
    1-bit.  Three kinds of job, each its own integration time:
      A (one per entry of `subbands`): a 32 MHz subband at 64 MS/s with all
        20 stations dual-pol (40 streams: the 64 MHz stations correlated at
        twice the job rate, the 16 MHz ones at half of it over their part of
        the band), 4096 channels, 2 s integrations;
      B (fine_subbands): the 12 32-MHz stations, 16384 channels (windowed
        FFTs of 32768 samples), 0.5 s integrations;
      C (narrow_subbands): a 16 MHz subband at 32 MS/s with the 8 other
        stations (the 64 MHz ones at four times the job rate), 256 channels,
        0.25 s integrations.
    Returns [Scenario]; each job's integrations cover the timeslice."""
    st = cubic_stations(20, seed=900 + seed, max_delay=1e-2, max_rate=3e-6)
    span = int(round(2_000_000 * scale))
    out = []
    for sb in subbands:
        modes = {st[i].number: (128_000_000, 2, -32_000_000 if sb % 2 else 0) for i in range(12, 18)}
        modes.update({st[i].number: (32_000_000, 1, 16_000_000 if sb % 2 else 0) for i in range(18, 20)})
        iu = span
        out.append(Scenario(stations=st, pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                            channel_freq=4_800_000_000 + sb * 32_000_000, nchan=4096, integration_us=iu,
                            n_integrations=max(1, span // iu), sub_integration_us=125000, lead_us=12000,
                            seed=seed * 10 + sb, block_bytes=2000, frequency_nr=sb, station_modes=modes))
    for sb in fine_subbands:
        iu = max(1, span // 4)
        out.append(Scenario(stations=st[:12], pols=("R", "L"), sample_rate=64_000_000, bandwidth=32_000_000, bits=2,
                            channel_freq=4_800_000_000 + sb * 32_000_000, nchan=16384, integration_us=iu,
                            n_integrations=max(1, span // iu), sub_integration_us=125000, lead_us=12000,
                            seed=seed * 10 + 5 + sb, block_bytes=2000, frequency_nr=8 + sb))
    for sb in narrow_subbands:
        iu = max(1, span // 8)
        modes = {st[i].number: (128_000_000, 2, -16_000_000 * (sb % 4)) for i in range(12, 18)}
        modes.update({st[i].number: (32_000_000, 1, 0) for i in range(18, 20)})
        out.append(Scenario(stations=st[12:], pols=("R", "L"), sample_rate=32_000_000, bandwidth=16_000_000, bits=2,
                            channel_freq=4_800_000_000 + sb * 16_000_000, nchan=256, integration_us=iu,
                            n_integrations=max(1, span // iu), sub_integration_us=125000, lead_us=12000,
                            seed=seed * 10 + 7 + sb, block_bytes=2000, frequency_nr=16 + sb, station_modes=modes))
    return out
