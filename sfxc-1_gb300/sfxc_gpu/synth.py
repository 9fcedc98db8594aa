"""Seeded synthetic VLBI station data: delay tables, quantised samples, VDIF frames.

The reference ships no station recordings, so every workload is generated.
Signal model (one subband, one polarisation):

    x_i(t) = g_i * [ sqrt(rho) * Re{ a(T) exp(-2 pi i f_lo tau_i(T)) } + sqrt(1-rho) * n_i(t) ]

where a is the analytic signal of a white band-limited Gaussian sky signal s,
T solves T + tau_i(T) = t (the station sees the wavefront tau_i later), n_i is
independent white noise, and f_lo is the subband's sky frequency at baseband
zero.  Correlating x_i at t = T + tau_i(T) -- which is what the correlator's
integer shift plus fractional-delay / fringe-rotation do with the delay table
written here -- recovers the common signal with a stationary phase.

Samples are quantised like a VLBI digitiser: 2-bit offset-binary codes at
thresholds {-0.98 sigma, 0, +0.98 sigma} (codes 0..3 map to -7,-2,+2,+7 in the
reference's unpack tables, sfxc/src/bit2float_worker.cc:4-10), or 1-bit sign
codes.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

from . import timebase

THRESH_2BIT = 0.98


# --------------------------------------------------------------------------
# delay tables (.del files; layout of sfxc/utils/delay/generate_delay_model_calc.c:440-467,636-642,
# read by Delay_table::open, sfxc/src/delay_table_akima.cc:238-372)
# --------------------------------------------------------------------------
@dataclass
class DelayPoly:
    """tau(t) = sum_k c[k] * (t - t0)^k seconds, t in seconds of day; phase and amplitude columns."""
    coeffs: tuple = (0.0,)
    t0: float = 0.0
    phase_coeffs: tuple = (0.0,)
    amp: float = 1.0

    def delay(self, sec_of_day):
        x = np.asarray(sec_of_day, dtype=np.float64) - self.t0
        r = np.zeros_like(x)
        for c in reversed(self.coeffs):
            r = r * x + c
        return r

    def phase(self, sec_of_day):
        x = np.asarray(sec_of_day, dtype=np.float64) - self.t0
        r = np.zeros_like(x)
        for c in reversed(self.phase_coeffs):
            r = r * x + c
        return r


def del_file_bytes(station: str, scans) -> bytes:
    """scans: list of (source, mjd, sec_start, n_rows, DelayPoly[, uvw]) with
    1-s row spacing; uvw(sec) -> (u, v, w) in metres fills those columns
    (zero without it)."""
    out = bytearray()
    name = station.encode()[:2].ljust(2, b"\0") + b"\0"
    out += struct.pack("<i", 3) + name
    for scan in scans:
        source, mjd, sec_start, n_rows, poly = scan[:5]
        uvw = scan[5] if len(scan) > 5 else None
        src = source.encode()[:80].ljust(80, b" ") + b"\0"
        out += src + struct.pack("<i", mjd)
        for k in range(n_rows):
            sec = float(sec_start + k)
            d = float(poly.delay(sec))
            ph = float(poly.phase(sec))
            u, v, w = (float(x) for x in uvw(sec)) if uvw else (0.0, 0.0, 0.0)
            out += struct.pack("<7d", sec, u, v, w, d, ph, poly.amp)
        out += struct.pack("<7d", *([0.0] * 7))
    return bytes(out)


def earth_rotation_uvw(baseline_m, dec, h0):
    """u, v, w (metres) of a station `baseline_m` (x, y, z) from the array
    centre towards a source at declination dec (rad), hour angle h0 + Earth
    rotation at sec 0: the textbook projection, as a smooth test model."""
    bx, by, bz = baseline_m

    def f(sec):
        h = h0 + 7.2921150e-5 * sec
        u = bx * math.sin(h) + by * math.cos(h)
        v = -bx * math.sin(dec) * math.cos(h) + by * math.sin(dec) * math.sin(h) + bz * math.cos(dec)
        w = bx * math.cos(dec) * math.cos(h) - by * math.cos(dec) * math.sin(h) + bz * math.sin(dec)
        return u, v, w
    return f


# --------------------------------------------------------------------------
# signal generation
# --------------------------------------------------------------------------
@dataclass
class StationSignal:
    poly: DelayPoly
    gain: float = 1.0
    sideband: str = "U"


@dataclass
class SubbandSignal:
    """Synthesis parameters shared by all stations of one subband/polarisation."""
    sample_rate: int
    f_lo: float                 # sky frequency of baseband zero (Hz)
    rho: float = 0.01           # correlated power fraction
    seed: int = 0
    tones: list = field(default_factory=list)   # [(baseband_freq_hz, amplitude_in_sigma)], common RFI


def _inverse_delay_time(t_abs, poly: DelayPoly, mjd_sec_offset: float):
    """Solve T + tau(T) = t (seconds of day) by fixed-point iteration."""
    T = t_abs - poly.delay(t_abs)
    for _ in range(4):
        T = t_abs - poly.delay(T)
    return T


def generate_station_samples(sub: SubbandSignal, stations: list, start_sec_of_day: float,
                             n_samples: int, block: int = 8192, pad: int = 512):
    """Real-valued station signals x_i(t) (float32 arrays, unit-ish variance).

    start_sec_of_day: time of sample 0 (identical for all stations: the
    recording start).  The common sky signal is drawn on a grid wide enough to
    cover every station's shift.
    """
    sr = sub.sample_rate
    rng = np.random.Generator(np.random.PCG64(sub.seed))
    t_samples = start_sec_of_day + np.arange(n_samples, dtype=np.float64) / sr
    # total shift range (samples) to size the sky-signal grid
    max_tau = max(float(np.max(np.abs(st.poly.delay(t_samples[[0, -1]])))) for st in stations)
    margin = int(max_tau * sr) + 4 * pad + block
    n_sky = n_samples + 2 * margin
    sky = rng.standard_normal(n_sky).astype(np.float64)
    sky0 = margin  # sky index of T = start_sec_of_day
    out = []
    for si, st in enumerate(stations):
        nrng = np.random.Generator(np.random.PCG64(sub.seed * 1000 + 17 + si))
        x = np.empty(n_samples, dtype=np.float64)
        for b0 in range(0, n_samples, block):
            b1 = min(n_samples, b0 + block)
            t = t_samples[b0:b1]
            T = _inverse_delay_time(t, st.poly, 0.0)
            # sample position of T on the sky grid (fractional)
            pos = (T - start_sec_of_day) * sr + sky0
            centre = 0.5 * (pos[0] + pos[-1])
            shift = centre - (b0 + (b1 - b0 - 1) * 0.5 + sky0)
            ishift = int(math.floor(shift))
            frac = shift - ishift
            lo = b0 + sky0 + ishift - pad
            seg = sky[lo:lo + (b1 - b0) + 2 * pad]
            L = seg.size
            F = np.fft.rfft(seg)
            f = np.arange(F.size) / L
            # analytic signal of the segment, advanced by frac samples
            A = np.zeros(L, dtype=np.complex128)
            A[:F.size] = F * 2.0
            A[0] = F[0]
            if L % 2 == 0:
                A[L // 2] = F[L // 2]
            A[:F.size] *= np.exp(2j * np.pi * f * frac)
            a = np.fft.ifft(A)[pad:pad + (b1 - b0)]
            # small residual drift of the shift across the block: linear correction
            resid = pos - (np.arange(b0, b1) + sky0 + shift)
            # derivative approximation of a for the residual (first order)
            da = np.gradient(a)
            a = a + da * resid
            phase = -2.0 * np.pi * sub.f_lo * st.poly.delay(T)
            sig = np.real(a * np.exp(1j * phase))
            noise = nrng.standard_normal(b1 - b0)
            xs = math.sqrt(sub.rho) * sig + math.sqrt(1.0 - sub.rho) * noise
            for (ftone, amp) in sub.tones:
                xs = xs + amp * np.cos(2 * np.pi * ftone * (t - start_sec_of_day))
            x[b0:b1] = st.gain * xs
        out.append(x.astype(np.float32))
    return out


def quantise(x: np.ndarray, bits: int) -> np.ndarray:
    """Digitiser codes (uint8): 2-bit offset binary at +-0.98 sigma, or 1-bit sign."""
    sigma = float(np.std(x.astype(np.float64)))
    if bits == 2:
        t = THRESH_2BIT * sigma
        return (np.digitize(x, [-t, 0.0, t])).astype(np.uint8)
    if bits == 1:
        return (x >= 0).astype(np.uint8)
    raise ValueError("bits must be 1 or 2")


def pack_codes(codes: np.ndarray, bits: int) -> np.ndarray:
    """Channel stream bytes: samples packed LSB-first (first sample in the lowest bits)."""
    spb = 8 // bits
    n = codes.size - codes.size % spb
    c = codes[:n].astype(np.uint8).reshape(-1, spb)
    out = np.zeros(c.shape[0], dtype=np.uint8)
    for k in range(spb):
        out |= (c[:, k] << (k * bits)).astype(np.uint8)
    return out


def unpack_codes(stream: np.ndarray, bits: int) -> np.ndarray:
    spb = 8 // bits
    mask = (1 << bits) - 1
    s = np.asarray(stream, dtype=np.uint8)
    return np.stack([(s >> (k * bits)) & mask for k in range(spb)], axis=1).reshape(-1)


# --------------------------------------------------------------------------
# VDIF framing (sfxc/include/vdif_reader.h:36-61)
# --------------------------------------------------------------------------
VDIF_HEADER_BYTES = 32


def vdif_ref_epoch(mjd: int) -> tuple:
    """(ref_epoch, mjd of that epoch): half-years since 2000 containing mjd."""
    best = (0, timebase.mjd_from_date(1, 1, 2000))
    for e in range(0, 64):
        y = 2000 + e // 2
        m = 1 + 6 * (e % 2)
        em = timebase.mjd_from_date(1, m, y)
        if em <= mjd:
            best = (e, em)
    return best


def vdif_header(sec_from_epoch: int, frame_in_second: int, ref_epoch: int, frame_bytes: int,
                log2_nchan: int, bits: int, thread_id: int = 0, station_id: int = 0,
                invalid: bool = False) -> bytes:
    w0 = (sec_from_epoch & 0x3FFFFFFF) | ((1 if invalid else 0) << 31)
    w1 = (frame_in_second & 0xFFFFFF) | ((ref_epoch & 0x3F) << 24)
    w2 = ((frame_bytes // 8) & 0xFFFFFF) | ((log2_nchan & 0x1F) << 24)
    w3 = (station_id & 0xFFFF) | ((thread_id & 0x3FF) << 16) | (((bits - 1) & 0x1F) << 26)
    return struct.pack("<8I", w0, w1, w2, w3, 0, 0, 0, 0)


def vdif_words_from_codes(chan_codes: list, bits: int) -> np.ndarray:
    """Interleave per-channel codes into 32-bit VDIF words.

    With C channels of b bits, a word carries 32/(C*b) samples of every
    channel; sample k of channel c sits at bit ((k*C)+c)*b.
    """
    C = len(chan_codes)
    per_word = 32 // (C * bits)
    if per_word < 1:
        raise ValueError("more bits per sample period than one word")
    n = min(c.size for c in chan_codes)
    n -= n % per_word
    words = np.zeros(n // per_word, dtype=np.uint32)
    for c in range(C):
        cc = chan_codes[c][:n].astype(np.uint32).reshape(-1, per_word)
        for k in range(per_word):
            words |= cc[:, k] << np.uint32(((k * C) + c) * bits)
    return words


def vdif_file_bytes(words: np.ndarray, *, payload_bytes: int, sample_rate: int, nchan: int, bits: int,
                    start_mjd: int, start_sec_of_day: int, invalid_frames=(), thread_id=0,
                    station_id=0) -> bytes:
    """Frame a word stream into VDIF frames (32-B header + payload).

    Sample 0 must fall on an integer second (start_sec_of_day) so that frame
    numbers restart at 0 each second.
    """
    ref_epoch, epoch_mjd = vdif_ref_epoch(start_mjd)
    words_per_frame = payload_bytes // 4
    samples_per_frame = payload_bytes * 8 // (bits * nchan)
    frames_per_second = sample_rate // samples_per_frame
    nframes = words.size // words_per_frame
    log2_nchan = int(round(math.log2(nchan)))
    inv = set(invalid_frames)
    payload = words[: nframes * words_per_frame].reshape(nframes, words_per_frame)
    out = bytearray()
    sec0 = (start_mjd - epoch_mjd) * 86400 + start_sec_of_day
    for f in range(nframes):
        sec = sec0 + f // frames_per_second
        fn = f % frames_per_second
        out += vdif_header(sec, fn, ref_epoch, payload_bytes + VDIF_HEADER_BYTES, log2_nchan, bits,
                           thread_id, station_id, f in inv)
        out += payload[f].tobytes()
    return bytes(out)


def vdif_frames_array(words: np.ndarray, *, payload_bytes: int, sample_rate: int, nchan: int, bits: int,
                      start_mjd: int, start_sec_of_day: int) -> np.ndarray:
    """vdif_file_bytes without invalid frames, built with whole-array
    operations (for recordings of gigabytes): a uint8 array of the frames."""
    ref_epoch, epoch_mjd = vdif_ref_epoch(start_mjd)
    wpf = payload_bytes // 4
    fps = sample_rate // (payload_bytes * 8 // (bits * nchan))
    nframes = words.size // wpf
    f = np.arange(nframes, dtype=np.int64)
    sec0 = (start_mjd - epoch_mjd) * 86400 + start_sec_of_day
    out = np.zeros((nframes, 8 + wpf), dtype=np.uint32)
    out[:, 0] = ((sec0 + f // fps) & 0x3FFFFFFF).astype(np.uint32)
    out[:, 1] = ((f % fps) & 0xFFFFFF).astype(np.uint32) | np.uint32((ref_epoch & 0x3F) << 24)
    out[:, 2] = np.uint32((((payload_bytes + VDIF_HEADER_BYTES) // 8) & 0xFFFFFF) |
                          ((int(round(math.log2(nchan))) & 0x1F) << 24))
    out[:, 3] = np.uint32(((bits - 1) & 0x1F) << 26)
    out[:, 8:] = words[:nframes * wpf].reshape(nframes, wpf)
    return out.reshape(-1).view(np.uint8)


# --------------------------------------------------------------------------
# Recordings with the irregularities the format readers handle
# --------------------------------------------------------------------------
VDIF_FILL_WORD = 0x11223344


def vdif_recording(nframes: int, *, payload_bytes: int, frames_per_second: int, start_mjd: int,
                   start_sec_of_day: int, log2_nchan: int, bits: int, legacy: bool = False, threads=(0,),
                   invalid=(), fill=(), drop=(), first_frame: int = 0, seed: int = 0) -> bytes:
    """VDIF frames with random payloads.  Frame k belongs to thread
    threads[k % len(threads)] and is that thread's (first_frame + k //
    len(threads))-th frame of the recording; `invalid` frames carry the
    invalid bit, `fill` frames are fill pattern throughout (header and
    payload), `drop` frames are left out.  Legacy frames have 16-byte headers."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ref_epoch, epoch_mjd = vdif_ref_epoch(start_mjd)
    sec0 = (start_mjd - epoch_mjd) * 86400 + start_sec_of_day
    hbytes = 16 if legacy else 32
    out = bytearray()
    for k in range(nframes):
        if k in drop:
            continue
        if k in fill:
            out += struct.pack("<I", VDIF_FILL_WORD) * ((hbytes + payload_bytes) // 4)
            continue
        n = first_frame + k // len(threads)
        h = bytearray(vdif_header(sec0 + n // frames_per_second, n % frames_per_second, ref_epoch,
                                  payload_bytes + hbytes, log2_nchan, bits, threads[k % len(threads)], 0,
                                  k in invalid))
        if legacy:
            h[3] |= 0x40  # legacy-mode bit (word 0, bit 30)
        out += bytes(h[:hbytes])
        out += rng.integers(0, 256, payload_bytes, dtype=np.uint8).tobytes()
    return bytes(out)


MK5B_SYNC = 0xABADDEED
MK5B_FRAME_BYTES = 10000


def _mk5b_crc_table():
    tab = []
    for i in range(256):
        c = (i << 8) & 0xFFFF
        for _ in range(8):
            c = ((c << 1) ^ 0x8005) & 0xFFFF if c & 0x8000 else (c << 1) & 0xFFFF
        tab.append(c)
    return tab


_MK5B_TAB = _mk5b_crc_table()


def _mk5b_register(b: bytes) -> int:
    """Mark5B header check register over words 2-3 (bytes of each word from
    the most significant), 32-bit and never masked: zero means valid."""
    crc = 0
    for word in (2, 3):
        for i in (3, 2, 1, 0):
            crc ^= b[word * 4 + i] << 8
            crc = ((crc << 8) ^ _MK5B_TAB[(crc >> 8) & 0xFF]) & 0xFFFFFFFF
    return crc


_MK5B_SOLVE = None


def mk5b_valid_crc(header16: bytes) -> int:
    """The CRC field value that makes the header check pass.  The register
    is affine over GF(2) in the 16 CRC bits, so R(x) = R(0) ^ A x with A fixed:
    tabulate A x once and look up R(0)."""
    global _MK5B_SOLVE
    b = bytearray(header16)
    if _MK5B_SOLVE is None:
        z = bytearray(16)
        r0 = _mk5b_register(bytes(z))
        cols = []
        for i in range(16):
            z[12:14] = struct.pack("<H", 1 << i)
            cols.append(_mk5b_register(bytes(z)) ^ r0)
        table = {}
        for x in range(1 << 16):
            v = 0
            for i in range(16):
                if x >> i & 1:
                    v ^= cols[i]
            table[v] = x
        _MK5B_SOLVE = table
    b[12:14] = b"\0\0"
    r = _mk5b_register(bytes(b))
    x = _MK5B_SOLVE.get(r)
    if x is None:
        raise ValueError("no CRC value passes the header check")
    return x


def _bcd(value: int, digits: int) -> int:
    return int("%0*d" % (digits, value), 16)


def mark5b_recording(nframes: int, *, mjd: int, sec_of_day: int, frames_per_second: int, seed: int = 0,
                     first_frame: int = 0, crc: str = "zero", bad_crc=(), bad_sync=(), garbage=None,
                     fill_runs=(), no_subsec=False, payload_words=None) -> bytes:
    """Mark5B frames (16-byte header + 10000 bytes) with random payloads,
    frame numbers counting within each second from first_frame.  crc: "zero"
    (the field left 0, accepted without a check) or "valid" (the value that
    passes the check); bad_crc frames get a failing value, bad_sync frames a
    wrong sync word; garbage = {frame: nbytes} inserts random bytes before a
    frame; fill_runs = [(frame, first word, nwords)] writes the fill word into
    payloads; no_subsec leaves the fractional-second field zero; payload_words
    (uint32, 2500 per frame) replaces the random payloads."""
    rng = np.random.Generator(np.random.PCG64(seed))
    garbage = garbage or {}
    out = bytearray()
    for k in range(nframes):
        if k in garbage:
            out += rng.integers(0, 256, garbage[k], dtype=np.uint8).tobytes()
        n = first_frame + k
        sec = sec_of_day + n // frames_per_second
        fn = n % frames_per_second
        day = mjd + sec // 86400
        sec %= 86400
        sub = 0 if no_subsec else (fn * 10000) // frames_per_second  # 0.1 ms units
        w1 = fn & 0x7FFF
        w2 = _bcd(day % 1000, 3) << 20 | _bcd(sec, 5)
        w3 = _bcd(sub, 4) << 16
        h = bytearray(struct.pack("<IIII", MK5B_SYNC if k not in bad_sync else 0xABADDEEE, w1, w2, w3))
        if crc == "valid" or k in bad_crc:
            c = mk5b_valid_crc(bytes(h))
            h[12:14] = struct.pack("<H", c ^ 0x0101 if k in bad_crc else c)
        if payload_words is not None:
            payload = bytearray(np.asarray(payload_words[k * 2500:(k + 1) * 2500], dtype="<u4").tobytes())
        else:
            payload = bytearray(rng.integers(0, 256, MK5B_FRAME_BYTES, dtype=np.uint8).tobytes())
        for (f, w0, nw) in fill_runs:
            if f == k:
                payload[4 * w0:4 * (w0 + nw)] = struct.pack("<I", VDIF_FILL_WORD) * nw
        out += bytes(h) + bytes(payload)
    return bytes(out)


# --------------------------------------------------------------------------
# the same signal model at benchmark sizes, on a GPU with torch
# --------------------------------------------------------------------------
@dataclass
class PulseModel:
    """A pulsar in the sky signal: amplitude 1 + peak * exp(-(phi - 1/2)^2 / (2 w^2))
    for pulse phase phi = frac((T - t_ref) / period), its arrival delayed by the
    dispersion delay 4148.808 DM / f_MHz^2 s at the subband's centre frequency
    (no sweep within the subband); w from the duty cycle (FWHM)."""
    period: float = 0.0334
    duty: float = 0.05
    peak: float = 20.0
    dm: float = 56.8
    t_ref: float = 0.0


def model_codes_torch(stations, pols, sample_rate, f_lo, n_samples, start_sec_of_day, rho, seed, tones=(),
                      pulse: PulseModel | None = None, band_centre_hz=None, device="cuda", chunk=1 << 24):
    """Yields ((station index, pol), packed 2-bit codes as a numpy uint8 array)
    for every stream in correlator order, generated on the GPU.

    The model of generate_station_samples -- the analytic sky signal a seen at
    T with T + tau_i(T) = t, fringe phase -2 pi f_lo tau_i(T) in FP64, gain g_i,
    correlated fraction rho, common RFI tones (amplitude in units of the
    unit-variance noise) -- with two simplifications that keep it fast at
    tens of gigasamples: the sky signal is taken at the nearest sample of T
    (no fractional interpolation), and a pulsar, if any, modulates the sky
    signal's amplitude.  2-bit quantisation at +-0.98 sigma of each stream."""
    import torch
    sr = float(sample_rate)
    max_tau = 0.0
    for st in stations:
        max_tau = max(max_tau, float(np.max(np.abs(st.poly.delay(
            np.array([start_sec_of_day, start_sec_of_day + n_samples / sr]))))))
    margin = int(max_tau * sr) + 1024
    n_sky = n_samples + 2 * margin
    n_sky += n_sky & 1
    gen = torch.Generator(device=device)
    for pi, pol in enumerate(pols):
        gen.manual_seed(seed * 100 + pi)
        sky = torch.randn(n_sky, generator=gen, device=device, dtype=torch.float32)
        F = torch.fft.rfft(sky)
        del sky
        A = torch.zeros(n_sky, dtype=torch.complex64, device=device)
        A[:F.numel()] = 2.0 * F
        A[0] = F[0]
        A[n_sky // 2] = F[n_sky // 2]
        del F
        a = torch.fft.ifft(A)  # analytic signal, real part = the sky signal
        del A
        for si, st in enumerate(stations):
            c = torch.tensor(st.poly.coeffs, dtype=torch.float64, device=device)

            def tau(t):
                x = t - st.poly.t0
                r = torch.zeros_like(x)
                for k in range(c.numel() - 1, -1, -1):
                    r = r * x + c[k]
                return r

            gen.manual_seed(seed * 1000 + 17 + si * 7 + pi)
            x = torch.empty(n_samples, dtype=torch.float32, device=device)
            for c0 in range(0, n_samples, chunk):
                c1 = min(n_samples, c0 + chunk)
                t = start_sec_of_day + torch.arange(c0, c1, dtype=torch.float64, device=device) / sr
                T = t - tau(t)
                for _ in range(4):
                    T = t - tau(T)
                pos = torch.round((T - start_sec_of_day) * sr).to(torch.int64) + margin
                sig = a[pos]
                ph = -f_lo * tau(T)
                ph = (ph - torch.floor(ph)).to(torch.float32) * (2.0 * math.pi)
                s = sig.real * torch.cos(ph) - sig.imag * torch.sin(ph)
                if pulse is not None:
                    fc = (band_centre_hz if band_centre_hz is not None else f_lo) * 1e-6
                    tp = T - pulse.t_ref - 4148.808 * pulse.dm / (fc * fc)
                    phi = tp / pulse.period
                    phi = (phi - torch.floor(phi)).to(torch.float32)
                    w = pulse.duty / 2.3548
                    s = s * (1.0 + pulse.peak * torch.exp(-((phi - 0.5) ** 2) / (2 * w * w)))
                noise = torch.randn(c1 - c0, generator=gen, device=device, dtype=torch.float32)
                xs = st.gain * (math.sqrt(rho) * s + math.sqrt(1.0 - rho) * noise)
                for (ftone, amp) in tones:
                    tph = ftone * (t - start_sec_of_day)
                    tph = (tph - torch.floor(tph)).to(torch.float32) * (2.0 * math.pi)
                    xs = xs + amp * torch.cos(tph)
                x[c0:c1] = xs
            sigma = float(x.double().std())
            thr = THRESH_2BIT * sigma
            codes = (x >= -thr).to(torch.uint8) + (x >= 0).to(torch.uint8) + (x >= thr).to(torch.uint8)
            del x
            n4 = codes.numel() // 4 * 4
            q = codes[:n4].view(-1, 4)
            packed = q[:, 0] | (q[:, 1] << 2) | (q[:, 2] << 4) | (q[:, 3] << 6)
            yield (si, pol), packed.cpu().numpy()
        del a
