"""Correlator time base: int64 clock ticks at 512 MHz since MJD 51544.

Mirrors the reference's `Time` class (sfxc/include/correlator_time.h:12-91,
sfxc/src/correlator_time.cc): ticks are the exact integer representation used
everywhere on the path, so every conversion here is integer arithmetic or the
same rounding the reference applies.
"""
import math

MAX_SAMPLE_RATE = 512_000_000          # ticks per second (sfxc/include/utils.h:36)
REFERENCE_MJD = 51544                  # correlator_time.h:9
SECONDS_PER_DAY = 86400
TICKS_PER_DAY = SECONDS_PER_DAY * MAX_SAMPLE_RATE


def ticks_from_mjd_sec(mjd: int, sec: float) -> int:
    """Time::set_time (correlator_time.h:76-78)."""
    return int((mjd - REFERENCE_MJD) * SECONDS_PER_DAY * float(MAX_SAMPLE_RATE)) + int(
        _round_half_away(sec * MAX_SAMPLE_RATE))


def ticks_from_usec(usec: float) -> int:
    """Time(double usec) constructor (correlator_time.cc:182-185)."""
    return int(_round_half_away(usec * (MAX_SAMPLE_RATE / 1_000_000)))


def ticks_per_sample(sample_rate: int) -> int:
    """Time::set_sample_rate: clock ticks per sample (correlator_time.cc:213-215)."""
    return int(_round_half_away(MAX_SAMPLE_RATE / sample_rate))


def mjd_of(ticks: int) -> float:
    """Time::get_mjd (correlator_time.cc:217-222)."""
    ndays = int(ticks / TICKS_PER_DAY) if ticks >= 0 else -int(-ticks // TICKS_PER_DAY)
    rem = ticks - ndays * TICKS_PER_DAY
    return REFERENCE_MJD + ndays + rem / float(MAX_SAMPLE_RATE) / SECONDS_PER_DAY


def mjd_from_date(day: int, month: int, year: int) -> int:
    """Modified Julian day of a calendar date (the reference's mjd(), sfxc/src/utils.cc:255-263)."""
    a = (14 - month) // 12
    y = year + 4800 - a
    m = month + 12 * a - 3
    jdn = day + ((153 * m + 2) // 5) + 365 * y + (y // 4) - (y // 100) + (y // 400) - 32045
    return int(jdn - 2400000.5)


def nr_ffts_per_integration_slice(integration_time_us: int, data_rate: int, fft_size: int) -> int:
    """Control_parameters::nr_ffts_per_integration_slice (sfxc/include/control_parameters.h:301-307).

    Both times are converted to ticks exactly as the reference's Time(usec) does,
    then the (double) tick ratio is floored.
    """
    t_int = ticks_from_usec(float(integration_time_us))
    t_fft = ticks_from_usec(fft_size / (data_rate / 1_000_000.0))
    return int(math.floor(t_int / t_fft))


def _round_half_away(x: float) -> float:
    # C's round(): halves away from zero
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)
