// Host-side model of the correlator-node path (see host.hpp).
#include "host.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace sfxc {

// ------------------------------------------------------------------- time --
ticks_t time_from_mjd_sec(int mjd, double sec) {
  return (ticks_t)((mjd - kReferenceMjd) * 86400 * kClockRate) + (ticks_t)std::round(sec * kClockRate);
}
ticks_t time_from_usec(double usec) { return (ticks_t)std::round(usec * (kClockRate / 1000000)); }
int ticks_per_sample(double sample_rate) { return (int)std::round(kClockRate / sample_rate); }
double time_mjd(ticks_t t) {
  int ndays = (int)(t / kTicksPerDay);
  double mjd = kReferenceMjd + ndays;
  return mjd + (t % kTicksPerDay) / kClockRate / 86400;
}
double time_usec_of_day(ticks_t t) { return (t % kTicksPerDay) / (kClockRate / 1000000); }
double time_sec_of_day(ticks_t t) { return (t % kTicksPerDay) / kClockRate; }
ticks_t time_mul(ticks_t t, double v) { return (ticks_t)std::round(t * v); }
ticks_t time_div(ticks_t t, double v) { return (ticks_t)std::round(t / v); }
int nr_ffts_per_integration_slice(double integration_time_us, int data_rate, int fft_size) {
  ticks_t ti = time_from_usec((double)(int)integration_time_us);
  ticks_t tf = time_from_usec(fft_size / (data_rate / 1000000.));
  return (int)std::floor((double)ti / (double)tf);
}

// ------------------------------------------------------------ delay table --
DelayTable DelayTable::parse(const uint8_t *p, size_t n) {
  DelayTable t;
  size_t pos = 0;
  auto need = [&](size_t k) {
    if (pos + k > n) throw Error(-2, "truncated delay table");
  };
  need(4);
  int32_t hs;
  std::memcpy(&hs, p, 4);
  pos = 4 + (size_t)hs;
  while (pos + 81 + 4 + 56 <= n) {
    int32_t mjd;
    double line[7];
    pos += 81;  // source name
    std::memcpy(&mjd, p + pos, 4);
    pos += 4;
    std::memcpy(line, p + pos, 56);
    pos += 56;
    Scan s{};
    double scan_start = line[0], scan_end = line[0];
    s.begin = time_from_mjd_sec(mjd, scan_start);
    s.first_row = (int)t.times.size();
    for (;;) {
      if (line[0] == 0 && line[4] == 0) {
        if ((int)t.times.size() - s.first_row < 2) throw Error(-2, "delay table scan with fewer than two rows");
        s.end = time_from_mjd_sec(mjd, scan_end);
        break;
      }
      t.times.push_back(line[0] - scan_start);
      t.us.push_back(line[1]);
      t.vs.push_back(line[2]);
      t.ws.push_back(line[3]);
      t.delays.push_back(line[4]);
      t.phases.push_back(line[5]);
      t.amps.push_back(line[6]);
      scan_end = line[0];
      if (pos + 56 > n) break;
      std::memcpy(line, p + pos, 56);
      pos += 56;
    }
    s.nrows = (int)t.times.size() - s.first_row;
    t.scans.push_back(s);
  }
  if (t.scans.empty()) throw Error(-2, "delay table holds no scan");
  return t;
}

// Akima (1970) slopes with GSL's non-periodic end conditions (two extra
// secant slopes extrapolated linearly at each end); cubic coefficients per
// interval b (slope), c (quadratic), d (cubic).
static void akima_coefficients(const double *x, const double *y, int n, double *b, double *c, double *d) {
  std::vector<double> mb(n + 4);
  double *m = mb.data() + 2;
  for (int i = 0; i <= n - 2; i++) m[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
  m[-2] = 3.0 * m[0] - 2.0 * m[1];
  m[-1] = 2.0 * m[0] - m[1];
  m[n - 1] = 2.0 * m[n - 2] - m[n - 3];
  m[n] = 3.0 * m[n - 2] - 2.0 * m[n - 3];
  for (int i = 0; i < n - 1; i++) {
    const double ne = std::fabs(m[i + 1] - m[i]) + std::fabs(m[i - 1] - m[i - 2]);
    if (ne == 0.0) {
      b[i] = m[i];
      c[i] = 0.0;
      d[i] = 0.0;
      continue;
    }
    const double h = x[i + 1] - x[i];
    const double ne_next = std::fabs(m[i + 2] - m[i + 1]) + std::fabs(m[i] - m[i - 1]);
    const double alpha = std::fabs(m[i - 1] - m[i - 2]) / ne;
    double t_next;
    if (ne_next == 0.0) {
      t_next = m[i];
    } else {
      const double alpha_next = std::fabs(m[i] - m[i - 1]) / ne_next;
      t_next = (1.0 - alpha_next) * m[i] + alpha_next * m[i + 1];
    }
    b[i] = (1.0 - alpha) * m[i - 1] + alpha * m[i];
    c[i] = (3.0 * m[i] - 2.0 * b[i] - t_next) / h;
    d[i] = (b[i] + t_next - 2.0 * m[i]) / (h * h);
  }
}

Spline Spline::create(const DelayTable &t, ticks_t start_, ticks_t duration, int pc) {
  int mjd_start = (int)std::floor(time_mjd(start_));
  double seconds_start = std::floor(time_usec_of_day(start_) / 1000000);
  ticks_t stop = start_ + duration;
  int mjd_stop = (int)std::floor(time_mjd(stop));
  double seconds_stop = std::ceil(time_usec_of_day(stop) / 1000000);
  ticks_t start = time_from_mjd_sec(mjd_start, seconds_start);
  int n_seconds = (int)((mjd_stop - mjd_start) * 86400 + seconds_stop - seconds_start);
  size_t sn = 0;
  while (sn < t.scans.size() && stop > t.scans[sn].end) sn++;
  if (sn == t.scans.size()) throw Error(-3, "time is not covered by the delay table");
  if (sn + pc >= t.scans.size() || t.scans[sn + pc].begin != t.scans[sn].begin)
    throw Error(-3, "the delay table has fewer phase centres than requested");
  const Scan &s = t.scans[sn + pc];
  if (time_diff(s.end, s.begin) < 4.) throw Error(-3, "delay table scan shorter than 4 s");
  const ticks_t onesec = time_from_usec(1000000.);
  ticks_t ib = start - time_mul(onesec, 2);
  ticks_t ie = start + time_mul(onesec, 2 + n_seconds);
  if (ib < s.begin) {
    ib = s.begin;
    if (time_diff(ie, ib) < 4) ie = ib + time_mul(onesec, 4);
  }
  if (ie > s.end) {
    ie = s.end;
    if (time_diff(ie, ib) < 4) ib = ie - time_mul(onesec, 4);
  }
  const std::vector<double> *const cols[3] = {&t.delays, &t.phases, &t.amps};
  return build(t, s, ib, ie, cols);
}

Spline Spline::build(const DelayTable &t, const Scan &s, ticks_t ib, ticks_t ie,
                     const std::vector<double> *const cols[3]) {
  const ticks_t onesec = time_from_usec(1000000.);
  Spline sp;
  sp.n = (int)((double)(ie - ib) / (double)onesec + 1);
  int idx = (int)time_diff(ib, s.begin);
  if (sp.n <= 4) throw Error(-3, "fewer than five delay-table rows cover the slice");
  if (idx < 0 || idx + sp.n > s.nrows) throw Error(-3, "delay-table rows do not cover the spline interval");
  const int r0 = s.first_row + idx;
  sp.x.assign(t.times.begin() + r0, t.times.begin() + r0 + sp.n);
  for (int k = 0; k < 3; k++) {
    sp.y[k].assign(cols[k]->begin() + r0, cols[k]->begin() + r0 + sp.n);
    sp.b[k].resize(sp.n);
    sp.c[k].resize(sp.n);
    sp.d[k].resize(sp.n);
    akima_coefficients(sp.x.data(), sp.y[k].data(), sp.n, sp.b[k].data(), sp.c[k].data(), sp.d[k].data());
  }
  sp.scan_begin = s.begin;
  sp.interval_begin = ib;
  sp.interval_end = ie;
  sp.clock_epoch = t.clock_epoch;
  sp.clock_offset = t.clock_offset;
  sp.clock_rate = t.clock_rate;
  return sp;
}

// ---------------------------------------------------------------- UVW model --
UvwModel::UvwModel(DelayTable t) : t_(std::move(t)) {
  scan_nr_ = 0;
  n_sources_ = 0;
  next_scan();  // open(): the first scan group
}

// initialise_next_scan (uvw_model.cc:244-257): the next group of scans with one start
bool UvwModel::next_scan() {
  if (scan_nr_ >= t_.scans.size() - (size_t)n_sources_) return false;
  scan_nr_ += (size_t)n_sources_;
  n_sources_ = 1;
  while (scan_nr_ + n_sources_ < t_.scans.size() &&
         t_.scans[scan_nr_ + n_sources_ - 1].begin == t_.scans[scan_nr_ + n_sources_].begin)
    n_sources_++;
  return true;
}

// create_akima_spline (uvw_model.cc:259-310): the second holding t, splines
// over [-2 s, +3 s] of it clamped to the scan (at least 4 s)
void UvwModel::create(ticks_t t) {
  while (t_.scans[scan_nr_].end < t)
    if (!next_scan()) throw Error(-3, "UVW model ends before the requested time");
  const int mjd_start = (int)std::floor(time_mjd(t));
  const double seconds_start = std::floor(time_usec_of_day(t) / 1000000);
  const ticks_t start = time_from_mjd_sec(mjd_start, seconds_start);
  const ticks_t onesec = time_from_usec(1000000.);
  interval_begin_ = start;
  interval_end_ = start + onesec;
  ticks_t ib = start - time_mul(onesec, 2), ie = start + time_mul(onesec, 3);
  const Scan &s0 = t_.scans[scan_nr_];
  if (ib < s0.begin) {
    ib = s0.begin;
    if (time_diff(ie, ib) < 4) ie = ib + time_mul(onesec, 4);
  }
  if (ie > s0.end) {
    ie = s0.end;
    if (time_diff(ie, ib) < 4) ib = ie - time_mul(onesec, 4);
  }
  const std::vector<double> *const cols[3] = {&t_.us, &t_.vs, &t_.ws};
  splines_.clear();
  for (int i = 0; i < n_sources_; i++) {
    Spline sp = Spline::build(t_, t_.scans[scan_nr_ + i], ib, ie, cols);
    sp.scan_begin = s0.begin;
    splines_.push_back(std::move(sp));
  }
}

void UvwModel::get(int pc, ticks_t t, double out[3]) {
  if (t > interval_end_) create(t);
  if (pc < 0 || pc >= (int)splines_.size()) throw Error(-1, "no such phase centre in the UVW model's scan");
  const double sec = time_diff(t, t_.scans[scan_nr_].begin);
  for (int k = 0; k < 3; k++) out[k] = splines_[(size_t)pc].eval_extended(k, sec);
}

// Interval search as GSL's gsl_interp_bsearch; the device uses the same rule.
int Spline::index(double v) const {
  if (v < x[0] || v > x[n - 1]) throw Error(-3, "delay model evaluated outside its interval");
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int i = (hi + lo) / 2;
    if (x[i] > v)
      hi = i;
    else
      lo = i;
  }
  return lo;
}
double Spline::eval(int col, double v) const {
  int i = index(v);
  const double dx = v - x[i];
  return y[col][i] + dx * (b[col][i] + dx * (c[col][i] + d[col][i] * dx));
}
// gsl_spline_eval as GSL 1.9 has it (interpolation/interp.c, gsl_interp_eval)
// checks no domain: outside the nodes its interval search returns the first
// or the last interval and akima_eval extends that interval's cubic.
// Uvw_model::get_uvw evaluates this way when a time steps back before its
// spline's window (the spline is only rebuilt for later times) or lies past a
// scan's last row.
double Spline::eval_extended(int col, double v) const {
  const int i = v < x[0] ? 0 : v > x[n - 1] ? n - 2 : index(v);
  const double dx = v - x[i];
  return y[col][i] + dx * (b[col][i] + dx * (c[col][i] + d[col][i] * dx));
}
double Spline::deriv(int col, double v) const {
  int i = index(v);
  double dx = v - x[i];
  return b[col][i] + dx * (2.0 * c[col][i] + 3.0 * d[col][i] * dx);
}
double Spline::delay(ticks_t t) const {
  if (t < interval_begin || t > interval_end) throw Error(-3, "delay requested outside the spline interval");
  double r = eval(0, time_diff(t, scan_begin));
  double drift = clock_offset + time_diff(t, clock_epoch) * clock_rate;
  return r + drift;
}
double Spline::rate(ticks_t t) const { return deriv(0, time_diff(t, scan_begin)) + clock_rate; }
double Spline::phase(ticks_t t) const { return eval(1, time_diff(t, scan_begin)); }
double Spline::amplitude(ticks_t t) const { return eval(2, time_diff(t, scan_begin)); }

// ---------------------------------------------------------- integer delays --
Delay integer_delay(const Spline &s, ticks_t t, int sample_rate, int bits) {
  const int spb = 8 / bits;
  int32_t samples = (int32_t)std::floor(s.delay(t) * sample_rate + .5);
  int32_t bytes = (int32_t)std::floor((samples - 1) * 1. / spb);
  int32_t rem = samples - bytes * spb;
  if (rem * bits == 8) {
    bytes++;
    rem = 0;
  }
  return Delay{t, bytes, rem};
}

static void bisect_delays(const Spline &s, ticks_t start, int64_t nsamples, int tps, int sr, int bits,
                          std::vector<Delay> &out) {
  ticks_t stop = start + nsamples * tps;
  Delay a = integer_delay(s, start, sr, bits), e = integer_delay(s, stop, sr, bits);
  if (a.bytes != e.bytes || a.rem != e.rem) {
    if (nsamples == 1) {
      out.push_back(e);
      return;
    }
  } else if (!(s.rate(start) * s.rate(stop) < 0 && nsamples >= 3)) {
    return;
  }
  bisect_delays(s, start, nsamples / 2, tps, sr, bits, out);
  bisect_delays(s, start + (nsamples / 2) * tps, nsamples - nsamples / 2, tps, sr, bits, out);
}

std::vector<Delay> interval_delays(const Spline &s, ticks_t start, ticks_t stop, int sample_rate, int bits) {
  std::vector<Delay> out;
  const int tps = ticks_per_sample(sample_rate);
  out.push_back(integer_delay(s, start, sample_rate, bits));
  int64_t nsamples = (stop - start) / tps;
  if (nsamples <= 0) throw Error(-1, "empty delay interval");
  bisect_delays(s, start, nsamples, tps, sample_rate, bits, out);
  return out;
}

// -------------------------------------------------------- protocol writer --
namespace {
struct RecordSink {
  std::vector<Record> &out;
  void delay(int rem) { out.push_back(Record{HEADER_DELAY, (int8_t)rem, 0, 0}); }
  void invalid(int n) {  // records of at most SHRT_MAX samples
    for (int w = 0; w < n;) {
      int k = std::min(n - w, (int)SHRT_MAX);
      out.push_back(Record{HEADER_INVALID, 0, k, 0});
      w += k;
    }
  }
  void data(int n, int64_t src) {
    for (int w = 0; w < n;) {
      int k = std::min(n - w, (int)SHRT_MAX);
      out.push_back(Record{HEADER_DATA, 0, k, src + w});
      w += k;
    }
  }
  void end() { out.push_back(Record{HEADER_ENDSTREAM, 0, 0, 0}); }
};
}  // namespace

std::vector<std::vector<Record>> write_protocol(const std::vector<ChannelBlock> &blocks,
                                                const std::vector<SliceRequest> &slices, int sr, int bits,
                                                double integration_time_us) {
  const int tps = ticks_per_sample(sr);
  const ticks_t byte_length = time_from_usec(8 * 1000000. / ((double)sr * bits));
  const ticks_t integration_time = time_from_usec(integration_time_us);
  const int spb = 8 / bits;
  std::vector<std::vector<Record>> outs(slices.size());
  ticks_t now = 0, slice_start = 0, iv_stop = 0;
  size_t next_interval = 0, writer = 0, bi = 0;
  bool active = false, sync = false;
  int di = 0;
  int64_t slice_size = slices.empty() ? 0 : slices[0].nr_samples;
  const std::vector<Delay> *cur = nullptr;
  int64_t block_size = 0;
  auto next_delay_pos = [&](ticks_t t) -> int {
    int p = (di < (int)cur->size() - 1) ? (int)((double)((*cur)[di + 1].time - t) / (double)byte_length) : INT_MAX / 2;
    return std::max(p, 0);
  };
  auto adjust = [&]() {  // slice size follows the inserted / dropped sample
    int d = (*cur)[di].rem - (*cur)[di - 1].rem;
    slice_size += (d > 1 || d == -1) ? -1 : 1;
  };
  for (long guard = 0;; guard++) {
    if (guard > 400000000L) throw Error(-4, "protocol writer did not terminate");
    if (writer >= slices.size()) break;
    if (!active && now >= iv_stop) {
      if (next_interval >= slices.size()) break;
      iv_stop = slices[next_interval].stop;
      di = 0;
      cur = &slices[next_interval].delays;
      now = slices[next_interval].start;
      next_interval++;
    }
    if (bi >= blocks.size()) break;
    const ChannelBlock &blk = blocks[bi];
    RecordSink o{outs[writer]};
    int64_t byte_offset = 0;
    const int nd = (int)cur->size();
    if (!active) {
      active = true;
      slice_start = now;
      sync = true;
    }
    if (sync) {
      block_size = blk.size;
      while (di < nd - 1 && (*cur)[di + 1].time <= now + byte_length) di++;
      int64_t dsamples = (now - blk.start) / tps;
      byte_offset = dsamples * bits / 8 + (*cur)[di].bytes;
      if (byte_offset < 0) {  // write_initial_invalid_data
        int initial = (*cur)[di].rem;
        o.delay((*cur)[di].rem);
        slice_size += (*cur)[di].rem;
        int64_t inval = std::min(-byte_offset * spb, slice_size);
        int64_t written = 0;
        while (written < inval) {
          int64_t ndp = (di < nd - 1) ? (int64_t)(spb * ((double)((*cur)[di + 1].time - now) / (double)byte_length))
                                      : slice_size * 2;
          if (written == ndp) {
            di++;
            o.delay((*cur)[di].rem);
            adjust();
            inval = std::min(-byte_offset * spb, slice_size);
          } else {
            int k = (int)std::min(ndp - written, inval - written);
            o.invalid(k);
            written += k;
          }
        }
        slice_size -= inval;
        now += (inval - initial) * tps;
        sync = false;
        continue;
      } else if (byte_offset >= block_size) {
        bi++;
        continue;
      }
      slice_size += (*cur)[di].rem;
      o.delay((*cur)[di].rem);
      now -= (ticks_t)(*cur)[di].rem * tps;
      sync = false;
    }
    int index = (int)byte_offset, inv_i = 0;
    int next_inv = blk.invalid.empty() ? (int)block_size + 1 : blk.invalid[0].begin;
    int ndp = next_delay_pos(now) + (int)byte_offset;
    auto total = [&]() { return (int)std::min(block_size - byte_offset, (slice_size + spb - 1) / spb); };
    int to_write = total();
    int end_index = to_write + (int)byte_offset;
    while (index < end_index) {
      if (index >= ndp) {
        di++;
        o.delay((*cur)[di].rem);
        adjust();
        ndp = next_delay_pos(now) + (int)byte_offset;
        to_write = total();
        end_index = to_write + (int)byte_offset;
      } else if (index >= next_inv) {
        int n = blk.invalid[inv_i].n;
        int end_pos = std::min(next_inv + n, ndp);
        int nr = std::min(std::max(0, end_pos - index), end_index - index);
        if (nr > 0) {
          o.invalid(nr * spb);
          index += nr;
        }
        if (end_pos == next_inv + n) {
          inv_i++;
          next_inv = (int)blk.invalid.size() > inv_i ? blk.invalid[inv_i].begin : (int)block_size + 1;
        }
      } else {
        int k = std::min(std::min(ndp - index, end_index - index), next_inv - index);
        if (k > 0) o.data(k, blk.src_offset + index);
        index += k;
      }
    }
    slice_size -= (int64_t)to_write * spb;
    now += (ticks_t)to_write * spb * tps;
    if (index >= block_size) bi++;
    if (slice_size <= 0) {
      o.end();
      now = slice_start + integration_time;
      active = false;
      writer++;
      if (writer < slices.size()) slice_size = slices[writer].nr_samples;
    }
  }
  return outs;
}

void serialize_protocol(const std::vector<Record> &recs, const uint8_t *stream, std::vector<uint8_t> &out) {
  for (const Record &r : recs) {
    out.push_back(r.type);
    if (r.type == HEADER_DELAY) {
      out.push_back((uint8_t)r.rem);
    } else if (r.type == HEADER_DATA || r.type == HEADER_INVALID) {
      int16_t k = (int16_t)r.n;
      out.push_back((uint8_t)(k & 0xff));
      out.push_back((uint8_t)((k >> 8) & 0xff));
      if (r.type == HEADER_DATA) out.insert(out.end(), stream + r.src, stream + r.src + r.n);
    }
  }
}

std::vector<Record> parse_protocol(const uint8_t *p, size_t n, int64_t base) {
  std::vector<Record> recs;
  size_t pos = 0;
  while (pos < n) {
    uint8_t h = p[pos];
    if (h == HEADER_ENDSTREAM) {
      recs.push_back(Record{h, 0, 0, 0});
      pos += 1;
    } else if (h == HEADER_DELAY) {
      if (pos + 2 > n) throw Error(-4, "truncated delay record");
      recs.push_back(Record{h, (int8_t)p[pos + 1], 0, 0});
      pos += 2;
    } else if (h == HEADER_DATA || h == HEADER_INVALID) {
      if (pos + 3 > n) throw Error(-4, "truncated protocol record");
      int k = p[pos + 1] | (p[pos + 2] << 8);
      if (h == HEADER_DATA) {
        if (pos + 3 + k > n) throw Error(-4, "truncated data record");
        if (k == 0) throw Error(-4, "empty data record");
        recs.push_back(Record{h, 0, k, base + (int64_t)pos + 3});
        pos += 3 + k;
      } else {
        recs.push_back(Record{h, 0, k, 0});
        pos += 3;
      }
    } else {
      throw Error(-4, "invalid header in the input protocol");
    }
  }
  return recs;
}

// ---------------------------------------------------------- unpack plan --
enum { S_IDLE = 0, S_INVALID = 1, S_DATA = 2, S_PURGE = 3 };

UnpackPlan plan_unpack(const std::vector<Record> &recs, StreamUnpackState &st, int n_blocks, int nfft_max,
                       int fft_size, int bits, int sample_rate, int tsys_freq, double delay_at_start) {
  UnpackPlan plan;
  plan.n_blocks = n_blocks;
  plan.nfft_max = nfft_max;
  const int spb = 8 / bits;
  // set_parameters: per-integration resets (state and bytes_left carry over)
  st.invalid_left = 0;
  st.sample_in_byte = 0;
  int cur_delay = -1;
  // payload position of the current data record (the reference's read pointer);
  // an integration always starts in IDLE or PURGE, so no payload carries over
  int64_t src = 0;
  plan.tsys.two_bit = bits == 2;
  plan.tsys.on0 = 1;
  if (bits == 2) {
    int delay_in_samples = (int)(delay_at_start * sample_rate);  // an int in the reference
    int full = sample_rate / tsys_freq, half = sample_rate / (2 * tsys_freq);
    int tc = (int)std::floor(delay_in_samples + 0.5);
    tc %= full;
    while (tc < 0) tc += full;
    plan.tsys.on0 = tc < half;
    tc %= half;
    plan.tsys.t0 = (half - tc) / 4;
    plan.tsys.period = half / 4;
  }
  auto push_seg = [&](int32_t out0, int32_t n, int64_t src_bit) {
    if (n <= 0) return;
    if (!plan.segs.empty()) {
      Segment &p = plan.segs.back();
      bool contiguous = p.out0 + p.n == out0 &&
                        ((p.src_bit < 0 && src_bit < 0) || (p.src_bit >= 0 && src_bit == p.src_bit + (int64_t)p.n * bits));
      if (contiguous) {
        p.n += n;
        return;
      }
    }
    plan.segs.push_back(Segment{out0, n, src_bit});
  };
  auto push_stat = [&](int64_t byte, int32_t n) {
    if (!plan.stats.empty()) {
      StatRange &p = plan.stats.back();
      if (p.src_byte + p.n == byte && p.cidx + p.n == plan.counted) {
        p.n += n;
        plan.counted += n;
        return;
      }
    }
    plan.stats.push_back(StatRange{byte, n, (int32_t)plan.counted});
    plan.counted += n;
  };
  int current_fft = 0;
  while (current_fft < n_blocks) {
    const int nfft = std::min(nfft_max, n_blocks - current_fft);
    const size_t size = (size_t)nfft * fft_size;
    const int32_t base = current_fft * fft_size;
    size_t out_index = 0;
    while (out_index != size) {
      switch (st.state) {
        case S_IDLE: {
          if (st.rec >= recs.size() || recs[st.rec].type == HEADER_ENDSTREAM)
            throw Error(-5, "input stream ended before the integration was complete");
          const Record &r = recs[st.rec++];
          st.rec_off = 0;
          if (r.type == HEADER_DATA) {
            st.bytes_left = r.n;
            src = r.src;
            st.state = S_DATA;
          } else if (r.type == HEADER_DELAY) {
            if (cur_delay < 0) {
              st.sample_in_byte = (uint64_t)(int64_t)r.rem;
            } else {
              int diff = r.rem - cur_delay;
              if (diff == -1 || diff > 1) {
                push_seg(base + (int32_t)out_index, 1, -1);  // insert a sample
                out_index++;
              } else {
                if (st.sample_in_byte != 0) throw Error(-5, "sample drop while a byte is partially consumed");
                st.sample_in_byte = 1;  // drop a sample
              }
            }
            cur_delay = r.rem;
            if (st.sample_in_byte >= 8) throw Error(-5, "delay record out of range");
          } else {
            st.invalid_left = (uint64_t)r.n;
            plan.n_invalid += r.n;
            plan.invalid.push_back(InvalidRun{base + (int32_t)out_index, r.n});
            st.state = S_INVALID;
          }
          break;
        }
        case S_INVALID: {
          uint64_t itw = std::min<uint64_t>(size - out_index, st.invalid_left);
          if (st.sample_in_byte > 0) {
            uint64_t drop = std::min(st.sample_in_byte, itw);
            st.sample_in_byte -= drop;
            itw -= drop;
            st.invalid_left -= drop;
          }
          if (itw > 0) {
            push_seg(base + (int32_t)out_index, (int32_t)itw, -1);
            st.invalid_left -= itw;
            out_index += itw;
          }
          if (st.invalid_left == 0) st.state = S_IDLE;
          break;
        }
        case S_DATA: {
          const uint64_t start = st.sample_in_byte;
          const uint64_t stw = std::min<uint64_t>(st.bytes_left * spb - start, size - out_index);
          push_seg(base + (int32_t)out_index, (int32_t)stw, src * 8 + (int64_t)start * bits);
          // counted bytes of this bit2float() call: the first byte always,
          // then whole bytes; a trailing partial byte is counted when finished
          if (start + stw >= (uint64_t)spb)
            push_stat(src, (int32_t)(1 + (stw - (spb - start)) / spb));
          else
            push_stat(src, 1);
          const uint64_t done = (stw + start) / spb;
          st.bytes_left -= done;
          src += (int64_t)done;
          st.rec_off += (int64_t)done;
          st.sample_in_byte = (stw + start) % spb;
          out_index += stw;
          if (st.bytes_left == 0) {
            if (st.sample_in_byte != 0) throw Error(-5, "data record ended inside a byte");
            st.state = S_IDLE;
          }
          break;
        }
        case S_PURGE: {  // skip the rest of the previous integration
          st.bytes_left = 0;
          if (st.rec >= recs.size()) throw Error(-5, "input stream ended while skipping the previous integration");
          const Record &r = recs[st.rec++];
          st.rec_off = 0;
          if (r.type == HEADER_ENDSTREAM)
            st.state = S_IDLE;
          else if (r.type == HEADER_DATA)
            st.bytes_left = r.n;
          break;
        }
      }
    }
    current_fft += nfft;
  }
  st.state = S_PURGE;
  return plan;
}

// ------------------------------------------------------------ baselines --
std::vector<Baseline> create_baselines(const std::vector<StationStream> &s, int ref) {
  std::vector<Baseline> bl;
  const int n = (int)s.size();
  for (int i = 0; i < n; i++) bl.push_back({i, i});
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      int s1 = s[i].station_number, s2 = s[j].station_number;
      if (s1 == s2) continue;
      if (ref >= 0 && ref != s1 && ref != s2) continue;
      if (s1 < s2)
        bl.push_back({i, j});
      else
        bl.push_back({j, i});
    }
  return bl;
}

void BitStats::levels(int out[5]) const {
  // the reference adds every byte bin's count into int accumulators, once per
  // code of the byte; the same sums from the code counts, wrapped to 32 bits
  int acc[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < (bits == 2 ? 4 : 2); k++) acc[k] = (int)(uint32_t)(uint64_t)(on[k] + off[k]);
  acc[4] += (int)n_invalid;
  for (int i = 0; i < 5; i++)
    out[i] = (int)(((uint64_t)base_sample_rate * (uint64_t)(int64_t)acc[i]) / (uint64_t)sample_rate);
}

void BitStats::tsys(int out[4]) const {
  out[0] = out[1] = out[2] = out[3] = 0;
  if (bits != 2) return;
  const int64_t *a = on, *b = off;
  out[0] = (int)(a[1] + a[2]);
  out[1] = (int)(a[0] + a[3]);
  out[2] = (int)(b[1] + b[2]);
  out[3] = (int)(b[0] + b[3]);
}

void find_invalid(const std::vector<StationStream> &s, int base_sr, const std::vector<Baseline> &bl,
                  const std::vector<const std::vector<InvalidRun> *> &inv, std::vector<std::pair<int64_t, int64_t>> &nfl) {
  const int nstreams = (int)s.size();
  nfl.assign(bl.size(), {0, 0});
  for (size_t b = nstreams; b < bl.size(); b++) {
    const int st2[2] = {bl[b].a, bl[b].b};
    const double scale[2] = {s[st2[0]].sample_rate * 1. / base_sr, s[st2[1]].sample_rate * 1. / base_sr};
    const std::vector<InvalidRun> *iv[2] = {inv[st2[0]], inv[st2[1]]};
    int index[2] = {0, 0}, nflagged[2] = {0, 0};
    int is[2] = {INT_MAX, INT_MAX}, ie[2] = {INT_MAX, INT_MAX};
    const int isz[2] = {(int)iv[0]->size(), (int)iv[1]->size()};
    for (int i = 0; i < 2; i++)
      if (isz[i] > 0) {
        is[i] = (int)std::floor((*iv[i])[0].begin / scale[i]);
        ie[i] = is[i] + (int)std::floor((*iv[i])[index[i]].n / scale[i]);
        index[i]++;
      }
    int i = is[0] < is[1] ? 0 : 1;
    while (is[i] < INT_MAX) {
      if (is[0] == is[1]) {
        if (ie[0] == ie[1]) {
          is[0] = ie[0] + 1;
          is[1] = ie[1] + 1;
        } else {
          int k = ie[0] < ie[1] ? 0 : 1;
          is[1 - k] = ie[k];
          is[k] = ie[k] + 1;
        }
      } else if (ie[i] < is[1 - i]) {
        nflagged[1 - i] += ie[i] - is[i];
        is[i] = ie[i] + 1;
      } else {
        nflagged[1 - i] += is[1 - i] - is[i];
        is[i] = is[1 - i];
      }
      for (int k = 0; k < 2; k++) {
        if (is[k] > ie[k]) {
          if (index[k] < isz[k]) {
            is[k] = (int)std::floor((*iv[k])[index[k]].begin / scale[k]);
            ie[k] = is[k] + (int)std::floor((*iv[k])[index[k]].n / scale[k]);
            index[k]++;
          } else {
            is[k] = ie[k] = INT_MAX;
          }
        }
      }
      i = is[0] < is[1] ? 0 : 1;
    }
    nfl[b].first += nflagged[0];
    nfl[b].second += nflagged[1];
  }
}

}  // namespace sfxc
