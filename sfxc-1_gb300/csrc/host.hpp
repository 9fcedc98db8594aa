// Host-side model of the correlator-node path: time base, delay tables and
// their Akima splines, integer delays, the input-node byte protocol, and the
// plan that maps one integration's protocol onto device work (sample
// segments, counted-byte ranges for the bit statistics, invalid runs).
//
// Everything here is integer work or FP64 setup; the per-sample arithmetic
// runs in the CUDA kernels.  Semantics follow the reference classes cited at
// each declaration (paths relative to the reference project).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace sfxc {

using ticks_t = int64_t;
constexpr double kClockRate = 512000000.0;  // MAX_SAMPLE_RATE, sfxc/include/utils.h:36
constexpr int kReferenceMjd = 51544;
constexpr ticks_t kTicksPerDay = (ticks_t)86400 * 512000000LL;
enum { HEADER_DATA = 0, HEADER_INVALID = 1, HEADER_DELAY = 2, HEADER_ENDSTREAM = 3 };  // utils.h:39-42
enum { WINDOW_NONE = 0, WINDOW_RECT = 1, WINDOW_COS = 2, WINDOW_HAMMING = 3, WINDOW_HANN = 4 };
constexpr int kCorrelatorBufferSize = 8192;  // utils.h:50

struct Error : std::exception {
  int code;
  std::string msg;
  Error(int c, std::string m) : code(c), msg(std::move(m)) {}
  const char *what() const noexcept override { return msg.c_str(); }
};

// ---- Time (sfxc/include/correlator_time.h:58-91, sfxc/src/correlator_time.cc)
ticks_t time_from_mjd_sec(int mjd, double sec);
ticks_t time_from_usec(double usec);
int ticks_per_sample(double sample_rate);
double time_mjd(ticks_t t);
double time_usec_of_day(ticks_t t);
double time_sec_of_day(ticks_t t);
inline double time_diff(ticks_t a, ticks_t b) { return (double)(a - b) / kClockRate; }
ticks_t time_mul(ticks_t t, double v);
ticks_t time_div(ticks_t t, double v);
// Control_parameters::nr_ffts_per_integration_slice (sfxc/include/control_parameters.h:301-307)
int nr_ffts_per_integration_slice(double integration_time_us, int data_rate, int fft_size);

// ---- Delay tables (.del reader: Delay_table::open, sfxc/src/delay_table_akima.cc:238-372)
struct Scan {
  ticks_t begin, end;
  int first_row, nrows;
};
struct DelayTable {
  std::vector<Scan> scans;
  std::vector<double> times, delays, phases, amps;  // row columns; times relative to scan start
  std::vector<double> us, vs, ws;                    // the u, v, w columns (metres)
  double clock_offset = 0, clock_rate = 0;
  ticks_t clock_epoch = 0;
  static DelayTable parse(const uint8_t *bytes, size_t n);
};

// Akima spline over a slice (Delay_table::create_akima_spline, delay_table_akima.cc:431-502).
// Coefficients are built with the published Akima (1970) method and the
// non-periodic end conditions of GSL's akima interpolator, in the same
// operation order, so host and device evaluations reproduce the reference's
// doubles.  Column 0 = delay, 1 = phase, 2 = amplitude.
struct Spline {
  int n = 0;
  std::vector<double> x, y[3], b[3], c[3], d[3];
  ticks_t scan_begin = 0, interval_begin = 0, interval_end = 0, clock_epoch = 0;
  double clock_offset = 0, clock_rate = 0;
  // pc: phase centre, the pc-th scan starting with the covering one (an
  // additional phase centre is a scan with the same start, 313-336, 478-494)
  static Spline create(const DelayTable &t, ticks_t start, ticks_t duration, int pc = 0);
  // the spline of three columns of scan s's rows over [ib, ie] (whole seconds from the scan start)
  static Spline build(const DelayTable &t, const Scan &s, ticks_t ib, ticks_t ie,
                      const std::vector<double> *const cols[3]);
  int index(double x) const;
  double eval(int col, double x) const;
  double eval_extended(int col, double x) const;  // no domain check, as GSL 1.9's gsl_spline_eval
  double deriv(int col, double x) const;
  double delay(ticks_t t) const;       // Delay_table_akima::delay (114-126)
  double rate(ticks_t t) const;        // ::rate (128-136)
  double phase(ticks_t t) const;       // ::phase (148-156)
  double amplitude(ticks_t t) const;   // ::amplitude (158-166)
};

// ---- UVW model (Uvw_model, sfxc/src/uvw_model.cc:79-330): Akima splines of
// a delay table's u, v, w columns over the six whole seconds around a time,
// rebuilt when a later time leaves the current second, one per phase
// centre of the scan (scans with the same start).
class UvwModel {
 public:
  explicit UvwModel(DelayTable t);
  // get_uvw (312-325): u, v, w of phase centre pc at time t
  void get(int pc, ticks_t t, double out[3]);

 private:
  DelayTable t_;
  size_t scan_nr_ = 0;
  int n_sources_ = 0;
  ticks_t interval_begin_ = 0, interval_end_ = 0;
  std::vector<Spline> splines_;
  bool next_scan();
  void create(ticks_t t);
};

// ---- Integer delays (Input_node_tasklet::get_delay/get_delays, sfxc/src/input_node_tasklet.cc:235-282)
struct Delay {
  ticks_t time;
  int32_t bytes, rem;
};
Delay integer_delay(const Spline &s, ticks_t t, int sample_rate, int bits);
// Delay list for one interval as built by add_time_interval (input_node_tasklet.cc:103-115).
std::vector<Delay> interval_delays(const Spline &s, ticks_t start, ticks_t stop, int sample_rate, int bits);

// ---- Input-node protocol (Input_node_data_writer, sfxc/src/input_node_data_writer.cc:107-229,389-500)
struct InvalidRun {
  int32_t begin, n;
};
struct ChannelBlock {  // one channel-extracted block (Channel_buffer_element)
  ticks_t start;
  int64_t src_offset;  // byte offset of the block in the channel stream buffer
  int32_t size;
  std::vector<InvalidRun> invalid;
};
struct SliceRequest {
  ticks_t start, stop;
  int64_t nr_samples;
  std::vector<Delay> delays;
};
// Protocol records.  DATA records refer to payload bytes by offset into a
// source buffer: the protocol byte buffer itself when the records are parsed
// from bytes, the channel stream buffer when the writer emits them directly.
struct Record {
  uint8_t type;  // HEADER_*
  int8_t rem;    // HEADER_DELAY
  int32_t n;     // HEADER_DATA bytes / HEADER_INVALID samples
  int64_t src;   // HEADER_DATA payload offset
};
// Writes the records of every slice (one vector per slice).
std::vector<std::vector<Record>> write_protocol(const std::vector<ChannelBlock> &blocks,
                                                const std::vector<SliceRequest> &slices, int sample_rate,
                                                int bits, double integration_time_us);
void serialize_protocol(const std::vector<Record> &recs, const uint8_t *stream, std::vector<uint8_t> &out);
// Parses protocol bytes into records (payload offsets into `bytes`, plus `base`).
std::vector<Record> parse_protocol(const uint8_t *bytes, size_t n, int64_t base);

// ---- Per-integration unpack plan (replica of Bit2float_worker, sfxc/src/bit2float_worker.cc:36-436)
struct Segment {  // output samples [out0, out0+n) read from src bit src_bit (+bits per sample); src_bit<0: zeros
  int32_t out0, n;
  int64_t src_bit;
};
struct StatRange {  // counted bytes [src_byte, src_byte+n) with counter indices [cidx, cidx+n)
  int64_t src_byte;
  int32_t n, cidx;
};
struct TsysParams {  // cal-diode phase of the counted bytes (bit2float_worker.cc:299-312,341-346)
  int32_t t0, period, on0, two_bit;
};
struct UnpackPlan {
  std::vector<Segment> segs;
  std::vector<StatRange> stats;
  std::vector<InvalidRun> invalid;  // Invalid{start, n_invalid}
  int64_t n_invalid = 0;            // bit_statistics::nInvalid
  int64_t counted = 0;
  TsysParams tsys{};
  int n_blocks = 0, nfft_max = 0;   // integration length in fft_size_delaycor blocks
};
struct StreamUnpackState {  // what carries over between integrations (state, bytes_left...)
  int state = 0;
  uint64_t bytes_left = 0, invalid_left = 0, sample_in_byte = 0;
  size_t rec = 0;      // next record
  int64_t rec_off = 0;  // bytes of that record already consumed
};
UnpackPlan plan_unpack(const std::vector<Record> &recs, StreamUnpackState &st, int n_blocks, int nfft_max,
                       int fft_size, int bits, int sample_rate, int tsys_freq, double delay_at_start);

// ---- Correlation setup and output (sfxc/src/correlation_core.cc)
struct StationStream {
  int32_t station_number, station_stream, sample_rate, bandwidth, bits, tsys_freq;
  int64_t channel_freq;
  char sideband, polarisation;
  double lo_offset;
};
struct Baseline {
  int a, b;
};
std::vector<Baseline> create_baselines(const std::vector<StationStream> &s, int reference_station);  // 134-171
struct BitStats {
  // per-code counts of the counted bytes (2-bit codes 0..3, or bit values 0/1
  // at indices 0/1), with the cal diode on and off
  int64_t on[4], off[4];
  int64_t n_invalid;
  int bits, sample_rate, base_sample_rate;
  void levels(int out[5]) const;  // bit_statistics::get_statistics (bit_statistics.cc:81-111)
  void tsys(int out[4]) const;    // ::get_tsys (113-139)
};
// Correlation_core::find_invalid (599-665): per cross baseline {flagged a, flagged b}
void find_invalid(const std::vector<StationStream> &s, int base_sr, const std::vector<Baseline> &bl,
                  const std::vector<const std::vector<InvalidRun> *> &inv, std::vector<std::pair<int64_t, int64_t>> &nfl);

}  // namespace sfxc
