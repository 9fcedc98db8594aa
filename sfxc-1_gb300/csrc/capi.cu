// C ABI of the correlator-node path (include/sfxc_gpu.h): job setup, per-
// integration planning on the host, kernel launches on one CUDA stream, and
// the byte layout of the correlator output (Correlation_core::integration_write,
// sfxc/src/correlation_core.cc:316-477; headers sfxc/include/output_header.h:100-148).
#include <algorithm>
#include <array>
#include <chrono>
#include <tuple>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "control.hpp"
#include "formats.hpp"
#include "host.hpp"
#include "kernels.hpp"
#include "sfxc_gpu.h"

using namespace sfxc;

namespace {

thread_local std::string g_error;

struct CudaError : Error {
  CudaError(cudaError_t e, const char *what)
      : Error(SFXC_GPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e)) {}
};
#define CK(x)                                  \
  do {                                         \
    cudaError_t e_ = (x);                      \
    if (e_ != cudaSuccess) throw CudaError(e_, #x); \
  } while (0)

// While a batch plans several integrations whose device work runs later,
// buffers that grow keep their old allocation alive (work already recorded
// refers to it) and free it once the batch has run.
thread_local std::vector<void *> *g_retired = nullptr;

// Device buffer that only grows.  Move-only: freeing device memory
// synchronises the whole device, so buffers are kept and handed on (swap)
// rather than freed between jobs.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), cap(o.cap) {
    o.p = nullptr;
    o.cap = 0;
  }
  void swap(DevBuf &o) noexcept {
    std::swap(p, o.p);
    std::swap(cap, o.cap);
  }
  void *ensure(size_t n) {
    if (n > cap) {
      if (p) {
        if (g_retired)
          g_retired->push_back(p);
        else
          cudaFree(p);
      }
      p = nullptr;
      cap = 0;
      CK(cudaMalloc(&p, n));
      cap = n;
    }
    return p;
  }
  template <class T>
  T *as() const { return reinterpret_cast<T *>(p); }
  ~DevBuf() {
    if (!p) return;
    if (g_retired)
      g_retired->push_back(p);
    else
      cudaFree(p);
  }
};

// Pinned host staging that only grows (asynchronous uploads; freeing pinned
// memory synchronises the device, so it is kept).
struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  HostBuf() = default;
  HostBuf(const HostBuf &) = delete;
  HostBuf &operator=(const HostBuf &) = delete;
  void *ensure(size_t n) {
    if (n > cap) {
      if (p) cudaFreeHost(p);
      p = nullptr;
      cap = 0;
      CK(cudaHostAlloc(&p, n, cudaHostAllocDefault));
      cap = n;
    }
    return p;
  }
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
};

struct StreamCtx {
  std::vector<Record> recs;
  StreamUnpackState ust;
  std::vector<Record> pending;  // records of the bytes pushed for the next integration
  int64_t dev_bytes = 0;        // bytes of that input already on the device
  bool pushed = false;
  UnpackPlan plan;
  BitStats stats{};
  Spline sp;
  std::vector<Spline> sp_pc;  // extra phase centres 1.. (host only: the uvshift parameters)
  int n_blocks = 0, nfft_max = 0, rot = 0, hop = 0;
  DevBuf src, segs, stat_rng, spline, bpar;
  void take_buffers(StreamCtx &o) {
    src.swap(o.src);
    segs.swap(o.segs);
    stat_rng.swap(o.stat_rng);
    spline.swap(o.spline);
    bpar.swap(o.bpar);
  }
};

struct Polyco {
  double tmid, dm, ref_phase, ref_freq, obs_freq;
  std::vector<double> coef;
};

// Device work of one integration, recorded while the host plans it and run
// afterwards, eagerly or under stream capture (a batch of jobs in one CUDA
// graph).  Buffers are sized while recording, so running allocates nothing;
// the payloads of the uploads are kept here and copied into the context's
// pinned arena before the work runs.
struct Ops {
  std::vector<std::function<cudaError_t(const uint8_t *)>> ops;  // argument: the pinned arena
  std::vector<uint8_t> host;                                     // upload payloads, 16-byte aligned
  void clear() {
    ops.clear();
    host.clear();
  }
  void upload(DevBuf &b, const void *src, size_t n, cudaStream_t st) {
    b.ensure(n ? n : 16);
    if (!n) return;
    const size_t off = (host.size() + 15) & ~(size_t)15;
    host.resize(off + n);
    std::memcpy(host.data() + off, src, n);
    void *dst = b.p;
    ops.push_back([=](const uint8_t *arena) { return cudaMemcpyAsync(dst, arena + off, n, cudaMemcpyHostToDevice, st); });
  }
  void memset(void *p, int v, size_t n, cudaStream_t st) {
    ops.push_back([=](const uint8_t *) { return cudaMemsetAsync(p, v, n, st); });
  }
  // a dependency between the context's streams (inside a capture: an edge of the graph)
  void record(cudaEvent_t e, cudaStream_t st) {
    ops.push_back([=](const uint8_t *) { return cudaEventRecord(e, st); });
  }
  // a timing mark (inside a capture: an event-record node, so that the
  // event's time can be read after the graph ran)
  void mark(cudaEvent_t e, cudaStream_t st) {
    ops.push_back([=](const uint8_t *) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      const cudaError_t r = cudaStreamIsCapturing(st, &cs);
      if (r != cudaSuccess) return r;
      return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal)
                                                 : cudaEventRecord(e, st);
    });
  }
  void wait(cudaStream_t st, cudaEvent_t e) {
    ops.push_back([=](const uint8_t *) { return cudaStreamWaitEvent(st, e, 0); });
  }
  template <class F>
  void op(F f) {  // f returns a cudaError_t
    ops.push_back([f](const uint8_t *) { return f(); });
  }
  template <class F>
  void kernel(F f) {  // f launches; the launch error is checked
    ops.push_back([f](const uint8_t *) {
      f();
      return cudaGetLastError();
    });
  }
};

// What finish_integration needs of an enqueued integration.
struct Pending {
  std::vector<int64_t> n_invalid;  // per stream, of this integration's unpack plan
  ticks_t start = 0;
  size_t nvis = 0, ev = 0;
  int nout = 0, nphs = 0, launches = 0;
  bool pulsar = false;
  std::vector<std::pair<int64_t, int64_t>> nfl;
  uint8_t *res = nullptr;
};

// One integration in flight: its recorded work, the pinned copy of its
// upload payloads, its pinned results, its timing events and what finishing
// it needs.  A context has one slot per integration that can be in flight
// at once (several when a batch runs several integrations of it in one
// graph).
struct Slot {
  Ops q;
  HostBuf arena, results;
  Pending pend;
  std::vector<cudaEvent_t> evs;   // timing marks
  std::vector<cudaEvent_t> deps;  // dependencies between the context's two streams
  cudaEvent_t ev0 = nullptr;
  ~Slot() {
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    for (cudaEvent_t e : deps) cudaEventDestroy(e);
    if (ev0) cudaEventDestroy(ev0);
  }
};

// Host-side per-launch tables uploaded once per job.
struct JobTables {
  std::vector<int> blmap, tiles, blpairs;
  int npad = 0, ntiles = 0;
};

// Device buffers of a recording (sfxc_gpu_recording_*), kept by the
// context for the next recording once one is destroyed.
struct RecordingBuffers {
  DevBuf own, frames, chan, tracks, list, gathered, counts, offs, runs, info;
  std::vector<DevBuf> proto;           // protocol bytes per channel
  std::map<int, DevBuf> plan_recs;     // the protocol records of the last plan of each group
  HostBuf staging;                     // decoded headers on their way to the host
};

}  // namespace

struct sfxc_gpu_ctx {
  int device = 0, x_mode = 0;
  cudaStream_t st = nullptr;
  // second stream: the next chunk's per-block parameters (FP64) beside the
  // current chunk's X-step
  cudaStream_t st2 = nullptr;
  // third stream: a chunk's X-step beside the next chunk's F-step
  cudaStream_t st3 = nullptr;
  float timings[7] = {};
  std::string err;
  bool have_job = false;
  // job
  sfxc_correlation_params p{};
  std::vector<StationStream> streams;
  std::vector<DelayTable> tables;
  std::vector<int> stream_table;
  std::vector<Polyco> polyco;
  int current_integration = 0;  // integrations finished (output written)
  int planned_integration = 0;  // integrations planned (several may be in flight in a batch)
  std::vector<StreamCtx> sc;
  std::vector<Baseline> bl;
  JobTables jt;
  int M = 0, K = 0, Nd = 0, kpad = 0, nffts = 0, nsub = 0, nbins = 1;
  // spectral reduction: output channels nch (< M when reducing), Kout = nch + 1;
  // mask (M + 1), lag window (2 nch), exp(-2 pi i k / 2M) (k < 2M), reduced output
  int nch = 0, Kout = 0, rnorm = 0;
  DevBuf rmask, rlag, rtw, rout;
  // extra phase centres: count (1: the pointing centre only), output file
  // index per centre, window-autocorrelation weights (create_weights), the
  // centres' accumulators [centre][baseline][kpad] and the chunks' uvshift
  // parameters [chunk][centre - 1][baseline]
  int npc = 1;
  std::vector<int32_t> pc_file;
  int phased = 0;  // phased-array core
  // UVW per stream and phase centre for the timeslice headers (sfxc_gpu_set_uvw)
  std::vector<double> uvw;
  std::vector<float> pc_weights;
  DevBuf pcacc, uvp;
  // device
  DevBuf streamdev, tw256, ts, spec, acc, out, norms, flagfac, blmap, tiles, blpairs, items, bins,
      offsets, derr;
  DevBuf rowlist, segs;  // pulsar binning on the tensor cores: rows of each channel sorted by bin, and the runs
  DevBuf xpart;          // FP32 X-step: partial sums of its row blocks
  int bins_rows = 0;     // rows of the last integration's bin table (pulsar)
  DevBuf xin, xtracks, xout;  // channel extraction
  // per windowed-FFT length (streams of different sample rates): window and
  // twiddle tables, and the stream descriptors grouped by length
  struct RotTables {
    DevBuf window, twrot;
  };
  std::map<int, RotTables> rot_tables;
  // integrations in flight (slot 0: the next one)
  std::vector<std::unique_ptr<Slot>> slots;
  // the last chunk of the last integration, for the autotuner: its stream
  // descriptors (block order, then grouped by windowed-FFT length), the
  // groups (rot, first, count) and the launch sizes
  struct TuneSpec {
    StreamDev *dchunk = nullptr;
    int nstreams = 0, max_blocks = 0, nrows = 0, max_rows = 0, M = 0, kpad = 0, tc_slots = 0, window = 0;
    float tc_scale = 1.f;
    void *spec = nullptr;
    std::vector<std::array<int, 3>> groups;
  } tune;
  // bit-statistics counters of all streams (8 per stream), and the pinned
  // landing area of an integration's results: visibilities, counters, the
  // X-step's error flag (one readback copy each)
  DevBuf hist;
  std::vector<StreamDev> hsd;
  // buffers of destroyed recordings, for the next ones
  std::vector<std::unique_ptr<RecordingBuffers>> rec_spare;
};

namespace {

// CTAs per SM of the per-block parameter launches beside the X-step (0:
// uncapped; caps of 1, 2 and 4 measured slower: the launch then runs longer
// and slows the X-step for longer)
constexpr int kSideParamCtas = 0;

// ---- plan cache of the autotuner: launch shapes of the F-step kernels per
// job shape, shared by every context of the process.  Keys: (kernel, and
// what decides its best shape); values: the variant (0 or absent: the
// launcher's default).  Only launch shapes that leave every result bit
// unchanged are tuned.
enum PlanKnob { kKnobBlockStage = 0, kKnobWindowFft = 1 };
std::mutex g_plan_mu;
std::map<std::array<int, 4>, int> g_plan;

int ilog2c(int x) {
  int l = 0;
  while ((1 << l) < x) l++;
  return l;
}
std::array<int, 4> block_key(int nstreams, int max_blocks) { return {kKnobBlockStage, nstreams, ilog2c(max_blocks), 0}; }
std::array<int, 4> window_key(int rot, int nstreams, int nrows) {
  return {kKnobWindowFft, rot, nstreams, ilog2c(nrows)};
}
int plan_get(const std::array<int, 4> &k) {
  std::lock_guard<std::mutex> lock(g_plan_mu);
  auto it = g_plan.find(k);
  return it == g_plan.end() ? 0 : it->second;
}
void plan_set(const std::array<int, 4> &k, int v) {
  std::lock_guard<std::mutex> lock(g_plan_mu);
  g_plan[k] = v;
}

int fail(sfxc_gpu_ctx *c, const Error &e) {
  if (c) c->err = e.msg;
  g_error = e.msg;
  return e.code;
}

void upload(DevBuf &b, const void *src, size_t n, cudaStream_t st) {
  b.ensure(n ? n : 16);
  if (n) CK(cudaMemcpyAsync(b.p, src, n, cudaMemcpyHostToDevice, st));
}

// Twiddle tables exp(-2 pi i m / n), computed in double and rounded once.
void twiddles(std::vector<float2> &v, int n) {
  for (int m = 0; m < n; m++) {
    double a = -2.0 * M_PI * (double)m / (double)n;
    v.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
  }
}

// Delay_correction::create_window (sfxc/src/delay_correction.cc:300-341)
std::vector<float> make_window(int type, int n) {
  std::vector<float> w(n);
  for (int i = 0; i < n; i++) {
    double v = 0;
    switch (type) {
      case WINDOW_NONE: v = i < n / 2 ? 1 : 0; break;
      case WINDOW_RECT: v = (i >= n / 4 && i < 3 * n / 4) ? 1 : 0; break;
      case WINDOW_COS: v = std::sin(M_PI * i / (n - 1)); break;
      case WINDOW_HAMMING: v = 0.54 - 0.46 * std::cos(2 * M_PI * i / (n - 1)); break;
      case WINDOW_HANN: v = 0.5 * (1 - std::cos(2 * M_PI * i / (n - 1))); break;
      default: throw Error(SFXC_GPU_EINVAL, "invalid window function");
    }
    w[i] = (float)v;
  }
  return w;
}

template <class T>
void put(std::vector<uint8_t> &o, const T &v) {
  const uint8_t *p = reinterpret_cast<const uint8_t *>(&v);
  o.insert(o.end(), p, p + sizeof(T));
}

// Lag window of the spectral reduction when the ctrl file gives none:
// Correlation_core::create_window (sfxc/src/correlation_core.cc:760-810) for
// n = 2 nch lags out of m = 2M, with the cos / hamming / hann functions of
// (n, i) and convolve (667-706), in FP64, kept in FP32 as the reference
// keeps it.  The convolutions cost O(n m): kept per (nch, M, window).
std::vector<float> reduction_window(int nch, int M, int window) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int>, std::vector<float>> cache;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(nch, M, window);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  const int n = 2 * nch, m = 2 * M;
  std::vector<double> w(n, 0.0);
  if (window == WINDOW_NONE || window == WINDOW_RECT) {
    w[0] = 1.;
    for (int i = 1; i < n / 2; i++) w[i] = w[n - i] = (1. - 2. * i / n) / (1. - 2. * i / m);
    w[n / 2] = 0.;
  } else {
    auto f = [window](int len, int i) {
      if (window == WINDOW_COS) return std::sin(M_PI * i / len);
      if (window == WINDOW_HAMMING) return 0.54 - 0.46 * std::cos(2 * M_PI * i / len);
      return 0.5 * (1 - std::cos(2 * M_PI * i / len));
    };
    std::vector<double> fn(n + 1), fm(m + 1);
    for (int j = 0; j <= n; j++) fn[j] = f(n, j);
    for (int j = 0; j <= m; j++) fm[j] = f(m, j);
    auto conv = [](const std::vector<double> &fv, int len, int i) {  // sum over j of f(j) f(i + len/2 - j)
      double sum = 0.0;
      i += len / 2;
      for (int j = 0; j <= len; j++) {
        if (i - j < 0 || i - j > len) continue;
        sum += fv[j] * fv[i - j];
      }
      return sum;
    };
    const int r = m / n;  // integer ratio, as in the reference
    w[0] = r * conv(fn, n, n / 2) / conv(fm, m, m / 2);
    for (int i = 1; i < n / 2; i++) w[i] = w[n - i] = r * conv(fn, n, n / 2 + i) / conv(fm, m, m / 2 + i);
    w[n / 2] = r * conv(fn, n, n) / conv(fm, m, (n + m) / 2);
  }
  std::vector<float> out(w.begin(), w.end());
  cache.emplace(key, out);
  return out;
}

// Amplitude weights of the extra phase centres: Correlation_core::
// create_weights (sfxc/src/correlation_core.cc:708-744) -- the
// autocorrelation of the window of 2M - 1 points (rect / cos / hamming /
// hann of (n, i), 667-690) zero-padded to 4M, normalised at lag 0, for lags
// below M.  The reference takes it through FP32 FFTs; here an FP64 direct
// sum (once per (M, window)), rounded to FP32.
std::vector<float> phase_center_weights(int M, int window) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::vector<float>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find({M, window});
  if (it != cache.end()) return it->second;
  const int n = 2 * M - 1;
  std::vector<double> f(2 * M);
  for (int i = 0; i < 2 * M; i++) {
    if (window == WINDOW_NONE || window == WINDOW_RECT)
      f[i] = (i >= n / 4 && i < (3 * n) / 4) ? 1.0 : 0.0;
    else if (window == WINDOW_COS)
      f[i] = std::sin(M_PI * i / n);
    else if (window == WINDOW_HAMMING)
      f[i] = 0.54 - 0.46 * std::cos(2 * M_PI * i / n);
    else
      f[i] = 0.5 * (1 - std::cos(2 * M_PI * i / n));
    f[i] = (float)f[i];  // the reference keeps the window in FP32
  }
  std::vector<double> r(M);
  for (int lag = 0; lag < M; lag++) {  // the zero padding makes the circular autocorrelation linear here
    double sum = 0.0;
    for (int i = 0; i + lag < 2 * M; i++) sum += f[i] * f[i + lag];
    r[lag] = sum;
  }
  std::vector<float> w(M);
  for (int lag = 0; lag < M; lag++) w[lag] = (float)(r[lag] / r[0]);
  cache.emplace(std::make_pair(M, window), w);
  return w;
}

void set_parameters(sfxc_gpu_ctx *c, const sfxc_correlation_params *p) {
  if (!p || p->n_streams <= 0 || !p->streams) throw Error(SFXC_GPU_EINVAL, "no streams");
  if (p->fft_size_delaycor != kNd) throw Error(SFXC_GPU_EINVAL, "fft_size_delaycor must be 256");
  if (p->number_channels < 2 || p->number_channels > p->fft_size_correlation ||
      (p->number_channels & (p->number_channels - 1)))
    throw Error(SFXC_GPU_EINVAL, "number_channels must be a power of two no larger than fft_size_correlation");
  if (p->fft_size_correlation < kNd || (p->fft_size_correlation & (p->fft_size_correlation - 1)))
    throw Error(SFXC_GPU_EINVAL, "fft_size_correlation must be a power of two >= 256");
  if (p->window < WINDOW_NONE || p->window > WINDOW_HANN) throw Error(SFXC_GPU_EINVAL, "invalid window");
  if (p->n_delay_tables <= 0 || !p->delay_tables) throw Error(SFXC_GPU_EINVAL, "no delay tables");
  c->p = *p;
  c->p.streams = nullptr;
  c->p.delay_tables = nullptr;
  c->p.mask = c->p.lag_window = nullptr;  // caller-owned; copied below
  c->p.polyco = nullptr;
  c->tables.clear();
  for (int i = 0; i < p->n_delay_tables; i++) {
    const sfxc_delay_table &t = p->delay_tables[i];
    if (!t.del_bytes || t.del_size < 4) throw Error(SFXC_GPU_EDELTAB, "empty delay table");
    DelayTable dt = DelayTable::parse(t.del_bytes, t.del_size);
    dt.clock_offset = t.clock_offset;
    dt.clock_rate = t.clock_rate;
    dt.clock_epoch = t.clock_epoch_ticks;
    c->tables.push_back(std::move(dt));
  }
  c->streams.clear();
  c->stream_table.clear();
  for (int i = 0; i < p->n_streams; i++) {
    const sfxc_station_stream &s = p->streams[i];
    if (s.bits_per_sample != 1 && s.bits_per_sample != 2) throw Error(SFXC_GPU_EINVAL, "bits_per_sample must be 1 or 2");
    if (s.sample_rate <= 0 || s.bandwidth <= 0) throw Error(SFXC_GPU_EINVAL, "bad stream sample rate or bandwidth");
    if (s.delay_table < 0 || s.delay_table >= p->n_delay_tables) throw Error(SFXC_GPU_EINVAL, "bad delay table index");
    // the node's input number of the stream (a station's second polarisation
    // numbered after every station's first; a station missing from the scan
    // leaves a gap): streams are taken in array order, the numbers only
    // have to be distinct
    if (s.station_stream < 0) throw Error(SFXC_GPU_EINVAL, "station_stream must not be negative");
    for (int j = 0; j < i; j++)
      if (p->streams[j].station_stream == s.station_stream) throw Error(SFXC_GPU_EINVAL, "station_stream repeated");
    if (s.bits_per_sample == 2 && s.tsys_freq <= 0) throw Error(SFXC_GPU_EINVAL, "tsys_freq must be positive");
    StationStream ss{s.station_number, s.station_stream, s.sample_rate, s.bandwidth, s.bits_per_sample, s.tsys_freq,
                     s.channel_freq, s.sideband, s.polarisation, s.lo_offset};
    c->streams.push_back(ss);
    c->stream_table.push_back(s.delay_table);
  }
  c->polyco.clear();
  c->nbins = 1;
  if (p->pulsar_nbins > 0) {
    if (p->n_polyco <= 0 || !p->polyco) throw Error(SFXC_GPU_EINVAL, "pulsar binning without polyco");
    for (int i = 0; i < p->n_polyco; i++) {
      const sfxc_polyco &q = p->polyco[i];
      if (q.n_coef < 2 || !q.coef) throw Error(SFXC_GPU_EINVAL, "polyco needs at least two coefficients");
      c->polyco.push_back(Polyco{q.tmid, q.dm, q.ref_phase, q.ref_freq, q.obs_freq,
                                 std::vector<double>(q.coef, q.coef + q.n_coef)});
    }
    c->nbins = p->pulsar_nbins + 1;
  }
  c->npc = std::max(1, (int)p->n_phase_centers);
  if (c->npc > 1 && c->nbins > 1) throw Error(SFXC_GPU_EINVAL, "extra phase centres cannot be combined with pulsar binning");
  c->pc_file.assign(c->npc, 0);
  if (p->phase_center_file_index) c->pc_file.assign(p->phase_center_file_index, p->phase_center_file_index + c->npc);
  c->p.phase_center_file_index = nullptr;
  c->uvw.assign((size_t)p->n_streams * c->npc * 3, 0.0);
  c->phased = p->phased_array != 0;
  if (c->phased && (c->nbins > 1 || c->npc > 1 || p->number_channels != p->fft_size_correlation))
    throw Error(SFXC_GPU_EINVAL,
                "the phased-array core takes no pulsar binning, extra phase centres or spectral reduction");
  c->M = p->fft_size_correlation;
  c->K = c->M + 1;
  c->nch = p->number_channels;
  c->Kout = c->nch + 1;
  if (c->npc > 1) c->pc_weights = phase_center_weights(c->M, p->window);
  if (c->nch < c->M) {  // spectral reduction tables
    std::vector<float> mk(p->mask ? p->mask : nullptr, p->mask ? p->mask + c->M + 1 : nullptr);
    if (!p->mask) mk.assign(c->M + 1, 1.0f);
    std::vector<float> lw = p->lag_window ? std::vector<float>(p->lag_window, p->lag_window + 2 * c->nch)
                                          : reduction_window(c->nch, c->M, p->window);
    std::vector<float2> tw(2 * (size_t)c->M);
    for (size_t k = 0; k < tw.size(); k++) {
      const double a = -M_PI * (double)k / c->M;
      tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    upload(c->rmask, mk.data(), mk.size() * sizeof(float), c->st);
    upload(c->rlag, lw.data(), lw.size() * sizeof(float), c->st);
    upload(c->rtw, tw.data(), tw.size() * sizeof(float2), c->st);
    c->rnorm = p->mask_normalize != 0;
  }
  c->Nd = p->fft_size_delaycor;
  c->kpad = c->M + 4;
  const int nr = nr_ffts_per_integration_slice((double)p->integration_time_us, p->sample_rate, c->M);
  c->nffts = nr - (p->window != WINDOW_NONE ? 1 : 0);
  c->nsub = nr_ffts_per_integration_slice((double)p->sub_integration_time_us, p->sample_rate, c->M);
  if (c->nffts <= 0) throw Error(SFXC_GPU_EINVAL, "integration shorter than two FFTs");
  {  // fresh stream state; the device buffers of the previous job are reused
    std::vector<StreamCtx> prev;
    prev.swap(c->sc);
    c->sc.resize(p->n_streams);
    for (size_t i = 0; i < prev.size() && i < c->sc.size(); i++) c->sc[i].take_buffers(prev[i]);
  }
  for (int i = 0; i < p->n_streams; i++) {
    StreamCtx &s = c->sc[i];
    const StationStream &ss = c->streams[i];
    const int nfft_min = std::max(c->M / c->Nd, 1);
    s.nfft_max = (int)(((uint64_t)std::max(kCorrelatorBufferSize / c->Nd, nfft_min) * (uint64_t)ss.sample_rate) /
                       p->sample_rate);
    s.n_blocks = (int)(((uint64_t)(c->M / c->Nd) * nr * (uint64_t)ss.sample_rate) / p->sample_rate);
    s.rot = (int)(((uint64_t)2 * c->M * (uint64_t)ss.sample_rate) / p->sample_rate);
    s.hop = s.rot / 2;
    if (s.rot & (s.rot - 1)) throw Error(SFXC_GPU_EINVAL, "FFT length per stream must be a power of two");
    if (s.rot > 32768 || s.rot < 512)
      throw Error(SFXC_GPU_EINVAL, "windowed FFT lengths must lie within 512..32768 samples");
  }
  c->bl = create_baselines(c->streams, p->reference_station);
  // stream-pair tiles of the X-step and the map pair -> baseline
  JobTables &jt = c->jt;
  const int N = p->n_streams;
  jt.npad = (N + 3) / 4 * 4;
  jt.blmap.assign((size_t)jt.npad * jt.npad, -1);
  jt.blpairs.clear();
  for (size_t b = 0; b < c->bl.size(); b++) {
    const int a = c->bl[b].a, bb = c->bl[b].b;
    const int i = std::min(a, bb), j = std::max(a, bb);
    jt.blmap[(size_t)i * jt.npad + j] = (int)(b << 1) | (a > bb ? 1 : 0);
    jt.blpairs.push_back(a);
    jt.blpairs.push_back(bb);
  }
  jt.tiles.clear();
  const int T4 = jt.npad / 4;
  for (int I = 0; I < T4; I++)
    for (int J = I; J < T4; J++) {
      bool used = false;
      for (int p_ = 0; p_ < 4; p_++)
        for (int q = 0; q < 4; q++) used |= jt.blmap[(size_t)(4 * I + p_) * jt.npad + 4 * J + q] >= 0;
      if (used) {
        jt.tiles.push_back(I);
        jt.tiles.push_back(J);
      }
    }
  jt.ntiles = (int)jt.tiles.size() / 2;
  if (xcorr_f32_plan(jt.ntiles, jt.npad).tpw <= 0)
    throw Error(SFXC_GPU_EINVAL, "the FP32 X-step takes at most 128 streams per job");
  if (c->x_mode == SFXC_GPU_X_TC_HILO && N > kTcSlotsWide)
    throw Error(SFXC_GPU_EINVAL, "the tensor-core X-step takes at most 64 streams per job");
  upload(c->blmap, jt.blmap.data(), jt.blmap.size() * 4, c->st);
  upload(c->tiles, jt.tiles.data(), jt.tiles.size() * 4, c->st);
  upload(c->blpairs, jt.blpairs.data(), jt.blpairs.size() * 4, c->st);
  // twiddle tables: 256/128 for the block stage, rot and rot/2 for the windowed FFT
  std::vector<float2> tw;
  twiddles(tw, 256);
  twiddles(tw, 128);
  upload(c->tw256, tw.data(), tw.size() * sizeof(float2), c->st);
  std::set<int> rots;
  for (const StreamCtx &s : c->sc) rots.insert(s.rot);
  for (int rot : rots) {  // one window and twiddle table per FFT length
    sfxc_gpu_ctx::RotTables &t = c->rot_tables[rot];
    std::vector<float2> twr;
    twiddles(twr, rot);
    twiddles(twr, rot / 2);
    upload(t.twrot, twr.data(), twr.size() * sizeof(float2), c->st);
    std::vector<float> win = make_window(p->window, rot);
    upload(t.window, win.data(), win.size() * 4, c->st);
  }
  CK(cudaStreamSynchronize(c->st));
  c->current_integration = 0;
  c->planned_integration = 0;
  c->have_job = true;
}

// Delay_correction output chunking (sfxc/src/delay_correction.cc:31-36) and the
// sub-integration dumps of Correlation_core::do_task (correlation_core.cc:48-72):
// returns the row ranges accumulated between dumps.
std::vector<std::pair<int, int>> subint_ranges(const sfxc_gpu_ctx *c) {
  const StreamCtx &s = c->sc[0];
  std::vector<std::pair<int, int>> r;
  int tb = 0, cur = 0, start = 0, next_sub = 1;
  const int minus = c->p.window != WINDOW_NONE ? 1 : 0;
  for (int c0 = 0; c0 < s.n_blocks; c0 += s.nfft_max) {
    const int nb = std::min(s.nfft_max, s.n_blocks - c0);
    const int nc = (nb * c->Nd + tb) / s.hop - minus;
    tb += nb * c->Nd - nc * s.hop;
    if (nc <= 0) continue;
    cur += nc;
    if (cur == c->nffts || (c->nsub > 0 && cur >= next_sub * c->nsub)) {
      r.push_back({start, cur});
      start = cur;
      if (cur != c->nffts) next_sub++;
    }
  }
  if (start != c->nffts) r.push_back({start, c->nffts});
  return r;
}

// bls: the baselines written (the job's, or the phased core's one (0, 0)
// entry per sub-integration, Correlation_core_phased::create_baselines).
void serialize_integration(sfxc_gpu_ctx *c, const std::vector<Baseline> &bls, const float2 *vis, int32_t source_nr,
                           int centre, const std::vector<std::pair<int64_t, int64_t>> &nfl, std::vector<uint8_t> &o) {
  const int N = (int)c->streams.size();
  const int nbl = (int)bls.size();
  put(o, source_nr);
  // stations in stream order, each with its first stream
  std::vector<std::pair<int, int>> stations;
  std::set<int> seen;
  for (int i = 0; i < N; i++)
    if (seen.insert(c->streams[i].station_number).second) stations.push_back({c->streams[i].station_number, i});
  put(o, (int32_t)(c->p.integration_nr + c->current_integration));
  put(o, (int32_t)nbl);
  put(o, (int32_t)stations.size());
  put(o, (int32_t)N);
  for (auto &s : stations) {
    put(o, (int32_t)s.first);
    put(o, (int32_t)0);
    for (int k = 0; k < 3; k++) put(o, c->uvw[((size_t)s.second * c->npc + centre) * 3 + k]);
  }
  for (int i = 0; i < N; i++) {
    o.push_back((uint8_t)c->streams[i].station_number);
    o.push_back((uint8_t)c->p.frequency_nr);
    o.push_back((uint8_t)(c->p.sideband == 'L' ? 0 : 1));
    o.push_back((uint8_t)(c->streams[i].polarisation == 'R' ? 0 : 1));
    int lv[5];
    c->sc[i].stats.levels(lv);
    int32_t l[5];
    if (c->streams[i].bits == 2) {
      l[0] = lv[0]; l[1] = lv[1]; l[2] = lv[2]; l[3] = lv[3];
    } else {
      l[0] = 0; l[1] = lv[0]; l[2] = lv[1]; l[3] = 0;
    }
    l[4] = lv[4];
    for (int k = 0; k < 5; k++) put(o, l[k]);
  }
  const int64_t total = (int64_t)c->nffts * c->M;
  const size_t K = (size_t)c->Kout;  // output channels + 1
  for (int b = 0; b < nbl; b++) {
    int lv[5];
    c->sc[bls[b].a].stats.levels(lv);
    int64_t w = bls[b].a == bls[b].b ? total - lv[4] : total - lv[4] - nfl[b].first;
    put(o, (int32_t)std::max<int64_t>(w, 0));
    o.push_back((uint8_t)c->streams[bls[b].a].station_number);
    o.push_back((uint8_t)c->streams[bls[b].b].station_number);
    o.push_back((uint8_t)((c->streams[bls[b].a].polarisation == 'R' ? 0 : 1) |
                          ((c->streams[bls[b].b].polarisation == 'R' ? 0 : 1) << 1) |
                          ((c->p.sideband == 'U' ? 1 : 0) << 2) | ((c->p.frequency_nr & 31) << 3)));
    o.push_back((uint8_t)' ');
    const uint8_t *d = reinterpret_cast<const uint8_t *>(vis + (size_t)b * K);
    o.insert(o.end(), d, d + K * sizeof(float2));
  }
}

// Node interval (the device search's answer) of the first block start of a
// launch; the block kernel walks forward from it.
int spline_lo_for(const StreamDev &d, const std::vector<double> &x) {
  const double v = (double)(d.start_ticks + (int64_t)d.block0 * kNd * d.tps - d.scan_begin) * (1.0 / 512000000.0);
  int lo = 0, hi = (int)x.size() - 1;
  while (hi > lo + 1) {
    const int i = (hi + lo) >> 1;
    if (x[i] > v)
      hi = i;
    else
      lo = i;
  }
  return lo;
}

// Host planning of the context's next integration, with its device work
// recorded into slot k (run by run_ops, eagerly or under stream capture) and
// what finish_integration needs kept there.  Sizes every device buffer
// and creates every event it uses, so running the work allocates nothing.
Slot &slot_of(sfxc_gpu_ctx *c, int k) {
  while ((int)c->slots.size() <= k) {
    std::unique_ptr<Slot> sl(new Slot());
    CK(cudaEventCreate(&sl->ev0));
    c->slots.push_back(std::move(sl));
  }
  return *c->slots[k];
}

void enqueue_integration(sfxc_gpu_ctx *c, int k = 0, bool require_push = true) {
  Slot &sl = slot_of(c, k);
  Ops &q = sl.q;
  q.clear();
  if (!c->have_job) throw Error(SFXC_GPU_ESTATE, "no parameters set");
  const int N = (int)c->streams.size();
  for (int i = 0; i < N; i++)
    if (require_push && !c->sc[i].pushed) throw Error(SFXC_GPU_ESTATE, "a stream has no input for this integration");
  const ticks_t tint = time_from_usec((double)c->p.integration_time_us);
  const ticks_t start = c->p.start_ticks + (ticks_t)c->planned_integration * tint;
  c->planned_integration++;
  const int M = c->M, K = c->K, kpad = c->kpad, nbl = (int)c->bl.size();
  cudaStream_t st = c->st;
  // ---- host planning per stream (Bit2float_worker state machine replica)
  c->hsd.assign(N, StreamDev{});
  c->hist.ensure((size_t)N * 64);
  q.memset(c->hist.p, 0, (size_t)N * 64, st);
  std::vector<int4> items;
  for (int i = 0; i < N; i++) {
    StreamCtx &s = c->sc[i];
    const StationStream &ss = c->streams[i];
    s.sp = Spline::create(c->tables[c->stream_table[i]], start, tint);
    s.sp_pc.clear();
    for (int pc = 1; pc < c->npc; pc++) s.sp_pc.push_back(Spline::create(c->tables[c->stream_table[i]], start, tint, pc));
    std::vector<Record> recs(s.recs.begin() + (long)s.ust.rec, s.recs.end());
    recs.insert(recs.end(), s.pending.begin(), s.pending.end());
    s.pending.clear();
    s.ust.rec = 0;
    s.recs.swap(recs);
    s.plan = plan_unpack(s.recs, s.ust, s.n_blocks, s.nfft_max, c->Nd, ss.bits, ss.sample_rate, ss.tsys_freq,
                         s.sp.delay(start));
    if (s.plan.segs.empty()) s.plan.segs.push_back(Segment{0, s.n_blocks * c->Nd, -1});
    q.upload(s.segs, s.plan.segs.data(), s.plan.segs.size() * sizeof(Segment), st);
    q.upload(s.stat_rng, s.plan.stats.data(), s.plan.stats.size() * sizeof(StatRange), st);
    std::vector<double> spl;
    spl.insert(spl.end(), s.sp.x.begin(), s.sp.x.end());
    for (int k = 0; k < 3; k++) {
      spl.insert(spl.end(), s.sp.y[k].begin(), s.sp.y[k].end());
      spl.insert(spl.end(), s.sp.b[k].begin(), s.sp.b[k].end());
      spl.insert(spl.end(), s.sp.c[k].begin(), s.sp.c[k].end());
      spl.insert(spl.end(), s.sp.d[k].begin(), s.sp.d[k].end());
    }
    q.upload(s.spline, spl.data(), spl.size() * 8, st);
    StreamDev &d = c->hsd[i];
    d.src = s.src.as<uint8_t>();
    d.segs = s.segs.as<DevSegment>();
    d.nsegs = (int)s.plan.segs.size();
    d.bits = ss.bits;
    d.stats = s.stat_rng.as<DevStatRange>();
    d.nstats = (int)s.plan.stats.size();
    d.tsys_t0 = s.plan.tsys.t0;
    d.tsys_period = s.plan.tsys.period;
    d.tsys_on0 = s.plan.tsys.on0;
    d.tsys_two_bit = s.plan.tsys.two_bit;
    d.spline = s.spline.as<double>();
    d.spline_n = s.sp.n;
    d.scan_begin = s.sp.scan_begin;
    d.clock_epoch = s.sp.clock_epoch;
    d.clock_offset = s.sp.clock_offset;
    d.clock_rate = s.sp.clock_rate;
    d.start_ticks = start;
    d.tps = ticks_per_sample(ss.sample_rate);
    d.n_blocks = s.n_blocks;
    const ticks_t fft_len = time_from_usec((double)c->Nd / (ss.sample_rate / 1000000));
    d.fft_len_ticks = fft_len;
    d.half_len_ticks = time_div(fft_len, 2);
    d.fft_len_sec = time_sec_of_day(fft_len);
    d.sample_rate = ss.sample_rate;
    d.bandwidth = ss.bandwidth;
    d.oversamp = (int)std::round(ss.sample_rate / (2 * (double)ss.bandwidth));
    d.frac_scale = -2.0 * M_PI / ss.sample_rate;
    d.int_phase_q = M_PI / (2 * d.oversamp);
    d.frac_scale_f = (float)d.frac_scale;
    d.int_phase_q_f = (float)d.int_phase_q;
    d.half_bw_f = (float)(0.5 * ss.bandwidth);
    d.rate_per_bin_f = (float)((double)ss.sample_rate / kNd);
    d.sideband = ss.sideband == 'L' ? -1 : 1;
    d.fringe_mult = -d.sideband * 2.0 * M_PI;
    d.center_freq = ss.channel_freq + d.sideband * ss.bandwidth * 0.5 + ss.lo_offset;
    d.lo_offset = ss.lo_offset;
    const double dt = time_diff(start, c->p.experiment_start_ticks);
    double sp0 = ss.lo_offset * (dt - std::trunc(dt)) + (ss.lo_offset - std::trunc(ss.lo_offset)) * std::trunc(dt);
    d.start_phase = sp0 - std::floor(sp0);
    d.rot = s.rot;
    d.slot = i;
    d.flip = c->p.sideband != ss.sideband;
    int64_t delta, freq = ss.channel_freq;  // delay_correction.cc:226-241
    if (c->p.sideband != ss.sideband) freq += (int64_t)d.sideband * ss.bandwidth;
    delta = c->p.sideband == 'L' ? freq - c->p.channel_freq : c->p.channel_freq - freq;
    if (delta > 0) {
      d.output_offset = (int)(delta * 2 * M / c->p.sample_rate);
      d.temp_fft_offset = 0;
    } else {
      d.output_offset = 0;
      d.temp_fft_offset = (int)(-delta * 2 * M / c->p.sample_rate);
    }
    d.hist = c->hist.as<unsigned long long>() + (size_t)i * 8;
    d.phase_zero = std::all_of(s.sp.y[1].begin(), s.sp.y[1].end(), [](double v) { return v == 0.0; });
    d.amp_one = std::all_of(s.sp.y[2].begin(), s.sp.y[2].end(), [](double v) { return v == 1.0; });
    d.no_clock = s.sp.clock_offset == 0.0 && s.sp.clock_rate == 0.0;
    // bit-statistics work: ranges up to 8 KB (one per protocol data block)
    // packed about 64 KB to an item, longer ones cut into 64 KB pieces
    const std::vector<StatRange> &st_r = s.plan.stats;
    for (int r = 0; r < (int)st_r.size();) {
      if (st_r[r].n > 8192) {
        for (int off = 0; off < st_r[r].n; off += 65536) items.push_back(make_int4(i, r, 0, off));
        r++;
        continue;
      }
      const int r0 = r;
      int64_t bytes = 0;
      while (r < (int)st_r.size() && st_r[r].n <= 8192 && r - r0 < 64 && bytes < 65536) bytes += st_r[r++].n;
      items.push_back(make_int4(i, r0, r - r0, 0));
    }
    s.pushed = false;
  }
  // ---- flagged samples and normalisation factors (host)
  std::vector<const std::vector<InvalidRun> *> inv;
  for (int i = 0; i < N; i++) inv.push_back(&c->sc[i].plan.invalid);
  std::vector<std::pair<int64_t, int64_t>> nfl;
  find_invalid(c->streams, c->p.sample_rate, c->bl, inv, nfl);
  const int64_t total = (int64_t)c->nffts * M;
  std::vector<double> flagfac(nbl, 1.0);
  auto inv_level = [&](int i) {  // bit_statistics::get_statistics()[4]
    return (int)(((uint64_t)c->p.sample_rate * (uint64_t)(int64_t)(int)c->sc[i].plan.n_invalid) /
                 (uint64_t)c->streams[i].sample_rate);
  };
  for (int b = N; b < nbl; b++) {
    const int64_t v1 = total - inv_level(c->bl[b].a), v2 = total - inv_level(c->bl[b].b);
    const double n1 = v1 > 0 ? 1 - nfl[b].first * 1. / v1 : 1;
    const double n2 = v2 > 0 ? 1 - nfl[b].second * 1. / v2 : 1;
    double n = n1 * n2;
    if (n < 0.01) n = 1;
    flagfac[b] = n;
  }
  q.upload(c->flagfac, flagfac.data(), flagfac.size() * 8, st);
  q.upload(c->items, items.data(), items.size() * sizeof(int4), st);
  // ---- device work
  // phased array: one buffer per sub-integration (Correlation_core_phased::create_baselines)
  const int nphs = c->phased ? c->nffts / c->nsub + 1 : 0;
  const size_t accn = (size_t)std::max(c->nbins * nbl, nphs) * kpad;
  c->acc.ensure(accn * sizeof(float2));
  q.memset(c->acc.p, 0, accn * sizeof(float2), st);
  const bool pulsar = c->nbins > 1;
  if (c->npc > 1) {
    c->pcacc.ensure((size_t)c->npc * nbl * kpad * sizeof(float2));
    q.memset(c->pcacc.p, 0, (size_t)c->npc * nbl * kpad * sizeof(float2), st);
  }
  std::vector<std::pair<int, int>> ranges;
  if (pulsar)
    ranges.push_back({0, c->nffts});  // no sub-integrations in Correlation_core_pulsar
  else
    ranges = subint_ranges(c);
  int max_rows = 0;
  for (auto &r : ranges) max_rows = std::max(max_rows, r.second - r.first);
  const int minus = c->p.window != WINDOW_NONE ? 0 : -1;  // one extra hop for overlapping windows
  const int hop = c->sc[0].hop;
  const bool chunked = hop % kNd == 0;
  if (!chunked) {
    if (c->npc > 1)
      throw Error(SFXC_GPU_EINVAL, "extra phase centres need windowed-FFT hops of whole 256-sample blocks");
    ranges.assign(1, {0, c->nffts});
    max_rows = c->nffts;
  }
  int max_blocks = 0;
  for (int i = 0; i < N; i++)  // each stream's own hop: streams at other rates need more or fewer blocks
    max_blocks = std::max(max_blocks, chunked ? (max_rows + 2) * c->sc[i].hop / kNd : c->sc[i].n_blocks);
  c->ts.ensure((size_t)N * max_blocks * kNd * sizeof(float));
  // tensor-core X-step (normal correlation and pulsar binning; the phased
  // array sums spectra and has no products); the spectra are scaled by a
  // power of two before the FP16 hi/lo split so that typical magnitudes sit
  // near 1 (|X| ~ sqrt(2M * 0.375 * E[x^2]) for a Hann window)
  const bool tc_x = c->x_mode == SFXC_GPU_X_TC_HILO && !c->phased;
  const int tc_slots = tc_x ? (N <= kTcSlots ? kTcSlots : kTcSlotsWide) : 0;
  // up to 32 streams without binning: the TMA-fed kernel; else the row-gathered one
  const bool tc_tma = tc_x && !pulsar && tc_slots == kTcSlots;
  const float tc_scale = std::ldexp(1.0f, -(int)std::lround(0.5 * std::log2(2.0 * M * 10.0)));
  // FP32 spectra: [stream][row][kpad]; TC spectra: [row][kpad][S stream slots], 8 bytes each
  // the TMA-fed kernel reads rows in groups of 8 (rows past a chunk's end cleared before its X-step)
  c->spec.ensure((size_t)(tc_x ? tc_slots : N) * (tc_x ? (max_rows + 7) / 8 * 8 : max_rows) * kpad * sizeof(float2));
  c->derr.ensure(sizeof(int));
  q.memset(c->derr.p, 0, sizeof(int), st);
  if (!tc_x && !pulsar && !c->phased)
    c->xpart.ensure(std::max<size_t>(16, xcorr_f32_scratch_bytes(c->jt.ntiles, c->jt.npad, K, max_rows, nbl, kpad)));
  // two sets of per-block records: chunk ch uses set ch & 1, so the next
  // chunk's are computed while the current chunk is still transformed
  for (int i = 0; i < N; i++) {
    c->sc[i].bpar.ensure((size_t)2 * max_blocks * sizeof(BlockPar));
  }
  // pulsar setup (Correlation_core_pulsar::set_parameters, correlation_core_pulsar.cc:46-95)
  double psr_start_phase = 0, psr_rate = 0, fft_duration = 0;
  if (pulsar) {
    const double us_per_day = (double)((int64_t)24 * 60 * 60 * 1000000);
    const double start_mjd = time_mjd(start);
    fft_duration = ((double)M * 1000000) / c->p.sample_rate;
    size_t closest = 0;
    double diff = std::fabs(c->polyco[0].tmid - start_mjd);
    for (size_t i = 1; i < c->polyco.size(); i++) {
      double nd = std::fabs(c->polyco[i].tmid - start_mjd);
      if (nd < diff) {
        diff = nd;
        closest = i;
      }
    }
    const Polyco &pc = c->polyco[closest];
    // Association of the reference as built with its own flags (-O2 -ffast-math,
    // sfxc/configure.ac:31): GCC evaluates (start_mjd - tmid) + fft_duration/us_per_day
    // as (start_mjd + fft_duration/us_per_day) - tmid.  The FP64 start MJD has
    // ~6e-7 s resolution, so the association moves the phase by up to ~1e-5
    // cycles and decides bins near a gate edge.
    double DT = c->p.window == WINDOW_NONE ? ((start_mjd + fft_duration / (2 * us_per_day)) - pc.tmid) * 1440
                                           : ((start_mjd + fft_duration / us_per_day) - pc.tmid) * 1440;
    const int nc = (int)pc.coef.size();
    double sp = 0;
    for (int i = nc - 1; i > 0; i--) sp = (sp + pc.coef[i]) * DT;
    sp += (pc.ref_phase - std::floor(pc.ref_phase)) + DT * 60 * pc.ref_freq + pc.coef[0];
    psr_start_phase = sp;
    psr_rate = pc.coef[1] + 60 * pc.ref_freq;
    const int sb = c->p.sideband == 'L' ? -1 : 1;
    const double base_freq = c->p.channel_freq * 1e-6;
    const double dfreq = sb * c->p.sample_rate * 1e-6 / (2 * M);
    const double inv2 = 1 / (pc.obs_freq * pc.obs_freq);
    double freq = 0;
    for (int i = nc - 1; i > 1; i--) freq = (freq + i * pc.coef[i]) * DT;
    freq = (freq + pc.coef[1]) / 60 + pc.ref_freq;
    std::vector<double> off(K);
    for (int i = 0; i < K; i++) {  // (4148.808*DM)*((...)*freq): the same build's association
      const double x = base_freq + i * dfreq;
      off[i] = (4148.808 * pc.dm) * ((1 / (x * x) - inv2) * freq);
    }
    q.upload(c->offsets, off.data(), off.size() * 8, st);
    c->bins.ensure((size_t)max_rows * K * sizeof(int16_t));
    if (tc_x) {  // per channel the rows sorted by bin (runs padded to 16 rows), and the runs
      c->rowlist.ensure((size_t)K * (max_rows + 16 * c->nbins) * sizeof(int));
      c->segs.ensure((size_t)K * c->nbins * sizeof(int2));
    }
  }
  // four timing marks per chunk (+2 for normalisation), recorded without
  // host syncs
  const size_t nev = ranges.size() * 5 + 2;
  while (sl.evs.size() < nev) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    sl.evs.push_back(e);
  }
  // the start, each chunk's parameters ready (second stream), each chunk's
  // windowed FFT done (main stream), each chunk's X-step done (third stream)
  while (sl.deps.size() < 1 + 3 * ranges.size()) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    sl.deps.push_back(e);
  }
  // ---- every chunk's stream descriptors, in job order and then grouped by
  // windowed-FFT length (job order within a group), in one asynchronous
  // upload from pinned memory: no host wait between the chunks' launches
  std::vector<int> order;                   // job index of each grouped position
  std::vector<std::pair<int, int>> groups;  // (rot, first grouped position)
  for (auto &rt : c->rot_tables) {
    const size_t first = order.size();
    for (int i = 0; i < N; i++)
      if (c->sc[i].rot == rt.first) order.push_back(i);
    if (order.size() > first) groups.push_back({rt.first, (int)first});
  }
  const size_t per_chunk = 2 * (size_t)N;
  std::vector<StreamDev> staged(ranges.size() * per_chunk);
  for (size_t ch = 0; ch < ranges.size(); ch++) {
    const int r0 = ranges[ch].first, r1 = ranges[ch].second;
    // block range of each stream for rows [r0, r1) (plus the overlapping half window)
    for (int i = 0; i < N; i++) {
      StreamDev &d = c->hsd[i];
      const int b0 = chunked ? r0 * c->sc[i].hop / kNd : 0;
      const int b1 = chunked ? std::min(c->sc[i].n_blocks, (r1 + 1 + minus) * c->sc[i].hop / kNd) : c->sc[i].n_blocks;
      d.ts = c->ts.as<float>() + (size_t)i * max_blocks * kNd;
      d.bpar = c->sc[i].bpar.as<BlockPar>() + (ch & 1) * (size_t)max_blocks;
      d.block0 = b0;
      d.n_blocks = b1 - b0;
      d.spline_lo = spline_lo_for(d, c->sc[i].sp.x);
      staged[ch * per_chunk + i] = d;
    }
    for (int k = 0; k < N; k++) staged[ch * per_chunk + N + k] = c->hsd[order[k]];
  }
  q.upload(c->streamdev, staged.data(), staged.size() * sizeof(StreamDev), st);
  // uvshift of every chunk (sub-integration), cross baseline and extra centre:
  // Correlation_core::sub_integration / uvshift (sfxc/src/correlation_core.cc:
  // 516-593) in FP64 on the host -- tmid of the sub-integration, residual
  // delays of the centre against the pointing centre, rates, amplitude from
  // the window-autocorrelation weight of the residual lag
  if (c->npc > 1) {
    const ticks_t tfft = (ticks_t)M * (ticks_t)std::lround(512000000.0 / c->p.sample_rate);
    const int sbs = c->p.sideband == 'L' ? -1 : 1;
    const double base_freq = (double)c->p.channel_freq, dfreq = c->p.sample_rate / (2. * M);
    std::vector<UvShift> uv(ranges.size() * (size_t)(c->npc - 1) * nbl, UvShift{0, 0, 0, 0});
    for (size_t ch = 0; ch < ranges.size(); ch++) {
      const int prev = ranges[ch].first, cur = ranges[ch].second;
      const ticks_t tmid = start + time_mul(tfft, prev + (cur - prev) / 2.);
      for (int pc = 1; pc < c->npc; pc++)
        for (int b = N; b < nbl; b++) {
          const StreamCtx &s1 = c->sc[c->bl[b].a], &s2 = c->sc[c->bl[b].b];
          const double delay1 = s1.sp.delay(tmid), delay2 = s2.sp.delay(tmid);
          const double dd1 = s1.sp_pc[pc - 1].delay(tmid) - delay1, dd2 = s2.sp_pc[pc - 1].delay(tmid) - delay2;
          const double r1 = s1.sp.rate(tmid), r2 = s2.sp.rate(tmid);
          float amplitude = 1;
          const int lag = std::abs((int)std::round((dd1 - dd2) * c->p.sample_rate));
          if (lag < M && c->pc_weights[lag] > 1e-4) amplitude = (float)(1. / c->pc_weights[lag]);
          double phi = base_freq * (dd1 * (1 - r1) - dd2 * (1 - r2));
          phi = 2 * M_PI * sbs * (phi - std::floor(phi));
          const double delta = 2 * M_PI * dfreq * (dd1 * (1 - r1) - dd2 * (1 - r2));
          uv[(ch * (c->npc - 1) + (pc - 1)) * nbl + b] = UvShift{phi, delta, amplitude, 0.0};
        }
    }
    q.upload(c->uvp, uv.data(), uv.size() * sizeof(UvShift), st);
  }
  q.mark(sl.ev0, st);
  q.record(sl.deps[0], st);
  // The per-block parameters (block_params_kernel, FP64-pipe bound, few
  // registers) run on the second stream: those of the first chunk beside the
  // bit statistics (memory bound), those of chunk ch + 1 once chunk ch's
  // windowed FFT is done, i.e. beside chunk ch's X-step, whose CTAs leave
  // registers and issue slots free.  Each chunk's transforms wait for them.
  q.wait(c->st2, sl.deps[0]);  // the descriptors are on the device
  StreamDev *const sdev = c->streamdev.as<StreamDev>();
  cudaStream_t st2 = c->st2;
  q.kernel([=] { launch_block_params(sdev, N, max_blocks, st2); });
  q.record(sl.deps[1], c->st2);
  // bit statistics read only chunk-independent fields (source bytes, ranges, histograms)
  {
    const int4 *ditems = c->items.as<int4>();
    const int nitems = (int)items.size();
    q.kernel([=] { launch_bitstat(sdev, ditems, nitems, st); });
  }
  int launches = items.empty() ? 0 : 1;
  size_t ev = 0;
  // Chunk ch's X-step runs on the third stream beside chunk ch + 1's F-step
  // (an X-step CTA and an F-step CTA fit an SM together); chunk ch + 1's
  // windowed FFT, which overwrites the spectra, waits for it (the phases'
  // times then overlap: each is its own kernels' elapsed time).  Measured
  // at 4096 channels: the FP32 X-step path 5-6 % faster overall (16- and
  // 32-stream jobs), a batch with row-gathered tensor-core X-steps (40-stream
  // jobs) 5 %; the TMA-fed X-step 1.3-3 % slower, whatever its CTA count
  // (with 129 KB of shared memory it leaves room for one of the F-step's four
  // CTAs per SM, so the F-step's time grows by about what the X-step takes),
  // so it stays on the main stream.
  const size_t R = ranges.size();
  cudaStream_t xs = tc_tma ? st : c->st3;
  for (size_t ch = 0; ch < R; ch++) {
    const int nrows = ranges[ch].second - ranges[ch].first;
    StreamDev *dchunk = sdev + ch * per_chunk;
    q.mark(sl.evs[ev], st);
    q.wait(st, sl.deps[1 + ch]);
    {
      const float2 *tw256 = c->tw256.as<float2>();
      const int fw = plan_get(block_key(N, max_blocks));
      q.kernel([=] { launch_fstep(dchunk, N, max_blocks, tw256, st, fw); });
    }
    q.mark(sl.evs[ev + 1], st);
    if (xs != st && ch > 0) q.wait(st, sl.deps[1 + 2 * R + ch - 1]);
    q.mark(sl.evs[ev + 2], st);
    for (size_t g = 0; g < groups.size(); g++) {
      const int rot = groups[g].first, first = groups[g].second;
      const int count = (g + 1 < groups.size() ? groups[g + 1].second : N) - first;
      const int nper = c->p.window == WINDOW_NONE ? rot / 2 : rot;
      const sfxc_gpu_ctx::RotTables &t = c->rot_tables.at(rot);
      const float *win = t.window.as<float>();
      const float2 *twr = t.twrot.as<float2>();
      void *spec = c->spec.p;
      const int ww = plan_get(window_key(rot, count, nrows));
      q.kernel([=] {
        launch_window_fft(dchunk + N + first, count, 0, nrows, max_rows, win, twr, rot, nper, M, kpad, spec, tc_slots,
                          tc_scale, st, ww);
      });
    }
    q.mark(sl.evs[ev + 3], st);
    q.record(sl.deps[1 + R + ch], st);
    q.wait(xs, sl.deps[1 + R + ch]);
    {
      // X-step of the chunk (pointers and sizes taken now; the buffers are sized above)
      const int r0c = ranges[ch].first, nsub = c->nsub, nbins = c->nbins, npad = c->jt.npad, ntiles = c->jt.ntiles;
      float2 *acc = c->acc.as<float2>();
      void *specp = c->spec.p;
      const int *blmap = c->blmap.as<int>(), *tiles = c->tiles.as<int>();
      int *derr = c->derr.as<int>();
      const float inv_s2 = 1.0f / (tc_scale * tc_scale);
      if (c->phased) {
        q.kernel([=] { launch_phased(static_cast<float2 *>(specp), max_rows, kpad, N, r0c, nrows, K, nsub, acc, xs); });
      } else if (pulsar) {
        // the bin of every (row, channel), then the binned X-step: tensor cores
        // over each channel's rows sorted by bin, or CUDA cores in row order
        const double *offs = c->offsets.as<double>();
        const double g0 = c->p.gate_start, g1 = c->p.gate_stop;
        int16_t *bins = c->bins.as<int16_t>();
        q.kernel([=] {
          launch_pulsar_bins(nrows, K, psr_start_phase, psr_rate, fft_duration, offs, g0, g1, nbins, bins, xs);
        });
        c->bins_rows = nrows;  // one chunk: the whole integration
        if (tc_x) {
          const int list_len = max_rows + 16 * nbins;
          int *rowlist = c->rowlist.as<int>();
          int2 *segs = c->segs.as<int2>();
          q.kernel([=] { launch_pulsar_sort(bins, nrows, K, nbins, list_len, rowlist, segs, xs); });
          q.op([=] {
            return launch_xcorr_tc_gather(specp, tc_slots, nrows, kpad, K, N, blmap, npad, nbl, nbins, rowlist,
                                          list_len, segs, inv_s2, acc, derr, xs);
          });
          launches += 1;
        } else {
          q.kernel([=] {
            launch_xcorr_f32(static_cast<float2 *>(specp), max_rows, kpad, N, npad, 0, nrows, K, tiles, ntiles, blmap,
                             nbl, bins, nrows, acc, nullptr, 0, xs);
          });
        }
      } else if (tc_tma) {
        if (nrows % 8)
          q.memset(static_cast<char *>(specp) + (size_t)nrows * kpad * kTcSlots * sizeof(float2), 0,
                   (size_t)(8 - nrows % 8) * kpad * kTcSlots * sizeof(float2), xs);
        q.op([=] { return launch_xcorr_tc(specp, nrows, kpad, K, blmap, npad, inv_s2, acc, derr, xs); });
      } else if (tc_x) {  // 33 to 64 streams: the row-gathered kernel over rows in order
        q.op([=] {
          return launch_xcorr_tc_gather(specp, tc_slots, nrows, kpad, K, N, blmap, npad, nbl, 1, nullptr, 0, nullptr,
                                        inv_s2, acc, derr, xs);
        });
      } else {
        float2 *xpart = c->xpart.as<float2>();
        const size_t xcap = c->xpart.cap;
        q.kernel([=] {
          launch_xcorr_f32(static_cast<float2 *>(specp), max_rows, kpad, N, npad, 0, nrows, K, tiles, ntiles, blmap, nbl,
                           nullptr, 0, acc, xpart, xcap, xs);
        });
      }
      if (c->npc > 1) {  // the sub-integration into every phase centre
        float2 *pcacc = c->pcacc.as<float2>();
        const UvShift *uvp = c->uvp.as<UvShift>() + ch * (size_t)(c->npc - 1) * nbl;
        const int npc = c->npc;
        q.kernel([=] { launch_pc_dump(acc, pcacc, uvp, N, nbl, kpad, K, npc, xs); });
        launches += 1;
      }
    }
    q.mark(sl.evs[ev + 4], xs);  // before the event the main stream joins on (a capture ends joined)
    q.record(sl.deps[1 + 2 * R + ch], xs);
    if (ch + 1 < R) {
      // chunk ch + 1's records go to the other set, last read by chunk ch - 1's
      // transforms.  (Starting them once chunk ch's transforms are done, to
      // fill the windowed FFT's tail, measured slower: their CTAs then hold
      // SMs when the X-step's persistent CTAs are placed.)
      q.wait(c->st2, sl.deps[1 + R + ch]);
      q.kernel([=] { launch_block_params(dchunk + per_chunk, N, max_blocks, st2, kSideParamCtas); });
      q.record(sl.deps[1 + ch + 1], c->st2);
    }
    ev += 5;
    launches += pulsar ? 5 : 4;  // parameters, blocks, window FFT, (pulsar bins,) X-step
  }
  {  // the last chunk, for the autotuner
    sfxc_gpu_ctx::TuneSpec &ts = c->tune;
    ts.dchunk = sdev + (ranges.size() - 1) * per_chunk;
    ts.nstreams = N;
    ts.max_blocks = max_blocks;
    ts.nrows = ranges.back().second - ranges.back().first;
    ts.max_rows = max_rows;
    ts.M = M;
    ts.kpad = kpad;
    ts.tc_slots = tc_slots;
    ts.tc_scale = tc_scale;
    ts.window = c->p.window;
    ts.spec = c->spec.p;
    ts.groups.clear();
    for (size_t g = 0; g < groups.size(); g++)
      ts.groups.push_back({groups[g].first, groups[g].second,
                           (g + 1 < groups.size() ? groups[g + 1].second : N) - groups[g].second});
  }
  // restore the whole-integration time base for inspection calls
  for (int i = 0; i < N; i++) {
    c->hsd[i].block0 = 0;
    c->hsd[i].n_blocks = c->sc[i].n_blocks;
    c->hsd[i].spline_lo = spline_lo_for(c->hsd[i], c->sc[i].sp.x);
  }
  // ---- normalisation and statistics, once the last X-step is done
  q.wait(st, sl.deps[3 * R]);
  q.mark(sl.evs[ev], st);
  c->norms.ensure((size_t)N * 8);
  // outputs: the pulsar bins, or the phase centres (each normalised on its
  // own); the phased array writes its sub-integration sums as they are
  const int nout = pulsar ? c->nbins : c->npc;
  const float2 *accs = c->npc > 1 ? c->pcacc.as<float2>() : c->acc.as<float2>();
  c->out.ensure((size_t)std::max(nout * nbl, nphs) * K * sizeof(float2));
  float2 *outp = c->out.as<float2>();
  if (c->phased) {
    const void *accp = c->acc.p;
    q.op([=] {
      return cudaMemcpy2DAsync(outp, K * sizeof(float2), accp, kpad * sizeof(float2), K * sizeof(float2), nphs,
                               cudaMemcpyDeviceToDevice, st);
    });
  } else {
    const int *blp = c->blpairs.as<int>();
    double *norms = c->norms.as<double>();
    const double *ff = c->flagfac.as<double>();
    q.kernel([=] {
      for (int bin = 0; bin < nout; bin++)
        launch_normalize(accs + (size_t)bin * nbl * kpad, kpad, M, N, nbl, blp, norms, ff, outp + (size_t)bin * nbl * K,
                         st);
    });
  }
  const float2 *vsrc = outp;
  if (c->nch < M) {
    c->rout.ensure((size_t)nout * nbl * c->Kout * sizeof(float2));
    const int nch = c->nch, rnorm = c->rnorm;
    const float *rmask = c->rmask.as<float>(), *rlag = c->rlag.as<float>();
    const float2 *rtw = c->rtw.as<float2>();
    float2 *rout = c->rout.as<float2>();
    q.op([=] { return launch_reduce(outp, nout * nbl, M, nch, rmask, rlag, rnorm, rtw, rout, st); });
    vsrc = rout;
    launches += 1;
  }
  const size_t nvis = c->phased ? (size_t)nphs * c->Kout : (size_t)nout * nbl * c->Kout;
  uint8_t *res = static_cast<uint8_t *>(sl.results.ensure(nvis * sizeof(float2) + (size_t)N * 64 + 16));
  {
    const void *histp = c->hist.p, *derrp = c->derr.p;
    q.op([=] { return cudaMemcpyAsync(res, vsrc, nvis * sizeof(float2), cudaMemcpyDeviceToHost, st); });
    q.op([=] { return cudaMemcpyAsync(res + nvis * sizeof(float2), histp, (size_t)N * 64, cudaMemcpyDeviceToHost, st); });
    q.op([=] {
      return cudaMemcpyAsync(res + nvis * sizeof(float2) + (size_t)N * 64, derrp, sizeof(int), cudaMemcpyDeviceToHost,
                             st);
    });
  }
  q.mark(sl.evs[ev + 1], st);
  launches += 2 * nout;
  Pending &pd = sl.pend;
  pd.start = start;
  pd.nvis = nvis;
  pd.nout = nout;
  pd.nphs = nphs;
  pd.ev = ev;
  pd.launches = launches;
  pd.pulsar = pulsar;
  pd.nfl = std::move(nfl);
  pd.res = res;
  pd.n_invalid.resize(N);
  for (int i = 0; i < N; i++) pd.n_invalid[i] = c->sc[i].plan.n_invalid;
}

// After the recorded work has run: device error flag, timings, statistics,
// output bytes to the sink.
// The host side of a finished integration: its output bytes and tsys
// records, made before any of them goes to the sink.
struct IntegrationOut {
  std::vector<uint8_t> cor;
  std::vector<std::vector<uint8_t>> tsys;
};

void prepare_outputs(sfxc_gpu_ctx *c, int k, IntegrationOut &out) {
  Slot &sl = *c->slots[k];
  Pending &pd = sl.pend;
  const int N = (int)c->streams.size(), nbl = (int)c->bl.size();
  const size_t nvis = pd.nvis, ev = pd.ev;
  const int nout = pd.nout, nphs = pd.nphs;
  const bool pulsar = pd.pulsar;
  const ticks_t start = pd.start;
  const int launches = pd.launches;
  const std::vector<std::pair<int64_t, int64_t>> &nfl = pd.nfl;
  uint8_t *res = pd.res;
  const float2 *vis = reinterpret_cast<const float2 *>(res);
  const unsigned long long *hist = reinterpret_cast<const unsigned long long *>(res + nvis * sizeof(float2));
  const int *dev_err = reinterpret_cast<const int *>(res + nvis * sizeof(float2) + (size_t)N * 64);
  cudaStream_t st = c->st;
  float t_f1 = 0, t_f2 = 0, t_x = 0;
  CK(cudaStreamSynchronize(st));
  if (*dev_err) throw Error(SFXC_GPU_ECUDA, "tensor-core X-step timed out waiting for its MMAs");
  // per chunk: F-step start and end, windowed FFT start (after the previous
  // X-step when that ran beside the F-step) and end, X-step end
  for (size_t q = 0; q + 5 <= ev; q += 5) {
    float a, b, x;
    CK(cudaEventElapsedTime(&a, sl.evs[q], sl.evs[q + 1]));
    CK(cudaEventElapsedTime(&b, sl.evs[q + 2], sl.evs[q + 3]));
    CK(cudaEventElapsedTime(&x, sl.evs[q + 3], sl.evs[q + 4]));
    t_f1 += a;
    t_f2 += b;
    t_x += x;
  }
  float tn, tall;
  CK(cudaEventElapsedTime(&tn, sl.evs[ev], sl.evs[ev + 1]));
  CK(cudaEventElapsedTime(&tall, sl.ev0, sl.evs[ev + 1]));
  c->timings[5] = (float)launches;
  c->timings[0] = t_f1;
  c->timings[1] = t_f2;
  c->timings[2] = t_x;
  c->timings[3] = tn;
  c->timings[4] = tall;
  float tb = 0;  // the bit statistics: between the start and the first chunk
  if (ev >= 5) CK(cudaEventElapsedTime(&tb, sl.ev0, sl.evs[0]));
  c->timings[6] = tb;
  for (int i = 0; i < N; i++) {
    BitStats &bs = c->sc[i].stats;
    for (int k = 0; k < 4; k++) {
      bs.on[k] = (int64_t)hist[(size_t)i * 8 + k];
      bs.off[k] = (int64_t)hist[(size_t)i * 8 + 4 + k];
    }
    bs.n_invalid = pd.n_invalid[i];
    bs.bits = c->streams[i].bits;
    bs.sample_rate = c->streams[i].sample_rate;
    bs.base_sample_rate = c->p.sample_rate;
  }
  // ---- output bytes (integration_write per bin) and tsys records
  std::vector<uint8_t> &o = out.cor;
  {
    const size_t per_out = 20 + (size_t)N * (32 + 24) + (size_t)std::max(nbl, nphs) * (8 + (size_t)c->Kout * 8);
    o.reserve(per_out * (size_t)std::max(1, nout));
  }
  if (c->phased) {
    serialize_integration(c, std::vector<Baseline>(nphs, Baseline{0, 0}), vis, 0, 0, nfl, o);
  } else {
    for (int bin = 0; bin < nout; bin++)
      serialize_integration(c, c->bl, vis + (size_t)bin * nbl * c->Kout, pulsar ? bin : c->pc_file[bin],
                            pulsar ? 0 : bin, nfl, o);
  }
  for (int i = 0; i < N && !c->phased; i++) {  // the phased core writes no tsys records
    out.tsys.emplace_back();
    std::vector<uint8_t> &t = out.tsys.back();
    t.push_back((uint8_t)c->streams[i].station_number);
    t.push_back((uint8_t)c->p.frequency_nr);
    t.push_back((uint8_t)(c->p.sideband == 'L' ? 0 : 1));
    t.push_back((uint8_t)(c->streams[i].polarisation == 'R' ? 0 : 1));
    int ts[4];
    c->sc[i].stats.tsys(ts);
    put(t, (int64_t)start);
    for (int k = 0; k < 4; k++) put(t, (int64_t)ts[k]);
  }
  c->current_integration++;
}

void deliver_outputs(const IntegrationOut &o, sfxc_output_sink sink, void *user) {
  if (!sink) return;
  if (sink(user, 0, o.cor.data(), o.cor.size()) != 0) throw Error(SFXC_GPU_EINVAL, "output sink refused the data");
  for (const std::vector<uint8_t> &t : o.tsys)
    if (sink(user, 1, t.data(), t.size()) != 0) throw Error(SFXC_GPU_EINVAL, "output sink refused the data");
}

int finish_integration(sfxc_gpu_ctx *c, int k, sfxc_output_sink sink, void *user) {
  IntegrationOut o;
  prepare_outputs(c, k, o);
  deliver_outputs(o, sink, user);
  return SFXC_GPU_OK;
}

// Copy the recorded uploads' payloads into the pinned arena (may allocate:
// before any stream capture).
void stage_ops(sfxc_gpu_ctx *c, int k) {
  Slot &sl = *c->slots[k];
  uint8_t *a = static_cast<uint8_t *>(sl.arena.ensure(std::max<size_t>(sl.q.host.size(), 16)));
  if (!sl.q.host.empty()) std::memcpy(a, sl.q.host.data(), sl.q.host.size());
}

// Issue the recorded work on the context's streams (allocates nothing).
void run_ops(sfxc_gpu_ctx *c, int k) {
  Slot &sl = *c->slots[k];
  const uint8_t *a = static_cast<const uint8_t *>(sl.arena.p);
  for (auto &f : sl.q.ops) CK(f(a));
}

int run_integration(sfxc_gpu_ctx *c, sfxc_output_sink sink, void *user) {
  try {
    enqueue_integration(c, 0);
    stage_ops(c, 0);
    run_ops(c, 0);
    return finish_integration(c, 0, sink, user);
  } catch (...) {
    c->planned_integration = c->current_integration;  // the failed integration is not counted
    throw;
  }
}

}  // namespace

// ------------------------------------------------------------ C entry points
extern "C" {

sfxc_gpu_ctx *sfxc_gpu_create(const sfxc_gpu_config *config) {
  std::unique_ptr<sfxc_gpu_ctx> c(new sfxc_gpu_ctx());
  try {
    if (config) {
      c->device = config->device;
      c->x_mode = config->x_mode;
    }
    if (c->x_mode != SFXC_GPU_X_FP32 && c->x_mode != SFXC_GPU_X_TC_HILO) throw Error(SFXC_GPU_EINVAL, "bad x_mode");
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (c->device < 0 || c->device >= n) throw Error(SFXC_GPU_EINVAL, "no such CUDA device");
    CK(cudaSetDevice(c->device));
    // Contexts of one process take successive stream priorities (cycling
    // through the device's range): jobs correlated side by side then finish
    // one after another instead of all together, so each job's host work
    // (output, next input, planning) overlaps the others' kernels rather than
    // leaving the GPU idle while every job does it at once.
    static std::atomic<unsigned> created{0};
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    // The second stream sits one level below the first and the third one
    // level above it, so that when a chunk's windowed FFT ends the X-step's
    // CTAs are placed before the next chunk's parameter and F-step CTAs fill
    // the room they leave.
    const int levels = least - greatest + 1;
    const int prio = greatest + 1 + (int)(created.fetch_add(1) % (unsigned)std::max(levels - 2, 1));
    CK(cudaStreamCreateWithPriority(&c->st, cudaStreamNonBlocking, std::min(prio, least)));
    CK(cudaStreamCreateWithPriority(&c->st2, cudaStreamNonBlocking, std::min(prio + 1, least)));
    CK(cudaStreamCreateWithPriority(&c->st3, cudaStreamNonBlocking, std::min(prio - 1, least)));
  } catch (const Error &e) {
    g_error = e.msg;
    return nullptr;
  }
  return c.release();
}

void sfxc_gpu_destroy(sfxc_gpu_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->st2) cudaStreamSynchronize(c->st2);
  if (c->st3) cudaStreamSynchronize(c->st3);
  c->slots.clear();
  if (c->st) cudaStreamDestroy(c->st);
  if (c->st2) cudaStreamDestroy(c->st2);
  if (c->st3) cudaStreamDestroy(c->st3);
  delete c;
}

const char *sfxc_gpu_last_error(const sfxc_gpu_ctx *c) { return c ? c->err.c_str() : g_error.c_str(); }
const char *sfxc_gpu_global_error(void) { return g_error.c_str(); }

int sfxc_gpu_set_parameters(sfxc_gpu_ctx *c, const sfxc_correlation_params *p) {
  if (!c) return SFXC_GPU_EINVAL;
  try {
    CK(cudaSetDevice(c->device));
    c->have_job = false;
    set_parameters(c, p);
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

namespace {
// Room for n more protocol bytes in a stream's device input, keeping what
// this integration already pushed.
void grow_stream_input(sfxc_gpu_ctx *c, StreamCtx &s, size_t n) {
  // 8 spare bytes: the unpack reads whole 32-bit words, one past the last sample
  const size_t need = (size_t)(s.dev_bytes + (int64_t)n) + 8;
  if (need <= s.src.cap) return;
  DevBuf grown;
  grown.ensure(std::max(need, s.src.cap * 3 / 2));
  if (s.dev_bytes) CK(cudaMemcpyAsync(grown.p, s.src.p, (size_t)s.dev_bytes, cudaMemcpyDeviceToDevice, c->st));
  std::swap(grown.p, s.src.p);
  std::swap(grown.cap, s.src.cap);
  CK(cudaStreamSynchronize(c->st));
}
}  // namespace

int sfxc_gpu_push_protocol(sfxc_gpu_ctx *c, int32_t stream, const uint8_t *bytes, size_t n) {
  if (!c) return SFXC_GPU_EINVAL;
  if (!c->have_job) return fail(c, Error(SFXC_GPU_ESTATE, "no parameters set"));
  if (stream < 0 || stream >= (int)c->sc.size()) return fail(c, Error(SFXC_GPU_EINVAL, "bad stream index"));
  if (n && !bytes) return fail(c, Error(SFXC_GPU_EINVAL, "null input"));
  StreamCtx &s = c->sc[stream];
  try {
    CK(cudaSetDevice(c->device));
    grow_stream_input(c, s, n);
    // the copy runs while the records are parsed; bytes past dev_bytes only
    // count once the parse has succeeded
    if (n) CK(cudaMemcpyAsync(s.src.as<uint8_t>() + s.dev_bytes, bytes, n, cudaMemcpyHostToDevice, c->st));
    std::vector<Record> recs;
    try {
      // records refer to the bytes by their offset in the stream's device buffer
      recs = parse_protocol(bytes, n, s.dev_bytes);
    } catch (...) {
      cudaStreamSynchronize(c->st);  // the caller owns the buffer again on return
      throw;
    }
    CK(cudaStreamSynchronize(c->st));  // the caller may reuse its buffer on return
    s.dev_bytes += (int64_t)n;
    s.pending.insert(s.pending.end(), recs.begin(), recs.end());
    s.pushed = true;
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_run_integration(sfxc_gpu_ctx *c, sfxc_output_sink sink, void *user) {
  if (!c) return SFXC_GPU_EINVAL;
  try {
    CK(cudaSetDevice(c->device));
    return run_integration(c, sink, user);
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_copy_unpacked(sfxc_gpu_ctx *c, int32_t stream, float *out, size_t n) {
  if (!c || !c->have_job) return SFXC_GPU_ESTATE;
  if (stream < 0 || stream >= (int)c->sc.size()) return fail(c, Error(SFXC_GPU_EINVAL, "bad stream index"));
  try {
    const StreamCtx &s = c->sc[stream];
    const size_t need = (size_t)s.n_blocks * c->Nd;
    if (n < need) throw Error(SFXC_GPU_EINVAL, "output buffer too small");
    StreamDev d = c->hsd[stream];
    DevBuf sd, dout;
    dout.ensure(need * sizeof(float));
    upload(sd, &d, sizeof(StreamDev), c->st);
    launch_unpack(sd.as<StreamDev>(), 1, s.n_blocks, dout.as<float>(), c->st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout.p, need * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return (int)need;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_autotune(sfxc_gpu_ctx *c, int32_t trials) {
  if (!c || !c->have_job) return SFXC_GPU_ESTATE;
  try {
    const sfxc_gpu_ctx::TuneSpec &t = c->tune;
    if (!t.dchunk) throw Error(SFXC_GPU_ESTATE, "no integration run yet");
    if (trials <= 0) trials = 3;
    CK(cudaSetDevice(c->device));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // best of `trials` timings of each candidate, the launches rewriting the
    // last chunk's own intermediates with the same values
    auto time_best = [&](auto launch) {
      float best = 1e30f;
      launch();
      for (int r = 0; r < trials; r++) {
        cudaEventRecord(e0, c->st);
        launch();
        cudaEventRecord(e1, c->st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
      }
      return best;
    };
    int tuned = 0;
    {
      const int cands[] = {4, 8, 12, 16, 24};
      int best_v = 12;
      float best_t = 1e30f;
      for (int v : cands) {
        const float ms = time_best([&] { launch_fstep(t.dchunk, t.nstreams, t.max_blocks, c->tw256.as<float2>(), c->st, v); });
        if (ms < best_t) {
          best_t = ms;
          best_v = v;
        }
      }
      plan_set(block_key(t.nstreams, t.max_blocks), best_v);
      tuned++;
    }
    for (const auto &g : t.groups) {
      const int rot = g[0], first = g[1], count = g[2];
      const int nper = t.window == WINDOW_NONE ? rot / 2 : rot;
      const sfxc_gpu_ctx::RotTables &rt = c->rot_tables.at(rot);
      int best_v = 2;
      float best_t = 1e30f;
      for (int v : {1, 2, 3, 4}) {
        const float ms = time_best([&] {
          launch_window_fft(t.dchunk + t.nstreams + first, count, 0, t.nrows, t.max_rows, rt.window.as<float>(),
                            rt.twrot.as<float2>(), rot, nper, t.M, t.kpad, t.spec, t.tc_slots, t.tc_scale, c->st, v);
        });
        if (ms < best_t) {
          best_t = ms;
          best_v = v;
        }
      }
      plan_set(window_key(rot, count, t.nrows), best_v);
      tuned++;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaGetLastError());
    return tuned;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_plan_cache(int32_t *out, int32_t capacity) {
  std::lock_guard<std::mutex> lock(g_plan_mu);
  int n = 0;
  for (const auto &kv : g_plan) {
    if (out && n < capacity) {
      for (int i = 0; i < 4; i++) out[5 * n + i] = kv.first[i];
      out[5 * n + 4] = kv.second;
    }
    n++;
  }
  return n;
}

int sfxc_gpu_copy_pulsar_bins(sfxc_gpu_ctx *c, int32_t *out, size_t n) {
  if (!c || !c->have_job) return SFXC_GPU_ESTATE;
  try {
    if (c->nbins <= 1 || c->bins_rows <= 0) throw Error(SFXC_GPU_ESTATE, "no pulsar bins: binning off or no integration yet");
    const size_t rows = (size_t)c->bins_rows, K = (size_t)c->K;
    if (!out || n < rows * K) throw Error(SFXC_GPU_EINVAL, "output buffer too small");
    CK(cudaSetDevice(c->device));
    std::vector<int16_t> b(rows * K);  // device table: [channel][row]
    CK(cudaMemcpyAsync(b.data(), c->bins.p, b.size() * sizeof(int16_t), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t k = 0; k < K; k++)
      for (size_t r = 0; r < rows; r++) out[r * K + k] = b[k * rows + r];
    return (int)(rows * K);
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_copy_spectra(sfxc_gpu_ctx *c, int32_t stream, float *out, size_t n) {
  if (!c || !c->have_job) return SFXC_GPU_ESTATE;
  if (stream < 0 || stream >= (int)c->sc.size()) return fail(c, Error(SFXC_GPU_EINVAL, "bad stream index"));
  try {
    // recompute the spectra of the whole last integration into a scratch buffer
    const StreamCtx &s = c->sc[stream];
    const size_t rows = (size_t)c->nffts, K = (size_t)c->M + 1;
    if (n < rows * K * 2) throw Error(SFXC_GPU_EINVAL, "output buffer too small");
    StreamDev d = c->hsd[stream];
    d.block0 = 0;
    d.n_blocks = s.n_blocks;
    d.spline_lo = spline_lo_for(d, s.sp.x);  // the block kernel walks the spline forward from block 0
    d.slot = 0;  // the only stream of this launch
    DevBuf ts, spec, sd, bp;
    ts.ensure((size_t)s.n_blocks * kNd * sizeof(float));
    spec.ensure(rows * c->kpad * sizeof(float2));
    bp.ensure((size_t)s.n_blocks * sizeof(BlockPar));
    d.ts = ts.as<float>();
    d.bpar = bp.as<BlockPar>();
    upload(sd, &d, sizeof(StreamDev), c->st);
    launch_fstep_block(sd.as<StreamDev>(), 1, s.n_blocks, c->tw256.as<float2>(), c->st);
    const int nper = c->p.window == WINDOW_NONE ? s.hop : s.rot;
    const sfxc_gpu_ctx::RotTables &t = c->rot_tables.at(s.rot);
    launch_window_fft(sd.as<StreamDev>(), 1, 0, (int)rows, (int)rows, t.window.as<float>(), t.twrot.as<float2>(),
                      s.rot, nper, c->M, c->kpad, spec.p, 0, 1.0f, c->st);
    CK(cudaGetLastError());
    CK(cudaMemcpy2DAsync(out, K * sizeof(float2), spec.p, c->kpad * sizeof(float2), K * sizeof(float2), rows,
                         cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return (int)(rows * K * 2);
  } catch (const Error &e) {
    return fail(c, e);
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free spectra inspection.  Some callers cannot allocate device
// memory at the moment they want to look at a stream's delay-corrected
// spectra: real-time correlator loops whose latency budget has no room for
// allocator synchronisation (cudaMalloc/cudaFree may wait for the whole
// device), and hosts that hand the GPU's memory out once at start-up.
// sfxc_gpu_copy_spectra_noalloc does the work of sfxc_gpu_copy_spectra with
// its scratch (fringe-stopped series, per-block delay parameters, the stream
// descriptor and the spectra before the copy out) in one file-scope device
// array of fixed size instead of fresh allocations.
namespace {
constexpr int kNoallocMaxBlocks = 8192;                 // 2,097,152 samples of one stream and integration
constexpr size_t kNoallocMaxSpectra = (size_t)1 << 20;  // rows x (fft_size_correlation + 4) complex values
constexpr size_t kNoallocTsOff = 0;
constexpr size_t kNoallocParOff = kNoallocTsOff + (size_t)kNoallocMaxBlocks * kNd * sizeof(float);
constexpr size_t kNoallocDescOff = kNoallocParOff + (size_t)kNoallocMaxBlocks * sizeof(BlockPar);
constexpr size_t kNoallocSpecOff = kNoallocDescOff + 1024;
constexpr size_t kNoallocBytes = kNoallocSpecOff + kNoallocMaxSpectra * sizeof(float2);  // 16.4 MiB
static_assert(sizeof(StreamDev) <= 1024, "stream descriptor slot too small");

// Held by every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

std::mutex g_noalloc_mu;
std::map<int, unsigned char *> g_noalloc_addr;  // device ordinal -> device address of the array

// Device address of the array on `device` (current device), resolved once
// per device: in host code the array's name only stands in for the symbol.
unsigned char *noalloc_scratch(int device) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  auto it = g_noalloc_addr.find(device);
  if (it != g_noalloc_addr.end()) return it->second;
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr) throw CudaError(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  g_noalloc_addr[device] = static_cast<unsigned char *>(ptr);
  return static_cast<unsigned char *>(ptr);
}
}  // namespace

extern "C" {

int sfxc_gpu_copy_spectra_noalloc(sfxc_gpu_ctx *c, int32_t stream, float *out, size_t n) {
  if (!c || !c->have_job) return SFXC_GPU_ESTATE;
  if (stream < 0 || stream >= (int)c->sc.size()) return fail(c, Error(SFXC_GPU_EINVAL, "bad stream index"));
  try {
    const StreamCtx &s = c->sc[stream];
    const size_t rows = (size_t)c->nffts, K = (size_t)c->M + 1;
    if (!out || n < rows * K * 2) throw Error(SFXC_GPU_EINVAL, "output buffer too small");
    if (s.n_blocks > kNoallocMaxBlocks)
      throw Error(SFXC_GPU_EINVAL, "integration of " + std::to_string(s.n_blocks) +
                                       " blocks exceeds the static scratch (at most " +
                                       std::to_string(kNoallocMaxBlocks) + " blocks of 256 samples per stream)");
    if (rows * (size_t)c->kpad > kNoallocMaxSpectra)
      throw Error(SFXC_GPU_EINVAL, "spectra of " + std::to_string(rows * (size_t)c->kpad) +
                                       " values exceed the static scratch (at most " +
                                       std::to_string(kNoallocMaxSpectra) + " complex values)");
    CK(cudaSetDevice(c->device));
    unsigned char *base = noalloc_scratch(c->device);
    StreamDev d = c->hsd[stream];
    d.block0 = 0;
    d.n_blocks = s.n_blocks;
    d.spline_lo = spline_lo_for(d, s.sp.x);  // the block kernel walks the spline forward from block 0
    d.slot = 0;  // the only stream of this launch
    d.ts = reinterpret_cast<float *>(base + kNoallocTsOff);
    d.bpar = reinterpret_cast<BlockPar *>(base + kNoallocParOff);
    StreamDev *dd = reinterpret_cast<StreamDev *>(base + kNoallocDescOff);
    float2 *spec = reinterpret_cast<float2 *>(base + kNoallocSpecOff);
    // every scratch element read below is written first by the same call, so
    // nothing is cleared; the descriptor copy is ordered on the context stream
    CK(cudaMemcpyAsync(dd, &d, sizeof(StreamDev), cudaMemcpyHostToDevice, c->st));
    launch_fstep_block(dd, 1, s.n_blocks, c->tw256.as<float2>(), c->st);
    const int nper = c->p.window == WINDOW_NONE ? s.hop : s.rot;
    const sfxc_gpu_ctx::RotTables &t = c->rot_tables.at(s.rot);
    launch_window_fft(dd, 1, 0, (int)rows, (int)rows, t.window.as<float>(), t.twrot.as<float2>(), s.rot, nper, c->M,
                      c->kpad, spec, 0, 1.0f, c->st);
    CK(cudaGetLastError());
    CK(cudaMemcpy2DAsync(out, K * sizeof(float2), spec, c->kpad * sizeof(float2), K * sizeof(float2), rows,
                         cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return (int)(rows * K * 2);
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_extract_channels(sfxc_gpu_ctx *c, const uint8_t *words, int64_t nwords, int32_t word_bytes,
                              int32_t bits, int32_t n_subbands, int32_t fan_out, const int32_t *tracks, uint8_t *out) {
  if (!c) return SFXC_GPU_EINVAL;
  try {
    if (!words || !tracks || !out || nwords <= 0 || word_bytes <= 0 || n_subbands <= 0)
      throw Error(SFXC_GPU_EINVAL, "bad arguments");
    if (fan_out <= 0 || fan_out > 8 || 8 % fan_out || (bits != 1 && bits != 2) || fan_out % bits)
      throw Error(SFXC_GPU_EINVAL, "fan_out must divide 8 and be a multiple of bits_per_sample");
    for (int i = 0; i < n_subbands * fan_out; i++)
      if (tracks[i] < 0 || tracks[i] >= word_bytes * 8) throw Error(SFXC_GPU_EINVAL, "track outside the word");
    const int spb = 8 / fan_out;
    if (nwords % spb) throw Error(SFXC_GPU_EINVAL, "word count must be a multiple of 8/fan_out");
    CK(cudaSetDevice(c->device));
    const int64_t nout = nwords / spb;
    upload(c->xin, words, (size_t)(nwords * word_bytes), c->st);
    upload(c->xtracks, tracks, (size_t)n_subbands * fan_out * 4, c->st);
    c->xout.ensure((size_t)(nout * n_subbands));
    launch_extract(c->xin.as<uint8_t>(), nout, word_bytes, bits, n_subbands, fan_out, c->xtracks.as<int>(),
                   c->xout.as<uint8_t>(), c->st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, c->xout.p, (size_t)(nout * n_subbands), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_extract_block(sfxc_gpu_ctx *c, const sfxc_reader_block *block, int32_t word_bytes, int32_t bits,
                           int32_t n_subbands, int32_t fan_out, const int32_t *tracks, uint8_t *out,
                           int32_t *out_invalid) {
  if (!c) return SFXC_GPU_EINVAL;
  if (!block || !block->data || block->size <= 0 || word_bytes <= 0 || block->size % word_bytes ||
      (block->n_invalid > 0 && (!block->invalid || !out_invalid)))
    return fail(c, Error(SFXC_GPU_EINVAL, "bad reader block"));
  const int rc = sfxc_gpu_extract_channels(c, block->data, block->size / word_bytes, word_bytes, bits, n_subbands,
                                           fan_out, tracks, out);
  if (rc != SFXC_GPU_OK) return rc;
  // invalid byte runs of the input words, in bytes of each subband's output
  // (channel_extractor_tasklet.cc:181-194)
  for (int k = 0; k < 2 * block->n_invalid; k++) out_invalid[k] = block->invalid[k] * fan_out / (8 * word_bytes);
  return SFXC_GPU_OK;
}

struct sfxc_gpu_phasecal {
  sfxc_gpu_ctx *ctx = nullptr;
  int device = 0;
  sfxc_phasecal_params p{};
  int P = 0, spb = 4;
  // fold state (do_phasecal's phasecal, phasecal_count, phasecal_time):
  // started once the first integration start was seen; row 0 of acc holds
  // the running integration between calls once live
  bool started = false, live = false;
  int64_t count = 0, time = 0;
  DevBuf data, runs, acc;
  HostBuf staging;
};

sfxc_gpu_phasecal *sfxc_gpu_phasecal_create(sfxc_gpu_ctx *c, const sfxc_phasecal_params *p) {
  if (!c) return nullptr;
  try {
    if (!p) throw Error(SFXC_GPU_EINVAL, "null parameters");
    if (p->bits_per_sample != 1 && p->bits_per_sample != 2) throw Error(SFXC_GPU_EINVAL, "bits_per_sample must be 1 or 2");
    if (p->integration_ticks <= 0) throw Error(SFXC_GPU_EINVAL, "phase-cal integration time must be positive");
    // phasecal.resize((size_t)(sample_rate / 10e3)), SFXC_ASSERT(size % samples_per_byte == 0)
    const int P = (int)(p->sample_rate / 10e3);
    const int spb = 8 / p->bits_per_sample;
    if (p->sample_rate <= 0 || P <= 0 || P % spb) throw Error(SFXC_GPU_EINVAL, "sample_rate / 10 kHz bins must be a positive multiple of 8 / bits_per_sample");
    auto *pc = new sfxc_gpu_phasecal();
    pc->ctx = c;
    pc->device = c->device;
    pc->p = *p;
    pc->P = P;
    pc->spb = spb;
    return pc;
  } catch (const Error &e) {
    fail(c, e);
    return nullptr;
  }
}

void sfxc_gpu_phasecal_destroy(sfxc_gpu_phasecal *pc) {
  if (!pc) return;
  cudaSetDevice(pc->device);  // its buffers are freed there (cudaFree waits for the device)
  delete pc;
}

int sfxc_gpu_phasecal_push(sfxc_gpu_phasecal *pc, const uint8_t *stream, int32_t n_blocks,
                           const sfxc_channel_block *blocks, sfxc_output_sink sink, void *user) {
  if (!pc) return SFXC_GPU_EINVAL;
  sfxc_gpu_ctx *c = pc->ctx;
  try {
    if (n_blocks < 0 || (n_blocks && (!blocks || !stream))) throw Error(SFXC_GPU_EINVAL, "bad block list");
    for (int b = 0; b < n_blocks; b++) {
      const sfxc_channel_block &k = blocks[b];
      if (k.size < 0 || k.n_invalid < 0 || (k.n_invalid && !k.invalid)) throw Error(SFXC_GPU_EINVAL, "bad channel block");
      for (int v = 0; v < 2 * k.n_invalid; v++)
        if (k.invalid[v] < 0) throw Error(SFXC_GPU_EINVAL, "negative invalid run");
    }
    const int P = pc->P, spb = pc->spb, pb = P / spb;
    const int64_t T = pc->p.integration_ticks;
    // Host pass over the blocks in order: the integrations they start and end,
    // and each counted stretch of bytes with the bin of its first byte.  Long
    // stretches are cut every 64 periods (same first bin) to bound the work of
    // one thread.
    const int64_t piece = (int64_t)64 * pb;
    struct Close { int64_t time, length; };
    std::vector<Close> closes;
    std::vector<PcalRun> runs;
    int row = 0;
    int64_t off = 0, used_end = 0;
    auto add_run = [&](int64_t src, int64_t n) {
      const int bin0 = (int)((pc->count % P) / spb);
      for (int64_t q = 0; q < n; q += piece)
        runs.push_back(PcalRun{src + q, (int32_t)std::min(piece, n - q), bin0, row, 0});
      pc->count = (pc->count + n * spb) % P;
      used_end = src + n;
    };
    for (int b = 0; b < n_blocks; b++) {
      const sfxc_channel_block &k = blocks[b];
      if (k.start_ticks % T == 0) {
        if (pc->started) {
          closes.push_back(Close{pc->time, k.start_ticks - pc->time});
          row++;
        }
        pc->started = true;
        pc->count = 0;
        pc->time = k.start_ticks;
      }
      if (pc->started) {
        // do_phasecal's byte loop as stretches: at byte i an invalid run
        // beginning there is skipped (its samples advance the bin) and the byte
        // after it is counted without a check, so the next run is only ever
        // matched where it begins after that byte
        const int size = k.size;
        int64_t i = 0;
        int iv = 0;
        while (i < size) {
          if (iv < k.n_invalid && i == k.invalid[2 * iv]) {
            const int64_t n = k.invalid[2 * iv + 1];
            i += n;
            pc->count = (pc->count + n * spb) % P;
            iv++;
            if (i >= size) break;
          }
          // (a run beginning at or past the block end is never reached)
          const int64_t end = (iv < k.n_invalid && k.invalid[2 * iv] > i) ? std::min<int64_t>(k.invalid[2 * iv], size)
                                                                            : (int64_t)size;
          add_run(off + i, end - i);
          i = end;
        }
      }
      off += k.size;
    }
    const int rows = row + 1;
    if (!pc->started || (runs.empty() && closes.empty())) return SFXC_GPU_OK;
    CK(cudaSetDevice(c->device));
    if ((size_t)rows * P * 4 > pc->acc.cap) {
      // grow, keeping the running integration of row 0
      DevBuf grown;
      grown.ensure((size_t)std::max(rows, 4) * P * 4);
      if (pc->live) {
        CK(cudaMemcpyAsync(grown.p, pc->acc.p, (size_t)P * 4, cudaMemcpyDeviceToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
      }
      pc->acc.swap(grown);
    }
    // a new integration's row starts from zero; row 0 keeps the running one
    const int first_clear = pc->live ? 1 : 0;
    if (rows > first_clear)
      CK(cudaMemsetAsync(pc->acc.as<int32_t>() + (size_t)first_clear * P, 0, (size_t)(rows - first_clear) * P * 4, c->st));
    pc->live = true;
    if (!runs.empty()) {
      upload(pc->data, stream, (size_t)used_end, c->st);
      upload(pc->runs, runs.data(), runs.size() * sizeof(PcalRun), c->st);
      launch_phasecal(pc->data.as<uint8_t>(), pc->runs.as<PcalRun>(), (int)runs.size(), pb, pc->p.bits_per_sample,
                      pc->acc.as<int32_t>(), c->st);
      CK(cudaGetLastError());
    }
    const size_t nclose = closes.size();
    int32_t *h = nullptr;
    if (nclose) {
      h = (int32_t *)pc->staging.ensure(nclose * P * 4);
      CK(cudaMemcpyAsync(h, pc->acc.p, nclose * P * 4, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(pc->acc.p, pc->acc.as<int32_t>() + (size_t)row * P, (size_t)P * 4, cudaMemcpyDeviceToDevice,
                         c->st));
    }
    CK(cudaStreamSynchronize(c->st));
    // MPI_Pack layout of the message (input_node_data_writer.cc:250-265)
    std::vector<uint8_t> msg(4 + 8 + 8 + 4 + (size_t)P * 4);
    for (size_t k = 0; k < nclose; k++) {
      msg[0] = (uint8_t)pc->p.station_number;
      msg[1] = (uint8_t)pc->p.frequency_number;
      msg[2] = (uint8_t)pc->p.sideband;
      msg[3] = (uint8_t)pc->p.polarisation;
      std::memcpy(&msg[4], &closes[k].time, 8);
      std::memcpy(&msg[12], &closes[k].length, 8);
      const int32_t ns = P;
      std::memcpy(&msg[20], &ns, 4);
      std::memcpy(&msg[24], h + k * P, (size_t)P * 4);
      if (sink && sink(user, 2, msg.data(), msg.size()) != 0) throw Error(SFXC_GPU_EINVAL, "output sink refused the data");
    }
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_set_uvw(sfxc_gpu_ctx *c, const double *uvw, size_t n) {
  if (!c) return SFXC_GPU_EINVAL;
  if (!c->have_job) return fail(c, Error(SFXC_GPU_ESTATE, "no parameters set"));
  if (!uvw || n != c->uvw.size()) return fail(c, Error(SFXC_GPU_EINVAL, "uvw must hold n_streams x phase centres x 3 values"));
  std::copy(uvw, uvw + n, c->uvw.begin());
  return SFXC_GPU_OK;
}

// ---- output node (Output_node::start / write_output / write_global_header,
// sfxc/src/output_node.cc:68-214)
struct sfxc_gpu_output {
  int n_files = 0;
  sfxc_output_sink sink = nullptr;
  void *user = nullptr;
  int64_t next_slice = 0;  // curr_slice
  std::map<int64_t, std::pair<std::vector<uint8_t>, int>> held;  // slice -> (bytes, bins)
  // set when a slice's write stopped part way (a refusing sink or a bad file
  // index): some files already hold part of that slice, so writing it again
  // would duplicate bytes; every later call fails
  std::string failed;
};

namespace {
// write_output: each of the slice's n_bins equal parts is an int32 file index
// and the bytes that go to that file
void output_write_slice(sfxc_gpu_output *o, const std::vector<uint8_t> &b, int bins) {
  const size_t per = b.size() / (size_t)bins;
  for (int k = 0; k < bins; k++) {
    int32_t file;
    std::memcpy(&file, &b[k * per], 4);
    if (file < 0 || file >= o->n_files) throw Error(SFXC_GPU_EINVAL, "output file index outside the files");
    if (o->sink(o->user, file, &b[k * per + 4], per - 4) != 0)
      throw Error(SFXC_GPU_EINVAL, "output sink refused the data");
  }
}
}  // namespace

sfxc_gpu_output *sfxc_gpu_output_create(const sfxc_output_global *g, int32_t n_files, sfxc_output_sink sink,
                                        void *user) {
  try {
    if (!g || !sink || n_files <= 0) throw Error(SFXC_GPU_EINVAL, "bad output parameters");
    // Output_header_global, 84 bytes, little-endian, no padding
    std::vector<uint8_t> h(84, 0);
    auto put32 = [&](size_t off, int32_t v) { std::memcpy(&h[off], &v, 4); };
    auto put16 = [&](size_t off, int32_t v) {
      const int16_t x = (int16_t)v;
      std::memcpy(&h[off], &x, 2);
    };
    put32(0, 84);
    // strcpy into a zeroed field (the name up to its terminator, at most 31 bytes)
    std::memcpy(&h[4], g->experiment, strnlen(g->experiment, 31));
    put16(36, g->start_year);
    put16(38, g->start_day);
    put32(40, g->start_time);
    put32(44, g->number_channels);
    put32(48, g->integration_time_us);
    put32(52, 1);  // OUTPUT_FORMAT_VERSION
    put32(56, g->correlator_version);
    h[60] = (uint8_t)(int8_t)g->polarisation_type;
    // strncpy(15) with the last byte cleared
    std::memcpy(&h[61], g->correlator_branch, strnlen(g->correlator_branch, 14));
    put32(76, g->job_nr);
    put32(80, g->subjob_nr);
    std::unique_ptr<sfxc_gpu_output> o(new sfxc_gpu_output());
    o->n_files = n_files;
    o->sink = sink;
    o->user = user;
    for (int f = 0; f < n_files; f++)
      if (sink(user, f, h.data(), h.size()) != 0) throw Error(SFXC_GPU_EINVAL, "output sink refused the data");
    return o.release();
  } catch (const Error &e) {
    g_error = e.msg;
    return nullptr;
  }
}

int sfxc_gpu_output_put_slice(sfxc_gpu_output *o, int64_t slice_nr, const uint8_t *bytes, size_t n, int32_t bins) {
  if (!o) return SFXC_GPU_EINVAL;
  try {
    if (!o->failed.empty()) throw Error(SFXC_GPU_ESTATE, "output failed earlier: " + o->failed);
    if ((n && !bytes) || bins <= 0 || n % (size_t)bins || n / (size_t)bins < 4)
      throw Error(SFXC_GPU_EINVAL, "slice bytes must be n_bins equal parts of at least 4 bytes");
    // set_weight_of_input_stream: a slice already written or already held is an error
    if (slice_nr < o->next_slice || o->held.count(slice_nr)) throw Error(SFXC_GPU_EINVAL, "slice given twice");
    o->held[slice_nr] = {std::vector<uint8_t>(bytes, bytes + n), bins};
    for (auto it = o->held.begin(); it != o->held.end() && it->first == o->next_slice; it = o->held.begin()) {
      try {
        output_write_slice(o, it->second.first, it->second.second);
      } catch (const Error &e) {
        o->failed = "slice " + std::to_string(it->first) + ": " + e.msg;
        o->held.clear();
        throw;
      }
      o->held.erase(it);
      o->next_slice++;
    }
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    g_error = e.msg;
    return e.code;
  }
}

int sfxc_gpu_output_finish(sfxc_gpu_output *o) {
  if (!o) return SFXC_GPU_EINVAL;
  if (!o->failed.empty()) {
    g_error = "output failed earlier: " + o->failed;
    return SFXC_GPU_ESTATE;
  }
  if (!o->held.empty()) {
    g_error = "slices held for a missing slice " + std::to_string(o->next_slice);
    return SFXC_GPU_ESTATE;
  }
  return SFXC_GPU_OK;
}

void sfxc_gpu_output_destroy(sfxc_gpu_output *o) { delete o; }

int sfxc_gpu_last_timings_n(const sfxc_gpu_ctx *c, float *ms, int32_t n) {
  if (!c || !ms || n < 0) return SFXC_GPU_EINVAL;
  for (int i = 0; i < std::min<int32_t>(n, 7); i++) ms[i] = c->timings[i];
  return SFXC_GPU_OK;
}

int sfxc_gpu_last_timings(const sfxc_gpu_ctx *c, float *ms6) { return sfxc_gpu_last_timings_n(c, ms6, 6); }

int sfxc_gpu_delay_list(const sfxc_delay_table *table, int64_t start, int64_t stop, int32_t sample_rate, int32_t bits,
                        int64_t *ticks, int32_t *bytes, int32_t *remaining, int32_t capacity) {
  try {
    if (!table || !table->del_bytes) throw Error(SFXC_GPU_EINVAL, "no delay table");
    if (bits != 1 && bits != 2) throw Error(SFXC_GPU_EINVAL, "bits_per_sample must be 1 or 2");
    if (stop <= start) throw Error(SFXC_GPU_EINVAL, "empty interval");
    DelayTable t = DelayTable::parse(table->del_bytes, table->del_size);
    t.clock_offset = table->clock_offset;
    t.clock_rate = table->clock_rate;
    t.clock_epoch = table->clock_epoch_ticks;
    Spline sp = Spline::create(t, start, stop - start);
    std::vector<Delay> d = interval_delays(sp, start, stop, sample_rate, bits);
    for (size_t i = 0; i < d.size() && (int)i < capacity; i++) {
      ticks[i] = d[i].time;
      bytes[i] = d[i].bytes;
      remaining[i] = d[i].rem;
    }
    return (int)d.size();
  } catch (const Error &e) {
    g_error = e.msg;
    return e.code;
  }
}

int64_t sfxc_gpu_write_protocol(const uint8_t *stream, int32_t n_blocks, const sfxc_channel_block *blocks,
                                int32_t n_slices, const sfxc_slice *slices, int32_t sample_rate, int32_t bits,
                                int64_t integration_time_us, uint8_t *out, int64_t capacity, int64_t *offsets) {
  try {
    if (!stream || !blocks || !slices || n_blocks < 0 || n_slices < 0) throw Error(SFXC_GPU_EINVAL, "bad arguments");
    std::vector<ChannelBlock> cb(n_blocks);
    int64_t off = 0;
    for (int i = 0; i < n_blocks; i++) {
      cb[i].start = blocks[i].start_ticks;
      cb[i].size = blocks[i].size;
      cb[i].src_offset = off;
      off += blocks[i].size;
      for (int k = 0; k < blocks[i].n_invalid; k++)
        cb[i].invalid.push_back(InvalidRun{blocks[i].invalid[2 * k], blocks[i].invalid[2 * k + 1]});
    }
    std::vector<SliceRequest> sl(n_slices);
    for (int i = 0; i < n_slices; i++) {
      sl[i].start = slices[i].start_ticks;
      sl[i].stop = slices[i].stop_ticks;
      sl[i].nr_samples = slices[i].nr_samples;
      for (int k = 0; k < slices[i].n_delays; k++)
        sl[i].delays.push_back(Delay{slices[i].delay_ticks[k], slices[i].delay_bytes[k], slices[i].delay_remaining[k]});
      if (sl[i].delays.empty()) throw Error(SFXC_GPU_EINVAL, "slice without delays");
    }
    auto recs = write_protocol(cb, sl, sample_rate, bits, (double)integration_time_us);
    int64_t total = 0;
    std::vector<uint8_t> buf;
    for (int i = 0; i < n_slices; i++) {
      buf.clear();
      serialize_protocol(recs[i], stream, buf);
      if (offsets) offsets[i] = total;
      if (out) {
        if (total + (int64_t)buf.size() > capacity) throw Error(SFXC_GPU_EINVAL, "output buffer too small");
        std::memcpy(out + total, buf.data(), buf.size());
      }
      total += (int64_t)buf.size();
    }
    if (offsets) offsets[n_slices] = total;
    return total;
  } catch (const Error &e) {
    g_error = e.msg;
    return e.code;
  }
}


namespace {
// Input_node_parameters as the readers take them (sfxc_reader_params).
ReaderParams reader_params(const sfxc_reader_params *p) {
  ReaderParams rp;
  rp.format = p->format;
  rp.ref_ticks = p->ref_ticks;
  rp.offset_ticks = p->offset_ticks;
  rp.track_bit_rate = p->track_bit_rate;
  rp.frame_size = p->frame_size;
  rp.n_tracks = p->n_tracks;
  rp.bits_per_sample = p->bits_per_sample;
  rp.tracks_per_channel = p->tracks_per_channel;
  rp.first_track.assign(p->first_track, p->first_track + p->n_channels);
  return rp;
}
}  // namespace

struct sfxc_gpu_reader {
  std::unique_ptr<FormatReader> r;
  ReaderBlock block;
};

sfxc_gpu_reader *sfxc_gpu_reader_create(const sfxc_reader_params *p, const uint8_t *bytes, size_t n) {
  try {
    if (!p || (n && !bytes)) throw Error(SFXC_GPU_EINVAL, "no reader parameters or data");
    if (p->n_channels <= 0 || !p->first_track) throw Error(SFXC_GPU_EINVAL, "no channels");
    std::unique_ptr<sfxc_gpu_reader> h(new sfxc_gpu_reader());
    try {
      h->r = FormatReader::create(reader_params(p), bytes, n);
    } catch (const std::exception &e) {
      throw Error(SFXC_GPU_EINVAL, e.what());
    }
    return h.release();
  } catch (const Error &e) {
    g_error = e.msg;
    return nullptr;
  }
}

int sfxc_gpu_reader_next(sfxc_gpu_reader *h, sfxc_reader_block *out) {
  if (!h || !out) return SFXC_GPU_EINVAL;
  if (!h->r->next(h->block)) return 0;
  out->data = h->block.data.data();
  out->size = (int32_t)h->block.data.size();
  out->channel = h->block.channel;
  out->start_ticks = h->block.start_ticks;
  out->n_invalid = (int32_t)(h->block.invalid.size() / 2);
  out->invalid = h->block.invalid.data();
  return 1;
}

void sfxc_gpu_reader_destroy(sfxc_gpu_reader *h) { delete h; }

// ---- recordings in device memory: the input node's reader, channel
// extractor and writer with the recording's bytes kept on the device (the
// headers decoded, the fill runs found, the channels extracted and the
// protocol bytes assembled by kernels; the readers' block decisions and the
// writer's records on the host)
namespace {
struct DeviceFrames : FrameSource {
  const uint8_t *rec = nullptr;
  int64_t n = 0;
  cudaStream_t st = nullptr;
  DevBuf *info = nullptr;
  HostBuf *staging = nullptr;
  int64_t size() const override { return n; }
  void decode(int format, int64_t pos0, int64_t stride, int64_t count, FrameInfo *out) override {
    if (count <= 0) return;
    const size_t bytes = (size_t)count * sizeof(FrameInfo);
    info->ensure(bytes);
    launch_decode_frames(rec, pos0, stride, count, format == FORMAT_MARK5B, info->as<FrameInfo>(), st);
    CK(cudaGetLastError());
    staging->ensure(bytes);
    CK(cudaMemcpyAsync(staging->p, info->p, bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memcpy(out, staging->p, bytes);
  }
  void fetch(int64_t pos, int64_t len, uint8_t *dst) override {
    if (len <= 0) return;
    CK(cudaMemcpyAsync(dst, rec + pos, (size_t)len, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
};
}  // namespace

// The writer's records for one set of slices and their serialised layout:
// shared by every subband of an extracted recording (same blocks, same
// invalid runs, payload offsets relative to the channel's bytes).
struct ProtoPlan {
  std::vector<int64_t> key;  // the slices and arguments it was made for
  int group = 0;             // channel (one channel per thread) or -1 (every subband)
  std::vector<int64_t> offsets;
  std::vector<std::vector<Record>> slice_recs;  // DATA payload offsets within the slice's bytes
  std::vector<ProtoRecord> dev_recs;  // also on the device, in the recording's plan buffer of its group
  int64_t total = 0;
};

struct sfxc_gpu_recording {
  sfxc_gpu_ctx *ctx = nullptr;
  ReaderParams p;
  std::unique_ptr<RecordingBuffers> buf;
  const uint8_t *rec = nullptr;
  int64_t n = 0;
  std::vector<FrameBlock> blocks;
  int nf = 0, fb = 0, block_size = 0;  // frames per block, frame payload bytes, block bytes
  // channel streams: channel c's bytes at buf->chan + chan_off[c], its
  // blocks (offsets within them) and their invalid runs as (begin, n) pairs
  bool per_thread = false;
  std::vector<int64_t> chan_off;
  // block lists: every subband of an extracted recording shares one, each
  // VDIF thread's channel has its own; chan_set[c] is channel c's
  std::vector<int> chan_set;
  std::vector<std::vector<ChannelBlock>> set_blocks;
  std::vector<std::vector<std::vector<int32_t>>> set_runs;
  const std::vector<ChannelBlock> &blocks_of(int c) const { return set_blocks[chan_set[c]]; }
  int n_channels() const { return (int)chan_set.size(); }
  // each channel's last protocol (its bytes in buf->proto[c])
  std::vector<std::shared_ptr<ProtoPlan>> proto;
  std::shared_ptr<ProtoPlan> last_plan;
};

namespace {
DeviceFrames device_frames(sfxc_gpu_recording *r) {
  DeviceFrames src;
  src.rec = r->rec;
  src.n = r->n;
  src.st = r->ctx->st;
  src.info = &r->buf->info;
  src.staging = &r->buf->staging;
  return src;
}

// The recording's blocks: `blocks` in order, each carrying the bytes of a
// walk block (its frames) or none (filled in: frame offsets -1, wholly
// invalid).  Mark5B blocks take the fill-pattern runs of their walk block,
// found on the device.
void install_blocks(sfxc_gpu_recording *r, const FrameWalk &walk, const std::vector<ScheduledBlock> &blocks) {
  sfxc_gpu_ctx *c = r->ctx;
  RecordingBuffers &B = *r->buf;
  const bool mk5b = r->p.format == FORMAT_MARK5B;
  r->blocks.clear();
  r->chan_set.clear();
  r->set_blocks.clear();
  r->set_runs.clear();
  r->chan_off.clear();
  r->proto.clear();
  r->last_plan.reset();
  if (!walk.blocks.empty()) {
    r->nf = walk.blocks[0].nframes;
    r->fb = walk.blocks[0].frame_bytes;
    r->block_size = walk.blocks[0].size;
  } else if (mk5b) {
    r->nf = kMk5bBlockFrames;
    r->fb = kMk5bFrame;
    r->block_size = kMk5bBlock;
  } else if (!blocks.empty()) {
    throw Error(SFXC_GPU_EINVAL, "no VDIF frame header in the recording: no block size for filled-in blocks");
  }
  const int nw = (int)walk.blocks.size();
  for (int b = 0; b < nw; b++)
    if (walk.blocks[b].nframes != r->nf || walk.blocks[b].size != r->block_size ||
        walk.blocks[b].first != (int64_t)b * r->nf)
      throw Error(SFXC_GPU_ESTATE, "uneven reader blocks");
  // fill-pattern runs of every Mark5B walk block: count, then write
  std::vector<std::vector<int32_t>> fill(mk5b ? nw : 0);
  if (mk5b && nw) {
    upload(B.frames, walk.frames.data(), walk.frames.size() * sizeof(int64_t), c->st);
    B.counts.ensure((size_t)nw * 4);
    launch_fill_runs(r->rec, B.frames.as<int64_t>(), r->nf, r->fb / 4, r->block_size / 4, nw, B.counts.as<int32_t>(),
                     nullptr, nullptr, c->st);
    CK(cudaGetLastError());
    std::vector<int32_t> cnt(nw);
    CK(cudaMemcpyAsync(cnt.data(), B.counts.p, (size_t)nw * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    std::vector<int64_t> off(nw + 1, 0);
    for (int b = 0; b < nw; b++) off[b + 1] = off[b] + cnt[b];
    if (off[nw]) {
      upload(B.offs, off.data(), (size_t)nw * 8, c->st);
      B.runs.ensure((size_t)off[nw] * 8);
      launch_fill_runs(r->rec, B.frames.as<int64_t>(), r->nf, r->fb / 4, r->block_size / 4, nw, nullptr,
                       B.offs.as<int64_t>(), B.runs.as<int32_t>(), c->st);
      CK(cudaGetLastError());
      std::vector<int32_t> runs((size_t)off[nw] * 2);
      CK(cudaMemcpyAsync(runs.data(), B.runs.p, runs.size() * 4, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      for (int b = 0; b < nw; b++) fill[b].assign(runs.begin() + 2 * off[b], runs.begin() + 2 * off[b + 1]);
    }
  }
  std::vector<int64_t> frames;
  frames.reserve(blocks.size() * (size_t)r->nf);
  for (const ScheduledBlock &sb : blocks) {
    FrameBlock fb;
    fb.channel = sb.channel;
    fb.start_ticks = sb.start_ticks;
    fb.size = r->block_size;
    fb.frame_bytes = r->fb;
    fb.nframes = r->nf;
    fb.first = (int64_t)frames.size();
    if (sb.whole_invalid || sb.block < 0) {
      frames.insert(frames.end(), (size_t)r->nf, (int64_t)-1);
      fb.invalid = {0, r->block_size};
      fb.invalid.insert(fb.invalid.end(), sb.invalid.begin(), sb.invalid.end());
    } else {
      const FrameBlock &w = walk.blocks[(size_t)sb.block];
      frames.insert(frames.end(), walk.frames.begin() + w.first, walk.frames.begin() + w.first + r->nf);
      fb.invalid = mk5b ? fill[(size_t)sb.block] : sb.invalid;
    }
    r->blocks.push_back(std::move(fb));
  }
  if (!frames.empty()) upload(B.frames, frames.data(), frames.size() * sizeof(int64_t), c->st);
  CK(cudaStreamSynchronize(c->st));
}
}  // namespace

sfxc_gpu_recording *sfxc_gpu_recording_create(sfxc_gpu_ctx *c, const sfxc_reader_params *params,
                                               const uint8_t *bytes, size_t n, int32_t bytes_on_device) {
  if (!c) return nullptr;
  try {
    if (!params || (n && !bytes)) throw Error(SFXC_GPU_EINVAL, "no reader parameters or data");
    if (params->n_channels <= 0 || !params->first_track) throw Error(SFXC_GPU_EINVAL, "no channels");
    CK(cudaSetDevice(c->device));
    std::unique_ptr<sfxc_gpu_recording> r(new sfxc_gpu_recording());
    r->ctx = c;
    r->p = reader_params(params);
    r->n = (int64_t)n;
    if (!c->rec_spare.empty()) {
      r->buf = std::move(c->rec_spare.back());
      c->rec_spare.pop_back();
    } else {
      r->buf.reset(new RecordingBuffers());
    }
    RecordingBuffers &B = *r->buf;
    if (bytes_on_device) {
      r->rec = bytes;
    } else {
      B.own.ensure(n + 16);
      if (n) CK(cudaMemcpyAsync(B.own.p, bytes, n, cudaMemcpyHostToDevice, c->st));
      r->rec = B.own.as<uint8_t>();
    }
    FrameWalk walk;
    {
      DeviceFrames src = device_frames(r.get());
      try {
        walk = walk_frames(r->p, src);
      } catch (const std::invalid_argument &e) {
        throw Error(SFXC_GPU_EINVAL, e.what());
      } catch (const std::logic_error &e) {
        throw Error(SFXC_GPU_ESTATE, e.what());
      }
    }
    std::vector<ScheduledBlock> all;
    for (size_t b = 0; b < walk.blocks.size(); b++)
      all.push_back(ScheduledBlock{walk.blocks[b].start_ticks, walk.blocks[b].channel, (int32_t)b, false,
                                   walk.blocks[b].invalid});
    install_blocks(r.get(), walk, all);
    CK(cudaStreamSynchronize(c->st));
    return r.release();
  } catch (const Error &e) {
    fail(c, e);
    return nullptr;
  }
}

void sfxc_gpu_recording_destroy(sfxc_gpu_recording *r) {
  if (!r) return;
  cudaSetDevice(r->ctx->device);
  cudaStreamSynchronize(r->ctx->st);
  r->ctx->rec_spare.push_back(std::move(r->buf));  // its buffers serve the context's next recording
  delete r;
}

int sfxc_gpu_recording_schedule(sfxc_gpu_recording *r, int32_t n_intervals, const int64_t *intervals) {
  if (!r) return SFXC_GPU_EINVAL;
  sfxc_gpu_ctx *c = r->ctx;
  try {
    if (n_intervals < 0 || (n_intervals && !intervals)) throw Error(SFXC_GPU_EINVAL, "bad intervals");
    CK(cudaSetDevice(c->device));
    std::vector<TimeInterval> iv;
    for (int k = 0; k < n_intervals; k++)
      iv.push_back(TimeInterval{intervals[3 * k], intervals[3 * k + 1], intervals[3 * k + 2]});
    DeviceFrames src = device_frames(r);
    Schedule sched;
    try {
      sched = schedule_blocks(r->p, src, iv);
    } catch (const std::invalid_argument &e) {
      throw Error(SFXC_GPU_EINVAL, e.what());
    } catch (const std::exception &e) {
      throw Error(SFXC_GPU_ESTATE, e.what());
    }
    install_blocks(r, sched.walk, sched.blocks);
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int32_t sfxc_gpu_recording_n_blocks(const sfxc_gpu_recording *r) { return r ? (int32_t)r->blocks.size() : 0; }

int sfxc_gpu_recording_block(sfxc_gpu_recording *r, int32_t i, sfxc_reader_block *out, uint8_t *data) {
  if (!r) return SFXC_GPU_EINVAL;
  sfxc_gpu_ctx *c = r->ctx;
  try {
    if (!out || i < 0 || i >= (int32_t)r->blocks.size()) throw Error(SFXC_GPU_EINVAL, "bad block index");
    const FrameBlock &b = r->blocks[i];
    out->data = data;
    out->size = b.size;
    out->channel = b.channel;
    out->start_ticks = b.start_ticks;
    out->n_invalid = (int32_t)(b.invalid.size() / 2);
    out->invalid = b.invalid.data();
    if (data) {  // the block's bytes, assembled from its frames on the device
      CK(cudaSetDevice(c->device));
      RecordingBuffers &B = *r->buf;
      upload(B.list, &i, 4, c->st);
      B.gathered.ensure((size_t)b.size);
      launch_gather_blocks(r->rec, B.frames.as<int64_t>(), r->nf, r->fb, r->block_size, B.list.as<int32_t>(), 1,
                           B.gathered.as<uint8_t>(), c->st);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(data, B.gathered.p, (size_t)b.size, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
    }
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_recording_extract(sfxc_gpu_recording *r, int32_t word_bytes, int32_t bits, int32_t n_subbands,
                               int32_t fan_out, const int32_t *tracks) {
  if (!r) return SFXC_GPU_EINVAL;
  sfxc_gpu_ctx *c = r->ctx;
  try {
    CK(cudaSetDevice(c->device));
    const int nb = (int)r->blocks.size();
    RecordingBuffers &B = *r->buf;
    r->chan_set.clear();
    r->set_blocks.clear();
    r->set_runs.clear();
    r->chan_off.clear();
    r->proto.clear();
    r->last_plan.reset();
    r->per_thread = word_bytes == 0;
    if (word_bytes == 0) {
      // one channel per VDIF thread (Channel_extractor_tasklet_VDIF::do_task,
      // sfxc/src/channel_extractor_tasklet_vdif.cc:25-49): each block is its
      // channel's next block as it is
      const int nch = (int)r->p.first_track.size();
      if (n_subbands != nch) throw Error(SFXC_GPU_EINVAL, "n_subbands must be the channel count");
      std::vector<std::vector<int32_t>> lists(nch);
      for (int b = 0; b < nb; b++) {
        const int ch = r->blocks[b].channel;
        if (ch < 0 || ch >= nch) throw Error(SFXC_GPU_EINVAL, "block of a channel outside the channel list");
        lists[ch].push_back(b);
      }
      r->set_blocks.resize(nch);
      r->set_runs.resize(nch);
      for (int ch = 0; ch < nch; ch++) r->chan_set.push_back(ch);
      int64_t total = 0;
      for (int ch = 0; ch < nch; ch++) {
        r->chan_off.push_back(total);
        total += (int64_t)lists[ch].size() * r->block_size;
      }
      B.chan.ensure((size_t)total + 16);
      std::vector<int32_t> all;
      for (auto &l : lists) all.insert(all.end(), l.begin(), l.end());
      upload(B.list, all.data(), all.size() * 4, c->st);
      int64_t e0 = 0;
      for (int ch = 0; ch < nch; ch++) {
        launch_gather_blocks(r->rec, B.frames.as<int64_t>(), r->nf, r->fb, r->block_size,
                             B.list.as<int32_t>() + e0, (int)lists[ch].size(),
                             B.chan.as<uint8_t>() + r->chan_off[ch], c->st);
        CK(cudaGetLastError());
        e0 += (int64_t)lists[ch].size();
        for (size_t j = 0; j < lists[ch].size(); j++) {
          const FrameBlock &b = r->blocks[lists[ch][j]];
          ChannelBlock cb;
          cb.start = b.start_ticks;
          cb.src_offset = (int64_t)j * r->block_size;
          cb.size = r->block_size;
          for (size_t k = 0; k + 1 < b.invalid.size(); k += 2) cb.invalid.push_back(InvalidRun{b.invalid[k], b.invalid[k + 1]});
          r->set_blocks[ch].push_back(cb);
          r->set_runs[ch].push_back(b.invalid);
        }
      }
    } else {
      // Channel_extractor_tasklet::do_task (sfxc/src/channel_extractor_tasklet.cc:120-220)
      // over every block, each block's words read from its frames
      if (!tracks || word_bytes <= 0 || n_subbands <= 0) throw Error(SFXC_GPU_EINVAL, "bad arguments");
      if (fan_out <= 0 || fan_out > 8 || 8 % fan_out || (bits != 1 && bits != 2) || fan_out % bits)
        throw Error(SFXC_GPU_EINVAL, "fan_out must divide 8 and be a multiple of bits_per_sample");
      for (int i = 0; i < n_subbands * fan_out; i++)
        if (tracks[i] < 0 || tracks[i] >= word_bytes * 8) throw Error(SFXC_GPU_EINVAL, "track outside the word");
      const int per_byte = 8 / fan_out * word_bytes;  // input bytes per output byte
      if (nb && (r->fb % word_bytes || r->block_size % per_byte))
        throw Error(SFXC_GPU_EINVAL, "frames are not whole words, or blocks not whole output bytes");
      const int64_t opb = nb ? r->block_size / per_byte : 0;
      const int64_t nout = (int64_t)nb * opb;
      B.chan.ensure((size_t)(nout * n_subbands) + 16);
      // each subband's tracks one bit field, as the extractor orders them
      // (2-bit samples: track pairs swapped)?  Then its lowest bit is enough.
      std::vector<int32_t> bases(n_subbands);
      bool fields = true;
      for (int sb = 0; sb < n_subbands && fields; sb++) {
        const int32_t *tr = tracks + sb * fan_out;
        bases[sb] = tr[bits == 2 ? 1 : 0];
        for (int q = 0; q < fan_out; q++)
          if (tr[bits == 2 ? (q ^ 1) : q] != bases[sb] + q) fields = false;
      }
      if (fields) {
        upload(B.tracks, bases.data(), bases.size() * 4, c->st);
        fields = launch_extract_fields(r->rec, B.frames.as<int64_t>(), r->nf, r->fb, opb, nout, word_bytes, fan_out,
                                       n_subbands, B.tracks.as<int>(), B.chan.as<uint8_t>(), c->st);
      }
      if (!fields) upload(B.tracks, tracks, (size_t)n_subbands * fan_out * 4, c->st);
      if (!fields && !launch_extract_frames(r->rec, B.frames.as<int64_t>(), r->nf, r->fb, opb, nout, word_bytes, bits,
                                 n_subbands, fan_out, B.tracks.as<int>(), B.chan.as<uint8_t>(), c->st))
        throw Error(SFXC_GPU_EINVAL, "more than 1024 tracks in all, or words over 8 bytes across frames");
      CK(cudaGetLastError());
      // every subband: the same blocks at the same offsets in its own bytes
      r->set_blocks.resize(1);
      r->set_runs.resize(1);
      r->set_blocks[0].reserve(nb);
      r->set_runs[0].reserve(nb);
      for (int b = 0; b < nb; b++) {
        ChannelBlock cb;
        cb.start = r->blocks[b].start_ticks;
        cb.src_offset = (int64_t)b * opb;
        cb.size = (int32_t)opb;
        // invalid byte runs in bytes of each subband (channel_extractor_tasklet.cc:181-194)
        std::vector<int32_t> runs;
        for (int32_t v : r->blocks[b].invalid) runs.push_back(v * fan_out / (8 * word_bytes));
        for (size_t k = 0; k + 1 < runs.size(); k += 2) cb.invalid.push_back(InvalidRun{runs[k], runs[k + 1]});
        r->set_blocks[0].push_back(std::move(cb));
        r->set_runs[0].push_back(std::move(runs));
      }
      for (int sb = 0; sb < n_subbands; sb++) {
        r->chan_off.push_back((int64_t)sb * nout);
        r->chan_set.push_back(0);
      }
    }
    r->proto.assign(r->n_channels(), nullptr);
    if ((int)B.proto.size() < r->n_channels()) B.proto.resize(r->n_channels());
    CK(cudaStreamSynchronize(c->st));
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int32_t sfxc_gpu_recording_channel(sfxc_gpu_recording *r, int32_t channel, int32_t capacity,
                                   sfxc_channel_block *blocks, uint8_t *data) {
  if (!r) return SFXC_GPU_EINVAL;
  sfxc_gpu_ctx *c = r->ctx;
  try {
    if (channel < 0 || channel >= r->n_channels()) throw Error(SFXC_GPU_EINVAL, "bad channel");
    const auto &cb = r->blocks_of(channel);
    const auto &runs = r->set_runs[r->chan_set[channel]];
    const int nb = (int)cb.size();
    if (blocks) {
      if (capacity < nb) throw Error(SFXC_GPU_EINVAL, "block array too small");
      for (int b = 0; b < nb; b++) {
        blocks[b].start_ticks = cb[b].start;
        blocks[b].size = cb[b].size;
        blocks[b].n_invalid = (int32_t)(runs[b].size() / 2);
        blocks[b].invalid = runs[b].data();
      }
    }
    if (data && nb) {
      CK(cudaSetDevice(c->device));
      const int64_t bytes = cb.back().src_offset + cb.back().size;
      CK(cudaMemcpyAsync(data, r->buf->chan.as<uint8_t>() + r->chan_off[channel], (size_t)bytes,
                         cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
    }
    return nb;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int64_t sfxc_gpu_recording_protocol(sfxc_gpu_recording *r, int32_t channel, int32_t n_slices,
                                    const sfxc_slice *slices, int32_t sample_rate, int32_t bits,
                                    int64_t integration_time_us, uint8_t *out, int64_t capacity,
                                    int64_t *out_offsets) {
  if (!r) return SFXC_GPU_EINVAL;
  sfxc_gpu_ctx *c = r->ctx;
  try {
    if (channel < 0 || channel >= r->n_channels()) throw Error(SFXC_GPU_EINVAL, "bad channel");
    if (!slices || n_slices < 0) throw Error(SFXC_GPU_EINVAL, "bad slices");
    CK(cudaSetDevice(c->device));
    std::vector<int64_t> key{sample_rate, bits, integration_time_us, n_slices};
    for (int i = 0; i < n_slices; i++) {
      key.insert(key.end(), {slices[i].start_ticks, slices[i].stop_ticks, slices[i].nr_samples, slices[i].n_delays});
      for (int k = 0; k < slices[i].n_delays; k++)
        key.insert(key.end(), {slices[i].delay_ticks[k], slices[i].delay_bytes[k], slices[i].delay_remaining[k]});
    }
    // every subband of an extracted recording has the same blocks and
    // invalid runs: the records of one serve them all
    const int group = r->per_thread ? channel : -1;
    std::shared_ptr<ProtoPlan> plan = r->last_plan;
    if (!plan || plan->group != group || plan->key != key) {
      std::vector<SliceRequest> sl(n_slices);
      for (int i = 0; i < n_slices; i++) {
        sl[i].start = slices[i].start_ticks;
        sl[i].stop = slices[i].stop_ticks;
        sl[i].nr_samples = slices[i].nr_samples;
        for (int k = 0; k < slices[i].n_delays; k++)
          sl[i].delays.push_back(
              Delay{slices[i].delay_ticks[k], slices[i].delay_bytes[k], slices[i].delay_remaining[k]});
        if (sl[i].delays.empty()) throw Error(SFXC_GPU_EINVAL, "slice without delays");
      }
      // the writer's records (Input_node_data_writer::do_task), then where their bytes go
      auto recs = write_protocol(r->blocks_of(channel), sl, sample_rate, bits, (double)integration_time_us);
      plan = std::make_shared<ProtoPlan>();
      plan->key = key;
      plan->group = group;
      plan->offsets.assign(1, 0);
      plan->slice_recs.assign(n_slices, {});
      int64_t total = 0;
      for (int i = 0; i < n_slices; i++) {
        const int64_t s0 = total;
        for (const Record &q : recs[i]) {
          plan->dev_recs.push_back(ProtoRecord{q.src, total, q.n, q.type, q.rem, 0});
          Record rel = q;
          if (q.type == HEADER_DATA) rel.src = total - s0 + 3;
          plan->slice_recs[i].push_back(rel);
          total += q.type == HEADER_ENDSTREAM ? 1 : q.type == HEADER_DELAY ? 2 : q.type == HEADER_DATA ? 3 + q.n : 3;
        }
        plan->offsets.push_back(total);
      }
      plan->total = total;
      upload(r->buf->plan_recs[group], plan->dev_recs.data(), plan->dev_recs.size() * sizeof(ProtoRecord), c->st);
      r->last_plan = plan;
    }
    if (out_offsets)
      for (int i = 0; i <= n_slices; i++) out_offsets[i] = plan->offsets[i];
    DevBuf &bytes = r->buf->proto[channel];
    bytes.ensure((size_t)plan->total + 16);
    launch_serialize_protocol(r->buf->plan_recs[group].as<ProtoRecord>(), (int)plan->dev_recs.size(),
                              r->buf->chan.as<uint8_t>() + r->chan_off[channel], bytes.as<uint8_t>(), c->st);
    CK(cudaGetLastError());
    r->proto[channel] = plan;
    if (out) {
      if (plan->total > capacity) throw Error(SFXC_GPU_EINVAL, "output buffer too small");
      CK(cudaMemcpyAsync(out, bytes.p, (size_t)plan->total, cudaMemcpyDeviceToHost, c->st));
    }
    CK(cudaStreamSynchronize(c->st));
    return plan->total;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

int sfxc_gpu_recording_push(sfxc_gpu_recording *r, int32_t channel, int32_t slice, sfxc_gpu_ctx *c, int32_t stream) {
  if (!r || !c) return SFXC_GPU_EINVAL;
  if (!c->have_job) return fail(c, Error(SFXC_GPU_ESTATE, "no parameters set"));
  if (stream < 0 || stream >= (int)c->sc.size()) return fail(c, Error(SFXC_GPU_EINVAL, "bad stream index"));
  try {
    if (c->device != r->ctx->device) throw Error(SFXC_GPU_EINVAL, "recording and correlator on different devices");
    if (channel < 0 || channel >= (int32_t)r->proto.size() || !r->proto[channel] || slice < 0 ||
        slice + 1 >= (int32_t)r->proto[channel]->offsets.size())
      throw Error(SFXC_GPU_EINVAL, "no protocol for that channel and slice");
    CK(cudaSetDevice(c->device));
    const ProtoPlan &pr = *r->proto[channel];
    const uint8_t *pbytes = r->buf->proto[channel].as<uint8_t>();
    const int64_t b0 = pr.offsets[slice], n = pr.offsets[slice + 1] - b0;
    StreamCtx &s = c->sc[stream];
    grow_stream_input(c, s, (size_t)n);
    // the protocol is complete on the recording's stream (its calls return
    // after it); the copy runs on the correlator's
    if (n) CK(cudaMemcpyAsync(s.src.as<uint8_t>() + s.dev_bytes, pbytes + b0, (size_t)n, cudaMemcpyDeviceToDevice,
                              c->st));
    for (Record q : pr.slice_recs[slice]) {
      if (q.type == HEADER_DATA) q.src += s.dev_bytes;
      s.pending.push_back(q);
    }
    CK(cudaStreamSynchronize(c->st));
    s.dev_bytes += n;
    s.pushed = true;
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    return fail(c, e);
  }
}

// ---- the UVW model (host only)
struct sfxc_gpu_uvw_model {
  std::unique_ptr<UvwModel> m;
};

sfxc_gpu_uvw_model *sfxc_gpu_uvw_create(const uint8_t *del_bytes, size_t n) {
  try {
    if (!del_bytes || !n) throw Error(SFXC_GPU_EINVAL, "no delay table");
    std::unique_ptr<sfxc_gpu_uvw_model> h(new sfxc_gpu_uvw_model());
    h->m.reset(new UvwModel(DelayTable::parse(del_bytes, n)));
    return h.release();
  } catch (const Error &e) {
    g_error = e.msg;
    return nullptr;
  }
}

int sfxc_gpu_uvw_get(sfxc_gpu_uvw_model *h, int32_t phase_center, int64_t time_ticks, double *uvw) {
  if (!h || !uvw) return SFXC_GPU_EINVAL;
  try {
    h->m->get(phase_center, time_ticks, uvw);
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    g_error = e.msg;
    return SFXC_GPU_EINVAL;
  }
}

void sfxc_gpu_uvw_destroy(sfxc_gpu_uvw_model *h) { delete h; }

// ---- correlation set-up from the control file and the VEX file

struct sfxc_gpu_control {
  Control c;
  std::string plan;
};

sfxc_gpu_control *sfxc_gpu_control_open(const char *ctrl_path, const char *vex_path) {
  try {
    if (!ctrl_path || !vex_path) throw Error(SFXC_GPU_EINVAL, "no control or vex file");
    std::unique_ptr<sfxc_gpu_control> h(new sfxc_gpu_control());
    h->c.initialise(ctrl_path, vex_path);
    return h.release();
  } catch (const Error &e) {
    g_error = e.msg;
  } catch (const std::exception &e) {
    g_error = e.what();
  }
  return nullptr;
}

int64_t sfxc_gpu_control_plan(sfxc_gpu_control *h, sfxc_station_time_fn station_time, void *user) {
  if (!h) return SFXC_GPU_EINVAL;
  try {
    std::function<ticks_t(int, int)> st;
    if (station_time) st = [station_time, user](int s, int scan) { return (ticks_t)station_time(user, s, scan); };
    Json j = plan_json(make_plan(h->c, st));
    j.set("ctrl", h->c.ctrl());
    Json ps = Json::parse("[]");
    for (const PulsarSpec &p : h->c.pulsars()) {
      Json x;
      x.set("name", Json::of_string(p.name));
      x.set("nbins", Json::of_int(p.nbins));
      x.set("gate_start", Json::of_double(p.gate_start));
      x.set("gate_stop", Json::of_double(p.gate_stop));
      Json pcs = Json::parse("[]");
      for (const PolycoBlock &pc : p.polyco) {
        Json y;
        y.set("name", Json::of_string(pc.name));
        y.set("tmid", Json::of_double(pc.tmid));
        y.set("dm", Json::of_double(pc.dm));
        y.set("ref_phase", Json::of_double(pc.ref_phase));
        y.set("ref_freq", Json::of_double(pc.ref_freq));
        y.set("obs_freq", Json::of_double(pc.obs_freq));
        y.set("data_span", Json::of_int(pc.data_span));
        Json co = Json::parse("[]");
        for (double v : pc.coef) co.append(Json::of_double(v));
        y.set("coef", co);
        pcs.append(y);
      }
      x.set("polyco", pcs);
      ps.append(x);
    }
    j.set("pulsars", ps);
    bool norm = false;
    std::vector<double> mask, window;
    if (h->c.mask(norm, mask, window)) {
      Json m, a = Json::parse("[]"), w = Json::parse("[]");
      for (double v : mask) a.append(Json::of_double(v));
      for (double v : window) w.append(Json::of_double(v));
      m.set("normalize", Json::of_bool(norm));
      m.set("mask", a);
      m.set("window", w);
      j.set("mask", m);
    }
    h->plan = j.dump();
    return (int64_t)h->plan.size();
  } catch (const Error &e) {
    g_error = e.msg;
  } catch (const std::exception &e) {
    g_error = e.what();
  }
  return SFXC_GPU_EINVAL;
}

const char *sfxc_gpu_control_plan_text(const sfxc_gpu_control *h) { return h ? h->plan.c_str() : ""; }

void sfxc_gpu_control_close(sfxc_gpu_control *h) { delete h; }

// ---- batches: the next integration of several jobs in one CUDA graph
struct sfxc_gpu_batch {
  std::vector<sfxc_gpu_ctx *> ctx;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr;
  std::vector<cudaEvent_t> join;
  float last_ms = 0.f;
  float host_ms[4] = {};  // the last run: planning, graph capture and update, launch to completion, outputs
  std::string err;
};

sfxc_gpu_batch *sfxc_gpu_batch_create(sfxc_gpu_ctx *const *ctxs, int32_t n) {
  try {
    if (!ctxs || n <= 0) throw Error(SFXC_GPU_EINVAL, "no contexts");
    std::unique_ptr<sfxc_gpu_batch> b(new sfxc_gpu_batch());
    for (int i = 0; i < n; i++) {
      if (!ctxs[i]) throw Error(SFXC_GPU_EINVAL, "null context");
      for (sfxc_gpu_ctx *o : b->ctx)
        if (o == ctxs[i]) throw Error(SFXC_GPU_EINVAL, "a context appears twice");
      if (i > 0 && ctxs[i]->device != ctxs[0]->device) throw Error(SFXC_GPU_EINVAL, "contexts on different devices");
      b->ctx.push_back(ctxs[i]);
    }
    b->device = ctxs[0]->device;
    CK(cudaSetDevice(b->device));
    CK(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b->e0));
    CK(cudaEventCreate(&b->e1));
    CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->join.resize(n);
    for (auto &e : b->join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return b.release();
  } catch (const Error &e) {
    g_error = e.msg;
    return nullptr;
  }
}

void sfxc_gpu_batch_destroy(sfxc_gpu_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->origin) cudaStreamSynchronize(b->origin);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (cudaEvent_t e : {b->e0, b->e1, b->fork})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
}

int sfxc_gpu_batch_run_counts(sfxc_gpu_batch *b, const int32_t *counts, sfxc_output_sink sink, void *const *users) {
  if (!b) return SFXC_GPU_EINVAL;
  size_t i = 0;
  const size_t n = b->ctx.size();
  std::vector<int> cnt(n, 1);
  try {
    if (counts)
      for (size_t k = 0; k < n; k++) {
        if (counts[k] < 0) throw Error(SFXC_GPU_EINVAL, "negative integration count");
        cnt[k] = counts[k];
      }
    CK(cudaSetDevice(b->device));
    for (size_t k = 0; k < n; k++) {
      sfxc_gpu_ctx *c = b->ctx[k];
      if (!cnt[k]) continue;
      if (!c->have_job) throw Error(SFXC_GPU_ESTATE, "a context of the batch has no parameters set");
      for (const StreamCtx &s : c->sc)
        if (!s.pushed) throw Error(SFXC_GPU_ESTATE, "a stream of the batch has no input for this integration");
    }
    // host planning of every integration of every job, its device work
    // recorded and its upload payloads staged in pinned memory: nothing
    // below allocates.  A job's later integrations take their input from the
    // bytes pushed beyond the first one's.  A buffer that grows for a later
    // integration keeps its old allocation (earlier work refers to it) until
    // the batch has run.
    struct Retire {
      std::vector<void *> list;
      Retire() { g_retired = &list; }
      ~Retire() {
        g_retired = nullptr;
        for (void *p : list) cudaFree(p);
      }
    } retire;
    using clock = std::chrono::steady_clock;
    auto ms_since = [](clock::time_point t) {
      return std::chrono::duration<float, std::milli>(clock::now() - t).count();
    };
    clock::time_point t0 = clock::now();
    {
      // the jobs planned at the same time, one host thread per context (a
      // job's integrations in order); each thread keeps its own list of
      // grown buffers, taken over by the batch's
      std::vector<std::vector<void *>> grown(n);
      std::vector<int> codes(n, SFXC_GPU_OK);
      std::vector<std::string> msgs(n);
      auto plan_job = [&](size_t k) {
        g_retired = &grown[k];
        try {
          CK(cudaSetDevice(b->device));
          for (int j = 0; j < cnt[k]; j++) {
            enqueue_integration(b->ctx[k], j, j == 0);
            stage_ops(b->ctx[k], j);
          }
        } catch (const Error &e) {
          codes[k] = e.code;
          msgs[k] = e.msg;
        } catch (const std::exception &e) {
          codes[k] = SFXC_GPU_ESTATE;
          msgs[k] = e.what();
        }
        g_retired = nullptr;
      };
      std::vector<std::thread> threads;
      for (size_t k = 0; k < n; k++)
        if (cnt[k]) threads.emplace_back(plan_job, k);
      for (std::thread &t : threads) t.join();
      for (auto &l : grown) retire.list.insert(retire.list.end(), l.begin(), l.end());
      for (size_t k = 0; k < n; k++)
        if (codes[k] != SFXC_GPU_OK) {
          i = k;
          throw Error(codes[k], msgs[k]);
        }
    }
    b->host_ms[0] = ms_since(t0);
    t0 = clock::now();
    g_retired = nullptr;  // nothing is allocated below; what grew is freed when the batch returns
    // all of it captured into one graph: each job on its own streams, its
    // integrations in order, forked from and joined back into the batch's
    // stream
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed));
    try {
      CK(cudaEventRecord(b->fork, b->origin));
      for (size_t k = 0; k < n; k++) {
        if (!cnt[k]) continue;
        sfxc_gpu_ctx *c = b->ctx[k];
        CK(cudaStreamWaitEvent(c->st, b->fork, 0));
        for (int j = 0; j < cnt[k]; j++) run_ops(c, j);
        CK(cudaEventRecord(b->join[k], c->st));
        CK(cudaStreamWaitEvent(b->origin, b->join[k], 0));
      }
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(b->origin, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    CK(cudaStreamEndCapture(b->origin, &graph));
    // the previous executable graph takes the new node parameters when the
    // topology is the same; else instantiate anew
    bool updated = false;
    if (b->exec) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(b->exec, graph, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
      }
    }
    if (!updated) {
      const cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        throw CudaError(e, "cudaGraphInstantiate");
      }
    }
    cudaGraphDestroy(graph);
    b->host_ms[1] = ms_since(t0);
    t0 = clock::now();
    CK(cudaEventRecord(b->e0, b->origin));
    CK(cudaGraphLaunch(b->exec, b->origin));
    CK(cudaEventRecord(b->e1, b->origin));
    CK(cudaStreamSynchronize(b->origin));
    CK(cudaEventElapsedTime(&b->last_ms, b->e0, b->e1));
    b->host_ms[2] = ms_since(t0);
    t0 = clock::now();
    // every job's output bytes made side by side (one host thread per
    // context, its integrations in order), then handed to the sink in job
    // order as one thread would
    std::vector<std::vector<IntegrationOut>> outs(n);
    std::vector<std::exception_ptr> errs(n);
    {
      auto prepare_job = [&](int k) {
        try {
          CK(cudaSetDevice(b->ctx[k]->device));
          outs[k].resize(cnt[k]);
          for (int j = 0; j < cnt[k]; j++) prepare_outputs(b->ctx[k], j, outs[k][j]);
        } catch (...) {
          errs[k] = std::current_exception();
        }
      };
      std::vector<std::thread> threads;
      for (size_t k = 0; k < n; k++)
        if (cnt[k]) threads.emplace_back(prepare_job, (int)k);
      for (std::thread &t : threads) t.join();
    }
    for (i = 0; i < n; i++)
      if (errs[i]) std::rethrow_exception(errs[i]);
    for (i = 0; i < n; i++)
      for (int j = 0; j < cnt[i]; j++) deliver_outputs(outs[i][j], sink, users ? users[i] : nullptr);
    b->host_ms[3] = ms_since(t0);
    return SFXC_GPU_OK;
  } catch (const Error &e) {
    b->err = e.msg;
    g_error = e.msg;
    if (i < n) b->ctx[i]->err = e.msg;
    for (sfxc_gpu_ctx *c : b->ctx) c->planned_integration = c->current_integration;
    return e.code;
  }
}

int sfxc_gpu_batch_run(sfxc_gpu_batch *b, sfxc_output_sink sink, void *const *users) {
  return sfxc_gpu_batch_run_counts(b, nullptr, sink, users);
}

float sfxc_gpu_batch_last_ms(const sfxc_gpu_batch *b) { return b ? b->last_ms : 0.f; }

int sfxc_gpu_batch_last_host_ms(const sfxc_gpu_batch *b, float *out4) {
  if (!b || !out4) return SFXC_GPU_EINVAL;
  for (int k = 0; k < 4; k++) out4[k] = b->host_ms[k];
  return SFXC_GPU_OK;
}

}  // extern "C"
