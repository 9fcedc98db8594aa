// Checker harness: drives the REFERENCE's own correlator-node classes
// (compiled from the reference sources by oracle/build_ref.py) on one job and
// writes their outputs to files.  Test infrastructure only: it generates the
// golden fixtures under tests/golden/ and pins the C restatement in
// oracle/sfxc_oracle.c.  Nothing in the product links or runs it.
//
// Modes
//   correlate <job> <outdir>  Bit2float_worker -> Delay_correction ->
//                             Correlation_core(_pulsar), wired as in
//                             Correlator_node::hook_added_data_reader
//                             (sfxc/src/correlator_node.cc:213-249) and polled
//                             as in Correlator_node::correlate (263-296).
//   delays <job> <outfile>    Input_node_tasklet::get_delay/get_delays as
//                             called by add_time_interval
//                             (sfxc/src/input_node_tasklet.cc:103-128,235-282).
//   protocol <job> <outfile>  Input_node_data_writer::do_task producing the
//                             correlator-node byte protocol
//                             (sfxc/src/input_node_data_writer.cc:107-229).
//   extract <job> <outfile>   Channel_extractor_5 (sfxc/src/channel_extractor_5.cc).
//
// Job files are "key value..." text lines (written by tests/golden/make_golden.py
// and oracle/refrun.py).
#define private public
#define protected public
#include "bit2float_worker.h"
#include "bit_statistics.h"
#include "channel_extractor_5.h"
#include "control_parameters.h"
#include "correlation_core.h"
#include "correlation_core_phased.h"
#include "correlation_core_pulsar.h"
#include "correlator_node_types.h"
#include "data_writer.h"
#include "delay_correction.h"
#include "delay_table_akima.h"
#include "input_node_data_writer.h"
#include "input_node_tasklet.h"
#include "data_reader_file.h"
#include "input_data_format_reader_tasklet.h"
#include "uvw_model.h"
#include "mark5b_reader.h"
#include "vdif_reader.h"
#undef private
#undef protected

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <sstream>
#include <set>
#include <algorithm>
#include <string>
#include <vector>

struct ShimMessage {
  int tag;
  std::vector<char> bytes;
};
extern std::vector<ShimMessage> g_shim_messages;

typedef std::map<std::string, std::vector<std::string> > Kv;

static void die(const std::string &m) {
  std::fprintf(stderr, "ref_harness: %s\n", m.c_str());
  std::exit(2);
}

// Reads "key v1 v2 ..." lines.  Repeated keys get an index suffix "#k".
static Kv read_job(const char *path) {
  std::ifstream in(path);
  if (!in) die(std::string("cannot open ") + path);
  Kv kv;
  std::map<std::string, int> count;
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ss(line);
    std::string key, v;
    ss >> key;
    std::vector<std::string> vals;
    while (ss >> v) vals.push_back(v);
    std::ostringstream k2;
    k2 << key << "#" << count[key]++;
    kv[k2.str()] = vals;
    if (count[key] == 1) kv[key] = vals;
  }
  return kv;
}

static const std::vector<std::string> &get(const Kv &kv, const std::string &k) {
  Kv::const_iterator it = kv.find(k);
  if (it == kv.end()) die("missing key " + k);
  return it->second;
}
static int geti(const Kv &kv, const std::string &k, int i = 0) { return std::atoi(get(kv, k)[i].c_str()); }
static long long getll(const Kv &kv, const std::string &k, int i = 0) { return std::atoll(get(kv, k)[i].c_str()); }
static double getd(const Kv &kv, const std::string &k, int i = 0) { return std::strtod(get(kv, k)[i].c_str(), 0); }
static bool has(const Kv &kv, const std::string &k) { return kv.find(k) != kv.end(); }
static int count_key(const Kv &kv, const std::string &k) {
  int n = 0;
  while (true) {
    std::ostringstream s;
    s << k << "#" << n;
    if (!has(kv, s.str())) return n;
    n++;
  }
}
static std::string idx(const std::string &k, int i) {
  std::ostringstream s;
  s << k << "#" << i;
  return s.str();
}

static std::vector<char> read_file(const std::string &path) {
  std::ifstream in(path.c_str(), std::ios::binary);
  if (!in) die("cannot open " + path);
  return std::vector<char>((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}
static void write_file(const std::string &path, const void *p, size_t n) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) die("cannot write " + path);
  if (n) std::fwrite(p, 1, n, f);
  std::fclose(f);
}

// Time from "ticks" (int64 clock ticks at 512 MHz since MJD 51544).
static Time ticks_time(long long ticks) {
  Time t;
  t.set_clock_ticks(ticks);
  return t;
}

class Memory_writer : public Data_writer {
 public:
  std::vector<char> bytes;
  bool can_write() { return true; }

 private:
  size_t do_put_bytes(size_t n, const char *buf) {
    bytes.insert(bytes.end(), buf, buf + n);
    return n;
  }
};

// Builds a Delay_table for one station: job keys "delfile#k", optional
// "clock#k offset rate epoch_ticks".
static Delay_table load_delay_table(const Kv &kv, int st) {
  Delay_table t;
  t.open(get(kv, idx("delfile", st))[0].c_str());
  if (has(kv, idx("clock", st))) {
    const std::vector<std::string> &c = get(kv, idx("clock", st));
    t.set_clock_offset(std::strtod(c[0].c_str(), 0), Time(), std::strtod(c[1].c_str(), 0),
                       ticks_time(std::atoll(c[2].c_str())));
  }
  return t;
}

// ---------------------------------------------------------------- delays ---
static int mode_delays(const Kv &kv, const char *outfile) {
  Delay_table table = load_delay_table(kv, 0);
  long long start_ticks = getll(kv, "start_ticks");
  long long stop_ticks = getll(kv, "stop_ticks");
  int sample_rate = geti(kv, "sample_rate");
  int bps = geti(kv, "bits_per_sample");

  // The tasklet is only used for its delay members; its reader/writer
  // members are never touched by get_delay/get_delays.
  void *mem = std::calloc(1, sizeof(Input_node_tasklet));
  Input_node_tasklet *t = static_cast<Input_node_tasklet *>(mem);
  new (&t->delay_table) Delay_table();
  new (&t->akima_delays) Delay_table_akima();
  t->delay_table.add_scans(table);
  t->sample_rate = sample_rate;
  t->bits_per_sample = bps;

  Time start_time = ticks_time(start_ticks), stop_time = ticks_time(stop_ticks);
  // add_time_interval (sfxc/src/input_node_tasklet.cc:103-115)
  t->akima_delays = t->delay_table.create_akima_spline(start_time, stop_time - start_time);
  std::vector<Delay> list;
  list.push_back(t->get_delay(start_time));
  start_time.set_sample_rate(sample_rate);
  stop_time.set_sample_rate(sample_rate);
  int64_t nsamples = stop_time.diff_samples(start_time);
  t->get_delays(start_time, nsamples, list);

  FILE *f = std::fopen(outfile, "w");
  for (size_t i = 0; i < list.size(); i++)
    std::fprintf(f, "%lld %d %d\n", (long long)list[i].time.get_clock_ticks(), list[i].bytes,
                 list[i].remaining_samples);
  // Also record spline evaluations at requested probe times (delay, rate, phase, amplitude).
  int np = count_key(kv, "probe");
  for (int i = 0; i < np; i++) {
    Time pt = ticks_time(getll(kv, idx("probe", i)));
    std::fprintf(f, "P %lld %.17g %.17g %.17g %.17g\n", (long long)pt.get_clock_ticks(),
                 t->akima_delays.delay(pt), t->akima_delays.rate(pt), t->akima_delays.phase(pt),
                 t->akima_delays.amplitude(pt));
  }
  std::fclose(f);
  return 0;
}

// -------------------------------------------------------------- protocol ---
// Input_node_data_writer over in-memory channel blocks.
//   sample_rate, bits_per_sample, integr_time_us, station_number
//   [channel_params <sideband> <polarisation> <frequency number>]
//   blockfile <path> ; blocks "block#k start_ticks offset size [inv_begin n]..."
//   delays <path to delay list from mode_delays>
//   slice#k start_ticks stop_ticks nr_samples
static int mode_protocol(const Kv &kv, const char *outfile) {
  Input_node_parameters param;
  int sample_rate = geti(kv, "sample_rate");
  int bps = geti(kv, "bits_per_sample");
  param.integr_time = Time((double)geti(kv, "integr_time_us"));
  param.phasecal_integr_time = Time();
  Input_node_parameters::Channel_parameters ch;
  ch.bits_per_sample = bps;
  ch.sideband = 'U';
  ch.polarisation = 'R';
  ch.frequency_number = 0;
  if (has(kv, "channel_params")) {  // sideband, polarisation, frequency number of the phase-cal messages
    const std::vector<std::string> &c = get(kv, "channel_params");
    ch.sideband = c[0][0];
    ch.polarisation = c[1][0];
    ch.frequency_number = std::atoi(c[2].c_str());
  }
  for (int b = 0; b < bps; b++) ch.tracks.push_back(b);
  param.channels.push_back(ch);
  param.track_bit_rate = sample_rate;  // sample_rate() = track_bit_rate * subsamples_per_sample
  param.n_tracks = bps;
  param.frame_size = -1;
  // phase-cal extraction (Input_node_data_writer::do_phasecal): its messages
  // (MPI_TAG_OUTPUT_NODE_WRITE_PHASECAL) are written after the slices
  param.phasecal_integr_time = ticks_time(has(kv, "phasecal_ticks") ? getll(kv, "phasecal_ticks") : 0);
  if (param.sample_rate() != sample_rate || param.bits_per_sample() != bps)
    die("Input_node_parameters accessors disagree with the job");

  Input_node_data_writer &w = *new Input_node_data_writer();
  Input_node_data_writer::Input_buffer_ptr q(new Input_node_data_writer::Input_buffer());
  w.connect_to(q);
  w.set_parameters(0, param, geti(kv, "station_number"));

  std::vector<char> data = read_file(get(kv, "blockfile")[0]);
  // Pools are leaked on purpose: the reference pools assert at destruction
  // that every element came back, and the writer still holds some at exit.
  Input_node_types::Data_memory_pool &pool = *new Input_node_types::Data_memory_pool(count_key(kv, "block") + 4);
  int nb = count_key(kv, "block");
  for (int b = 0; b < nb; b++) {
    const std::vector<std::string> &v = get(kv, idx("block", b));
    Input_node_types::Channel_buffer_element e;
    e.start_time = ticks_time(std::atoll(v[0].c_str()));
    size_t off = std::atoll(v[1].c_str()), size = std::atoll(v[2].c_str());
    e.channel_data = pool.allocate();
    e.channel_data.data().data.assign(data.begin() + off, data.begin() + off + size);
    for (size_t k = 3; k + 1 < v.size(); k += 2) {
      Input_node_types::Invalid_block ib;
      ib.invalid_begin = std::atoi(v[k].c_str());
      ib.nr_invalid = std::atoi(v[k + 1].c_str());
      e.invalid.push_back(ib);
    }
    q->push(e);
  }

  Delay_memory_pool &dpool = *new Delay_memory_pool(count_key(kv, "slice") + 2);
  std::vector<boost::shared_ptr<Memory_writer> > writers;
  int ns = count_key(kv, "slice");
  for (int s = 0; s < ns; s++) {
    const std::vector<std::string> &v = get(kv, idx("slice", s));
    Time start = ticks_time(std::atoll(v[0].c_str())), stop = ticks_time(std::atoll(v[1].c_str()));
    // Delay list for this slice: "dlist#s" file from mode_delays
    std::ifstream din(get(kv, idx("dlist", s))[0].c_str());
    Delay_memory_pool_element de = dpool.allocate();
    de.data().resize(0);
    std::string line;
    while (std::getline(din, line)) {
      if (line.empty() || line[0] == 'P') continue;
      std::istringstream ss(line);
      long long tk;
      Delay d;
      ss >> tk >> d.bytes >> d.remaining_samples;
      d.time = ticks_time(tk);
      d.time.set_sample_rate(sample_rate);
      de.data().push_back(d);
    }
    start.set_sample_rate(sample_rate);
    stop.set_sample_rate(sample_rate);
    w.add_delay(de);
    w.add_time_interval(start, stop);
    boost::shared_ptr<Memory_writer> mw(new Memory_writer());
    writers.push_back(mw);
    w.add_timeslice(mw, std::atoll(v[2].c_str()));
  }
  int guard = 0;
  while (w.has_work()) {
    w.do_task();
    if (++guard > 100000000) die("protocol writer did not terminate");
  }
  std::vector<char> all;
  FILE *f = std::fopen(outfile, "wb");
  for (size_t s = 0; s < writers.size(); s++) {
    uint64_t n = writers[s]->bytes.size();
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(&writers[s]->bytes[0], 1, n, f);
  }
  std::fclose(f);
  if (has(kv, "phasecal_out")) {
    FILE *pf = std::fopen(get(kv, "phasecal_out")[0].c_str(), "wb");
    for (size_t m = 0; m < g_shim_messages.size(); m++)
      std::fwrite(&g_shim_messages[m].bytes[0], 1, g_shim_messages[m].bytes.size(), pf);
    std::fclose(pf);
    g_shim_messages.clear();
  }
  return 0;
}

// --------------------------------------------------------------- extract ---
//   word_bytes N, bits_per_sample, nsamples, infile, subband#k track...
static int mode_extract(const Kv &kv, const char *outfile) {
  int N = geti(kv, "word_bytes");
  int bps = geti(kv, "bits_per_sample");
  int nsamples = geti(kv, "nsamples");
  std::vector<char> in = read_file(get(kv, "infile")[0]);
  std::vector<std::vector<int> > tracks;
  int nsub = count_key(kv, "subband");
  for (int s = 0; s < nsub; s++) {
    const std::vector<std::string> &v = get(kv, idx("subband", s));
    std::vector<int> t;
    for (size_t k = 0; k < v.size(); k++) t.push_back(std::atoi(v[k].c_str()));
    tracks.push_back(t);
  }
  int fan_out = tracks[0].size();
  if ((int)in.size() < nsamples * N) die("extract input too short");
  Channel_extractor_5 ex;
  ex.initialise(tracks, N, nsamples, bps);
  std::vector<std::vector<unsigned char> > out(nsub, std::vector<unsigned char>(nsamples * fan_out / 8 + 8));
  std::vector<unsigned char *> ptrs(nsub);
  for (int s = 0; s < nsub; s++) ptrs[s] = &out[s][0];
  ex.extract((unsigned char *)&in[0], &ptrs[0]);
  FILE *f = std::fopen(outfile, "wb");
  for (int s = 0; s < nsub; s++) std::fwrite(&out[s][0], 1, nsamples * fan_out / 8, f);
  std::fclose(f);
  return 0;
}

// ------------------------------------------------------------- correlate ---
struct Stream_chain {
  bit_statistics_ptr stats;
  Correlator_node_types::Channel_circular_input_buffer *ring;
  Bit2float_worker_sptr b2f;
  Correlator_node_types::Channel_queue_ptr b2f_to_dc;  // harness tap between the stages
  boost::shared_ptr<Delay_correction> dc;
  Delay_correction::Output_buffer_ptr dc_to_core;
  std::vector<char> protocol;
  size_t protocol_pos;
  std::vector<float> unpacked;          // all bit2float output of the current integration
  std::vector<std::complex<float> > rows;  // all Delay_correction rows (stride M+4)
};

static void push_bytes(Correlator_node_types::Channel_circular_input_buffer *r, const char *p, size_t n) {
  if (n > r->bytes_free()) die("protocol larger than the correlator-node ring buffer");
  for (size_t i = 0; i < n; i++) r->data[(r->write + i) % r->size] = p[i];
  r->write += n;
}

static int mode_correlate(const Kv &kv, const char *outdir) {
  const int nstreams = count_key(kv, "stream");
  const int nstations = count_key(kv, "delfile");
  const bool dump = has(kv, "dump") && geti(kv, "dump") != 0;
  const int n_int = geti(kv, "n_integrations");
  const int M = geti(kv, "fft_size_correlation");

  std::vector<Delay_table> tables;
  for (int s = 0; s < nstations; s++) tables.push_back(load_delay_table(kv, s));

  Correlation_parameters p;
  p.experiment_start = ticks_time(getll(kv, "experiment_start_ticks"));
  p.integration_time = Time((double)getll(kv, "integration_time_us"));
  p.sub_integration_time = Time((double)getll(kv, "sub_integration_time_us"));
  p.number_channels = geti(kv, "number_channels");
  p.fft_size_delaycor = geti(kv, "fft_size_delaycor");
  p.fft_size_correlation = M;
  p.slice_offset = 1;
  p.sample_rate = geti(kv, "sample_rate");
  p.channel_freq = getll(kv, "channel_freq");
  p.bandwidth = geti(kv, "bandwidth");
  p.sideband = get(kv, "sideband")[0][0];
  p.frequency_nr = geti(kv, "frequency_nr");
  p.polarisation = get(kv, "polarisation")[0][0];
  p.cross_polarize = geti(kv, "cross_polarize") != 0;
  p.reference_station = geti(kv, "reference_station");
  p.window = geti(kv, "window");
  std::memset(p.source, 0, sizeof(p.source));
  std::strncpy(p.source, get(kv, "source")[0].c_str(), 10);
  p.n_phase_centers = has(kv, "n_phase_centers") ? geti(kv, "n_phase_centers") : 1;
  // the pulsar core for a pulsar source; pulsar mode for any other source of
  // a pulsar-binning run (Correlator_node::set_parameters,
  // sfxc/src/correlator_node.cc:351-361): the normal core, file index 1
  const bool pulsar_core = has(kv, "pulsar");
  p.pulsar_binning = pulsar_core || (has(kv, "pulsar_mode") && geti(kv, "pulsar_mode") != 0) ? 1 : 0;
  p.pulsar_parameters = 0;
  p.mask_parameters = 0;
  // Mask_parameters of the ctrl file: float32 files of the mask (M + 1) and
  // the lag window (2 number_channels), and the normalisation flag
  Mask_parameters mask_params;
  if (has(kv, "mask_normalize") || has(kv, "mask") || has(kv, "lag_window")) {
    mask_params.normalize = has(kv, "mask_normalize") && geti(kv, "mask_normalize") != 0;
    if (has(kv, "mask")) {
      const std::vector<char> b = read_file(get(kv, "mask")[0]);
      for (size_t q = 0; q + 4 <= b.size(); q += 4) {
        float v;
        std::memcpy(&v, &b[q], 4);
        mask_params.mask.push_back(v);
      }
    }
    if (has(kv, "lag_window")) {
      const std::vector<char> b = read_file(get(kv, "lag_window")[0]);
      for (size_t q = 0; q + 4 <= b.size(); q += 4) {
        float v;
        std::memcpy(&v, &b[q], 4);
        mask_params.window.push_back(v);
      }
    }
    p.mask_parameters = &mask_params;
  }
  std::vector<int> stream_station_index;  // delay table per stream
  for (int i = 0; i < nstreams; i++) {
    const std::vector<std::string> &v = get(kv, idx("stream", i));
    // station_number station_stream sample_rate channel_freq bandwidth sideband pol bps LO_offset tsys_freq table_index
    Correlation_parameters::Station_parameters sp;
    sp.station_number = std::atoi(v[0].c_str());
    sp.station_stream = std::atoi(v[1].c_str());
    sp.sample_rate = std::atoi(v[2].c_str());
    sp.channel_freq = std::atoll(v[3].c_str());
    sp.bandwidth = std::atoi(v[4].c_str());
    sp.sideband = v[5][0];
    sp.polarisation = v[6][0];
    sp.bits_per_sample = std::atoi(v[7].c_str());
    sp.LO_offset = std::strtod(v[8].c_str(), 0);
    sp.tsys_freq = std::atoi(v[9].c_str());
    stream_station_index.push_back(std::atoi(v[10].c_str()));
    p.station_streams.push_back(sp);
  }

  Pulsar_parameters::Pulsar pulsar;
  if (pulsar_core) {
    const std::vector<std::string> &v = get(kv, "pulsar");  // nbins gate_start gate_stop
    std::memset(pulsar.name, 0, sizeof(pulsar.name));
    std::strncpy(pulsar.name, p.source, 10);
    pulsar.nbins = std::atoi(v[0].c_str());
    pulsar.interval.start = std::strtod(v[1].c_str(), 0);
    pulsar.interval.stop = std::strtod(v[2].c_str(), 0);
    int npc = count_key(kv, "polyco");
    for (int k = 0; k < npc; k++) {
      // tmid DM ref_phase ref_freq obs_freq coef...
      const std::vector<std::string> &c = get(kv, idx("polyco", k));
      Pulsar_parameters::Polyco_params pp;
      std::memset(&pp, 0, (char *)&pp.coef - (char *)&pp);
      pp.tmid = std::strtod(c[0].c_str(), 0);
      pp.DM = std::strtod(c[1].c_str(), 0);
      pp.ref_phase = std::strtod(c[2].c_str(), 0);
      pp.ref_freq = std::strtod(c[3].c_str(), 0);
      pp.obs_freq = std::strtod(c[4].c_str(), 0);
      for (size_t j = 5; j < c.size(); j++) pp.coef.push_back(std::strtod(c[j].c_str(), 0));
      pp.n_coef = pp.coef.size();
      pulsar.polyco_params.push_back(pp);
    }
  }

  // Build the per-stream chains (Correlator_node::hook_added_data_reader).
  int max_stream = 0;
  for (int i = 0; i < nstreams; i++) max_stream = std::max(max_stream, (int)p.station_streams[i].station_stream);
  std::vector<Stream_chain> chains(max_stream + 1);
  // Correlator_node::Correlator_node (sfxc/src/correlator_node.cc:37-38): the phased-array core
  boost::shared_ptr<Correlation_core> core_normal(has(kv, "phased_array") && geti(kv, "phased_array") != 0
                                                      ? (Correlation_core *)new Correlation_core_phased()
                                                      : new Correlation_core());
  boost::shared_ptr<Correlation_core_pulsar> core_pulsar(new Correlation_core_pulsar());
  Correlation_core *core = pulsar_core ? (Correlation_core *)core_pulsar.get() : core_normal.get();
  // the manager's source list of a multiple-phase-centre run
  // (correlator_node_controller.cc:76-82): each centre's output then carries
  // its source's place in the list as file index (correlation_core.cc:55-58)
  if (has(kv, "source_list")) {
    const std::vector<std::string> &v = get(kv, "source_list");
    std::map<std::string, int> m;
    for (size_t q = 0; q < v.size(); q++) m[v[q]] = (int)q;
    core_normal->add_source_list(m);
  }
  boost::shared_ptr<Memory_writer> out(new Memory_writer());
  core->set_data_writer(out);
  const size_t ring_size = has(kv, "ring_bytes") ? (size_t)getll(kv, "ring_bytes") : (size_t)37100000;
  for (int i = 0; i < nstreams; i++) {
    int s = p.station_streams[i].station_stream;
    Stream_chain &c = chains[s];
    c.stats = bit_statistics_ptr(new bit_statistics());
    c.ring = new Correlator_node_types::Channel_circular_input_buffer(ring_size);
    c.b2f = Bit2float_worker::new_sptr(s, c.stats);
    c.b2f->connect_to(c.ring);
    c.b2f_to_dc = Correlator_node_types::Channel_queue_ptr(new Correlator_node_types::Channel_queue());
    c.dc = boost::shared_ptr<Delay_correction>(new Delay_correction(s));
    c.dc->connect_to(c.b2f_to_dc);
    c.dc_to_core = Delay_correction::Output_buffer_ptr(new Delay_correction::Output_buffer());
    core->connect_to(s, c.stats, c.dc_to_core);
    core->connect_to(s, c.b2f->get_invalid());
    c.protocol = read_file(get(kv, idx("protocol", i))[0]);
    c.protocol_pos = 0;
  }

  // UVW per integration, stream (job order) and phase centre: float64 file
  std::vector<double> uvw_in;
  if (has(kv, "uvw")) {
    const std::vector<char> b = read_file(get(kv, "uvw")[0]);
    uvw_in.resize(b.size() / sizeof(double));
    if (!uvw_in.empty()) std::memcpy(&uvw_in[0], &b[0], uvw_in.size() * sizeof(double));
    if (uvw_in.size() < (size_t)n_int * nstreams * 3 * p.n_phase_centers) die("uvw file too short");
  }
  std::string od(outdir);
  FILE *tsys_f = std::fopen((od + "/tsys.bin").c_str(), "wb");
  FILE *stats_f = std::fopen((od + "/stats.txt").c_str(), "w");
  for (int it = 0; it < n_int; it++) {
    p.integration_nr = geti(kv, "integration_nr") + it;
    p.slice_nr = p.integration_nr;
    p.start_time = ticks_time(getll(kv, "start_ticks") + (long long)it * p.integration_time.get_clock_ticks());
    p.stop_time = p.start_time + p.integration_time;
    for (int i = 0; i < nstreams; i++) {
      p.station_streams[i].start_time = p.start_time;
      p.station_streams[i].stop_time = p.stop_time;
    }
    // Correlator_node::set_parameters (sfxc/src/correlator_node.cc:311-406)
    std::vector<Delay_table_akima> akima(max_stream + 1);
    std::vector<std::vector<double> > uvw(max_stream + 1, std::vector<double>(3 * p.n_phase_centers, 0.0));
    for (int i = 0; i < nstreams; i++) {
      int s = p.station_streams[i].station_stream;
      akima[s] = tables[stream_station_index[i]].create_akima_spline(p.start_time, p.integration_time);
      // the UVW model's values at the integration's mid-time, as given by the job
      if (!uvw_in.empty())
        for (int q = 0; q < 3 * p.n_phase_centers; q++)
          uvw[s][q] = uvw_in[((size_t)it * nstreams + i) * 3 * p.n_phase_centers + q];
    }
    if (pulsar_core)
      core_pulsar->set_parameters(p, pulsar, akima, uvw, 0);
    else
      core_normal->set_parameters(p, akima, uvw, 0);
    for (int i = 0; i < nstreams; i++) {
      int s = p.station_streams[i].station_stream;
      chains[s].dc->set_parameters(p, akima[s]);
      chains[s].b2f->set_new_parameters(p, akima[s]);
      chains[s].unpacked.clear();
      chains[s].rows.clear();
    }
    // Feed this integration's protocol (length-prefixed per integration).
    for (int i = 0; i < nstreams; i++) {
      int s = p.station_streams[i].station_stream;
      Stream_chain &c = chains[s];
      if (c.protocol_pos + 8 > c.protocol.size()) die("protocol file exhausted");
      uint64_t n;
      std::memcpy(&n, &c.protocol[c.protocol_pos], 8);
      c.protocol_pos += 8;
      push_bytes(c.ring, &c.protocol[c.protocol_pos], n);
      c.protocol_pos += n;
    }
    // Poll like the bit2float thread + main thread (single-threaded).
    long guard = 0;
    while (!core->finished()) {
      bool work = false;
      for (int i = 0; i < nstreams; i++) {
        Stream_chain &c = chains[p.station_streams[i].station_stream];
        while (c.b2f->has_work()) {
          c.b2f->do_task();
          work = true;
        }
        // Tap: copy bit2float output, then hand the element to Delay_correction.
        Correlator_node_types::Channel_queue_ptr src = c.b2f->get_output_buffer();
        while (!src->empty()) {
          Correlator_node_types::Channel_memory_pool_element e = src->front_and_pop();
          if (dump) c.unpacked.insert(c.unpacked.end(), &e.data().data[0], &e.data().data[0] + e.data().data.size());
          c.b2f_to_dc->push(e);
        }
        while (c.dc->has_work()) {
          c.dc->do_task();
          work = true;
        }
        Delay_correction::Output_buffer_ptr dsrc = c.dc->get_output_buffer();
        while (!dsrc->empty()) {
          Delay_correction::Output_buffer_element e = dsrc->front_and_pop();
          if (dump) c.rows.insert(c.rows.end(), &e->data[0], &e->data[0] + e->data.size());
          c.dc_to_core->push(e);
        }
      }
      while (core->has_work() && !core->finished()) {
        core->do_task();
        work = true;
      }
      if (!work && ++guard > 1000) die("pipeline stalled (protocol shorter than the integration?)");
    }
    // Statistics as the core saw them at integration end.
    for (int i = 0; i < nstreams; i++) {
      Stream_chain &c = chains[p.station_streams[i].station_stream];
      int *lv = c.stats->get_statistics();
      int *ts = c.stats->get_tsys();
      std::fprintf(stats_f, "%d %d %d %d %d %d %d %d %d %d %d\n", it, lv[0], lv[1], lv[2], lv[3], lv[4],
                   ts[0], ts[1], ts[2], ts[3], (int)c.b2f->get_invalid()->size());
      std::vector<Bit2float_worker::Invalid> *inv = c.b2f->get_invalid();
      for (size_t k = 0; k < inv->size(); k++)
        std::fprintf(stats_f, "I %d %d %d\n", i, (*inv)[k].start, (*inv)[k].n_invalid);
      if (dump) {
        std::ostringstream a, b;
        a << od << "/unpacked_i" << it << "_s" << i << ".f32";
        b << od << "/rows_i" << it << "_s" << i << ".c64";
        write_file(a.str(), c.unpacked.empty() ? 0 : &c.unpacked[0], c.unpacked.size() * 4);
        write_file(b.str(), c.rows.empty() ? 0 : &c.rows[0], c.rows.size() * 8);
      }
    }
    if (dump && pulsar_core) {
      // The reference's own bin table of this integration: dedisperse_buffer()
      // recomputed per FFT after the integration (its scratch buffer is zero,
      // so the accumulators are unchanged), plus its phase constants.
      std::ostringstream a;
      a << od << "/bins_i" << it << ".i32";
      FILE *bf = std::fopen(a.str().c_str(), "wb");
      const int nr = core_pulsar->number_ffts_in_integration;
      for (int r = 0; r < nr; r++) {
        core_pulsar->current_fft = r;
        core_pulsar->dedisperse_buffer();
        std::fwrite(&core_pulsar->bins[0], 4, core_pulsar->bins.size(), bf);
      }
      core_pulsar->current_fft = nr;
      std::fclose(bf);
      std::ostringstream b;
      b << od << "/pulsar_i" << it << ".txt";
      FILE *pf = std::fopen(b.str().c_str(), "w");
      std::fprintf(pf, "%.17g %.17g %.17g\n", core_pulsar->start_phase, core_pulsar->fft_duration,
                   p.start_time.get_mjd());
      for (size_t q = 0; q < core_pulsar->offsets.size(); q++) std::fprintf(pf, "%.17g\n", core_pulsar->offsets[q]);
      std::fclose(pf);
    }
    for (size_t m = 0; m < g_shim_messages.size(); m++)
      std::fwrite(&g_shim_messages[m].bytes[0], 1, g_shim_messages[m].bytes.size(), tsys_f);
    g_shim_messages.clear();
  }
  std::fclose(tsys_f);
  std::fclose(stats_f);
  write_file(od + "/out.cor", out->bytes.empty() ? 0 : &out->bytes[0], out->bytes.size());
  return 0;
}

// Format readers (VDIF_reader, Mark5b_reader, sfxc/src/vdif_reader.cc,
// sfxc/src/mark5b_reader.cc) over a file, as Input_data_format_reader_tasklet
// drives them: open_input_stream, then read_new_block with the frame's
// invalid list emptied in between.  Per block: channel, start ticks, payload
// size and invalid byte runs (blocks.txt); payloads back to back (data.bin).
//   format vdif|mark5b ; file <path> ; ref_ticks ; offset_ticks ;
//   track_bit_rate ; frame_size ; n_tracks ; bits ; channel#k <tracks...> ;
//   max_blocks
static int mode_reader(Kv &kv, const std::string &od) {
  Input_node_parameters p;
  p.track_bit_rate = geti(kv, "track_bit_rate");
  p.frame_size = geti(kv, "frame_size");
  p.n_tracks = geti(kv, "n_tracks");
  p.offset = ticks_time(getll(kv, "offset_ticks"));
  const int nch = count_key(kv, "channel");
  for (int c = 0; c < nch; c++) {
    Input_node_parameters::Channel_parameters cp;
    cp.bits_per_sample = geti(kv, "bits");
    const std::vector<std::string> &tr = get(kv, idx("channel", c));
    for (size_t k = 0; k < tr.size(); k++) cp.tracks.push_back(std::atoi(tr[k].c_str()));
    cp.sideband = 'U';
    cp.polarisation = 'R';
    cp.frequency_number = c;
    p.channels.push_back(cp);
  }
  boost::shared_ptr<Data_reader> dr(new Data_reader_file("file://" + get(kv, "file")[0]));
  Input_node_types::Data_memory_pool &pool = *new Input_node_types::Data_memory_pool(4);  // leaked, see above
  Input_data_format_reader::Data_frame data;
  data.buffer = pool.allocate();
  const Time ref = ticks_time(getll(kv, "ref_ticks"));
  const std::string fmt = get(kv, "format")[0];
  Input_data_format_reader *r;
  if (fmt == "vdif")
    r = new VDIF_reader(dr, data, ref);
  else if (fmt == "mark5b")
    r = new Mark5b_reader(dr, data, ref);
  else
    die("unknown format " + fmt);
  r->set_parameters(p);
  FILE *bf = std::fopen((od + "/blocks.txt").c_str(), "w");
  FILE *df = std::fopen((od + "/data.bin").c_str(), "wb");
  if (!bf || !df) die("cannot write reader output");
  const int maxb = geti(kv, "max_blocks");
  bool ok = r->open_input_stream(data);
  int n = 0;
  while (ok && n < maxb) {
    const std::vector<unsigned char> &b = data.buffer->data;
    std::fprintf(bf, "%d %lld %d", data.channel, (long long)data.start_time.get_clock_ticks(), (int)b.size());
    for (size_t k = 0; k < data.invalid.size(); k++)
      std::fprintf(bf, " %d %d", data.invalid[k].invalid_begin, data.invalid[k].nr_invalid);
    std::fprintf(bf, "\n");
    if (!b.empty()) std::fwrite(&b[0], 1, b.size(), df);
    n++;
    data.invalid.clear();
    ok = r->read_new_block(data);
  }
  std::fclose(bf);
  std::fclose(df);
  return 0;
}

// Readers that note, per data buffer, whether the last read into it
// succeeded (a failed read can leave part of a frame and older bytes there).
static std::map<const void *, bool> g_last_read_ok;
class Logged_vdif_reader : public VDIF_reader {
 public:
  Logged_vdif_reader(boost::shared_ptr<Data_reader> dr, Data_frame &d, Time ref) : VDIF_reader(dr, d, ref) {}
  bool read_new_block(Data_frame &d) {
    const bool ok = VDIF_reader::read_new_block(d);
    g_last_read_ok[&d.buffer->data] = ok;
    return ok;
  }
};
class Logged_mark5b_reader : public Mark5b_reader {
 public:
  Logged_mark5b_reader(boost::shared_ptr<Data_reader> dr, Data_frame &d, Time ref) : Mark5b_reader(dr, d, ref) {}
  bool read_new_block(Data_frame &d) {
    const bool ok = Mark5b_reader::read_new_block(d);
    g_last_read_ok[&d.buffer->data] = ok;
    return ok;
  }
};

// The reader tasklet (Input_data_format_reader_tasklet,
// sfxc/src/input_data_format_reader_tasklet.cc) over a file: the reader as in
// mode_reader, the tasklet given the job's time intervals (start, stop,
// leave ticks) and run to its end in this thread; per block it pushed:
// channel, start ticks, size, the number of its data buffer (blocks pushed
// with the same buffer share its bytes as they were last written), whether
// the buffer's bytes are not a block's (the last read into it failed, or
// none was made) and invalid runs (schedule.txt), payloads of blocks that
// are not wholly invalid back to back (data.bin).
//   as mode_reader, plus interval#k <start> <stop> <leave>
static int mode_schedule(Kv &kv, const std::string &od) {
  Input_node_parameters p;
  p.track_bit_rate = geti(kv, "track_bit_rate");
  p.frame_size = geti(kv, "frame_size");
  p.n_tracks = geti(kv, "n_tracks");
  p.offset = ticks_time(getll(kv, "offset_ticks"));
  p.data_modulation = 0;
  p.exit_on_empty_datastream = false;
  const int nch = count_key(kv, "channel");
  for (int c = 0; c < nch; c++) {
    Input_node_parameters::Channel_parameters cp;
    cp.bits_per_sample = geti(kv, "bits");
    const std::vector<std::string> &tr = get(kv, idx("channel", c));
    for (size_t k = 0; k < tr.size(); k++) cp.tracks.push_back(std::atoi(tr[k].c_str()));
    cp.sideband = 'U';
    cp.polarisation = 'R';
    cp.frequency_number = c;
    p.channels.push_back(cp);
  }
  boost::shared_ptr<Data_reader> dr(new Data_reader_file("file://" + get(kv, "file")[0]));
  // every pushed block stays in the output queue until the end: a pool large enough for all of them
  boost::shared_ptr<Input_node_types::Data_memory_pool> pool(new Input_node_types::Data_memory_pool(20000));
  Input_data_format_reader::Data_frame data;
  data.buffer = pool->allocate();
  const Time ref = ticks_time(getll(kv, "ref_ticks"));
  const std::string fmt = get(kv, "format")[0];
  boost::shared_ptr<Input_data_format_reader> r;
  if (fmt == "vdif")
    r.reset(new Logged_vdif_reader(dr, data, ref));
  else if (fmt == "mark5b")
    r.reset(new Logged_mark5b_reader(dr, data, ref));
  else
    die("unknown format " + fmt);
  r->set_parameters(p);
  Input_data_format_reader_tasklet t(r, pool);
  t.set_parameters(p);
  const int niv = count_key(kv, "interval");
  for (int k = 0; k < niv; k++) {
    const std::vector<std::string> &v = get(kv, idx("interval", k));
    Time a = ticks_time(std::atoll(v[0].c_str())), b = ticks_time(std::atoll(v[1].c_str())),
         c = ticks_time(std::atoll(v[2].c_str()));
    t.add_time_interval(a, b, c);
  }
  t.stop();
  t.do_execute();
  FILE *bf = std::fopen((od + "/schedule.txt").c_str(), "w");
  FILE *df = std::fopen((od + "/data.bin").c_str(), "wb");
  if (!bf || !df) die("cannot write schedule output");
  Input_node_types::Input_buffer_ptr q = t.get_output_buffer();
  std::map<const void *, int> buffers;
  while (!q->empty()) {
    Input_node_types::Input_data_frame &e = q->front();
    const std::vector<unsigned char> &b = e.buffer->data;
    const void *key = &b;
    if (!buffers.count(key)) {
      const int id = (int)buffers.size();
      buffers[key] = id;
    }
    const bool stale = !g_last_read_ok.count(key) || !g_last_read_ok[key];
    std::fprintf(bf, "%d %lld %d %d %d", e.channel, (long long)e.start_time.get_clock_ticks(), (int)b.size(),
                 buffers[key], stale ? 1 : 0);
    bool whole = false;
    for (size_t k = 0; k < e.invalid.size(); k++) {
      std::fprintf(bf, " %d %d", e.invalid[k].invalid_begin, e.invalid[k].nr_invalid);
      if (e.invalid[k].invalid_begin == 0 && e.invalid[k].nr_invalid >= (int)b.size()) whole = true;
    }
    std::fprintf(bf, "\n");
    if (!whole && !b.empty()) std::fwrite(&b[0], 1, b.size(), df);
    q->pop();
  }
  std::fclose(bf);
  std::fclose(df);
  return 0;
}

// The reference's UVW model (Uvw_model, sfxc/src/uvw_model.cc) of one .del
// file evaluated at probes, in order: u v w per line (%.17g).
//   delfile <path> ; probe#k <phase centre> <ticks>
static int mode_uvw(Kv &kv, const std::string &out) {
  Uvw_model m;
  m.open(get(kv, "delfile")[0].c_str());
  FILE *f = std::fopen(out.c_str(), "w");
  if (!f) die("cannot write " + out);
  const int np = count_key(kv, "probe");
  for (int k = 0; k < np; k++) {
    const std::vector<std::string> &v = get(kv, idx("probe", k));
    double u, vv, w;
    m.get_uvw(std::atoi(v[0].c_str()), ticks_time(std::atoll(v[1].c_str())), &u, &vv, &w);
    std::fprintf(f, "%.17g %.17g %.17g\n", u, vv, w);
  }
  std::fclose(f);
  return 0;
}

// ---- control: the reference's Control_parameters over a control file and a
// VEX file, with Manager_node's dealing of the jobs restated around it (the
// manager itself needs MPI).  Writes the plan as JSON in the form
// Json plan_json() of the library writes.
//   ctrl <path> ; vex <path> ; station_time#k <station> <scan> <ticks>

struct Jw {  // a small JSON writer
  std::string s;
  std::vector<int> count;  // items written so far in each open container
  bool after_key;
  Jw() : after_key(false) {}
  void pre() {
    if (after_key) {
      after_key = false;
      return;
    }
    if (!count.empty() && count.back()++) s += ",";
  }
  void key(const char *k) {
    if (!count.empty() && count.back()++) s += ",";
    s += "\"";
    s += k;
    s += "\":";
    after_key = true;
  }
  void val(const std::string &raw) {
    pre();
    s += raw;
  }
  void open(char c) {
    pre();
    s += c;
    count.push_back(0);
  }
  void close(char c) {
    count.pop_back();
    s += c;
  }
  void str(const std::string &v) {
    std::string q = "\"";
    for (size_t i = 0; i < v.size(); i++) {
      unsigned char c = v[i];
      if (c == '"' || c == '\\') {
        q += '\\';
        q += (char)c;
      } else if (c < 0x20) {
        char b[8];
        std::snprintf(b, sizeof b, "\\u%04x", c);
        q += b;
      } else {
        q += (char)c;
      }
    }
    val(q + "\"");
  }
  void num(long long v) {
    char b[32];
    std::snprintf(b, sizeof b, "%lld", v);
    val(b);
  }
  void dbl(double v) {
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", v);
    val(b);
  }
  void boolean(bool v) { val(v ? "true" : "false"); }
  void chr(char c) { str(c ? std::string(1, c) : std::string()); }
};

static void put_input(Jw &w, const Input_node_parameters &p, const std::string &fmt) {
  w.open('{');
  w.key("data_format"); w.str(fmt);
  w.key("n_tracks"); w.num(p.n_tracks);
  w.key("track_bit_rate"); w.num(p.track_bit_rate);
  w.key("frame_size"); w.num(p.frame_size);
  w.key("fft_size"); w.num(p.fft_size);
  w.key("data_modulation"); w.num(p.data_modulation);
  w.key("integr_time"); w.num(p.integr_time.get_clock_ticks());
  w.key("offset"); w.num(p.offset.get_clock_ticks());
  w.key("phasecal_integr_time"); w.num(p.phasecal_integr_time.get_clock_ticks());
  w.key("exit_on_empty_datastream"); w.boolean(p.exit_on_empty_datastream);
  w.key("channels");
  w.open('[');
  for (size_t i = 0; i < p.channels.size(); i++) {
    const Input_node_parameters::Channel_parameters &c = p.channels[i];
    w.open('{');
    w.key("bits_per_sample"); w.num(c.bits_per_sample);
    w.key("sideband"); w.chr(c.sideband);
    w.key("polarisation"); w.chr(c.polarisation);
    w.key("frequency_number"); w.num(c.frequency_number);
    w.key("tracks");
    w.open('[');
    for (size_t k = 0; k < c.tracks.size(); k++) w.num(c.tracks[k]);
    w.close(']');
    w.close('}');
  }
  w.close(']');
  w.close('}');
}

static int mode_control(Kv &kv, const std::string &out) {
  Control_parameters cp;
  if (!cp.initialise(get(kv, "ctrl")[0].c_str(), get(kv, "vex")[0].c_str(), std::cerr)) {
    write_file(out, "{\"error\":\"initialise\"}", 22);
    return 0;
  }
  const Vex &vex = cp.get_vex();
  const int nst = (int)cp.number_stations();
  std::map<std::string, int> to_input;
  for (int s = 0; s < nst; s++) to_input[cp.station(s)] = s;
  std::map<std::pair<int, int>, long long> station_time;
  for (int k = 0; k < count_key(kv, "station_time"); k++) {
    const std::vector<std::string> &v = get(kv, idx("station_time", k));
    station_time[std::make_pair(std::atoi(v[0].c_str()), std::atoi(v[1].c_str()))] = std::atoll(v[2].c_str());
  }
  Time start = cp.get_start_time(), stop = cp.get_stop_time();
  Time tint = cp.integration_time();
  Jw w;
  w.open('{');
  w.key("start"); w.num(start.get_clock_ticks());
  w.key("stop"); w.num(stop.get_clock_ticks());
  // Manager_node::initialise (manager_node.cc:402-418)
  int current_scan = cp.scan(start.date_string());
  if (current_scan == -1) die("no scan at the start time");
  // output files (420-472)
  std::vector<std::string> files, sources;
  std::string base = cp.get_output_file();
  if (cp.pulsar_binning()) {
    Pulsar_parameters pp(std::cerr);
    if (!cp.get_pulsar_parameters(pp)) die("pulsar parameters");
    int max_nbins = 2;
    for (std::map<std::string, Pulsar_parameters::Pulsar>::iterator it = pp.pulsars.begin(); it != pp.pulsars.end(); it++)
      max_nbins = std::max(it->second.nbins + 1, max_nbins);
    for (int b = 0; b < max_nbins; b++) {
      std::ostringstream f;
      f << base << ".bin" << b;
      files.push_back(f.str());
    }
  } else if (cp.multi_phase_center()) {
    Vex::Date st(cp.get_start_time().date_string()), sp(cp.get_stop_time().date_string());
    std::string first = vex.get_scan_name(st);
    Vex::Node::const_iterator it = vex.get_root_node()["SCHED"][first];
    std::set<std::string> srcs;
    while (it != vex.get_root_node()["SCHED"]->end() && vex.start_of_scan(it.key()) < sp) {
      for (Vex::Node::const_iterator si = it->begin("source"); si != it->end("source"); si++) srcs.insert(si->to_string());
      it++;
    }
    for (std::set<std::string>::iterator si = srcs.begin(); si != srcs.end(); si++) {
      sources.push_back(*si);
      files.push_back(base + "_" + *si);
    }
  } else {
    files.push_back(base);
  }
  w.key("output_files");
  w.open('[');
  for (size_t i = 0; i < files.size(); i++) w.str(files[i]);
  w.close(']');
  w.key("sources");
  w.open('[');
  for (size_t i = 0; i < sources.size(); i++) w.str(sources[i]);
  w.close(']');
  // send_global_header (660-683)
  {
    int y, d;
    start.get_date(y, d);
    w.key("header");
    w.open('{');
    w.key("experiment"); w.str(cp.get_exper_name());
    w.key("start_year"); w.num(y);
    w.key("start_day"); w.num(d);
    w.key("start_time"); w.num((int)start.get_time());
    w.key("number_channels"); w.num(cp.number_channels());
    w.key("integration_time"); w.num((int)tint.get_time_usec());
    w.key("polarisation_type"); w.num(cp.polarisation_type_for_global_output_header(vex.get_mode(cp.scan(current_scan))));
    w.key("job_nr"); w.num(cp.job_nr());
    w.key("subjob_nr"); w.num(cp.subjob_nr());
    w.close('}');
  }
  // the state machine of Manager_node::start (150-277) and
  // start_next_timeslice_on_node (284-391)
  Jw jobs;
  jobs.open('[');
  w.key("scans");
  w.open('[');
  int slice = 0, out_slice = 0, scan_index = 0;
  const int nch = (int)cp.number_frequency_channels();
  bool done = false;
  while (!done) {
    // initialise_scan (493-626)
    const std::string scan = cp.scan(current_scan);
    Vex::Date sos = vex.start_of_scan(scan), eos = vex.stop_of_scan(scan);
    Time scan_start(mjd(1, 1, sos.year) + sos.day - 1, sos.to_miliseconds() / 1000.);
    if (start + tint * slice < scan_start) {
      Time iv = scan_start - start;
      slice = (int)(iv / tint);
      if ((iv % tint) != Time()) slice++;
    }
    Time stop_scan(mjd(1, 1, eos.year) + eos.day - 1, eos.to_miliseconds() / 1000.);
    if (stop < stop_scan) stop_scan = stop;
    stop_scan -= (stop_scan - start) % tint;
    const std::string mode = vex.get_mode(scan);
    Jw sw;  // this scan's entry (written only if the scan is correlated)
    sw.open('{');
    sw.key("name"); sw.str(scan);
    sw.key("mode"); sw.str(mode);
    sw.key("source"); sw.str(cp.scan_source(scan));
    sw.key("n_sources"); sw.num(vex.n_sources(scan));
    sw.key("start"); sw.num(scan_start.get_clock_ticks());
    sw.key("stop"); sw.num(stop_scan.get_clock_ticks());
    sw.key("stations");
    sw.open('[');
    const Vex::Node &root = vex.get_root_node();
    for (int s = 0; s < nst; s++) {
      const std::string name = cp.station(s);
      if (!cp.station_in_scan(scan, name)) continue;
      std::string delay_file = cp.get_delay_table_name(name);
      // clock (532-576)
      Vex::Node::const_iterator clock = root["STATION"][name]["CLOCK"];
      const std::string clock_name = clock->to_string();
      Time cstart, epoch;
      double offset = 0.0, rate = 0.0;
      for (clock = root["CLOCK"][clock_name]->begin("clock_early"); clock != root["CLOCK"][clock_name]->end("clock_early"); clock++) {
        if (scan_start < Time(clock[0]->to_string())) continue;
        if (cstart > Time(clock[0]->to_string())) continue;
        cstart = Time(clock[0]->to_string());
        offset = clock[1]->to_double_amount("sec");
        rate = 0.0;
        if (clock->size() > 3) {
          if (clock[3]->to_string().find_first_of("\t ") != std::string::npos)
            rate = clock[3]->to_double_amount("sec/sec");
          else
            rate = clock[3]->to_double() * 1e-6;
          epoch = Time(clock[2]->to_string());
        }
      }
      if (cstart == Time()) die("clock does not cover the scan");
      double reader_offset = round(offset / 1.0) * 1.0;
      offset = offset - reader_offset;
      cp.set_reader_offset(name, Time(reader_offset * 1e6));
      Input_node_parameters ip = cp.get_input_node_parameters(mode, name);
      sw.open('{');
      sw.key("station"); sw.num(s);
      sw.key("name"); sw.str(name);
      sw.key("delay_file"); sw.str(delay_file);
      sw.key("clock_offset"); sw.dbl(offset);
      sw.key("clock_rate"); sw.dbl(rate);
      sw.key("clock_start"); sw.num(cstart.get_clock_ticks());
      sw.key("clock_epoch"); sw.num(epoch.get_clock_ticks());
      sw.key("reader_offset"); sw.num(Time(reader_offset * 1e6).get_clock_ticks());
      sw.key("stop_time"); sw.num(cp.stop_time(scan, name).get_clock_ticks());
      sw.key("input");
      put_input(sw, ip, cp.data_format(name));
      sw.close('}');
    }
    sw.close(']');
    std::vector<std::vector<int> > chs(nch, std::vector<int>(nst, -1));
    std::vector<int> last(nst, -1);
    for (int i = 0; i < nch; i++)
      for (int s = 0; s < nst; s++)
        if (cp.station_in_scan(scan, cp.station(s)) && !cp.frequency_channel(i, mode, cp.station(s)).empty())
          chs[i][s] = ++last[s];
    sw.key("ch_number_in_scan");
    sw.open('[');
    for (int i = 0; i < nch; i++) {
      sw.open('[');
      for (int s = 0; s < nst; s++) sw.num(chs[i][s]);
      sw.close(']');
    }
    sw.close(']');
    // START_NEW_SCAN (164-208)
    for (int s = 0; s < nst; s++) {
      bool in = false;
      for (int i = 0; i < nch; i++) in = in || chs[i][s] >= 0;
      if (!in) continue;
      std::map<std::pair<int, int>, long long>::iterator t = station_time.find(std::make_pair(s, scan_index));
      if (t == station_time.end()) continue;
      Time st = ticks_time(t->second);
      if (st > start + tint * slice) slice = (int)((st - start) / tint);
    }
    if (stop <= start + tint * slice) break;
    sw.key("first_slice_start"); sw.num((start + tint * slice).get_clock_ticks());
    sw.close('}');
    w.val(sw.s.substr(0));
    // time slices
    const bool xpol = cp.cross_polarize();
    for (;;) {
      int ch = 0;
      while (ch < nch) {
        int xch = xpol ? cp.cross_channel(ch, mode) : -1;
        Correlation_parameters c = cp.get_correlation_parameters(scan, ch, to_input);
        c.start_time = start + tint * slice;
        c.stop_time = start + tint * (slice + 1);
        c.integration_nr = slice;
        c.slice_nr = out_slice;
        strncpy(c.source, cp.scan_source(scan).c_str(), 11);
        c.pulsar_binning = cp.pulsar_binning();
        c.n_phase_centers = cp.multi_phase_center() ? vex.n_sources(scan) : 1;
        jobs.open('{');
        jobs.key("scan"); jobs.num(scan_index);
        jobs.key("channel"); jobs.num(ch);
        jobs.key("cross_channel"); jobs.num(xch);
        jobs.key("experiment_start"); jobs.num(c.experiment_start.get_clock_ticks());
        jobs.key("start_time"); jobs.num(c.start_time.get_clock_ticks());
        jobs.key("stop_time"); jobs.num(c.stop_time.get_clock_ticks());
        jobs.key("integration_time"); jobs.num(c.integration_time.get_clock_ticks());
        jobs.key("sub_integration_time"); jobs.num(c.sub_integration_time.get_clock_ticks());
        jobs.key("number_channels"); jobs.num(c.number_channels);
        jobs.key("fft_size_delaycor"); jobs.num(c.fft_size_delaycor);
        jobs.key("fft_size_correlation"); jobs.num(c.fft_size_correlation);
        jobs.key("window"); jobs.num(c.window);
        jobs.key("integration_nr"); jobs.num(c.integration_nr);
        jobs.key("slice_nr"); jobs.num(c.slice_nr);
        jobs.key("slice_offset"); jobs.num(c.slice_offset);
        jobs.key("sample_rate"); jobs.num(c.sample_rate);
        jobs.key("bandwidth"); jobs.num(c.bandwidth);
        jobs.key("frequency_nr"); jobs.num(c.frequency_nr);
        jobs.key("channel_freq"); jobs.num(c.channel_freq);
        jobs.key("sideband"); jobs.chr(c.sideband);
        jobs.key("polarisation"); jobs.chr(c.polarisation);
        jobs.key("cross_polarize"); jobs.boolean(c.cross_polarize);
        jobs.key("reference_station"); jobs.num(c.reference_station);
        jobs.key("n_phase_centers"); jobs.num(c.n_phase_centers);
        jobs.key("pulsar_binning"); jobs.boolean(c.pulsar_binning != 0);
        jobs.key("source"); jobs.str(std::string(c.source, strnlen(c.source, 11)));
        jobs.key("stations");
        jobs.open('[');
        for (size_t k = 0; k < c.station_streams.size(); k++) {
          const Correlation_parameters::Station_parameters &p = c.station_streams[k];
          jobs.open('{');
          jobs.key("station_number"); jobs.num(p.station_number);
          jobs.key("station_stream"); jobs.num(p.station_stream);
          jobs.key("start_time"); jobs.num(p.start_time.get_clock_ticks());
          jobs.key("stop_time"); jobs.num(p.stop_time.get_clock_ticks());
          jobs.key("sample_rate"); jobs.num(p.sample_rate);
          jobs.key("channel_freq"); jobs.num(p.channel_freq);
          jobs.key("bandwidth"); jobs.num(p.bandwidth);
          jobs.key("sideband"); jobs.chr(p.sideband);
          jobs.key("polarisation"); jobs.chr(p.polarisation);
          jobs.key("bits_per_sample"); jobs.num(p.bits_per_sample);
          jobs.key("lo_offset"); jobs.dbl(p.LO_offset);
          jobs.key("tsys_freq"); jobs.num(p.tsys_freq);
          jobs.close('}');
        }
        jobs.close(']');
        jobs.key("inputs");
        jobs.open('[');
        for (int s = 0; s < nst; s++) {
          int stream = 0;
          if (chs[ch][s] >= 0) {
            jobs.open('{');
            jobs.key("station"); jobs.num(s);
            jobs.key("channel_in_scan"); jobs.num(chs[ch][s]);
            jobs.key("stream"); jobs.num(s);
            jobs.close('}');
            stream = 1;
          }
          if (xch != -1 && chs[xch][s] >= 0) {
            jobs.open('{');
            jobs.key("station"); jobs.num(s);
            jobs.key("channel_in_scan"); jobs.num(chs[xch][s]);
            jobs.key("stream"); jobs.num(stream ? s + nst : s);
            jobs.close('}');
          }
        }
        jobs.close(']');
        jobs.close('}');
        out_slice++;
        ch++;
        if (xpol) {
          int x = cp.cross_channel(ch, mode);
          while (ch < nch && x >= 0 && x < ch) {
            ch++;
            x = cp.cross_channel(ch, mode);
          }
        }
      }
      slice++;
      if (start + tint * (slice + 1) > stop) {
        done = true;
        break;
      }
      if (start + tint * (slice + 1) > stop_scan) {
        if (++current_scan == (int)cp.number_scans()) done = true;
        break;
      }
    }
    scan_index++;
  }
  w.close(']');
  jobs.close(']');
  w.key("jobs");
  w.val(jobs.s);
  // pulsars and the mask
  w.key("pulsars");
  w.open('[');
  if (cp.pulsar_binning()) {
    Pulsar_parameters pp(std::cerr);
    cp.get_pulsar_parameters(pp);
    for (std::map<std::string, Pulsar_parameters::Pulsar>::iterator it = pp.pulsars.begin(); it != pp.pulsars.end(); it++) {
      const Pulsar_parameters::Pulsar &ps = it->second;
      w.open('{');
      w.key("name"); w.str(std::string(ps.name, strnlen(ps.name, 11)));
      w.key("nbins"); w.num(ps.nbins);
      w.key("gate_start"); w.dbl(ps.interval.start);
      w.key("gate_stop"); w.dbl(ps.interval.stop);
      w.key("polyco");
      w.open('[');
      for (size_t k = 0; k < ps.polyco_params.size(); k++) {
        const Pulsar_parameters::Polyco_params &pc = ps.polyco_params[k];
        w.open('{');
        w.key("name"); w.str(std::string(pc.name, strnlen(pc.name, 11)));
        w.key("tmid"); w.dbl(pc.tmid);
        w.key("dm"); w.dbl(pc.DM);
        w.key("ref_phase"); w.dbl(pc.ref_phase);
        w.key("ref_freq"); w.dbl(pc.ref_freq);
        w.key("obs_freq"); w.dbl(pc.obs_freq);
        w.key("data_span"); w.num(pc.data_span);
        w.key("coef");
        w.open('[');
        for (size_t q = 0; q < pc.coef.size(); q++) w.dbl(pc.coef[q]);
        w.close(']');
        w.close('}');
      }
      w.close(']');
      w.close('}');
    }
  }
  w.close(']');
  Mask_parameters mp;
  if (cp.get_mask_parameters(mp)) {
    w.key("mask");
    w.open('{');
    w.key("normalize"); w.boolean(mp.normalize);
    w.key("mask");
    w.open('[');
    for (size_t k = 0; k < mp.mask.size(); k++) w.dbl(mp.mask[k]);
    w.close(']');
    w.key("window");
    w.open('[');
    for (size_t k = 0; k < mp.window.size(); k++) w.dbl(mp.window[k]);
    w.close(']');
    w.close('}');
  }
  w.close('}');
  write_file(out, w.s.data(), w.s.size());
  return 0;
}

int main(int argc, char **argv) {
  if (argc != 4) die("usage: ref_harness correlate|delays|protocol|extract|reader|schedule|uvw|control <job> <out>");
  Kv kv = read_job(argv[2]);
  std::string m(argv[1]);
  if (m == "correlate") return mode_correlate(kv, argv[3]);
  if (m == "delays") return mode_delays(kv, argv[3]);
  if (m == "protocol") return mode_protocol(kv, argv[3]);
  if (m == "extract") return mode_extract(kv, argv[3]);
  if (m == "reader") return mode_reader(kv, argv[3]);
  if (m == "schedule") return mode_schedule(kv, argv[3]);
  if (m == "uvw") return mode_uvw(kv, argv[3]);
  if (m == "control") return mode_control(kv, argv[3]);
  die("unknown mode " + m);
  return 2;
}
