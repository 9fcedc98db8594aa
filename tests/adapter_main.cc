// Driver of the Correlator_node adapter (sfxc-1_gb300/adapter/correlator_node_gpu.h),
// compiled against the reference's own headers (test infrastructure).
//
//   adapter_main <job file> <out dir> <x_mode>
//
// Reads a job in the key-value format of the checkers' 'correlate' mode,
// fills the reference's Correlation_parameters (and Pulsar_parameters::Pulsar,
// Mask_parameters) as a correlator node receives them, flattens them through
// the adapter and writes every field of the resulting sfxc_correlation_params
// to <out dir>/params.txt.  Then it creates the adapter on device 0 -- where
// the library refuses (no GPU), the adapter calls the reference's sfxc_abort
// -- and, on a GPU, correlates every integration into <out dir>/out.cor.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "correlator_node_gpu.h"

typedef std::map<std::string, std::vector<std::string> > Keys;

static void fail(const std::string &m) {
  std::fprintf(stderr, "adapter_main: %s\n", m.c_str());
  std::exit(2);
}

// "key v1 v2 ..." lines; the k-th occurrence of a key is also stored as "key#k"
static Keys parse(const char *path) {
  std::ifstream in(path);
  if (!in) fail(std::string("cannot open ") + path);
  Keys keys;
  std::map<std::string, int> seen;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string key, v;
    if (!(ss >> key)) continue;
    std::vector<std::string> vals;
    while (ss >> v) vals.push_back(v);
    std::ostringstream nth;
    nth << key << "#" << seen[key]++;
    keys[nth.str()] = vals;
    if (seen[key] == 1) keys[key] = vals;
  }
  return keys;
}
static bool has(const Keys &k, const std::string &key) { return k.find(key) != k.end(); }
static const std::vector<std::string> &val(const Keys &k, const std::string &key) {
  Keys::const_iterator it = k.find(key);
  if (it == k.end()) fail("missing key " + key);
  return it->second;
}
static std::string nth(const std::string &key, int i) {
  std::ostringstream s;
  s << key << "#" << i;
  return s.str();
}
static int count(const Keys &k, const std::string &key) {
  int n = 0;
  while (has(k, nth(key, n))) n++;
  return n;
}
static long long ll(const Keys &k, const std::string &key) { return std::atoll(val(k, key)[0].c_str()); }
static std::vector<char> file_bytes(const std::string &path) {
  std::ifstream in(path.c_str(), std::ios::binary);
  if (!in) fail("cannot open " + path);
  return std::vector<char>((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}
static std::vector<double> f32_file(const std::string &path) {
  const std::vector<char> b = file_bytes(path);
  std::vector<double> v;
  for (size_t q = 0; q + 4 <= b.size(); q += 4) {
    float x;
    std::memcpy(&x, &b[q], 4);
    v.push_back(x);
  }
  return v;
}

class Bytes_writer : public Data_writer {
public:
  std::vector<char> bytes;
  bool can_write() { return true; }

private:
  size_t do_put_bytes(size_t n, const char *buf) {
    bytes.insert(bytes.end(), buf, buf + n);
    return n;
  }
};

int main(int argc, char **argv) {
  if (argc < 4) fail("usage: adapter_main <job file> <out dir> <x_mode>");
  const Keys k = parse(argv[1]);
  const std::string out = argv[2];
  const int x_mode = std::atoi(argv[3]);

  Correlation_parameters p;
  Time t;
  t.set_clock_ticks(ll(k, "experiment_start_ticks"));
  p.experiment_start = t;
  t.set_clock_ticks(ll(k, "start_ticks"));
  p.start_time = t;
  p.integration_time = Time((double)ll(k, "integration_time_us"));
  p.sub_integration_time = Time((double)ll(k, "sub_integration_time_us"));
  p.number_channels = (int32_t)ll(k, "number_channels");
  p.fft_size_delaycor = (int32_t)ll(k, "fft_size_delaycor");
  p.fft_size_correlation = (int32_t)ll(k, "fft_size_correlation");
  p.integration_nr = (int32_t)ll(k, "integration_nr");
  p.sample_rate = (int32_t)ll(k, "sample_rate");
  p.channel_freq = ll(k, "channel_freq");
  p.bandwidth = (int32_t)ll(k, "bandwidth");
  p.sideband = val(k, "sideband")[0][0];
  p.frequency_nr = (int32_t)ll(k, "frequency_nr");
  p.polarisation = val(k, "polarisation")[0][0];
  p.cross_polarize = ll(k, "cross_polarize") != 0;
  p.reference_station = (int32_t)ll(k, "reference_station");
  p.window = (int)ll(k, "window");
  std::memset(p.source, 0, sizeof(p.source));
  std::strncpy(p.source, val(k, "source")[0].c_str(), 10);
  p.n_phase_centers = has(k, "n_phase_centers") ? (int32_t)ll(k, "n_phase_centers") : 1;
  p.pulsar_binning = has(k, "pulsar") ? 1 : 0;
  p.pulsar_parameters = 0;
  p.mask_parameters = 0;
  Mask_parameters mask;
  if (has(k, "mask") || has(k, "lag_window") || has(k, "mask_normalize")) {
    if (has(k, "mask")) mask.mask = f32_file(val(k, "mask")[0]);
    if (has(k, "lag_window")) mask.window = f32_file(val(k, "lag_window")[0]);
    mask.normalize = has(k, "mask_normalize") && ll(k, "mask_normalize") != 0;
    p.mask_parameters = &mask;
  }
  std::vector<int> stream_table;
  const int nstreams = count(k, "stream");
  for (int i = 0; i < nstreams; i++) {
    // station_number station_stream sample_rate channel_freq bandwidth sideband pol bits LO_offset tsys_freq table
    const std::vector<std::string> &v = val(k, nth("stream", i));
    Correlation_parameters::Station_parameters s;
    s.station_number = std::atoi(v[0].c_str());
    s.station_stream = std::atoi(v[1].c_str());
    s.sample_rate = std::atoi(v[2].c_str());
    s.channel_freq = std::atoll(v[3].c_str());
    s.bandwidth = std::atoi(v[4].c_str());
    s.sideband = v[5][0];
    s.polarisation = v[6][0];
    s.bits_per_sample = std::atoi(v[7].c_str());
    s.LO_offset = std::strtod(v[8].c_str(), 0);
    s.tsys_freq = std::atoi(v[9].c_str());
    stream_table.push_back(std::atoi(v[10].c_str()));
    p.station_streams.push_back(s);
  }
  std::vector<std::vector<char> > del_files;
  for (int i = 0; i < count(k, "delfile"); i++) del_files.push_back(file_bytes(val(k, nth("delfile", i))[0]));
  Pulsar_parameters::Pulsar pulsar;
  if (p.pulsar_binning) {
    const std::vector<std::string> &v = val(k, "pulsar");  // nbins gate_start gate_stop
    std::memset(pulsar.name, 0, sizeof(pulsar.name));
    pulsar.nbins = std::atoi(v[0].c_str());
    pulsar.interval.start = std::strtod(v[1].c_str(), 0);
    pulsar.interval.stop = std::strtod(v[2].c_str(), 0);
    for (int q = 0; q < count(k, "polyco"); q++) {
      const std::vector<std::string> &c = val(k, nth("polyco", q));  // tmid DM ref_phase ref_freq obs_freq coef...
      Pulsar_parameters::Polyco_params pp;
      pp.tmid = std::strtod(c[0].c_str(), 0);
      pp.DM = std::strtod(c[1].c_str(), 0);
      pp.ref_phase = std::strtod(c[2].c_str(), 0);
      pp.ref_freq = std::strtod(c[3].c_str(), 0);
      pp.obs_freq = std::strtod(c[4].c_str(), 0);
      for (size_t j = 5; j < c.size(); j++) pp.coef.push_back(std::strtod(c[j].c_str(), 0));
      pp.n_coef = (int32_t)pp.coef.size();
      pulsar.polyco_params.push_back(pp);
    }
  }
  std::vector<int32_t> file_index;
  if (has(k, "pc_file_index"))
    for (size_t q = 0; q < val(k, "pc_file_index").size(); q++)
      file_index.push_back(std::atoi(val(k, "pc_file_index")[q].c_str()));

  // the adapter's flattening, field by field
  Correlator_node_gpu::Job j;
  Correlator_node_gpu::flatten(p, del_files, stream_table, file_index, p.pulsar_binning ? &pulsar : 0, j);
  FILE *f = std::fopen((out + "/params.txt").c_str(), "w");
  if (!f) fail("cannot write params.txt");
  const sfxc_correlation_params &c = j.c;
  std::fprintf(f, "experiment_start_ticks %lld\nstart_ticks %lld\n", (long long)c.experiment_start_ticks,
               (long long)c.start_ticks);
  std::fprintf(f, "integration_time_us %lld\nsub_integration_time_us %lld\n", (long long)c.integration_time_us,
               (long long)c.sub_integration_time_us);
  std::fprintf(f, "number_channels %d\nfft_size_delaycor %d\nfft_size_correlation %d\n", c.number_channels,
               c.fft_size_delaycor, c.fft_size_correlation);
  std::fprintf(f, "sample_rate %d\nbandwidth %d\nfrequency_nr %d\nchannel_freq %lld\n", c.sample_rate, c.bandwidth,
               c.frequency_nr, (long long)c.channel_freq);
  std::fprintf(f, "sideband %d\npolarisation %d\ncross_polarize %d\nreference_station %d\nwindow %d\n", c.sideband,
               c.polarisation, c.cross_polarize, c.reference_station, c.window);
  std::fprintf(f, "integration_nr %d\nn_streams %d\nn_delay_tables %d\n", c.integration_nr, c.n_streams,
               c.n_delay_tables);
  for (int i = 0; i < c.n_streams; i++) {
    const sfxc_station_stream &s = c.streams[i];
    std::fprintf(f, "stream %d %d %d %d %d %d %lld %d %d %d %.17g\n", s.station_number, s.station_stream,
                 s.sample_rate, s.bandwidth, s.bits_per_sample, s.tsys_freq, (long long)s.channel_freq, s.sideband,
                 s.polarisation, s.delay_table, s.lo_offset);
  }
  for (int i = 0; i < c.n_delay_tables; i++) std::fprintf(f, "delay_table %d %zu\n", i, c.delay_tables[i].del_size);
  std::fprintf(f, "pulsar_nbins %d\ngate %.17g %.17g\nn_polyco %d\n", c.pulsar_nbins, c.gate_start, c.gate_stop,
               c.n_polyco);
  for (int i = 0; i < c.n_polyco; i++) {
    const sfxc_polyco &q = c.polyco[i];
    std::fprintf(f, "polyco %.17g %.17g %.17g %.17g %.17g %d", q.tmid, q.dm, q.ref_phase, q.ref_freq, q.obs_freq,
                 q.n_coef);
    for (int e = 0; e < q.n_coef; e++) std::fprintf(f, " %.17g", q.coef[e]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "mask %d lag_window %d mask_normalize %d\n", c.mask ? (int)j.mask.size() : 0,
               c.lag_window ? (int)j.lag_window.size() : 0, c.mask_normalize);
  std::fprintf(f, "n_phase_centers %d\nphased_array %d\n", c.n_phase_centers, c.phased_array);
  std::fclose(f);

  // the node: the library refuses without a GPU, and the adapter aborts as the reference does
  Correlator_node_gpu node(0, x_mode != 0);
  node.set_parameters(p, del_files, stream_table, file_index, p.pulsar_binning ? &pulsar : 0);
  std::vector<std::vector<char> > protocols;
  for (int i = 0; i < nstreams; i++) protocols.push_back(file_bytes(val(k, nth("protocol", i))[0]));
  std::vector<size_t> pos(nstreams, 0);
  std::vector<char> cor;
  for (long long it = 0; it < ll(k, "n_integrations"); it++) {
    for (int i = 0; i < nstreams; i++) {  // each stream's chunk: uint64 length, then the bytes
      uint64_t n = 0;
      std::memcpy(&n, &protocols[i][pos[i]], 8);
      node.push(i, &protocols[i][pos[i] + 8], (size_t)n);
      pos[i] += 8 + (size_t)n;
    }
    Bytes_writer w;
    node.correlate(w, RANK_OUTPUT_NODE);
    cor.insert(cor.end(), w.bytes.begin(), w.bytes.end());
  }
  f = std::fopen((out + "/out.cor").c_str(), "wb");
  if (!f) fail("cannot write out.cor");
  if (!cor.empty()) std::fwrite(&cor[0], 1, cor.size(), f);
  std::fclose(f);
  return 0;
}
