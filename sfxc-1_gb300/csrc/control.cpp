// Control file + VEX -> job and reader parameters, and the manager's plan;
// see control.hpp.  Each function restates the reference function named in
// its comment (sfxc/src/control_parameters.cc, sfxc/src/manager_node.cc).
#include "control.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <set>
#include <sstream>
#include <stdexcept>

#include "frames.hpp"

namespace sfxc {

namespace {

constexpr double kClock = 512000000.0;  // ticks per second (MAX_SAMPLE_RATE)
constexpr int kRefMjd = 51544;
enum { W_NONE = 0, W_RECT = 1, W_COS = 2, W_HAMMING = 3, W_HANN = 4 };  // SFXC_WINDOW_* (utils.h)

[[noreturn]] void fail(const std::string &msg) { throw std::runtime_error(msg); }

ticks_t ticks_usec(double usec) { return (ticks_t)std::llround(usec * (kClock / 1000000)); }
ticks_t ticks_mjd_sec(int mjd, double sec) {
  return (ticks_t)((mjd - kRefMjd) * 86400 * kClock) + (ticks_t)std::llround(sec * kClock);
}

// Read an unsigned decimal of at most `width` digits (strptime's numeric fields).
bool read_num(const char *&p, int width, int lo, int hi, int &out) {
  while (*p == ' ') p++;
  if (!std::isdigit((unsigned char)*p)) return false;
  int v = 0, n = 0;
  while (n < width && std::isdigit((unsigned char)*p)) {
    v = v * 10 + (*p - '0');
    p++;
    n++;
  }
  if (v < lo || v > hi) return false;
  out = v;
  return true;
}

// Time(const std::string&) (sfxc/src/correlator_time.cc:20-40): "YYYYyDDDdHHhMMmSS[.fff]s",
// or without the seconds, minutes, hours
ticks_t time_of_string(const std::string &text) {
  int y = 0, j = 1, h = 0, m = 0, s = 0;
  const char *p = text.c_str();
  auto lit = [&p](char c) {
    if (*p != c) return false;
    p++;
    return true;
  };
  bool ok = read_num(p, 4, 0, 9999, y) && lit('y') && read_num(p, 3, 1, 366, j) && lit('d');
  if (!ok) fail("invalid date-time '" + text + "'");
  const char *after_day = p;
  if (read_num(p, 2, 0, 23, h) && lit('h')) {
    const char *after_h = p;
    if (read_num(p, 2, 0, 59, m) && lit('m')) {
      const char *after_m = p;
      if (read_num(p, 2, 0, 61, s)) {
        if (*p == '.') {
          p++;
          while (std::isdigit((unsigned char)*p)) p++;
        }
        if (*p == 's') p++;
      } else {
        p = after_m;
      }
    } else {
      p = after_h;
      m = 0;
    }
  } else {
    p = after_day;
    h = 0;
  }
  if (*p) fail("invalid date-time '" + text + "'");
  int mjd = mjd_from_date(1, 1, y) + (j - 1);
  return ticks_mjd_sec(mjd, 60 * (60 * h + m) + s);
}

// Time::get_date (correlator_time.cc:77-86)
void date_of_ticks(ticks_t t, int &year, int &day) {
  const ticks_t per_day = (ticks_t)(86400 * kClock);
  double mjd = kRefMjd + (double)(int)(t / per_day) + (double)(t % per_day) / kClock / 86400;
  int ndays = (int)(mjd - 15385);
  int p1 = ndays / (365 * 4 + 1);
  int p2 = (ndays - p1 * (365 * 4 + 1)) / 365;
  year = 4 * p1 + p2 + 1901;
  day = 1 + (ndays - p1 * (365 * 4 + 1)) % 365;
}

std::string dirname_of(const std::string &path) {
  size_t k = path.find_last_of('/');
  if (k == std::string::npos) return ".";
  if (k == 0) return "/";
  return path.substr(0, k);
}

std::string read_file(const std::string &path, const char *what) {
  std::ifstream in(path, std::ios::binary);
  if (!in) fail(std::string("could not open ") + what + " [" + path + "]");
  std::ostringstream ss;
  ss << in.rdbuf();
  return ss.str();
}

// A def of a block; a missing one is an error (the reference asserts or aborts).
const VexNode *require_def(const Vex &v, const std::string &block, const std::string &name) {
  const VexNode *d = v.def(block, name);
  if (!d) fail("cannot find " + name + " in $" + block + " block");
  return d;
}

}  // namespace

// ---------------------------------------------------------------- initialise

void Control::initialise(const std::string &ctrl_path, const std::string &vex_path) {
  initialise_text(read_file(ctrl_path, "control file"), read_file(vex_path, "vex file"), dirname_of(ctrl_path));
}

// Control_parameters::initialise (control_parameters.cc:29-230)
void Control::initialise_text(const std::string &ctrl_text, const std::string &vex_text,
                              const std::string &ctrl_dir) {
  ctrl_ = Json::parse(ctrl_text);
  if (ctrl_.type() != Json::OBJECT) fail("ctrl file: the document is not an object");
  vex_ = Vex(parse_vex(vex_text));
  ctrl_dir_ = ctrl_dir;
  station_map_.clear();
  Json &c = ctrl_;

  if (c["delay_directory"].is_null()) c.set("delay_directory", Json::of_string("file:///tmp/"));
  if (c["channels"].is_null()) {  // every channel name of every $FREQ def, sorted
    std::set<std::string> names;
    for (const auto &fd : vex_.block("FREQ").dict)
      for (const VexNode *cd : fd.second.all("chan_def")) names.insert(cd->at(4).str());
    Json ch = Json::parse("[]");
    for (const auto &n : names) ch.append(Json::of_string(n));
    c.set("channels", ch);
  }
  if (c["scans"].is_null()) {
    Json sc = Json::parse("[]");
    for (const auto &s : vex_.scans()) sc.append(Json::of_string(s));
    c.set("scans", sc);
  }
  if (c["reference_station"].is_null()) c.set("reference_station", Json::of_string(""));
  if (c["message_level"].is_null()) c.set("message_level", Json::of_int(1));
  if (c["pulsar_binning"].is_null()) {
    c.set("pulsar_binning", Json::of_bool(false));
  } else if (c["pulsar_binning"].as_bool()) {
    if (c["pulsars"].is_null()) fail("No pulsars block in control file");
    Json ps = c["pulsars"];
    if (ps.size() == 0 || ps.members().empty() || ps.members().begin()->second.is_null())
      fail("Empty pulsars block in control file");
    Json filled;
    for (const auto &kv : ps.members()) {
      Json p = kv.second;
      if (p["interval"].is_null()) {
        Json iv;
        iv.append(Json::of_double(0.0));
        iv.append(Json::of_double(1.0));
        p.set("interval", iv);
      }
      if (p["nbins"].is_null()) p.set("nbins", Json::of_int(0));
      filled.set(kv.first, p);
    }
    c.set("pulsars", filled);
  }
  if (c["phased_array"].is_null()) c.set("phased_array", Json::of_bool(false));
  if (c["multi_phase_center"].is_null()) {
    bool multi = false;
    if (!c["pulsar_binning"].as_bool())
      for (const auto &s : vex_.block("SCHED").dict)
        if (s.second.all("source").size() > 1) {
          multi = true;
          break;
        }
    c.set("multi_phase_center", Json::of_bool(multi));
  } else if (c["multi_phase_center"].as_bool() && c["pulsar_binning"].as_bool()) {
    fail("Pulsar binning cannot be used together with multiple phase centers");
  }
  if (c["phased_array"].as_bool() && c["pulsar_binning"].as_bool())
    fail("Pulsar binning cannot be used in phase array mode");
  if (c["window_function"].is_null())
    c.set("window_function", Json::of_string(c["multi_phase_center"].as_bool() ? "NONE" : "HANN"));
  if (c["fft_size_correlation"].is_null()) {
    int min_size = c["multi_phase_center"].as_bool() ? 4096 : 256;
    if (!c["fft_size_delaycor"].is_null()) min_size = std::max(min_size, c["fft_size_delaycor"].as_int());
    c.set("fft_size_correlation", Json::of_int(std::max(min_size, number_channels())));
  }
  if (c["fft_size_delaycor"].is_null())
    c.set("fft_size_delaycor", Json::of_int(std::min(256, c["fft_size_correlation"].as_int())));
  if (c["sub_integr_time"].is_null()) {
    const ticks_t per_day = (ticks_t)(86400 * kClock);
    double int_us = std::round((double)(integration_time() % per_day) / (kClock / 1000000));
    c.set("sub_integr_time", Json::of_double(std::min(int_us, c["multi_phase_center"].as_bool() ? 20480. : 125000.)));
  }
  if (c["phasecal_integr_time"].is_null())
    c.set("phasecal_integr_time", Json::of_int(c["phasecal_file"].as_bool() ? 10 : 0));
  if (c["exit_on_empty_datastream"].is_null()) c.set("exit_on_empty_datastream", Json::of_bool(true));
  if (c["start"].as_string() == "now") {
    std::time_t t = std::time(nullptr);
    std::tm tm;
    gmtime_r(&t, &tm);
    char b[64];
    std::snprintf(b, sizeof b, "%dy%dd%dh%dm%ds", tm.tm_year + 1900, tm.tm_yday + 1, tm.tm_hour, tm.tm_min,
                  tm.tm_sec);
    c.set("start", Json::of_string(b));
  }
  if (c["stop"].as_string() == "end") c.set("stop", Json::of_string(vex_.stop_time_of_experiment()));
}

// ---------------------------------------------------------------- control file

ticks_t Control::start_time() const { return time_of_string(ctrl_["start"].as_string()); }
ticks_t Control::stop_time() const { return time_of_string(ctrl_["stop"].as_string()); }
ticks_t Control::integration_time() const {
  return ticks_usec(std::round(ctrl_["integr_time"].as_double() * 1000000));
}
ticks_t Control::sub_integration_time() const { return ticks_usec(ctrl_["sub_integr_time"].as_double()); }
ticks_t Control::phasecal_integration_time() const {
  return ticks_usec((double)(ctrl_["phasecal_integr_time"].as_int() * 1000000));
}

int Control::window_function() const {  // 643-662
  if (ctrl_["window_function"].is_null()) return W_NONE;
  std::string w = ctrl_["window_function"].as_string();
  for (auto &ch : w) ch = (char)std::toupper((unsigned char)ch);
  if (w == "RECTANGULAR") return W_RECT;
  if (w == "COSINE") return W_COS;
  if (w == "HAMMING") return W_HAMMING;
  if (w == "HANN") return W_HANN;
  return W_NONE;
}

std::string Control::setup_station() const {
  return ctrl_["setup_station"].is_null() ? station(0) : ctrl_["setup_station"].as_string();
}

int Control::reference_station_number() const {
  std::string r = ctrl_["reference_station"].as_string();
  return r.empty() ? -1 : station_number(r);
}

double Control::lo_offset(const std::string &st) const { return ctrl_["LO_offset"][st].as_double(); }

int Control::tsys_freq(const std::string &st) const {
  return ctrl_["tsys_freq"][st].is_null() ? 80 : ctrl_["tsys_freq"][st].as_int();
}

// create_path (2061-2078): "file://x" with a relative x is taken relative to the control file
std::string Control::create_path(const std::string &path) const {
  if (path.compare(0, 7, "file://") == 0 && path.size() > 7 && path[7] != '/')
    return "file://" + ctrl_dir_ + "/" + path.substr(7);
  return path;
}

std::vector<std::string> Control::data_sources(const std::string &st) const {
  const Json &d = ctrl_["data_sources"][st];
  if (d.is_null()) fail("ctrl file: no data_sources for station " + st);
  std::vector<std::string> out;
  for (size_t i = 0; i < d.size(); i++) out.push_back(create_path(d[i].as_string()));
  return out;
}

// get_delay_table_name (2025-2048), without running the delay model generator
std::string Control::delay_table_name(const std::string &st) const {
  std::string dir = ctrl_["delay_directory"].as_string();
  if (dir.compare(0, 7, "file://") != 0) fail("Ctrl-file: Delay directory doesn't start with 'file://'");
  std::string name = exper_name() + "_" + st + ".del";
  if (dir.size() == 7) return name;
  return dir.substr(7) + "/" + name;  // as written: a relative directory is relative to the working directory
}

std::vector<PolycoBlock> parse_polyco(const std::string &path) {
  std::ifstream inp(path);
  if (!inp) fail("Could not open polyco file [" + path + "]");
  std::vector<PolycoBlock> out;
  std::string line, tmp;
  int line_nr = 0, coef_idx = 0, n_coef = 0, block = 0, end_prev = 0;
  bool completed = false, error = false;
  std::getline(inp, line);
  while (!inp.eof()) {  // a last line without a line end is not read, as in the reference
    std::istringstream ls(line);
    if (line_nr - end_prev == 0) {
      out.resize(block + 1);
      PolycoBlock &p = out[block];
      ls >> tmp;
      p.name = tmp.substr(0, 10);
      ls >> tmp;
      p.date = tmp.substr(0, 9);
      ls >> p.utc >> p.tmid >> p.dm >> p.doppler >> p.residual;
      completed = false;
      error = ls.fail();
    } else if (line_nr - end_prev == 1) {
      PolycoBlock &p = out[block];
      ls >> p.ref_phase >> p.ref_freq >> tmp;
      p.site = tmp.substr(0, 5);
      ls >> p.data_span >> p.n_coef;
      n_coef = p.n_coef;
      p.coef.assign(n_coef > 0 ? n_coef : 0, 0.0);
      ls >> p.obs_freq;
      error = ls.fail();
      ls >> p.bin_phase[0];
      if (!ls.fail()) {
        ls >> p.bin_phase[1];
        error = ls.fail();
      } else {
        p.bin_phase[0] = p.bin_phase[1] = 0;
      }
    } else {
      PolycoBlock &p = out[block];
      while (!ls.eof() && !ls.fail() && coef_idx < n_coef) {
        ls >> p.coef[coef_idx];
        coef_idx++;
      }
      if (!ls.fail() && coef_idx == n_coef) {
        completed = true;
        block++;
        coef_idx = 0;
        end_prev = line_nr + 1;
      }
      error = ls.fail();
    }
    if (error) fail("Error parsing line " + std::to_string(line_nr + 1) + " of polyco file [" + path + "]");
    line_nr++;
    std::getline(inp, line);
  }
  if (!completed) fail("Eof reached prematurely while parsing polyco file [" + path + "]");
  if ((int)out.size() > block) out.resize(block);
  return out;
}

// get_pulsar_parameters (719-739)
std::vector<PulsarSpec> Control::pulsars() const {
  std::vector<PulsarSpec> out;
  if (!pulsar_binning()) return out;
  for (const auto &kv : ctrl_["pulsars"].members()) {
    PulsarSpec p;
    p.name = kv.first.substr(0, 10);
    p.nbins = kv.second["nbins"].as_int();
    p.gate_start = kv.second["interval"][0].as_double();
    p.gate_stop = kv.second["interval"][1].as_double();
    std::string f = kv.second["polyco_file"].as_string();
    p.polyco = parse_polyco(f.size() > 7 ? f.substr(7) : std::string());  // "file://" dropped, the rest as written
    out.push_back(p);
  }
  return out;
}

bool Control::mask(bool &normalize, std::vector<double> &mask, std::vector<double> &window) const {
  const Json &m = ctrl_["mask"];
  if (m.is_null()) return false;
  normalize = m["normalize"].as_bool();
  auto read_list = [this](const Json &f, std::vector<double> &dst) {
    std::string path = create_path(f.as_string());
    std::ifstream in(path.size() > 7 ? path.substr(7) : path);
    if (!in) fail("Could not open mask/window file " + path);
    double d;
    while (in >> d) dst.push_back(d);
  };
  if (!m["mask"].is_null()) read_list(m["mask"], mask);
  if (!m["window"].is_null()) read_list(m["window"], window);
  return true;
}

// ---------------------------------------------------------------- VEX file

std::string Control::exper_name() const {  // 1030-1044
  const VexNode *g = vex_.root().get("GLOBAL");
  const VexNode *e = g ? g->get("EXPER") : nullptr;
  if (!e) fail("Cannot find EXPER in $GLOBAL block");
  const VexNode *d = vex_.def("EXPER", e->str());
  if (!d) fail("Cannot find " + e->str() + " in $EXPER block");
  const VexNode *n = d->get("exper_name");
  return n ? n->str() : std::string();
}

int Control::station_number(const std::string &st) const {  // 1846-1865
  if (station_map_.empty()) {
    int k = 0;
    for (const auto &kv : vex_.block("STATION").dict)
      if (!station_map_.count(kv.first)) station_map_[kv.first] = 0;
    for (auto &kv : station_map_) kv.second = k++;
  }
  auto it = station_map_.find(st);
  return it == station_map_.end() ? 0 : it->second;  // an unknown name reads as 0, as map::operator[] gives
}

std::string Control::transport_type(const std::string &st) const {  // 1558-1573
  const VexNode &sd = *require_def(vex_, "STATION", st);
  for (const VexNode *das : sd.all("DAS")) {
    const VexNode &d = *require_def(vex_, "DAS", das->str());
    if (const VexNode *t = d.get("record_transport_type")) return t->str();
  }
  return std::string();
}

std::string Control::rack_type(const std::string &st) const {  // 1603-1618
  const VexNode &sd = *require_def(vex_, "STATION", st);
  for (const VexNode *das : sd.all("DAS")) {
    const VexNode &d = *require_def(vex_, "DAS", das->str());
    if (const VexNode *t = d.get("electronics_rack_type")) return t->str();
  }
  return std::string();
}

std::string Control::data_format(const std::string &st) const {  // 1575-1601
  std::string tt = transport_type(st), rt = rack_type(st);
  if (tt == "Mark5A") return rt == "VLBA4" ? "Mark4" : rt;
  if (tt == "Mark5B" && (rt == "DVP" || rt == "RDBE2" || rt == "WIDAR")) return "VDIF";
  if (tt == "Mark5C" && (rt == "DBBC" || rt == "DVP" || rt == "RDBE2" || rt == "WIDAR")) return "VDIF";
  if (tt == "None" && rt == "DBBC") return "VDIF";
  return tt;
}

const VexNode &Control::freq_def(const std::string &mode, const std::string &st) const {
  std::string f = vex_.section("FREQ", mode, st);
  if (f.empty()) fail("Cannot find $FREQ reference for " + st + " in mode " + mode);
  return *require_def(vex_, "FREQ", f);
}

int Control::bits_per_sample(const std::string &mode, const std::string &st) const {  // 773-818
  std::string fmt = data_format(st);
  if (fmt == "VDIF") {
    std::string tn = vex_.section("THREADS", mode, st);
    const VexNode &th = *require_def(vex_, "THREADS", tn);
    auto threads = th.all("thread");
    if (!threads.empty()) return threads[0]->at(5).to_int();
  }
  if (fmt == "Mark5B") {
    std::string bn = vex_.section("BITSTREAMS", mode, st);
    if (!bn.empty()) {
      const VexNode &bs = *require_def(vex_, "BITSTREAMS", bn);
      for (const VexNode *sd : bs.all("stream_def"))
        if (sd->at(1).str() == "mag") return 2;
      return 1;
    }
  }
  if (fmt == "Mark4" || fmt == "VLBA" || fmt == "Mark5B") {
    const VexNode &tr = *require_def(vex_, "TRACKS", vex_.section("TRACKS", mode, st));
    for (const VexNode *fd : tr.all("fanout_def"))
      if (fd->at(2).str() == "mag") return 2;
    return 1;
  }
  fail("Unable to determine bits/sample");
}

int Control::sample_rate(const std::string &mode, const std::string &st) const {  // 820-828
  const VexNode *sr = freq_def(mode, st).get("sample_rate");
  if (!sr) fail("no sample_rate in the $FREQ def of " + st);
  return (int)(sr->to_double_amount("Ms/sec") * 1e6);
}

int Control::bandwidth(const std::string &mode, const std::string &st, const std::string &ch) const {
  for (const VexNode *cd : freq_def(mode, st).all("chan_def"))
    if (cd->at(4).str() == ch) return (int)cd->at(3).to_double_amount("Hz");
  fail("channel " + ch + " not in the $FREQ def of " + st);
}

int64_t Control::channel_freq(const std::string &mode, const std::string &st, const std::string &ch) const {
  for (const VexNode *cd : freq_def(mode, st).all("chan_def"))
    if (cd->at(4).str() == ch) return (int64_t)std::llround(cd->at(1).to_double_amount("Hz"));
  fail("channel " + ch + " not in the $FREQ def of " + st);
}

std::string Control::scan_source(const std::string &scan) const {
  const VexNode *s = vex_.def("SCHED", scan);
  if (!s || !s->get("source")) fail("scan " + scan + " has no source");
  return s->get("source")->str();
}

// scan(const Time&) (866-876): the first scan whose stop is after t
int Control::scan_at(ticks_t t) const {
  // Time::date_string's "%04dy%03dd%02dh%02dm%02d.%03ds" read back by Date (fraction dropped)
  int year, day;
  date_of_ticks(t, year, day);
  const ticks_t per_day = (ticks_t)(86400 * kClock);
  double frac = (double)(t % per_day) / (kClock * 86400);
  int ms = (int)std::round(86400.0 * 1000 * frac);
  VexDate d;
  d.year = year;
  d.day = day;
  d.hour = ms / 3600000;
  d.minute = (ms / 60000) % 60;
  d.second = (ms / 1000) % 60;
  for (size_t i = 0; i < number_scans(); i++)
    if (d < vex_.stop_of_scan(scan(i))) return (int)i;
  return -1;
}

bool Control::station_in_scan(const std::string &scan, const std::string &st) const {
  const VexNode &s = *require_def(vex_, "SCHED", scan);
  for (const VexNode *e : s.all("station"))
    if (e->at(0).str() == st) return true;
  return false;
}

// stop_time(scan, station) (891-902): scan start + the station's duration in microseconds... of
// "N sec" read as seconds
ticks_t Control::station_stop_time(const std::string &scan, const std::string &st) const {
  const VexNode &s = *require_def(vex_, "SCHED", scan);
  ticks_t start = time_of_string(vex_.start_of_scan(scan).to_string());
  for (const VexNode *e : s.all("station"))
    if (e->at(0).str() == st) return start + ticks_usec(e->at(2).to_double_amount("usec"));
  return start;
}

// frequency_channel (942-994)
std::string Control::frequency_channel(size_t nr, const std::string &mode, const std::string &st) const {
  if (nr >= number_frequency_channels()) fail("channel number out of range");
  const std::string setup = setup_station(), chn = channel(nr);
  char pol = polarisation(chn, setup, mode);
  if (pol == ' ') return std::string();
  int64_t fmin, fmax;
  if (sideband(chn, setup, mode) == 'L') {
    fmax = channel_freq(mode, setup, chn);
    fmin = fmax - bandwidth(mode, setup, chn);
  } else {
    fmin = channel_freq(mode, setup, chn);
    fmax = fmin + bandwidth(mode, setup, chn);
  }
  for (const VexNode *cd : freq_def(mode, st).all("chan_def")) {
    int64_t cmin, cmax;
    if (cd->at(2).to_char() == 'L') {
      cmax = (int64_t)std::llround(cd->at(1).to_double_amount("Hz"));
      cmin = cmax - (int)cd->at(3).to_double_amount("Hz");
    } else {
      cmin = (int64_t)std::llround(cd->at(1).to_double_amount("Hz"));
      cmax = cmin + (int)cd->at(3).to_double_amount("Hz");
    }
    const std::string &name = cd->at(4).str();
    // the subband lies inside this channel, or this channel inside the subband
    if (fmin >= cmin && fmax <= cmax && pol == polarisation(name, st, mode)) return name;
    if (cmin >= fmin && cmax <= fmax && pol == polarisation(name, st, mode)) return name;
  }
  return std::string();
}

// frequency_number (996-1022): rank of the channel's frequency among the setup station's
int Control::frequency_number(size_t nr, const std::string &mode) const {
  const std::string chn = channel(nr);
  std::set<int64_t> freqs;
  int64_t f = INT64_MIN;
  for (const VexNode *cd : freq_def(mode, setup_station()).all("chan_def")) {
    int64_t v = (int64_t)std::llround(cd->at(1).to_double_amount("Hz"));
    if (cd->at(4).str() == chn) f = v;
    freqs.insert(v);
  }
  int k = 0;
  for (int64_t v : freqs) {
    if (v == f) return k;
    k++;
  }
  return -1;
}

bool Control::cross_polarize() const {  // 1620-1634
  if (!ctrl_["cross_polarize"].as_bool()) return false;
  for (const auto &m : vex_.block("MODE").dict)
    for (size_t i = 0; i < number_frequency_channels(); i++)
      if (cross_channel((int)i, m.first) != -1) return true;
  return false;
}

int Control::cross_channel(int nr, const std::string &mode) const {
  if (nr < 0 || nr >= (int)number_frequency_channels()) return -1;
  return cross_channel(channel(nr), mode);
}

// cross_channel (1644-1667): same frequency and sideband, other polarisation
int Control::cross_channel(const std::string &chn, const std::string &mode) const {
  const std::string setup = setup_station();
  std::string f = frequency(chn, setup, mode);
  if (f.empty()) return -1;
  char side = sideband(chn, setup, mode), pol = polarisation(chn, setup, mode);
  if (pol == ' ') return -1;
  for (size_t i = 0; i < number_frequency_channels(); i++) {
    std::string other = channel(i);
    if (other != chn && f == frequency(other, setup, mode) && side == sideband(other, setup, mode) &&
        pol != polarisation(other, setup, mode))
      return (int)i;
  }
  return -1;
}

// polarisation (1669-1735): chan_def -> BBC -> IF -> its polarisation
char Control::polarisation(const std::string &chn, const std::string &st, const std::string &mode) const {
  require_def(vex_, "MODE", mode);
  const VexNode &fd = freq_def(mode, st);
  std::string ifn = vex_.section("IF", mode, st);
  if (ifn.empty()) fail("Cannot find $IF reference for " + st + " in mode " + mode);
  require_def(vex_, "IF", ifn);
  std::string bbcn = vex_.section("BBC", mode, st);
  if (bbcn.empty()) fail("Cannot find $BBC reference for " + st + " in mode " + mode);
  const VexNode &bbc = *require_def(vex_, "BBC", bbcn);
  std::string bbc_ref, if_ref;
  for (const VexNode *cd : fd.all("chan_def"))
    if (cd->at(4).str() == chn) bbc_ref = cd->at(5).str();
  for (const VexNode *ba : bbc.all("BBC_assign"))
    if (ba->at(0).str() == bbc_ref) if_ref = ba->at(2).str();
  return vex_.polarisation(ifn, if_ref);
}

namespace {
// The def name of the first element of each `ref $<sec>` line of a mode in
// which `station` appears at any position (the reference's loops over every
// element, control_parameters.cc:1774-1783,1796-1823); the last match wins.
std::string mode_ref_any(const Vex &v, const std::string &mode, const std::string &sec, const std::string &st,
                         size_t from) {
  std::string r;
  const VexNode *m = v.def("MODE", mode);
  if (!m) return r;
  for (const VexNode *ref : m->all(sec)) {
    if (ref->kind == VexNode::STR) {
      if (from == 0 && ref->s == st) r = ref->s;
      continue;
    }
    for (size_t i = from; i < ref->list.size(); i++)
      if (ref->list[i].kind == VexNode::STR && ref->list[i].s == st) r = ref->list[0].s;
  }
  return r;
}
}  // namespace

// frequency (1767-1795): the chan_def's frequency text
std::string Control::frequency(const std::string &chn, const std::string &st, const std::string &mode) const {
  std::string fn = mode_ref_any(vex_, mode, "FREQ", st, 0);
  if (fn.empty()) return std::string();
  const VexNode &fd = *require_def(vex_, "FREQ", fn);
  for (const VexNode *cd : fd.all("chan_def"))
    if (cd->at(4).str() == chn) return cd->at(1).str();
  return std::string();
}

// sideband (1797-1844): field 2 of the chan_def that names the channel anywhere
char Control::sideband(const std::string &chn, const std::string &st, const std::string &mode) const {
  std::string fn = mode_ref_any(vex_, mode, "FREQ", st, 0);
  const VexNode *fd = vex_.def("FREQ", fn);
  if (!fd) fail("Cannot find $FREQ reference for " + st + " in mode " + mode);
  char sb = 'x';
  for (const VexNode *cd : fd->all("chan_def")) {
    if (cd->kind != VexNode::LIST) continue;
    for (const VexNode &e : cd->list)
      if (e.kind == VexNode::STR && e.s == chn) sb = cd->at(2).to_char();
  }
  return sb;
}

int Control::number_correlation_cores_per_timeslice(const std::string &mode) const {  // 920-931
  if (!cross_polarize()) return (int)number_frequency_channels();
  int n = 0;
  for (int i = 0; i < (int)number_frequency_channels(); i++) {
    int x = cross_channel(i, mode);
    if (x == -1 || x > i) n++;
  }
  return n;
}

int Control::polarisation_type_for_global_output_header(const std::string &mode) const {  // 1737-1765
  if (cross_polarize()) return 3;
  bool left = false, right = false;
  std::string st = setup_station();
  for (size_t i = 0; i < number_frequency_channels(); i++) {
    std::string name = frequency_channel(i, mode, st);
    if (name.empty()) continue;
    char pol = (char)std::toupper((unsigned char)polarisation(name, st, mode));
    if (pol == 'L') left = true;
    if (pol == 'R') right = true;
  }
  if (left && right) return 2;
  if (left) return 0;
  if (!right) fail("no channel with a polarisation for the global header");
  return 1;
}

// ---------------------------------------------------------------- input node parameters

void Control::fill_channel(InputChannel &c, size_t ch_nr, const std::string &mode) const {
  const std::string setup = setup_station();
  c.sideband = sideband(channel(ch_nr), setup, mode);
  c.polarisation = polarisation(channel(ch_nr), setup, mode);
  c.frequency_number = frequency_number(ch_nr, mode);
}

// get_vdif_tracks (1285-1376)
void Control::vdif_tracks(const std::string &mode, const std::string &st, InputParams &p) const {
  std::string tn = vex_.section("THREADS", mode, st);
  if (tn.empty()) fail("Cannot find $THREADS reference for " + st + " in mode" + mode);
  const VexNode &th = *require_def(vex_, "THREADS", tn);
  auto threads = th.all("thread");
  auto chans = th.all("channel");
  p.frame_size = 0;
  if (!threads.empty()) p.frame_size = threads[0]->at(8).to_int();
  const int bits = bits_per_sample(mode, st);
  if (threads.size() == chans.size()) {  // one channel per thread: no extraction
    p.n_tracks = 0;
    for (size_t ch = 0; ch < number_frequency_channels(); ch++) {
      std::string name = frequency_channel(ch, mode, st);
      InputChannel c;
      int thread_id = -1;
      for (const VexNode *e : chans)
        if (e->at(0).str() == name) thread_id = e->at(1).to_int();
      c.bits_per_sample = bits;
      fill_channel(c, ch, mode);
      c.tracks = {thread_id, -1};
      p.channels.push_back(c);
    }
    return;
  }
  const int n_tracks = bits * (int)chans.size();
  p.n_tracks = n_tracks;
  for (size_t ch = 0; ch < number_frequency_channels(); ch++) {
    std::string name = frequency_channel(ch, mode, st);
    if (name.empty()) continue;
    InputChannel c;
    c.bits_per_sample = bits;
    fill_channel(c, ch, mode);
    const int word = n_tracks <= 32 ? 32 : n_tracks;
    for (int i = 0; i < word; i += n_tracks)
      for (const VexNode *e : chans)
        if (e->at(0).str() == name)
          for (int t = bits - 1; t >= 0; t--) c.tracks.push_back(e->at(2).to_int() * bits + t + i);
    p.channels.push_back(c);
  }
}

// get_mark5b_tracks (1143-1283)
void Control::mark5b_tracks(const std::string &mode, const std::string &st, InputParams &p) const {
  auto expand = [](InputChannel &c, int sign, int mag, int n_streams) {
    const int word = n_streams <= 32 ? 32 : 64;
    for (int i = 0; i < word / n_streams; i++) {
      c.tracks.push_back(sign + i * n_streams);
      if (c.bits_per_sample == 2) c.tracks.push_back(mag + i * n_streams);
    }
  };
  std::string bn = vex_.section("BITSTREAMS", mode, st);
  if (!bn.empty()) {
    const VexNode &bs = *require_def(vex_, "BITSTREAMS", bn);
    auto defs = bs.all("stream_def");
    p.n_tracks = (int)defs.size();
    for (size_t ch = 0; ch < number_frequency_channels(); ch++) {
      std::string name = frequency_channel(ch, mode, st);
      if (name.empty()) continue;
      InputChannel c;
      c.bits_per_sample = 1;
      fill_channel(c, ch, mode);
      int sign = INT32_MIN, mag = INT32_MIN;
      for (const VexNode *d : defs)
        if (d->at(0).str() == name) {
          if (d->at(1).str() == "sign") {
            sign = d->at(3).to_int();
          } else {
            c.bits_per_sample = 2;
            mag = d->at(3).to_int();
          }
        }
      if (sign == INT32_MIN || (c.bits_per_sample == 2 && mag == INT32_MIN))
        fail("no sign/magnitude bitstream for channel " + name);
      expand(c, sign, mag, (int)defs.size());
      p.channels.push_back(c);
    }
    return;
  }
  std::string tn = vex_.section("TRACKS", mode, st);
  if (!tn.empty()) {
    const VexNode &tr = *require_def(vex_, "TRACKS", tn);
    const VexNode *ff = tr.get("track_frame_format");
    if (!ff) fail("no track_frame_format in $TRACKS def " + tn);
    if (ff->str() == "Mark5B" || ff->str() == "MARK5B") {
      auto fds = tr.all("fanout_def");
      int n = 0;
      for (const VexNode *fd : fds) n += fd->kind == VexNode::LIST && fd->list.size() > 4 ? (int)fd->list.size() - 4 : 0;
      p.n_tracks = n;
      for (size_t ch = 0; ch < number_frequency_channels(); ch++) {
        std::string name = frequency_channel(ch, mode, st);
        if (name.empty()) continue;
        InputChannel c;
        c.bits_per_sample = 1;
        fill_channel(c, ch, mode);
        int sign = INT32_MIN, mag = INT32_MIN;
        for (const VexNode *fd : fds)
          if (fd->at(1).str() == name) {
            if (fd->at(2).str() == "sign") {
              sign = fd->at(4).to_int() - 2;
            } else {
              c.bits_per_sample = 2;
              mag = fd->at(4).to_int() - 2;
            }
          }
        if (sign == INT32_MIN || (c.bits_per_sample == 2 && mag == INT32_MIN))
          fail("no sign/magnitude track for channel " + name);
        expand(c, sign, mag, (int)fds.size());
        p.channels.push_back(c);
      }
      return;
    }
  }
  mark5b_standard_mapping(mode, st, p);
}

// get_mark5b_standard_mapping (1378-1481): upper sidebands of the BBCs in
// BBC-number order, then the lower ones, one bitstream (pair) each
void Control::mark5b_standard_mapping(const std::string &mode, const std::string &st, InputParams &p) const {
  const int bits = bits_per_sample(mode, st);
  std::string bbcn = vex_.section("BBC", mode, st), fn = vex_.section("FREQ", mode, st);
  if (bbcn.empty()) fail("Error : couldn't find BBC section for station " + st + ".");
  if (fn.empty()) fail("Error : couldn't find FREQ section for station " + st + ".");
  std::map<int, std::string> by_nr;
  for (const VexNode *ba : require_def(vex_, "BBC", bbcn)->all("BBC_assign")) by_nr[ba->at(1).to_int()] = ba->at(0).str();
  std::map<std::string, int> track_of;
  int stream = 0;
  auto cds = require_def(vex_, "FREQ", fn)->all("chan_def");
  for (const char *sbd : {"U", "L"})
    for (const auto &kv : by_nr)
      for (const VexNode *cd : cds)
        if (cd->at(2).str() == sbd && cd->at(5).str() == kv.second) track_of[cd->at(4).str()] = stream++;
  const int nstreams = (int)track_of.size() * bits;
  p.n_tracks = nstreams;
  for (size_t ch = 0; ch < number_frequency_channels(); ch++) {
    std::string name = frequency_channel(ch, mode, st);
    if (name.empty()) continue;
    auto it = track_of.find(name);
    int b = (it == track_of.end() ? 0 : it->second) * bits;
    InputChannel c;
    c.bits_per_sample = bits;
    fill_channel(c, ch, mode);
    for (; b < 32; b += nstreams) {
      c.tracks.push_back(b);
      if (bits == 2) c.tracks.push_back(b + 1);
    }
    p.channels.push_back(c);
  }
}

// get_mark5a_tracks (1046-1141): track numbers of the head stacks compacted
// into bit positions
void Control::mark5a_tracks(const std::string &mode, const std::string &st, InputParams &p) const {
  const VexNode &tr = *require_def(vex_, "TRACKS", vex_.section("TRACKS", mode, st));
  auto fds = tr.all("fanout_def");
  std::vector<int> pos(64, 0);
  int n = 0;
  for (const VexNode *fd : fds) {
    int hs = fd->at(3).to_int();
    for (size_t k = 4; k < fd->list.size(); k++) {
      int idx = 32 * (hs - 1) + fd->list[k].to_int() - 2;
      if (idx < 0 || idx >= 64) fail("track number out of range in $TRACKS");
      pos[idx] = 1;
      n++;
    }
  }
  for (int i = 0, bit = -1; i < 64; i++) {
    bit += pos[i];
    pos[i] *= bit;
  }
  p.n_tracks = n;
  const VexNode *mod = tr.get("data_modulation");
  p.data_modulation = mod && mod->kind == VexNode::STR && mod->s == "on" ? 1 : 0;
  for (size_t ch = 0; ch < number_frequency_channels(); ch++) {
    std::string name = frequency_channel(ch, mode, st);
    if (name.empty()) continue;
    InputChannel c;
    c.bits_per_sample = 1;
    fill_channel(c, ch, mode);
    std::vector<int> sign, mag;
    for (const VexNode *fd : fds) {
      if (fd->at(1).str() != name) continue;
      int hs = fd->at(3).to_int();
      bool is_sign = fd->at(2).str() == "sign";
      if (!is_sign) c.bits_per_sample = 2;
      for (size_t k = 4; k < fd->list.size(); k++)
        (is_sign ? sign : mag).push_back(pos[(hs - 1) * 32 + fd->list[k].to_int() - 2]);
    }
    if (c.bits_per_sample == 2 && mag.size() != sign.size())
      fail("Number of magnitude tracks do not match the number of sign tracks");
    for (size_t i = 0; i < sign.size(); i++) {
      c.tracks.push_back(sign[i]);
      if (c.bits_per_sample == 2) c.tracks.push_back(mag[i]);
    }
    p.channels.push_back(c);
  }
}

// get_input_node_parameters (1483-1555)
InputParams Control::input_node_parameters(const std::string &mode, const std::string &st,
                                          ticks_t reader_offset) const {
  InputParams p;
  p.fft_size = std::max(fft_size_delaycor(), fft_size_correlation());
  p.integr_time = integration_time();
  p.offset = reader_offset;
  p.phasecal_integr_time = phasecal_integration_time();
  p.exit_on_empty_datastream = exit_on_empty_datastream();
  require_def(vex_, "MODE", mode);
  freq_def(mode, st);
  std::string ifn = vex_.section("IF", mode, st);
  if (ifn.empty()) fail("Cannot find $IF reference for " + st + " in mode " + mode);
  require_def(vex_, "IF", ifn);
  std::string bbcn = vex_.section("BBC", mode, st);
  if (bbcn.empty()) fail("Cannot find $BBC reference for " + st + " in mode " + mode);
  require_def(vex_, "BBC", bbcn);
  // mixed bandwidths: enough samples for the widest station
  p.fft_size = (int)(((uint64_t)p.fft_size * (uint64_t)sample_rate(mode, st)) / (uint64_t)sample_rate(mode, setup_station()));
  if (p.fft_size == 0) fail("fft size 0 for station " + st);
  p.track_bit_rate = sample_rate(mode, st);
  p.data_format = data_format(st);
  if (p.data_format == "VDIF")
    vdif_tracks(mode, st, p);
  else if (p.data_format == "Mark4" || p.data_format == "VLBA")
    mark5a_tracks(mode, st, p);
  else if (p.data_format == "Mark5B")
    mark5b_tracks(mode, st, p);
  else
    fail("station " + st + ": data format '" + p.data_format + "' is not supported");
  if (p.channels.empty() || p.channels[0].tracks.empty()) fail("station " + st + " has no channel in mode " + mode);
  p.track_bit_rate /= (int)p.channels[0].tracks.size() / p.channels[0].bits_per_sample;
  return p;
}

// ---------------------------------------------------------------- correlation parameters

// get_correlation_parameters (1867-2022)
JobParams Control::correlation_parameters(const std::string &scan, size_t channel_nr,
                                          const std::map<std::string, int> &to_input) const {
  const VexNode &sc = *require_def(vex_, "SCHED", scan);
  const std::string mode = vex_.mode(scan);
  const VexNode &md = *require_def(vex_, "MODE", mode);
  const std::string setup = setup_station();
  const std::string chn = frequency_channel(channel_nr, mode, setup);
  JobParams j;
  j.experiment_start = time_of_string(vex_.start_time_of_experiment());
  j.start_time = ticks_usec((double)(vex_.start_of_scan(scan).ms_of_day() * 1000));
  j.stop_time = ticks_usec((double)(vex_.stop_of_scan(scan).ms_of_day() * 1000));
  j.integration_time = integration_time();
  j.sub_integration_time = sub_integration_time();
  j.number_channels = number_channels();
  j.fft_size_delaycor = fft_size_delaycor();
  j.fft_size_correlation = fft_size_correlation();
  j.window = window_function();
  j.slice_offset = number_correlation_cores_per_timeslice(mode);
  j.sample_rate = sample_rate(mode, setup);
  j.sideband = ' ';
  std::string bbc_nr;
  for (const VexNode *cd : freq_def(mode, setup).all("chan_def"))
    if (cd->at(4).str() == chn) {
      j.channel_freq = (int64_t)std::llround(cd->at(1).to_double_amount("Hz"));
      j.bandwidth = (int)cd->at(3).to_double_amount("Hz");
      j.sideband = cd->at(2).to_char();
      bbc_nr = cd->at(5).str();
    }
  j.frequency_nr = frequency_number(channel_nr, mode);
  std::string if_mode = mode_ref_any(vex_, mode, "IF", setup, 0);
  std::string bbc_mode = mode_ref_any(vex_, mode, "BBC", setup, 1);
  (void)md;
  std::string if_nr;
  if (const VexNode *bb = vex_.def("BBC", bbc_mode)) {
    for (const auto &kv : bb->dict) {
      const VexNode &e = kv.second;
      if (e.kind != VexNode::LIST) continue;
      for (const VexNode &x : e.list)
        if (x.kind == VexNode::STR && x.s == bbc_nr) if_nr = e.at(2).str();
    }
  } else {
    fail("Cannot find $BBC reference for " + setup + " in mode " + mode);
  }
  j.polarisation = vex_.polarisation(if_mode, if_nr);
  if (j.sideband != 'L' && j.sideband != 'U') fail("channel " + channel(channel_nr) + " has no sideband for " + setup);
  j.cross_polarize = cross_polarize() && cross_channel(chn, mode) != -1;
  j.reference_station = reference_station_number();

  auto add_stations = [&](size_t nr, bool second) {
    std::set<int> seen;
    for (const JobStation &s : j.stations) seen.insert(s.station_number);
    for (const VexNode *e : sc.all("station")) {
      const std::string name = e->at(0).str();
      auto it = to_input.find(name);
      if (it == to_input.end() || it->second < 0) continue;
      const std::string cn = frequency_channel(nr, mode, name);
      if (cn.empty()) continue;
      JobStation s;
      s.station_number = station_number(name);
      s.station_stream = second && seen.count(s.station_number) ? it->second + (int)number_stations() : it->second;
      s.start_time = ticks_usec((double)e->at(1).to_int_amount("sec"));
      s.stop_time = ticks_usec((double)e->at(2).to_int_amount("sec"));
      s.bits_per_sample = bits_per_sample(mode, name);
      s.sample_rate = sample_rate(mode, name);
      s.channel_freq = channel_freq(mode, name, cn);
      s.bandwidth = bandwidth(mode, name, cn);
      s.sideband = sideband(cn, name, mode);
      s.polarisation = polarisation(cn, name, mode);
      s.lo_offset = lo_offset(name);
      s.tsys_freq = tsys_freq(name);
      j.stations.push_back(s);
    }
  };
  add_stations(channel_nr, false);
  if (!cross_polarize()) return j;
  int x = cross_channel((int)channel_nr, mode);
  if (x < 0) fail("cross-polarised correlation: channel " + channel(channel_nr) + " has no partner");
  add_stations((size_t)x, true);
  return j;
}

// Manager_node::initialise_scan (manager_node.cc:532-576): the clock_early
// line in force at the scan start, the whole seconds moved to the reader
ClockModel Control::clock(const std::string &st, ticks_t scan_start, const std::string &scan) const {
  const VexNode &sd = *require_def(vex_, "STATION", st);
  const VexNode *cr = sd.get("CLOCK");
  if (!cr) fail("Cannot find $CLOCK reference for " + st);
  const VexNode &cd = *require_def(vex_, "CLOCK", cr->str());
  auto lines = cd.all("clock_early");
  if (lines.empty()) fail("Cannot find clock for " + st);
  ClockModel m;
  bool found = false;
  for (const VexNode *l : lines) {
    ticks_t t = time_of_string(l->at(0).str());
    if (scan_start < t) continue;
    if (m.start > t) continue;
    m.start = t;
    found = true;
    m.offset = l->at(1).to_double_amount("sec");
    m.rate = 0;
    if (l->size() > 3) {
      const std::string &r = l->at(3).str();
      if (r.find_first_of("\t ") != std::string::npos)
        m.rate = l->at(3).to_double_amount("sec/sec");
      else
        m.rate = l->at(3).to_double() * 1e-6;  // a rate without units is in usec/sec
      m.epoch = time_of_string(l->at(2).str());
    }
  }
  if (!found || m.start == 0) fail("Clock doesn't cover scan " + scan + " for station " + st);
  double reader = std::round(m.offset / 1.0) * 1.0;
  m.offset -= reader;
  m.reader_offset = ticks_usec(reader * 1e6);
  return m;
}

// ---------------------------------------------------------------- the manager's plan

Plan make_plan(const Control &c, const std::function<ticks_t(int, int)> &station_time) {
  Plan plan;
  const Vex &vex = c.vex();
  const int nst = (int)c.number_stations();
  if (nst <= 0) fail("ctrl file: no stations");
  plan.start = c.start_time();
  plan.stop = c.stop_time();
  const ticks_t tint = c.integration_time();
  if (tint <= 0) fail("ctrl file: integr_time must be positive");
  std::map<std::string, int> to_input;
  for (int s = 0; s < nst; s++) to_input[c.station(s)] = s;

  int scan_nr = c.scan_at(plan.start);  // Manager_node::initialise (manager_node.cc:402-418)
  if (scan_nr < 0) fail("Cannot find scan corresponding to the start time");

  // output files (420-472)
  const std::string out = c.output_file();
  if (c.pulsar_binning()) {
    int maxbins = 2;
    for (const PulsarSpec &p : c.pulsars()) maxbins = std::max(p.nbins + 1, maxbins);
    for (int b = 0; b < maxbins; b++) plan.output_files.push_back(out + ".bin" + std::to_string(b));
  } else if (c.multi_phase_center()) {
    // the sources of the scans from the one holding the start time until the stop
    VexDate t0(""), t1("");
    {
      int y, d;
      date_of_ticks(plan.start, y, d);
      const ticks_t per_day = (ticks_t)(86400 * kClock);
      int ms0 = (int)std::round(86400.0 * 1000 * ((double)(plan.start % per_day) / (kClock * 86400)));
      t0.year = y, t0.day = d, t0.hour = ms0 / 3600000, t0.minute = (ms0 / 60000) % 60, t0.second = (ms0 / 1000) % 60;
      date_of_ticks(plan.stop, y, d);
      int ms1 = (int)std::round(86400.0 * 1000 * ((double)(plan.stop % per_day) / (kClock * 86400)));
      t1.year = y, t1.day = d, t1.hour = ms1 / 3600000, t1.minute = (ms1 / 60000) % 60, t1.second = (ms1 / 1000) % 60;
    }
    std::string first = vex.scan_name(t0);
    std::set<std::string> sources;
    const auto &sched = vex.block("SCHED").dict;
    for (auto it = sched.find(first); it != sched.end() && vex.start_of_scan(it->first) < t1; ++it)
      for (const VexNode *s : it->second.all("source")) sources.insert(s->str());
    for (const auto &s : sources) {
      plan.sources.push_back(s);
      plan.output_files.push_back(out + "_" + s);
    }
  } else {
    plan.output_files.push_back(out);
  }

  // global header (send_global_header, manager_node.cc:660-683)
  plan.header.experiment = c.exper_name();
  date_of_ticks(plan.start, plan.header.start_year, plan.header.start_day);
  {
    const ticks_t per_day = (ticks_t)(86400 * kClock);
    plan.header.start_time = (int)((double)(plan.start % per_day) / kClock);
    plan.header.integration_time = (int)((double)(tint % per_day) / (kClock / 1000000));
  }
  plan.header.number_channels = c.number_channels();
  plan.header.polarisation_type = c.polarisation_type_for_global_output_header(vex.mode(c.scan(scan_nr)));
  plan.header.job_nr = c.job_nr();
  plan.header.subjob_nr = c.subjob_nr();

  // the manager's state machine (start, 150-277; start_next_timeslice_on_node, 284-391)
  int slice_nr = 0, output_slice = 0;
  const int nch = (int)c.number_frequency_channels();
  bool stop = false;
  while (!stop) {
    // START_NEW_SCAN: initialise_scan (493-626)
    const std::string scan = c.scan(scan_nr);
    PlannedScan ps;
    ps.name = scan;
    ps.mode = vex.mode(scan);
    ps.source = c.scan_source(scan);
    ps.n_sources = vex.n_sources(scan);
    VexDate ds = vex.start_of_scan(scan), de = vex.stop_of_scan(scan);
    ticks_t scan_start = ticks_mjd_sec(mjd_from_date(1, 1, ds.year) + ds.day - 1, ds.ms_of_day() / 1000.);
    if (plan.start + tint * slice_nr < scan_start) {
      ticks_t iv = scan_start - plan.start;
      slice_nr = (int)((double)iv / (double)tint);
      if (iv % tint != 0) slice_nr++;
    }
    ticks_t stop_scan = ticks_mjd_sec(mjd_from_date(1, 1, de.year) + de.day - 1, de.ms_of_day() / 1000.);
    if (plan.stop < stop_scan) stop_scan = plan.stop;
    if ((stop_scan - plan.start) % tint < 0) fail("scan " + scan + " ends before the correlation start");
    stop_scan -= (stop_scan - plan.start) % tint;
    ps.start = scan_start;
    ps.stop = stop_scan;
    for (int s = 0; s < nst; s++) {
      const std::string st = c.station(s);
      if (!c.station_in_scan(scan, st)) continue;
      ScanStation ss;
      ss.station = s;
      ss.name = st;
      ss.delay_file = c.delay_table_name(st);
      ss.clock = c.clock(st, scan_start, scan);
      ss.input = c.input_node_parameters(ps.mode, st, ss.clock.reader_offset);
      ss.stop_time = c.station_stop_time(scan, st);
      ps.stations.push_back(ss);
    }
    // which channels each station takes part in, numbered per station (606-625)
    std::vector<int> last(nst, -1);
    ps.ch_number_in_scan.assign(nch, std::vector<int>(nst, -1));
    for (int i = 0; i < nch; i++)
      for (int s = 0; s < nst; s++) {
        if (!c.station_in_scan(scan, c.station(s))) continue;
        if (!c.frequency_channel(i, ps.mode, c.station(s)).empty()) ps.ch_number_in_scan[i][s] = ++last[s];
      }
    // the input nodes' times can start the scan later (171-182)
    std::vector<bool> in_scan(nst, false);
    for (int s = 0; s < nst; s++)
      for (int i = 0; i < nch; i++)
        if (ps.ch_number_in_scan[i][s] >= 0) in_scan[s] = true;
    if (station_time)
      for (int s = 0; s < nst; s++) {
        if (!in_scan[s]) continue;
        ticks_t t = station_time(s, (int)plan.scans.size());
        if (t > plan.start + tint * slice_nr) slice_nr = (int)((double)(t - plan.start) / (double)tint);
      }
    if (plan.stop <= plan.start + tint * slice_nr) break;
    ps.first_slice_start = plan.start + tint * slice_nr;
    const int scan_index = (int)plan.scans.size();
    plan.scans.push_back(ps);
    const PlannedScan &cur = plan.scans.back();
    const bool xpol = c.cross_polarize();
    for (;;) {
      // START_CORRELATION_TIME_SLICE .. START_CORRELATOR_NODES_FOR_TIME_SLICE
      int ch = 0;
      while (ch < nch) {
        int xch = xpol ? c.cross_channel(ch, cur.mode) : -1;
        if (xch != -1 && xch <= ch) fail("cross channel ordering");
        PlannedJob job;
        job.scan = scan_index;
        job.channel = ch;
        job.cross_channel = xch;
        job.params = c.correlation_parameters(scan, ch, to_input);
        job.params.start_time = plan.start + tint * slice_nr;
        job.params.stop_time = plan.start + tint * (slice_nr + 1);
        job.params.integration_nr = slice_nr;
        job.params.slice_nr = output_slice;
        job.params.source = cur.source.substr(0, 11);  // strncpy into char[11]
        job.params.pulsar_binning = c.pulsar_binning();
        job.params.n_phase_centers = c.multi_phase_center() ? cur.n_sources : 1;
        for (int s = 0; s < nst; s++) {
          int stream = 0;  // stream numbers of one correlator node: main, then cross
          if (cur.ch_number_in_scan[ch][s] >= 0) {
            job.inputs.push_back({s, cur.ch_number_in_scan[ch][s], s});
            stream = 1;
          }
          if (xch != -1 && cur.ch_number_in_scan[xch][s] >= 0)
            job.inputs.push_back({s, cur.ch_number_in_scan[xch][s], stream ? s + nst : s});
        }
        plan.jobs.push_back(job);
        output_slice++;
        ch++;
        if (xpol) {
          int x = c.cross_channel(ch, cur.mode);
          while (ch < nch && x >= 0 && x < ch) {
            ch++;
            x = c.cross_channel(ch, cur.mode);
          }
        }
      }
      // GOTO_NEXT_TIMESLICE
      slice_nr++;
      if (plan.start + tint * (slice_nr + 1) > plan.stop) {
        stop = true;
        break;
      }
      if (plan.start + tint * (slice_nr + 1) > stop_scan) {
        if (++scan_nr == (int)c.number_scans()) stop = true;
        break;
      }
    }
  }
  return plan;
}

// ---------------------------------------------------------------- JSON form

namespace {
Json chr(char ch) { return Json::of_string(ch ? std::string(1, ch) : std::string()); }
Json ints(const std::vector<int32_t> &v) {
  Json a;
  for (int x : v) a.append(Json::of_int(x));
  if (v.empty()) a = Json::parse("[]");
  return a;
}
Json input_json(const InputParams &p) {
  Json j;
  j.set("data_format", Json::of_string(p.data_format));
  j.set("n_tracks", Json::of_int(p.n_tracks));
  j.set("track_bit_rate", Json::of_int(p.track_bit_rate));
  j.set("frame_size", Json::of_int(p.frame_size));
  j.set("fft_size", Json::of_int(p.fft_size));
  j.set("data_modulation", Json::of_int(p.data_modulation));
  j.set("integr_time", Json::of_int(p.integr_time));
  j.set("offset", Json::of_int(p.offset));
  j.set("phasecal_integr_time", Json::of_int(p.phasecal_integr_time));
  j.set("exit_on_empty_datastream", Json::of_bool(p.exit_on_empty_datastream));
  Json chs = Json::parse("[]");
  for (const InputChannel &ch : p.channels) {
    Json x;
    x.set("bits_per_sample", Json::of_int(ch.bits_per_sample));
    x.set("sideband", chr(ch.sideband));
    x.set("polarisation", chr(ch.polarisation));
    x.set("frequency_number", Json::of_int(ch.frequency_number));
    x.set("tracks", ints(ch.tracks));
    chs.append(x);
  }
  j.set("channels", chs);
  return j;
}
Json job_json(const PlannedJob &pj) {
  const JobParams &p = pj.params;
  Json j;
  j.set("scan", Json::of_int(pj.scan));
  j.set("channel", Json::of_int(pj.channel));
  j.set("cross_channel", Json::of_int(pj.cross_channel));
  j.set("experiment_start", Json::of_int(p.experiment_start));
  j.set("start_time", Json::of_int(p.start_time));
  j.set("stop_time", Json::of_int(p.stop_time));
  j.set("integration_time", Json::of_int(p.integration_time));
  j.set("sub_integration_time", Json::of_int(p.sub_integration_time));
  j.set("number_channels", Json::of_int(p.number_channels));
  j.set("fft_size_delaycor", Json::of_int(p.fft_size_delaycor));
  j.set("fft_size_correlation", Json::of_int(p.fft_size_correlation));
  j.set("window", Json::of_int(p.window));
  j.set("integration_nr", Json::of_int(p.integration_nr));
  j.set("slice_nr", Json::of_int(p.slice_nr));
  j.set("slice_offset", Json::of_int(p.slice_offset));
  j.set("sample_rate", Json::of_int(p.sample_rate));
  j.set("bandwidth", Json::of_int(p.bandwidth));
  j.set("frequency_nr", Json::of_int(p.frequency_nr));
  j.set("channel_freq", Json::of_int(p.channel_freq));
  j.set("sideband", chr(p.sideband));
  j.set("polarisation", chr(p.polarisation));
  j.set("cross_polarize", Json::of_bool(p.cross_polarize));
  j.set("reference_station", Json::of_int(p.reference_station));
  j.set("n_phase_centers", Json::of_int(p.n_phase_centers));
  j.set("pulsar_binning", Json::of_bool(p.pulsar_binning));
  j.set("source", Json::of_string(p.source));
  Json st = Json::parse("[]");
  for (const JobStation &s : p.stations) {
    Json x;
    x.set("station_number", Json::of_int(s.station_number));
    x.set("station_stream", Json::of_int(s.station_stream));
    x.set("start_time", Json::of_int(s.start_time));
    x.set("stop_time", Json::of_int(s.stop_time));
    x.set("sample_rate", Json::of_int(s.sample_rate));
    x.set("channel_freq", Json::of_int(s.channel_freq));
    x.set("bandwidth", Json::of_int(s.bandwidth));
    x.set("sideband", chr(s.sideband));
    x.set("polarisation", chr(s.polarisation));
    x.set("bits_per_sample", Json::of_int(s.bits_per_sample));
    x.set("lo_offset", Json::of_double(s.lo_offset));
    x.set("tsys_freq", Json::of_int(s.tsys_freq));
    st.append(x);
  }
  j.set("stations", st);
  Json in = Json::parse("[]");
  for (const JobInput &i : pj.inputs) {
    Json x;
    x.set("station", Json::of_int(i.station));
    x.set("channel_in_scan", Json::of_int(i.channel_in_scan));
    x.set("stream", Json::of_int(i.stream));
    in.append(x);
  }
  j.set("inputs", in);
  return j;
}
}  // namespace

Json plan_json(const Plan &p) {
  Json j;
  j.set("start", Json::of_int(p.start));
  j.set("stop", Json::of_int(p.stop));
  Json h;
  h.set("experiment", Json::of_string(p.header.experiment));
  h.set("start_year", Json::of_int(p.header.start_year));
  h.set("start_day", Json::of_int(p.header.start_day));
  h.set("start_time", Json::of_int(p.header.start_time));
  h.set("number_channels", Json::of_int(p.header.number_channels));
  h.set("integration_time", Json::of_int(p.header.integration_time));
  h.set("polarisation_type", Json::of_int(p.header.polarisation_type));
  h.set("job_nr", Json::of_int(p.header.job_nr));
  h.set("subjob_nr", Json::of_int(p.header.subjob_nr));
  j.set("header", h);
  Json of = Json::parse("[]"), src = Json::parse("[]");
  for (const auto &f : p.output_files) of.append(Json::of_string(f));
  for (const auto &s : p.sources) src.append(Json::of_string(s));
  j.set("output_files", of);
  j.set("sources", src);
  Json scans = Json::parse("[]");
  for (const PlannedScan &s : p.scans) {
    Json x;
    x.set("name", Json::of_string(s.name));
    x.set("mode", Json::of_string(s.mode));
    x.set("source", Json::of_string(s.source));
    x.set("n_sources", Json::of_int(s.n_sources));
    x.set("start", Json::of_int(s.start));
    x.set("stop", Json::of_int(s.stop));
    x.set("first_slice_start", Json::of_int(s.first_slice_start));
    Json sts = Json::parse("[]");
    for (const ScanStation &ss : s.stations) {
      Json y;
      y.set("station", Json::of_int(ss.station));
      y.set("name", Json::of_string(ss.name));
      y.set("delay_file", Json::of_string(ss.delay_file));
      y.set("clock_offset", Json::of_double(ss.clock.offset));
      y.set("clock_rate", Json::of_double(ss.clock.rate));
      y.set("clock_start", Json::of_int(ss.clock.start));
      y.set("clock_epoch", Json::of_int(ss.clock.epoch));
      y.set("reader_offset", Json::of_int(ss.clock.reader_offset));
      y.set("stop_time", Json::of_int(ss.stop_time));
      y.set("input", input_json(ss.input));
      sts.append(y);
    }
    x.set("stations", sts);
    Json chs = Json::parse("[]");
    for (const auto &row : s.ch_number_in_scan) chs.append(ints(row));
    x.set("ch_number_in_scan", chs);
    scans.append(x);
  }
  j.set("scans", scans);
  Json jobs = Json::parse("[]");
  for (const PlannedJob &pj : p.jobs) jobs.append(job_json(pj));
  j.set("jobs", jobs);
  return j;
}

}  // namespace sfxc
