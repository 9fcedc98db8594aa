// The correlator control file and the VEX schedule turned into what the
// correlator-node path needs: the parameters of every (time slice, subband)
// job and of every station's reader, as the reference's Control_parameters
// derives them (sfxc/src/control_parameters.cc) and its manager deals them
// out (Manager_node, sfxc/src/manager_node.cc:164-391,402-683).
#pragma once
#include <cstdint>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "json.hpp"
#include "vex.hpp"

namespace sfxc {

using ticks_t = int64_t;

// Input_node_parameters::Channel_parameters (sfxc/include/control_parameters.h:20-33)
struct InputChannel {
  int bits_per_sample = -1;
  std::vector<int32_t> tracks;  // bit positions of the tracks (VDIF threads: {thread id, -1})
  char sideband = 0, polarisation = 0;
  int frequency_number = -1;
};
// Input_node_parameters (control_parameters.h:15-65)
struct InputParams {
  std::string data_format;  // VDIF, Mark5B, Mark4, VLBA
  std::vector<InputChannel> channels;
  int n_tracks = 0, track_bit_rate = 0, frame_size = -1, fft_size = -1, data_modulation = 0;
  ticks_t integr_time = 0, offset = 0, phasecal_integr_time = 0;
  bool exit_on_empty_datastream = true;
};
// Correlation_parameters::Station_parameters (control_parameters.h:125-142)
struct JobStation {
  int station_number = 0, station_stream = 0;
  ticks_t start_time = 0, stop_time = 0;  // the scan line's offsets, as the reference stores them
  int sample_rate = 0, bandwidth = 0, bits_per_sample = 0, tsys_freq = 80;
  int64_t channel_freq = 0;
  char sideband = 0, polarisation = 0;
  double lo_offset = 0;
};
// Correlation_parameters (control_parameters.h:117-182) as the manager hands it out
struct JobParams {
  ticks_t experiment_start = 0, start_time = 0, stop_time = 0, integration_time = 0, sub_integration_time = 0;
  int number_channels = 0, fft_size_delaycor = 0, fft_size_correlation = 0, window = 0;
  int integration_nr = -1, slice_nr = -1, slice_offset = -1, sample_rate = 0, bandwidth = 0, frequency_nr = -1;
  int64_t channel_freq = 0;
  char sideband = 0, polarisation = 0;
  bool cross_polarize = false, pulsar_binning = false;
  int reference_station = -1, n_phase_centers = 1;
  std::string source;
  std::vector<JobStation> stations;
};

// Delay_table::set_clock_offset arguments of a station in a scan
// (Manager_node::initialise_scan, manager_node.cc:532-576)
struct ClockModel {
  double offset = 0, rate = 0;  // seconds (after the reader's whole-second part), s/s
  ticks_t start = 0, epoch = 0;
  ticks_t reader_offset = 0;    // whole seconds moved into the reader's time
};

// Pulsar_parameters::Polyco_params (control_parameters.h:74-90)
struct PolycoBlock {
  std::string name, date, site;
  float utc = 0, doppler = 0, residual = 0, bin_phase[2] = {0, 0};
  double tmid = 0, dm = 0, ref_phase = 0, ref_freq = 0, obs_freq = 0;
  int32_t data_span = 0, n_coef = 0;
  std::vector<double> coef;
};
struct PulsarSpec {
  std::string name;  // at most 10 characters
  int nbins = 0;
  double gate_start = 0, gate_stop = 1;
  std::vector<PolycoBlock> polyco;
};
// Pulsar_parameters::parse_polyco (control_parameters.cc:2256-2336); throws on
// a malformed file
std::vector<PolycoBlock> parse_polyco(const std::string &path);

class Control {
 public:
  // Control_parameters::initialise (control_parameters.cc:29-230): reads
  // both files and fills in the control file's defaults.  Throws
  // std::runtime_error with the reason.
  void initialise(const std::string &ctrl_path, const std::string &vex_path);
  // the same from texts; ctrl_dir stands for the control file's directory
  void initialise_text(const std::string &ctrl_text, const std::string &vex_text, const std::string &ctrl_dir);

  const Json &ctrl() const { return ctrl_; }
  const Vex &vex() const { return vex_; }

  // ---- the control file
  ticks_t start_time() const;
  ticks_t stop_time() const;
  ticks_t integration_time() const;      // integr_time [s] -> ticks, rounded to microseconds
  ticks_t sub_integration_time() const;  // sub_integr_time [us]
  ticks_t phasecal_integration_time() const;
  int number_channels() const { return ctrl_["number_channels"].as_int(); }
  int fft_size_delaycor() const { return ctrl_["fft_size_delaycor"].as_int(); }
  int fft_size_correlation() const { return ctrl_["fft_size_correlation"].as_int(); }
  int window_function() const;
  size_t number_stations() const { return ctrl_["stations"].size(); }
  std::string station(size_t i) const { return ctrl_["stations"][i].as_string(); }
  size_t number_scans() const { return ctrl_["scans"].size(); }
  std::string scan(size_t i) const { return ctrl_["scans"][i].as_string(); }
  size_t number_frequency_channels() const { return ctrl_["channels"].size(); }
  std::string channel(size_t i) const { return ctrl_["channels"][i].as_string(); }
  std::string setup_station() const;
  int reference_station_number() const;
  double lo_offset(const std::string &station) const;
  int tsys_freq(const std::string &station) const;
  bool pulsar_binning() const { return ctrl_["pulsar_binning"].as_bool(); }
  bool phased_array() const { return ctrl_["phased_array"].as_bool(); }
  bool multi_phase_center() const { return ctrl_["multi_phase_center"].as_bool(); }
  bool exit_on_empty_datastream() const { return ctrl_["exit_on_empty_datastream"].as_bool(); }
  int job_nr() const { return ctrl_["job"].as_int(); }
  int subjob_nr() const { return ctrl_["subjob"].as_int(); }
  // file:// paths relative to the control file's directory made absolute (create_path)
  std::string create_path(const std::string &path) const;
  std::vector<std::string> data_sources(const std::string &station) const;
  std::string output_file() const { return create_path(ctrl_["output_file"].as_string()); }
  // get_delay_table_name without running the delay model generator: the file must exist
  std::string delay_table_name(const std::string &station) const;
  std::vector<PulsarSpec> pulsars() const;                              // get_pulsar_parameters
  // get_mask_parameters: false without a "mask" section
  bool mask(bool &normalize, std::vector<double> &mask, std::vector<double> &window) const;

  // ---- the VEX file
  std::string exper_name() const;
  int station_number(const std::string &station) const;  // index among the $STATION defs, sorted
  std::string transport_type(const std::string &station) const;
  std::string rack_type(const std::string &station) const;
  std::string data_format(const std::string &station) const;
  int bits_per_sample(const std::string &mode, const std::string &station) const;
  int sample_rate(const std::string &mode, const std::string &station) const;
  int bandwidth(const std::string &mode, const std::string &station, const std::string &channel) const;
  int64_t channel_freq(const std::string &mode, const std::string &station, const std::string &channel) const;
  std::string scan_source(const std::string &scan) const;
  int scan_at(ticks_t t) const;  // index of the first scan that ends after t, or -1
  bool station_in_scan(const std::string &scan, const std::string &station) const;
  ticks_t station_stop_time(const std::string &scan, const std::string &station) const;
  std::string frequency_channel(size_t channel_nr, const std::string &mode, const std::string &station) const;
  int frequency_number(size_t channel_nr, const std::string &mode) const;
  bool cross_polarize() const;
  int cross_channel(int channel_nr, const std::string &mode) const;
  int cross_channel(const std::string &channel, const std::string &mode) const;
  char polarisation(const std::string &channel, const std::string &station, const std::string &mode) const;
  std::string frequency(const std::string &channel, const std::string &station, const std::string &mode) const;
  char sideband(const std::string &channel, const std::string &station, const std::string &mode) const;
  int number_correlation_cores_per_timeslice(const std::string &mode) const;
  int polarisation_type_for_global_output_header(const std::string &mode) const;

  InputParams input_node_parameters(const std::string &mode, const std::string &station,
                                    ticks_t reader_offset) const;
  JobParams correlation_parameters(const std::string &scan, size_t channel_nr,
                                   const std::map<std::string, int> &station_to_input) const;
  ClockModel clock(const std::string &station, ticks_t scan_start, const std::string &scan) const;

 private:
  Json ctrl_;
  Vex vex_;
  std::string ctrl_dir_;
  mutable std::map<std::string, int> station_map_;

  const VexNode &freq_def(const std::string &mode, const std::string &station) const;
  void vdif_tracks(const std::string &mode, const std::string &station, InputParams &p) const;
  void mark5b_tracks(const std::string &mode, const std::string &station, InputParams &p) const;
  void mark5b_standard_mapping(const std::string &mode, const std::string &station, InputParams &p) const;
  void mark5a_tracks(const std::string &mode, const std::string &station, InputParams &p) const;
  void fill_channel(InputChannel &c, size_t ch_nr, const std::string &mode) const;
};

// ---- The manager's plan of a whole correlation (single process, one GPU):
// every scan's station set-up and every job in output slice order.
struct ScanStation {
  int station = 0;  // index in the control file's station list
  std::string name, delay_file;
  ClockModel clock;
  InputParams input;
  ticks_t stop_time = 0;  // the station's stop in this scan (Control_parameters::stop_time)
};
struct JobInput {  // Manager_node::start_next_timeslice_on_node's input_node_set_time_slice
  int station = 0, channel_in_scan = 0, stream = 0;
};
struct PlannedJob {
  int scan = 0;      // index into Plan::scans
  int channel = 0;   // channel number (cross channel: cross_channel, else -1)
  int cross_channel = -1;
  JobParams params;
  std::vector<JobInput> inputs;
};
struct PlannedScan {
  std::string name, mode, source;
  int n_sources = 1;
  ticks_t start = 0, stop = 0;  // scan start; stop aligned to the integrations (stop_time_scan)
  ticks_t first_slice_start = 0;
  std::vector<ScanStation> stations;
  std::vector<std::vector<int>> ch_number_in_scan;  // [channel][station]
};
struct OutputHeader {  // Output_header_global fields the manager fills (manager_node.cc:660-683)
  std::string experiment;
  int start_year = 0, start_day = 0, start_time = 0, number_channels = 0, integration_time = 0;
  int polarisation_type = 0, job_nr = 0, subjob_nr = 0;
};
struct Plan {
  ticks_t start = 0, stop = 0;
  OutputHeader header;
  std::vector<std::string> output_files;  // one per pulsar bin / phase-centre source, else one
  std::vector<std::string> sources;       // the multi-phase-centre source list (file index order)
  std::vector<PlannedScan> scans;
  std::vector<PlannedJob> jobs;
};
// station_time(station index, scan index): the input node's current time when
// the scan starts (its reader's position), which can move the first slice of
// the scan later (manager_node.cc:171-182); null: never later than the start.
Plan make_plan(const Control &c, const std::function<ticks_t(int, int)> &station_time = nullptr);
// The plan as JSON (the form the tests compare)
Json plan_json(const Plan &p);

}  // namespace sfxc
