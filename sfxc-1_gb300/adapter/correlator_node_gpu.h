// correlator_node_gpu.h -- the GB300 chain behind SFXC's Correlator_node.
//
// What a maintainer adds to the reference to replace the three task objects
// a correlator node wires up per job -- Bit2float_worker, Delay_correction
// and Correlation_core(_pulsar) (sfxc/src/correlator_node.cc:213-249, polled
// in 263-296) -- with libsfxc_gpu.so.  It is written against the reference's
// own headers and C++ dialect (C++03): Correlation_parameters and
// Pulsar_parameters (sfxc/include/control_parameters.h:69-182), Data_writer
// (sfxc/include/data_writer.h:18-60), sfxc_abort (sfxc/include/utils.h:139),
// the MPI tags of sfxc/include/sfxc_mpi.h.  Build it into the reference with
// -I<repo>/include -L<repo>/sfxc-1_gb300/lib -lsfxc_gpu.
//
// Errors: every library call returns 0 or a negative status; the adapter
// turns a negative status into sfxc_abort(message), which is what the
// reference does on the same conditions (sfxc/src/utils.cc:44-90).
#ifndef CORRELATOR_NODE_GPU_H
#define CORRELATOR_NODE_GPU_H

#include <cstring>
#include <vector>

#include "control_parameters.h"
#include "data_writer.h"
#include "sfxc_gpu.h"
#include "sfxc_mpi.h"
#include "utils.h"

class Correlator_node_gpu {
public:
  // A job in the C ABI's form (sfxc_correlation_params) together with the
  // storage its pointers refer to.  Not copyable: the pointers point into it.
  struct Job {
    Job() { std::memset(&c, 0, sizeof(c)); }
    sfxc_correlation_params c;
    std::vector<sfxc_station_stream> streams;
    std::vector<sfxc_delay_table> tables;
    std::vector<float> mask, lag_window;
    std::vector<sfxc_polyco> polyco;
    std::vector<std::vector<double> > coef;
    std::vector<int32_t> file_index;
  private:
    Job(const Job &);
    Job &operator=(const Job &);
  };

  // Correlation_parameters as Correlator_node::set_parameters receives them
  // (sfxc/src/correlator_node.cc:311-406), flattened: the station streams,
  // the node's delay tables (the bytes of each station's .del file and its
  // clock model; stream_table[i] is stream i's table), the pulsar and its
  // polycos when binning, the ctrl file's Mask_parameters when reducing, and
  // each phase centre's output file index (the manager's source list).
  static void flatten(const Correlation_parameters &p, const std::vector<std::vector<char> > &del_files,
                      const std::vector<int> &stream_table, const std::vector<int32_t> &source_file_index,
                      const Pulsar_parameters::Pulsar *pulsar, Job &j) {
    j.streams.resize(p.station_streams.size());
    for (size_t i = 0; i < j.streams.size(); i++) {
      const Correlation_parameters::Station_parameters &q = p.station_streams[i];
      sfxc_station_stream &o = j.streams[i];
      std::memset(&o, 0, sizeof(o));
      o.station_number = q.station_number;
      o.station_stream = (int32_t)i;  // the stream's position in the job
      o.sample_rate = q.sample_rate;
      o.bandwidth = q.bandwidth;
      o.bits_per_sample = q.bits_per_sample;
      o.tsys_freq = q.tsys_freq;
      o.channel_freq = q.channel_freq;
      o.sideband = q.sideband;
      o.polarisation = q.polarisation;
      o.delay_table = stream_table[i];
      o.lo_offset = q.LO_offset;
    }
    j.tables.resize(del_files.size());
    for (size_t i = 0; i < j.tables.size(); i++) {
      sfxc_delay_table &t = j.tables[i];
      t.del_bytes = del_files[i].empty() ? 0 : (const uint8_t *)&del_files[i][0];
      t.del_size = del_files[i].size();
      t.clock_offset = 0;  // the station's $CLOCK values (Delay_table::set_clock_offset)
      t.clock_rate = 0;
      t.clock_epoch_ticks = 0;
    }
    sfxc_correlation_params &c = j.c;
    std::memset(&c, 0, sizeof(c));
    c.experiment_start_ticks = p.experiment_start.get_clock_ticks();
    c.start_ticks = p.start_time.get_clock_ticks();
    c.integration_time_us = (int64_t)(p.integration_time.get_time_usec() + 0.5);
    c.sub_integration_time_us = (int64_t)(p.sub_integration_time.get_time_usec() + 0.5);
    c.number_channels = p.number_channels;
    c.fft_size_delaycor = p.fft_size_delaycor;
    c.fft_size_correlation = p.fft_size_correlation;
    c.sample_rate = p.sample_rate;
    c.bandwidth = p.bandwidth;
    c.frequency_nr = p.frequency_nr;
    c.channel_freq = p.channel_freq;
    c.sideband = p.sideband;
    c.polarisation = p.polarisation;
    c.cross_polarize = p.cross_polarize ? 1 : 0;
    c.reference_station = p.reference_station;
    c.window = p.window;
    c.integration_nr = p.integration_nr;
    c.n_streams = (int32_t)j.streams.size();
    c.streams = j.streams.empty() ? 0 : &j.streams[0];
    c.n_delay_tables = (int32_t)j.tables.size();
    c.delay_tables = j.tables.empty() ? 0 : &j.tables[0];
    if (p.pulsar_binning && pulsar) {
      c.pulsar_nbins = pulsar->nbins;
      c.gate_start = pulsar->interval.start;
      c.gate_stop = pulsar->interval.stop;
      j.coef.resize(pulsar->polyco_params.size());
      j.polyco.resize(pulsar->polyco_params.size());
      for (size_t k = 0; k < j.polyco.size(); k++) {
        const Pulsar_parameters::Polyco_params &q = pulsar->polyco_params[k];
        j.coef[k] = q.coef;
        sfxc_polyco &o = j.polyco[k];
        o.tmid = q.tmid;
        o.dm = q.DM;
        o.ref_phase = q.ref_phase;
        o.ref_freq = q.ref_freq;
        o.obs_freq = q.obs_freq;
        o.n_coef = (int32_t)j.coef[k].size();
        o.coef = j.coef[k].empty() ? 0 : &j.coef[k][0];
      }
      c.n_polyco = (int32_t)j.polyco.size();
      c.polyco = j.polyco.empty() ? 0 : &j.polyco[0];
    }
    if (p.mask_parameters && p.number_channels < p.fft_size_correlation) {
      // the ctrl file's mask and lag window (doubles there), in FP32 as the core applies them
      j.mask.assign(p.mask_parameters->mask.begin(), p.mask_parameters->mask.end());
      j.lag_window.assign(p.mask_parameters->window.begin(), p.mask_parameters->window.end());
      c.mask = j.mask.empty() ? 0 : &j.mask[0];
      c.lag_window = j.lag_window.empty() ? 0 : &j.lag_window[0];
      c.mask_normalize = p.mask_parameters->normalize ? 1 : 0;
    }
    c.n_phase_centers = p.n_phase_centers;
    j.file_index = source_file_index;
    c.phase_center_file_index = j.file_index.empty() ? 0 : &j.file_index[0];
  }

  Correlator_node_gpu(int device, bool tensor_cores) {
    sfxc_gpu_config cfg = {device, tensor_cores ? SFXC_GPU_X_TC_HILO : SFXC_GPU_X_FP32};
    ctx_ = sfxc_gpu_create(&cfg);
    if (!ctx_) sfxc_abort(sfxc_gpu_global_error());
  }
  ~Correlator_node_gpu() { sfxc_gpu_destroy(ctx_); }

  // Correlator_node::set_parameters: one job (time slice x subband)
  void set_parameters(const Correlation_parameters &p, const std::vector<std::vector<char> > &del_files,
                      const std::vector<int> &stream_table, const std::vector<int32_t> &source_file_index,
                      const Pulsar_parameters::Pulsar *pulsar) {
    flatten(p, del_files, stream_table, source_file_index, pulsar, job_);
    check(sfxc_gpu_set_parameters(ctx_, &job_.c));
  }

  // The reader thread: the bytes Correlator_node_data_reader_tasklet puts in
  // the stream's Channel_circular_input_buffer
  void push(int stream, const char *buf, size_t n) {
    check(sfxc_gpu_push_protocol(ctx_, stream, (const uint8_t *)buf, n));
  }

  // The UVW values Correlator_node::set_parameters evaluates at the
  // integration's mid-time: [stream][phase centre][u, v, w]
  void set_uvw(const std::vector<double> &uvw) { check(sfxc_gpu_set_uvw(ctx_, &uvw[0], uvw.size())); }

  // Correlator_node::correlate until the core has finished the integration:
  // integration_write to the writer, tsys_write to the output node
  void correlate(Data_writer &writer, int output_node_rank) {
    Sink s = {&writer, output_node_rank};
    check(sfxc_gpu_run_integration(ctx_, &Correlator_node_gpu::sink, &s));
  }

  sfxc_gpu_ctx *context() { return ctx_; }

private:
  struct Sink {
    Data_writer *w;
    int rank;
  };
  static int sink(void *u, int32_t kind, const void *data, size_t n) {
    Sink *s = (Sink *)u;
    if (kind == 0)
      s->w->put_bytes(n, (const char *)data);  // integration_write
    else
      MPI_Send((void *)data, (int)n, MPI_PACKED, s->rank, MPI_TAG_OUTPUT_NODE_WRITE_TSYS,  // tsys_write
               MPI_COMM_WORLD);
    return 0;
  }
  void check(int rc) {
    if (rc < 0) sfxc_abort(sfxc_gpu_last_error(ctx_));
  }
  Correlator_node_gpu(const Correlator_node_gpu &);
  Correlator_node_gpu &operator=(const Correlator_node_gpu &);

  sfxc_gpu_ctx *ctx_;
  Job job_;
};

#endif
