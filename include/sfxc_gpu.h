/*
 * sfxc_gpu.h -- C ABI of the GB300 correlator-node path.
 *
 * Drop-in boundary for the reference's in-process correlator-node task
 * interface (paths relative to the reference project):
 *
 *   Correlator_node::set_parameters / receive_parameters
 *       sfxc/src/correlator_node.cc:298-406            -> sfxc_gpu_set_parameters
 *   Correlator_node_data_reader_tasklet -> Channel_circular_input_buffer
 *       sfxc/src/correlator_node_data_reader_tasklet.cc:28-109,
 *       sfxc/include/correlator_node_types.h:14-31     -> sfxc_gpu_push_protocol
 *   Bit2float_worker + Delay_correction + Correlation_core(_pulsar)::do_task
 *   until finished(), integration_write via Data_writer::put_bytes, tsys_write
 *       sfxc/src/correlator_node.cc:263-296, sfxc/include/delay_correction.h:39-55,
 *       sfxc/include/correlation_core.h:27-59,
 *       sfxc/include/correlation_core_pulsar.h:10-16,
 *       sfxc/include/data_writer.h:28                  -> sfxc_gpu_run_integration
 *   Input_node_tasklet::get_delay / get_delays (add_time_interval)
 *       sfxc/src/input_node_tasklet.cc:103-128,235-282 -> sfxc_gpu_delay_list
 *   Input_node_data_writer::do_task (byte protocol to the correlator node)
 *       sfxc/src/input_node_data_writer.cc:107-229,389-500 -> sfxc_gpu_write_protocol
 *   Channel_extractor_5::extract (bit gather into per-subband streams)
 *       sfxc/src/channel_extractor_5.cc:27-99          -> sfxc_gpu_extract_channels
 *
 * Conventions: plain pointers and sizes; every call returns 0 or a negative
 * status (SFXC_GPU_E*), with a message from sfxc_gpu_last_error().  Input
 * buffers belong to the caller and are not referenced after a call returns.
 * One host thread drives one context; a context owns three CUDA streams on
 * one device (the second carries per-block parameters ahead of the first, the
 * third a sub-integration chunk's X-step beside the next chunk's F-step).
 * Contexts created in one process get successive stream priorities
 * (cycling through the device's range), so that jobs correlated side by side
 * on one GPU finish in turn and their host work overlaps each other's kernels.
 * The library has no CPU fallback: without a usable GPU, sfxc_gpu_create
 * fails.
 */
#ifndef SFXC_GPU_H
#define SFXC_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFXC_GPU_OK 0
#define SFXC_GPU_EINVAL (-1)   /* bad parameters */
#define SFXC_GPU_EDELTAB (-2)  /* malformed delay table */
#define SFXC_GPU_EDELAY (-3)   /* delay model does not cover the request */
#define SFXC_GPU_EPROTO (-4)   /* malformed input protocol */
#define SFXC_GPU_ESTREAM (-5)  /* input ended before the integration was complete */
#define SFXC_GPU_ESTATE (-6)   /* call out of order */
#define SFXC_GPU_ECUDA (-10)   /* CUDA runtime error */

/* X-step arithmetic */
#define SFXC_GPU_X_FP32 0      /* FP32 spectra, FP32 CUDA-core multiply-accumulate */
#define SFXC_GPU_X_TC_HILO 1   /* FP16 hi+lo spectra, tensor-core products, FP32 accumulation;
                                  pulsar binning too; the phased array (sums of spectra, no
                                  products) keeps FP32 spectra in either mode */
/* Stream limits per job: FP32 up to 128 streams, tensor-core up to 64;
 * sfxc_gpu_set_parameters returns SFXC_GPU_EINVAL beyond them. */

typedef struct sfxc_gpu_ctx sfxc_gpu_ctx;

typedef struct {
  int32_t device; /* CUDA device ordinal */
  int32_t x_mode; /* SFXC_GPU_X_* */
} sfxc_gpu_config;

/* Correlation_parameters::Station_parameters (sfxc/include/control_parameters.h:125-142) */
typedef struct {
  int32_t station_number;
  int32_t station_stream; /* the node's input number: distinct per stream (gaps allowed); the
                             streams are taken in array order */
  int32_t sample_rate;
  int32_t bandwidth;
  int32_t bits_per_sample;
  int32_t tsys_freq;
  int64_t channel_freq;
  char sideband;     /* 'U' or 'L' */
  char polarisation; /* 'R' or 'L' */
  char pad_[2];
  int32_t delay_table; /* index into sfxc_correlation_params.delay_tables */
  double lo_offset;
} sfxc_station_stream;

/* A station delay table: the bytes of its .del file (layout of
 * sfxc/utils/delay/generate_delay_model_calc.c:440-467) and the clock model of
 * Delay_table::set_clock_offset (sfxc/src/delay_table_akima.cc:221-229). */
typedef struct {
  const uint8_t *del_bytes;
  size_t del_size;
  double clock_offset;
  double clock_rate;
  int64_t clock_epoch_ticks;
} sfxc_delay_table;

/* Pulsar_parameters::Polyco_params (sfxc/include/control_parameters.h:74-90) */
typedef struct {
  double tmid, dm, ref_phase, ref_freq, obs_freq;
  int32_t n_coef;
  const double *coef;
} sfxc_polyco;

/* Correlation_parameters (sfxc/include/control_parameters.h:117-182).  Times
 * are clock ticks at 512 MHz since MJD 51544 (the reference's Time). */
typedef struct {
  int64_t experiment_start_ticks;
  int64_t start_ticks;             /* start of the first integration */
  int64_t integration_time_us;
  int64_t sub_integration_time_us;
  int32_t number_channels;
  int32_t fft_size_delaycor;
  int32_t fft_size_correlation;
  int32_t sample_rate;
  int32_t bandwidth;
  int32_t frequency_nr;
  int64_t channel_freq;
  char sideband;
  char polarisation;
  char pad_[2];
  int32_t cross_polarize;
  int32_t reference_station;
  int32_t window;                  /* SFXC_WINDOW_* ids of sfxc/include/utils.h */
  int32_t integration_nr;
  int32_t n_streams;
  const sfxc_station_stream *streams;
  int32_t n_delay_tables;
  const sfxc_delay_table *delay_tables;
  /* pulsar binning (Correlation_core_pulsar); pulsar_nbins == 0 disables it */
  int32_t pulsar_nbins;            /* Pulsar::nbins (one off-pulse bin is added) */
  double gate_start, gate_stop;    /* Pulsar::interval */
  int32_t n_polyco;
  const sfxc_polyco *polyco;
  /* spectral reduction, number_channels < fft_size_correlation
   * (Correlation_core::integration_write, sfxc/src/correlation_core.cc:413-439):
   * the ctrl file's Mask_parameters -- a mask over fft_size_correlation + 1
   * channels and a lag window over 2 number_channels lags (NULL: ones, and
   * the window that create_window derives from `window`), and normalisation
   * of every channel to unit amplitude before the mask (non-zero: on) */
  const float *mask;
  const float *lag_window;
  int32_t mask_normalize;
  /* extra phase centres (Correlation_parameters::n_phase_centers; 0 or 1:
   * the pointing centre only): each .del table then holds, per scan, that
   * many scans with the same start, one per source; every centre's
   * visibilities are written as their own output with the file index given
   * here (the manager's source list; NULL: 0 for all).  Not with pulsar
   * binning (Correlator_node::set_parameters, sfxc/src/correlator_node.cc:348-366). */
  int32_t n_phase_centers;
  const int32_t *phase_center_file_index;
  /* phased-array core (Correlation_core_phased, sfxc/src/correlation_core_phased.cc;
   * Correlator_node::Correlator_node, sfxc/src/correlator_node.cc:37-38):
   * non-zero sums every station's spectra per sub-integration and writes one
   * spectrum per sub-integration instead of the baselines; no tsys records.
   * Not with pulsar binning, extra phase centres or spectral reduction. */
  int32_t phased_array;
} sfxc_correlation_params;

sfxc_gpu_ctx *sfxc_gpu_create(const sfxc_gpu_config *config);
void sfxc_gpu_destroy(sfxc_gpu_ctx *ctx);
const char *sfxc_gpu_last_error(const sfxc_gpu_ctx *ctx);
/* Message of the last failed context-free call (create, delay list, protocol). */
const char *sfxc_gpu_global_error(void);

/* Set up a job (one subband, one or more integrations). */
int sfxc_gpu_set_parameters(sfxc_gpu_ctx *ctx, const sfxc_correlation_params *params);

/* Append correlator-node protocol bytes (HEADER_DATA/INVALID/DELAY/ENDSTREAM
 * records, sfxc/include/utils.h:39-42) for stream index `stream` (position in
 * params.streams): the bytes of the next integration. */
int sfxc_gpu_push_protocol(sfxc_gpu_ctx *ctx, int32_t stream, const uint8_t *bytes, size_t n);

/* Output sink, the Data_writer::put_bytes of the reference.  kind 0: bytes of
 * the correlator output slice (file index, timeslice/uvw/statistics headers,
 * baseline headers and visibilities, byte-identical layout to
 * Correlation_core::integration_write); kind 1: one tsys record per stream
 * (the packed message of Correlation_core::tsys_write).  Return 0 to go on. */
typedef int (*sfxc_output_sink)(void *user, int32_t kind, const void *data, size_t n);

/* UVW coordinates for the timeslice headers of the next and later
 * integrations (until set again; sfxc_gpu_set_parameters resets them to
 * zero): n_streams x max(1, n_phase_centers) x 3 doubles, u, v, w of each
 * stream (params.streams order) and phase centre.  Correlator_node::
 * set_parameters evaluates its UVW model at the integration's mid-time and
 * hands these to Correlation_core::set_parameters (sfxc/src/correlator_node.cc:
 * 327-357); integration_write puts those of the first stream of each station
 * in the header, for the centre being written (pulsar bins and the phased
 * array: centre 0) (sfxc/src/correlation_core.cc:350-364). */
int sfxc_gpu_set_uvw(sfxc_gpu_ctx *ctx, const double *uvw, size_t n_doubles);

/* Correlate the next integration of the job (all streams must have pushed). */
int sfxc_gpu_run_integration(sfxc_gpu_ctx *ctx, sfxc_output_sink sink, void *user);

/* Inspection of the last integration (for verification).  Copies stream
 * `stream`'s unpacked samples (n_blocks * fft_size_delaycor floats, the
 * output of Bit2float_worker) or its delay-corrected spectra (rows of
 * fft_size_correlation + 1 complex values, the output of Delay_correction). */
int sfxc_gpu_copy_unpacked(sfxc_gpu_ctx *ctx, int32_t stream, float *out, size_t n_floats);
int sfxc_gpu_copy_spectra(sfxc_gpu_ctx *ctx, int32_t stream, float *out, size_t n_floats);
/* Pulsar bin of every FFT row and channel of the last integration (the bins
 * of Correlation_core_pulsar::dedisperse_buffer, sfxc/src/correlation_core_pulsar.cc:
 * 210-238: 0 off-pulse, 1..nbins on-pulse): nffts x (fft_size_correlation + 1)
 * int32, row-major; returns the count.  SFXC_GPU_ESTATE without binning. */
int sfxc_gpu_copy_pulsar_bins(sfxc_gpu_ctx *ctx, int32_t *out, size_t n);
/* sfxc_gpu_copy_spectra without any allocation.  This call has no
 * counterpart in the reference; it exists for callers that cannot allocate
 * device memory when they inspect a stream: real-time correlator loops that
 * cannot wait on the allocator (cudaMalloc and cudaFree may synchronise the
 * whole device, stalling every other job's kernels), and hosts that hand out
 * the GPU's memory once at start-up under a fixed budget shared with other
 * processes.  Its scratch -- the fringe-stopped samples, the per-block delay
 * parameters, the stream descriptor and the spectra before the copy out --
 * lives in one static device array of 16.4 MiB that every GPU loading the
 * library holds until the process exits.  Limits: at most 8192 blocks of
 * fft_size_delaycor samples (2,097,152 samples) per stream and integration,
 * and at most 2^20 values of nffts x (fft_size_correlation + 4); larger
 * requests return SFXC_GPU_EINVAL and touch nothing.  The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  The call runs on the context's
 * own stream and waits for it.  All calls share the array and it keeps the
 * last call's contents (each call writes every element it reads); calls that
 * overlap on the GPU -- from different contexts or threads -- race on it.
 * Arguments and result as sfxc_gpu_copy_spectra. */
int sfxc_gpu_copy_spectra_noalloc(sfxc_gpu_ctx *ctx, int32_t stream, float *out, size_t n_floats);
/* Device time (ms) of the last integration, CUDA events on the context's
 * streams: [0] unpack and fringe stopping, with any wait for the per-block
 * delay and phase parameters, which run on the context's second stream (the
 * first sub-integration chunk's beside the bit statistics, later chunks'
 * during the previous chunk's X-step), [1] windowed FFT, [2] X-step, [3]
 * normalisation and result copies, [4] total from the first kernel to the
 * last copy; [5] number of kernel launches.  Where a chunk's X-step runs on
 * the context's third stream beside the next chunk's F-step (every X-step
 * but the TMA-fed tensor-core one), [0] and [2] overlap and [0] to [3] add
 * up to more than [4]. */
int sfxc_gpu_last_timings(const sfxc_gpu_ctx *ctx, float *out6);
/* The same times and, as [6], the bit statistics (which run before the first
 * chunk); writes the first min(n, 7) entries. */
int sfxc_gpu_last_timings_n(const sfxc_gpu_ctx *ctx, float *out, int32_t n);

/* Integer delay list of one interval (Input_node_tasklet::add_time_interval):
 * writes up to `capacity` entries (ticks, bytes, remaining samples) and
 * returns the count (or a negative status). */
int sfxc_gpu_delay_list(const sfxc_delay_table *table, int64_t start_ticks, int64_t stop_ticks, int32_t sample_rate,
                        int32_t bits_per_sample, int64_t *ticks, int32_t *bytes, int32_t *remaining,
                        int32_t capacity);

/* Input-node byte protocol for consecutive slices of one channel.
 * Channel blocks: start ticks, byte size and invalid runs (begin, n) of each
 * block of the channel stream `stream` (blocks stored back to back).  Slices:
 * start/stop ticks, sample count and delay list (as returned by
 * sfxc_gpu_delay_list).  Output: slice k's bytes at out + out_offsets[k],
 * length out_offsets[k+1] - out_offsets[k]; returns the total byte count, or
 * the needed capacity as a negative-free count when out is NULL. */
typedef struct {
  int64_t start_ticks;
  int32_t size;
  int32_t n_invalid;
  const int32_t *invalid; /* 2*n_invalid: begin, n */
} sfxc_channel_block;
typedef struct {
  int64_t start_ticks, stop_ticks, nr_samples;
  int32_t n_delays;
  const int64_t *delay_ticks;
  const int32_t *delay_bytes;
  const int32_t *delay_remaining;
} sfxc_slice;
int64_t sfxc_gpu_write_protocol(const uint8_t *stream, int32_t n_blocks, const sfxc_channel_block *blocks,
                                int32_t n_slices, const sfxc_slice *slices, int32_t sample_rate,
                                int32_t bits_per_sample, int64_t integration_time_us, uint8_t *out,
                                int64_t capacity, int64_t *out_offsets);

/* Channel extraction on the GPU: `nwords` input words of `word_bytes` bytes
 * (host memory); subband s takes tracks tracks[s*fan_out .. +fan_out) (bit
 * positions within a word, first track = high bit of a sample code).  Writes
 * nwords*fan_out/8 bytes per subband, back to back, into `out` (host). */
int sfxc_gpu_extract_channels(sfxc_gpu_ctx *ctx, const uint8_t *words, int64_t nwords, int32_t word_bytes,
                              int32_t bits_per_sample, int32_t n_subbands, int32_t fan_out, const int32_t *tracks,
                              uint8_t *out);

/* Station recordings read into input-node blocks: the reference's VDIF and
 * Mark5B readers as Input_data_format_reader_tasklet drives them
 * (VDIF_reader::open_input_stream / read_new_block / set_parameters,
 * sfxc/src/vdif_reader.cc:19-36,77-190,202-226; Mark5b_reader, same calls,
 * sfxc/src/mark5b_reader.cc:23-38,111-162,241-327; fill-pattern runs,
 * sfxc/src/input_data_format_reader.cc:20-72).  Host only, no GPU needed. */
#define SFXC_GPU_FORMAT_VDIF 0
#define SFXC_GPU_FORMAT_MARK5B 1
/* Input_node_parameters (sfxc/include/control_parameters.h:16-66) as the readers use it. */
typedef struct {
  int32_t format;             /* SFXC_GPU_FORMAT_* */
  int64_t ref_ticks;          /* reference time; its day is the reader's reference MJD */
  int64_t offset_ticks;       /* subtracted from every block time */
  int32_t track_bit_rate;     /* samples/s per track (Mark5B: whole Mb/s) */
  int32_t frame_size;         /* VDIF payload bytes per frame */
  int32_t n_tracks;           /* VDIF: 0 = one thread per channel; Mark5B: bitstreams */
  int32_t bits_per_sample;    /* 1 or 2 */
  int32_t tracks_per_channel; /* sample rate = track_bit_rate * tracks_per_channel / bits_per_sample */
  int32_t n_channels;
  const int32_t *first_track; /* per channel: its first track (VDIF thread id when n_tracks == 0) */
} sfxc_reader_params;
typedef struct sfxc_gpu_reader sfxc_gpu_reader;
/* One reader block (Input_node_types::Input_data_frame). */
typedef struct {
  const uint8_t *data;    /* payload; valid until the next call on the reader */
  int32_t size;
  int32_t channel;        /* VDIF thread's channel, -1 for Mark5B */
  int64_t start_ticks;
  int32_t n_invalid;      /* invalid byte runs: invalid[2k] first byte, invalid[2k+1] length */
  const int32_t *invalid;
} sfxc_reader_block;
/* Reader over bytes[0, n), which must stay valid until sfxc_gpu_reader_destroy;
 * NULL on bad parameters (message from sfxc_gpu_global_error). */
sfxc_gpu_reader *sfxc_gpu_reader_create(const sfxc_reader_params *params, const uint8_t *bytes, size_t n);
/* The next block: 1 and *out filled, 0 at the end of the data (or when no
 * valid block follows within the readers' search limits). */
int sfxc_gpu_reader_next(sfxc_gpu_reader *reader, sfxc_reader_block *out);
void sfxc_gpu_reader_destroy(sfxc_gpu_reader *reader);
/* Channel_extractor_tasklet::do_task (sfxc/src/channel_extractor_tasklet.cc:120-220)
 * for one reader block of word_bytes-byte words: the subbands' bytes as
 * sfxc_gpu_extract_channels writes them (block->size / word_bytes words), and
 * the block's invalid runs in bytes of each subband's output
 * (begin * fan_out / (8 * word_bytes), length likewise) into out_invalid
 * (2 * block->n_invalid ints). */
int sfxc_gpu_extract_block(sfxc_gpu_ctx *ctx, const sfxc_reader_block *block, int32_t word_bytes, int32_t bits,
                           int32_t n_subbands, int32_t fan_out, const int32_t *tracks, uint8_t *out,
                           int32_t *out_invalid);

/* The same input-node front end with the recording's bytes kept on the
 * device: the reader (sfxc_gpu_reader_*), the channel extractor
 * (sfxc_gpu_extract_block) and the writer (sfxc_gpu_write_protocol) over a
 * whole recording, the frame headers decoded, the Mark5B fill-pattern runs
 * found, the channels extracted and the protocol bytes assembled by kernels
 * (the readers' block, skip and resync decisions and the writer's records
 * stay on the host).  It replaces, per station, Input_data_format_reader_tasklet
 * -> Channel_extractor_tasklet(_VDIF) -> Input_node_data_writer::do_task
 * (sfxc/src/input_data_format_reader_tasklet.cc:93-160,
 * sfxc/src/channel_extractor_tasklet.cc:120-220,
 * sfxc/src/channel_extractor_tasklet_vdif.cc:25-49,
 * sfxc/src/input_node_data_writer.cc:107-229) and the transfer of its bytes
 * into the correlator node's input buffer
 * (sfxc/src/correlator_node_data_reader_tasklet.cc:28-109).
 *
 * create: bytes[0, n) in host memory (copied to the device), or in device
 * memory of the context's device when bytes_on_device (not copied: it must
 * stay valid until destroy).  The blocks are those sfxc_gpu_reader_next
 * returns for the same bytes, except that where a truncated Mark5B recording
 * ends inside a resync the reader may return one more block whose bytes are
 * partly left over from its previous block; the walk ends before it.  NULL
 * on bad parameters (message from sfxc_gpu_last_error(ctx)). */
typedef struct sfxc_gpu_recording sfxc_gpu_recording;
sfxc_gpu_recording *sfxc_gpu_recording_create(sfxc_gpu_ctx *ctx, const sfxc_reader_params *params,
                                               const uint8_t *bytes, size_t n, int32_t bytes_on_device);
/* The reader tasklet's blocks instead (Input_data_format_reader_tasklet,
 * sfxc/src/input_data_format_reader_tasklet.cc:33-260): for the time
 * intervals intervals[3k] start, [3k+1] stop, [3k+2] leave (ticks; the input
 * node's reader intervals, Input_node_tasklet::add_time_interval,
 * sfxc/src/input_node_tasklet.cc:101-128), the blocks it pushes, with
 * wholly invalid blocks where frames are missing, the data ended or a
 * stream fell behind (the reference fills those with random bytes marked
 * invalid).  A block the reference pushes from a data buffer a failed read
 * wrote into (the data ended inside it) goes out wholly invalid here, and a
 * block keeps its own bytes where the reference's next read into the same
 * buffer can replace them before its consumer takes it.  Replaces the
 * recording's blocks (and any channels extracted). */
int sfxc_gpu_recording_schedule(sfxc_gpu_recording *rec, int32_t n_intervals, const int64_t *intervals);
int32_t sfxc_gpu_recording_n_blocks(const sfxc_gpu_recording *rec);
/* Reader block i (as sfxc_gpu_reader_next fills it; out->invalid valid
 * until destroy); when data is not NULL, the block's out->size bytes,
 * assembled from its frames on the device, are copied there (and out->data = data). */
int sfxc_gpu_recording_block(sfxc_gpu_recording *rec, int32_t i, sfxc_reader_block *out, uint8_t *data);
/* Channel streams of every block, on the device: subbands as for
 * sfxc_gpu_extract_block (each frame's payload a whole number of output
 * bytes), or with word_bytes == 0 one channel per VDIF thread (n_subbands =
 * the channel count; each block goes to its channel as it is). */
int sfxc_gpu_recording_extract(sfxc_gpu_recording *rec, int32_t word_bytes, int32_t bits, int32_t n_subbands,
                               int32_t fan_out, const int32_t *tracks);
/* Channel `channel`'s blocks after sfxc_gpu_recording_extract (start, size,
 * invalid runs in its bytes; up to capacity of them into blocks, if not NULL)
 * and its bytes (into data, if not NULL); returns the block count. */
int32_t sfxc_gpu_recording_channel(sfxc_gpu_recording *rec, int32_t channel, int32_t capacity,
                                   sfxc_channel_block *blocks, uint8_t *data);
/* The writer's protocol for consecutive slices of one channel, as
 * sfxc_gpu_write_protocol (same slices and arguments) writes it, assembled on
 * the device and kept there for sfxc_gpu_recording_push; copied to out
 * (host, capacity bytes) when out is not NULL; slice k's bytes at
 * out_offsets[k] (n_slices + 1 entries, if not NULL).  Returns the byte count. */
int64_t sfxc_gpu_recording_protocol(sfxc_gpu_recording *rec, int32_t channel, int32_t n_slices,
                                    const sfxc_slice *slices, int32_t sample_rate, int32_t bits_per_sample,
                                    int64_t integration_time_us, uint8_t *out, int64_t capacity,
                                    int64_t *out_offsets);
/* sfxc_gpu_push_protocol of slice `slice` of that protocol into stream
 * `stream` of a correlator context on the same device, device to device. */
int sfxc_gpu_recording_push(sfxc_gpu_recording *rec, int32_t channel, int32_t slice, sfxc_gpu_ctx *ctx,
                            int32_t stream);
void sfxc_gpu_recording_destroy(sfxc_gpu_recording *rec);

/* The UVW model of a station (Uvw_model, sfxc/src/uvw_model.cc:79-330): u, v
 * and w (metres) of a phase centre at a time, from the u, v, w columns of the
 * station's .del file (Akima splines over the six whole seconds around the
 * time, rebuilt when a later time leaves the current second, as the
 * reference's get_uvw does) -- the values Correlator_node::set_parameters
 * evaluates at each integration's mid-time for sfxc_gpu_set_uvw
 * (sfxc/src/correlator_node.cc:327-357).  Host only, no GPU needed.  NULL on
 * a table it cannot read (message from sfxc_gpu_global_error). */
typedef struct sfxc_gpu_uvw_model sfxc_gpu_uvw_model;
sfxc_gpu_uvw_model *sfxc_gpu_uvw_create(const uint8_t *del_bytes, size_t n);
/* phase_center: the phase centre's index among the scans with the covering
 * scan's start; uvw: 3 doubles.  SFXC_GPU_EINVAL beyond the table. */
int sfxc_gpu_uvw_get(sfxc_gpu_uvw_model *model, int32_t phase_center, int64_t time_ticks, double *uvw);
void sfxc_gpu_uvw_destroy(sfxc_gpu_uvw_model *model);

/* The correlation set-up of a control file and a VEX file: what
 * Control_parameters derives from them (sfxc/src/control_parameters.cc:
 * 29-230 defaults, 1483-1555 reader parameters, 1867-2022 job parameters)
 * and how the manager deals out the jobs (Manager_node::initialise,
 * initialise_scan, start, start_next_timeslice_on_node, send_global_header;
 * sfxc/src/manager_node.cc:150-391,402-683).  Host only, no GPU needed.
 * NULL on a file it cannot read or parse, or a set-up the reference refuses
 * (message from sfxc_gpu_global_error). */
typedef struct sfxc_gpu_control sfxc_gpu_control;
sfxc_gpu_control *sfxc_gpu_control_open(const char *ctrl_path, const char *vex_path);
/* The input node's current time (clock ticks) of control-file station
 * `station` when the manager starts scan number `scan` of the plan; the
 * manager moves the scan's first slice to the latest of these. */
typedef int64_t (*sfxc_station_time_fn)(void *user, int32_t station, int32_t scan);
/* Works out the whole plan and keeps it as JSON text: the global output
 * header, the output files, per scan its stations (delay table, clock model,
 * reader parameters with their track lists, stop time) and channel numbers,
 * and every job in output slice order (its Correlation_parameters and the
 * station channels feeding its streams); also "ctrl" (the control file with
 * its defaults), "pulsars" (polyco files read) and "mask".  station_time may
 * be NULL.  Returns the text's length, or a negative status. */
int64_t sfxc_gpu_control_plan(sfxc_gpu_control *control, sfxc_station_time_fn station_time, void *user);
/* The text of the last plan (NUL-terminated, owned by the handle). */
const char *sfxc_gpu_control_plan_text(const sfxc_gpu_control *control);
void sfxc_gpu_control_close(sfxc_gpu_control *control);

/* Phase-cal extraction of one channel (Input_node_data_writer::do_phasecal,
 * sfxc/src/input_node_data_writer.cc:230-312, with its parameters from
 * Input_node_data_writer::set_parameters, 328-346): the channel's samples,
 * block after block as the input node's writer takes them up, folded into
 * sample_rate / 10 kHz int32 bins (values -7, -2, 2, 7 for 2-bit codes,
 * -5, 5 for 1-bit, the samples of a byte LSB first).  A block whose start is
 * a multiple of integration_ticks ends the running integration (the first
 * such block starts one; the blocks before it are not counted) and restarts
 * the fold at bin 0.  Inside a block, an invalid run is skipped (its samples
 * still advance the bin) when the byte loop reaches its first byte; a run
 * that begins where the previous skipped run ends, or before it, is not
 * skipped, and neither are the block's runs after it -- the reference's
 * loop behaves so and the fold keeps that.  Every finished integration goes
 * to the sink as kind 2, the packed message of MPI_TAG_OUTPUT_NODE_WRITE_PHASECAL:
 * uint8 station, frequency number, sideband, polarisation; int64 start ticks;
 * int64 length in ticks; int32 bin count P; P int32 bins.  The last,
 * unfinished integration is never sent (the reference's behaviour). */
typedef struct {
  int32_t sample_rate;       /* samples/s; P = sample_rate / 10 kHz bins, a multiple of 8 / bits_per_sample */
  int32_t bits_per_sample;   /* 1 or 2 */
  int64_t integration_ticks; /* phasecal_integr_time in 512 MHz ticks, > 0 */
  int32_t station_number, frequency_number;
  int32_t sideband;          /* 1: upper ('U'), 0: lower, as packed */
  int32_t polarisation;      /* 1: left ('L'), 0: right, as packed */
} sfxc_phasecal_params;
typedef struct sfxc_gpu_phasecal sfxc_gpu_phasecal;
/* One channel's phase-cal state on ctx's device and stream; NULL on bad
 * parameters (message from sfxc_gpu_last_error(ctx)). */
sfxc_gpu_phasecal *sfxc_gpu_phasecal_create(sfxc_gpu_ctx *ctx, const sfxc_phasecal_params *params);
/* Fold the next n_blocks channel blocks (stored back to back from `stream`,
 * described as for sfxc_gpu_write_protocol); finished integrations go to
 * sink(user, 2, message, bytes) in order before the call returns.  After a
 * failed call the fold state is undefined: destroy it and start again. */
int sfxc_gpu_phasecal_push(sfxc_gpu_phasecal *pc, const uint8_t *stream, int32_t n_blocks,
                           const sfxc_channel_block *blocks, sfxc_output_sink sink, void *user);
/* Frees the state; before or after ctx is destroyed. */
void sfxc_gpu_phasecal_destroy(sfxc_gpu_phasecal *pc);

/* Output node (Output_node, sfxc/src/output_node.cc:68-214): the correlator
 * output of consecutive time slices into the output files.  Each file starts
 * with the global header (Output_header_global, sfxc/include/output_header.h:
 * 70-97, 84 bytes, filled as Manager_node::send_global_header does,
 * sfxc/src/manager_node.cc:670-703); slices are written in slice order from
 * slice 0, whatever order they arrive in; a slice's bytes are n_bins equal
 * parts (pulsar bins or phase centres), each an int32 file index followed by
 * that output, and each output goes, without its index, to that file.  For
 * this object the sink's `kind` is the file index. */
typedef struct {
  char experiment[32];
  int32_t start_year, start_day;  /* day of year; both stored as int16 */
  int32_t start_time;             /* seconds since midnight */
  int32_t number_channels;
  int32_t integration_time_us;
  int32_t correlator_version;
  int32_t polarisation_type;      /* 0 L, 1 R, 2 L+R, 3 L+R with crosses */
  char correlator_branch[15];
  int32_t job_nr, subjob_nr;
} sfxc_output_global;
typedef struct sfxc_gpu_output sfxc_gpu_output;
/* Writes the global header to files 0 .. n_files - 1; NULL on bad arguments
 * (message from sfxc_gpu_global_error). */
sfxc_gpu_output *sfxc_gpu_output_create(const sfxc_output_global *global, int32_t n_files, sfxc_output_sink sink,
                                        void *user);
/* One slice's bytes (copied); written now if it is the next slice in order,
 * with any later slices already held. */
int sfxc_gpu_output_put_slice(sfxc_gpu_output *out, int64_t slice_nr, const uint8_t *bytes, size_t n,
                              int32_t n_bins);
/* SFXC_GPU_ESTATE while slices are held for a missing earlier one. */
int sfxc_gpu_output_finish(sfxc_gpu_output *out);
void sfxc_gpu_output_destroy(sfxc_gpu_output *out);

/* Batches (no single counterpart in the reference, where each subband job of
 * a timeslice goes to its own correlator node: Manager_node deals them,
 * sfxc/src/manager_node.cc:201-257,288-391).  A batch holds several contexts
 * on one device -- jobs of one timeslice, of any mix of stream counts,
 * sample rates, bit depths, FFT lengths and integration times -- and
 * correlates the next integration of every one of them together: the host
 * plans all jobs first, then their device work goes to the GPU as one CUDA
 * graph (each job on its own streams, forked from and joined back into the
 * batch's stream), launched once.  Each context must have its parameters set
 * and its input pushed, as for sfxc_gpu_run_integration; the results equal
 * that call's.  The sink gets each job's output in batch order, with
 * users[i] (NULL: NULL) for job i, after every job's output bytes have been
 * made (one host thread per context); a sink that refuses data stops the
 * delivery there, the later jobs' integrations having run without their
 * output reaching the sink.  The first integration of a new shape
 * sizes the jobs' buffers; later ones with the same shapes reuse them and
 * the executable graph.  A context belongs to at most one batch at a time. */
typedef struct sfxc_gpu_batch sfxc_gpu_batch;
/* NULL on bad arguments (message from sfxc_gpu_global_error). */
sfxc_gpu_batch *sfxc_gpu_batch_create(sfxc_gpu_ctx *const *ctxs, int32_t n);
int sfxc_gpu_batch_run(sfxc_gpu_batch *batch, sfxc_output_sink sink, void *const *users);
/* The next counts[i] integrations of context i (0: none), all in the one
 * graph -- a timeslice's jobs of different integration times (the input of
 * all of them pushed beforehand); each job's outputs reach the sink in
 * integration order. */
int sfxc_gpu_batch_run_counts(sfxc_gpu_batch *batch, const int32_t *counts, sfxc_output_sink sink,
                              void *const *users);
/* Device time (ms, CUDA events around the graph launch) of the last run. */
float sfxc_gpu_batch_last_ms(const sfxc_gpu_batch *batch);
/* Host wall time (ms) of the last run's phases: [0] planning every
 * integration (host tables, upload payloads staged), [1] graph capture and
 * update (or instantiation), [2] launch to completion, [3] outputs to the
 * sink (statistics, output bytes, tsys records). */
int sfxc_gpu_batch_last_host_ms(const sfxc_gpu_batch *batch, float *out4);
void sfxc_gpu_batch_destroy(sfxc_gpu_batch *batch);

/* Autotuner (no counterpart in the reference): times the launch-shape
 * variants of the block stage (CTAs per SM) and of each windowed-FFT length
 * (waves of resident CTAs) on the last integration's final chunk -- the
 * launches rewrite that chunk's intermediates with the same values --
 * `trials` times each (<= 0: 3), and keeps the fastest per job shape in a
 * plan cache that every context of the process uses from its next
 * integration on.  Tuned shapes change no result bit.  Returns the number of
 * shapes tuned, or a negative status (SFXC_GPU_ESTATE before any
 * integration). */
int sfxc_gpu_autotune(sfxc_gpu_ctx *ctx, int32_t trials);
/* The plan cache: up to `capacity` entries of 5 int32 (kernel: 0 block stage,
 * 1 windowed FFT; two or three shape values; the chosen variant); returns the
 * number of entries. */
int sfxc_gpu_plan_cache(int32_t *out, int32_t capacity);

/* Compute peaks of `device` for the rooflines (no counterpart in the
 * reference: a measurement aid).  Times one short kernel of independent FP32
 * fused multiply-adds on the CUDA cores and one of FP16 tensor-core MMAs with
 * FP32 accumulation (128 x 256 x 16, operands in shared memory), each the best
 * of three CUDA-event timings after a warm-up; changes no device setting.
 * out4: [0] FP32 TFLOP/s, [1] FP16 tensor TFLOP/s, [2] and [3] their kernel
 * times in ms. */
int sfxc_gpu_measure_peaks(int32_t device, double *out4);

#ifdef __cplusplus
}
#endif
#endif
