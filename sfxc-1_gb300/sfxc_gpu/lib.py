"""ctypes binding of libsfxc_gpu.so (declarations in include/sfxc_gpu.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_PKG, "lib", "libsfxc_gpu.so")

OK = 0
EINVAL, EDELTAB, EDELAY, EPROTO, ESTREAM, ESTATE, ECUDA = -1, -2, -3, -4, -5, -6, -10
X_FP32, X_TC_HILO = 0, 1

EXPORTS = [
    "sfxc_gpu_create", "sfxc_gpu_destroy", "sfxc_gpu_last_error", "sfxc_gpu_global_error",
    "sfxc_gpu_set_parameters", "sfxc_gpu_push_protocol", "sfxc_gpu_run_integration",
    "sfxc_gpu_copy_unpacked", "sfxc_gpu_copy_spectra", "sfxc_gpu_last_timings", "sfxc_gpu_last_timings_n",
    "sfxc_gpu_delay_list",
    "sfxc_gpu_write_protocol", "sfxc_gpu_extract_channels", "sfxc_gpu_copy_spectra_noalloc",
    "sfxc_gpu_copy_pulsar_bins", "sfxc_gpu_measure_peaks", "sfxc_gpu_batch_create", "sfxc_gpu_batch_run",
    "sfxc_gpu_batch_run_counts", "sfxc_gpu_autotune", "sfxc_gpu_plan_cache",
    "sfxc_gpu_batch_last_ms", "sfxc_gpu_batch_last_host_ms", "sfxc_gpu_batch_destroy",
    "sfxc_gpu_reader_create", "sfxc_gpu_reader_next", "sfxc_gpu_reader_destroy", "sfxc_gpu_extract_block",
    "sfxc_gpu_phasecal_create", "sfxc_gpu_phasecal_push", "sfxc_gpu_phasecal_destroy", "sfxc_gpu_set_uvw",
    "sfxc_gpu_output_create", "sfxc_gpu_output_put_slice", "sfxc_gpu_output_finish", "sfxc_gpu_output_destroy",
    "sfxc_gpu_recording_create", "sfxc_gpu_recording_schedule", "sfxc_gpu_recording_n_blocks", "sfxc_gpu_recording_block",
    "sfxc_gpu_recording_extract", "sfxc_gpu_recording_channel", "sfxc_gpu_recording_protocol",
    "sfxc_gpu_recording_push", "sfxc_gpu_recording_destroy",
    "sfxc_gpu_uvw_create", "sfxc_gpu_uvw_get", "sfxc_gpu_uvw_destroy",
    "sfxc_gpu_control_open", "sfxc_gpu_control_plan", "sfxc_gpu_control_plan_text", "sfxc_gpu_control_close",
]
FORMAT_VDIF, FORMAT_MARK5B = 0, 1


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("x_mode", C.c_int32)]


class StationStream(C.Structure):
    _fields_ = [("station_number", C.c_int32), ("station_stream", C.c_int32), ("sample_rate", C.c_int32),
                ("bandwidth", C.c_int32), ("bits_per_sample", C.c_int32), ("tsys_freq", C.c_int32),
                ("channel_freq", C.c_int64), ("sideband", C.c_char), ("polarisation", C.c_char),
                ("pad_", C.c_char * 2), ("delay_table", C.c_int32), ("lo_offset", C.c_double)]


class DelayTable(C.Structure):
    _fields_ = [("del_bytes", C.POINTER(C.c_uint8)), ("del_size", C.c_size_t), ("clock_offset", C.c_double),
                ("clock_rate", C.c_double), ("clock_epoch_ticks", C.c_int64)]


class Polyco(C.Structure):
    _fields_ = [("tmid", C.c_double), ("dm", C.c_double), ("ref_phase", C.c_double), ("ref_freq", C.c_double),
                ("obs_freq", C.c_double), ("n_coef", C.c_int32), ("coef", C.POINTER(C.c_double))]


class CorrelationParams(C.Structure):
    _fields_ = [("experiment_start_ticks", C.c_int64), ("start_ticks", C.c_int64),
                ("integration_time_us", C.c_int64), ("sub_integration_time_us", C.c_int64),
                ("number_channels", C.c_int32), ("fft_size_delaycor", C.c_int32),
                ("fft_size_correlation", C.c_int32), ("sample_rate", C.c_int32), ("bandwidth", C.c_int32),
                ("frequency_nr", C.c_int32), ("channel_freq", C.c_int64), ("sideband", C.c_char),
                ("polarisation", C.c_char), ("pad_", C.c_char * 2), ("cross_polarize", C.c_int32),
                ("reference_station", C.c_int32), ("window", C.c_int32), ("integration_nr", C.c_int32),
                ("n_streams", C.c_int32), ("streams", C.POINTER(StationStream)),
                ("n_delay_tables", C.c_int32), ("delay_tables", C.POINTER(DelayTable)),
                ("pulsar_nbins", C.c_int32), ("gate_start", C.c_double), ("gate_stop", C.c_double),
                ("n_polyco", C.c_int32), ("polyco", C.POINTER(Polyco)),
                ("mask", C.POINTER(C.c_float)), ("lag_window", C.POINTER(C.c_float)),
                ("mask_normalize", C.c_int32), ("n_phase_centers", C.c_int32),
                ("phase_center_file_index", C.POINTER(C.c_int32)), ("phased_array", C.c_int32)]


class ChannelBlock(C.Structure):
    _fields_ = [("start_ticks", C.c_int64), ("size", C.c_int32), ("n_invalid", C.c_int32),
                ("invalid", C.POINTER(C.c_int32))]


class Slice(C.Structure):
    _fields_ = [("start_ticks", C.c_int64), ("stop_ticks", C.c_int64), ("nr_samples", C.c_int64),
                ("n_delays", C.c_int32), ("delay_ticks", C.POINTER(C.c_int64)),
                ("delay_bytes", C.POINTER(C.c_int32)), ("delay_remaining", C.POINTER(C.c_int32))]


class ReaderParams(C.Structure):
    _fields_ = [("format", C.c_int32), ("ref_ticks", C.c_int64), ("offset_ticks", C.c_int64),
                ("track_bit_rate", C.c_int32), ("frame_size", C.c_int32), ("n_tracks", C.c_int32),
                ("bits_per_sample", C.c_int32), ("tracks_per_channel", C.c_int32), ("n_channels", C.c_int32),
                ("first_track", C.POINTER(C.c_int32))]


class ReaderBlock(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_uint8)), ("size", C.c_int32), ("channel", C.c_int32),
                ("start_ticks", C.c_int64), ("n_invalid", C.c_int32), ("invalid", C.POINTER(C.c_int32))]


class PhasecalParams(C.Structure):
    _fields_ = [("sample_rate", C.c_int32), ("bits_per_sample", C.c_int32), ("integration_ticks", C.c_int64),
                ("station_number", C.c_int32), ("frequency_number", C.c_int32), ("sideband", C.c_int32),
                ("polarisation", C.c_int32)]


class OutputGlobal(C.Structure):
    _fields_ = [("experiment", C.c_char * 32), ("start_year", C.c_int32), ("start_day", C.c_int32),
                ("start_time", C.c_int32), ("number_channels", C.c_int32), ("integration_time_us", C.c_int32),
                ("correlator_version", C.c_int32), ("polarisation_type", C.c_int32),
                ("correlator_branch", C.c_char * 15), ("job_nr", C.c_int32), ("subjob_nr", C.c_int32)]


SINK = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t)
STATION_TIME = C.CFUNCTYPE(C.c_int64, C.c_void_p, C.c_int32, C.c_int32)

_lib = None


def load(path=None):
    """Load the library (build it first with sfxc-1_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libsfxc_gpu.so not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    lib.sfxc_gpu_create.restype = C.c_void_p
    lib.sfxc_gpu_create.argtypes = [C.POINTER(Config)]
    lib.sfxc_gpu_destroy.argtypes = [C.c_void_p]
    lib.sfxc_gpu_last_error.restype = C.c_char_p
    lib.sfxc_gpu_last_error.argtypes = [C.c_void_p]
    lib.sfxc_gpu_global_error.restype = C.c_char_p
    lib.sfxc_gpu_set_parameters.argtypes = [C.c_void_p, C.POINTER(CorrelationParams)]
    lib.sfxc_gpu_push_protocol.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_run_integration.argtypes = [C.c_void_p, SINK, C.c_void_p]
    lib.sfxc_gpu_set_uvw.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_copy_unpacked.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_copy_spectra.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_copy_spectra_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_copy_pulsar_bins.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_measure_peaks.argtypes = [C.c_int32, C.c_void_p]
    lib.sfxc_gpu_batch_create.restype = C.c_void_p
    lib.sfxc_gpu_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32]
    lib.sfxc_gpu_batch_run.argtypes = [C.c_void_p, SINK, C.POINTER(C.c_void_p)]
    lib.sfxc_gpu_batch_run_counts.argtypes = [C.c_void_p, C.POINTER(C.c_int32), SINK, C.POINTER(C.c_void_p)]
    lib.sfxc_gpu_autotune.argtypes = [C.c_void_p, C.c_int32]
    lib.sfxc_gpu_plan_cache.argtypes = [C.c_void_p, C.c_int32]
    lib.sfxc_gpu_batch_last_ms.restype = C.c_float
    lib.sfxc_gpu_batch_last_ms.argtypes = [C.c_void_p]
    lib.sfxc_gpu_batch_last_host_ms.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    lib.sfxc_gpu_batch_destroy.argtypes = [C.c_void_p]
    lib.sfxc_gpu_last_timings.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    lib.sfxc_gpu_last_timings_n.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int32]
    lib.sfxc_gpu_delay_list.argtypes = [C.POINTER(DelayTable), C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                        C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        C.c_int32]
    lib.sfxc_gpu_write_protocol.restype = C.c_int64
    lib.sfxc_gpu_write_protocol.argtypes = [C.c_void_p, C.c_int32, C.POINTER(ChannelBlock), C.c_int32,
                                            C.POINTER(Slice), C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                                            C.c_int64, C.POINTER(C.c_int64)]
    lib.sfxc_gpu_extract_channels.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int32, C.POINTER(C.c_int32), C.c_void_p]
    lib.sfxc_gpu_reader_create.restype = C.c_void_p
    lib.sfxc_gpu_reader_create.argtypes = [C.POINTER(ReaderParams), C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_reader_next.argtypes = [C.c_void_p, C.POINTER(ReaderBlock)]
    lib.sfxc_gpu_reader_destroy.argtypes = [C.c_void_p]
    lib.sfxc_gpu_extract_block.argtypes = [C.c_void_p, C.POINTER(ReaderBlock), C.c_int32, C.c_int32, C.c_int32,
                                           C.c_int32, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_int32)]
    lib.sfxc_gpu_recording_create.restype = C.c_void_p
    lib.sfxc_gpu_recording_create.argtypes = [C.c_void_p, C.POINTER(ReaderParams), C.c_void_p, C.c_size_t,
                                              C.c_int32]
    lib.sfxc_gpu_recording_schedule.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]
    lib.sfxc_gpu_recording_n_blocks.restype = C.c_int32
    lib.sfxc_gpu_recording_n_blocks.argtypes = [C.c_void_p]
    lib.sfxc_gpu_recording_block.argtypes = [C.c_void_p, C.c_int32, C.POINTER(ReaderBlock), C.c_void_p]
    lib.sfxc_gpu_recording_extract.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                               C.POINTER(C.c_int32)]
    lib.sfxc_gpu_recording_channel.restype = C.c_int32
    lib.sfxc_gpu_recording_channel.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(ChannelBlock),
                                               C.c_void_p]
    lib.sfxc_gpu_recording_protocol.restype = C.c_int64
    lib.sfxc_gpu_recording_protocol.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(Slice), C.c_int32,
                                                C.c_int32, C.c_int64, C.c_void_p, C.c_int64,
                                                C.POINTER(C.c_int64)]
    lib.sfxc_gpu_recording_push.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32]
    lib.sfxc_gpu_recording_destroy.argtypes = [C.c_void_p]
    lib.sfxc_gpu_uvw_create.restype = C.c_void_p
    lib.sfxc_gpu_uvw_create.argtypes = [C.c_void_p, C.c_size_t]
    lib.sfxc_gpu_uvw_get.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)]
    lib.sfxc_gpu_uvw_destroy.argtypes = [C.c_void_p]
    lib.sfxc_gpu_control_open.restype = C.c_void_p
    lib.sfxc_gpu_control_open.argtypes = [C.c_char_p, C.c_char_p]
    lib.sfxc_gpu_control_plan.restype = C.c_int64
    lib.sfxc_gpu_control_plan.argtypes = [C.c_void_p, STATION_TIME, C.c_void_p]
    lib.sfxc_gpu_control_plan_text.restype = C.c_char_p
    lib.sfxc_gpu_control_plan_text.argtypes = [C.c_void_p]
    lib.sfxc_gpu_control_close.argtypes = [C.c_void_p]
    lib.sfxc_gpu_phasecal_create.restype = C.c_void_p
    lib.sfxc_gpu_phasecal_create.argtypes = [C.c_void_p, C.POINTER(PhasecalParams)]
    lib.sfxc_gpu_phasecal_push.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(ChannelBlock), SINK,
                                           C.c_void_p]
    lib.sfxc_gpu_phasecal_destroy.argtypes = [C.c_void_p]
    lib.sfxc_gpu_output_create.restype = C.c_void_p
    lib.sfxc_gpu_output_create.argtypes = [C.POINTER(OutputGlobal), C.c_int32, SINK, C.c_void_p]
    lib.sfxc_gpu_output_put_slice.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_size_t, C.c_int32]
    lib.sfxc_gpu_output_finish.argtypes = [C.c_void_p]
    lib.sfxc_gpu_output_destroy.argtypes = [C.c_void_p]
    _lib = lib
    return lib


class SfxcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code
