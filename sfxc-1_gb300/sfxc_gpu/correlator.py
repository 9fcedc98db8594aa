"""Host-side interface of the GB300 correlator-node path.

Mirrors the reference's correlator-node task interface: a
`CorrelatorNode` takes the Correlation_parameters of a job (set_parameters,
sfxc/src/correlator_node.cc:311-406), receives each stream's byte protocol as
the input-node writer produced it (push_protocol; the reference's
Channel_circular_input_buffer), and correlates one integration at a time,
handing the output bytes to a writer (Data_writer::put_bytes) and the tsys
records to the output node.  Errors raise SfxcError with the library's
status code, where the reference would abort (sfxc/src/utils.cc:44-90).

Input-node helpers (`delay_list`, `write_protocol`, `extract_channels`)
expose Input_node_tasklet::get_delays, Input_node_data_writer and the channel
extractor through the same library.
"""
import ctypes as C
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import lib as L


def _bytes_ptr(b):
    arr = (C.c_uint8 * len(b)).from_buffer_copy(b) if len(b) else (C.c_uint8 * 1)()
    return arr


def correlation_params(job):
    """The sfxc_correlation_params of a job dict (the keys of
    oracle/jobs.correlate: the same dicts drive the reference checker, the C
    restatement and this library), and the ctypes objects its pointers refer
    to (keep them alive while the parameters are used)."""
    keep = []
    tables = (L.DelayTable * len(job["del_bytes"]))()
    for k, db in enumerate(job["del_bytes"]):
        buf = _bytes_ptr(db)
        keep.append(buf)
        clock = job.get("clocks", [None] * len(job["del_bytes"]))[k]
        off, rate, epoch = clock if clock is not None else (0.0, 0.0, 0)
        tables[k] = L.DelayTable(C.cast(buf, C.POINTER(C.c_uint8)), len(db), off, rate, epoch)
    streams = (L.StationStream * len(job["streams"]))()
    for i, s in enumerate(job["streams"]):
        (station_number, station_stream, sr, cf, bw, sb, pol, bits, lo, tsys_freq, table) = s
        streams[i] = L.StationStream(station_number, station_stream, sr, bw, bits, tsys_freq, cf,
                                     sb.encode(), pol.encode(), b"\0\0", table, lo)
    p = L.CorrelationParams()
    p.experiment_start_ticks = job["experiment_start_ticks"]
    p.start_ticks = job["start_ticks"]
    p.integration_time_us = job["integration_time_us"]
    p.sub_integration_time_us = job["sub_integration_time_us"]
    p.number_channels = job["number_channels"]
    p.fft_size_delaycor = job["fft_size_delaycor"]
    p.fft_size_correlation = job["fft_size_correlation"]
    p.sample_rate = job["sample_rate"]
    p.bandwidth = job["bandwidth"]
    p.frequency_nr = job["frequency_nr"]
    p.channel_freq = job["channel_freq"]
    p.sideband = job["sideband"].encode()
    p.polarisation = job["polarisation"].encode()
    p.cross_polarize = job["cross_polarize"]
    p.reference_station = job["reference_station"]
    p.window = job["window"]
    p.integration_nr = job["integration_nr"]
    p.n_streams = len(job["streams"])
    p.streams = streams
    p.n_delay_tables = len(job["del_bytes"])
    p.delay_tables = tables
    if "pulsar" in job:
        nb, g0, g1 = job["pulsar"]
        p.pulsar_nbins = int(nb)
        p.gate_start = float(g0)
        p.gate_stop = float(g1)
        pcs = (L.Polyco * len(job["polyco"]))()
        for k, pc in enumerate(job["polyco"]):
            coef = (C.c_double * (len(pc) - 5))(*pc[5:])
            keep.append(coef)
            pcs[k] = L.Polyco(pc[0], pc[1], pc[2], pc[3], pc[4], len(pc) - 5, coef)
        p.n_polyco = len(job["polyco"])
        p.polyco = pcs
        keep.append(pcs)
    # Mask_parameters of the spectral reduction
    for key in ("mask", "lag_window"):
        if job.get(key) is not None:
            arr = np.ascontiguousarray(job[key], dtype=np.float32)
            setattr(p, key, arr.ctypes.data_as(C.POINTER(C.c_float)))
            keep.append(arr)
    p.mask_normalize = int(bool(job.get("mask_normalize", 0)))
    p.n_phase_centers = int(job.get("n_phase_centers", 1))
    p.phased_array = int(bool(job.get("phased_array", 0)))
    if job.get("pc_file_index") is not None:
        fi = (C.c_int32 * len(job["pc_file_index"]))(*[int(x) for x in job["pc_file_index"]])
        p.phase_center_file_index = fi
        keep.append(fi)
    keep += [tables, streams]
    return p, keep


class CorrelatorNode:
    """One CUDA context on one device.  x_mode: L.X_FP32 or L.X_TC_HILO."""

    def __init__(self, device=0, x_mode=L.X_FP32):
        self._lib = L.load()
        cfg = L.Config(device, x_mode)
        self._h = self._lib.sfxc_gpu_create(C.byref(cfg))
        if not self._h:
            raise L.SfxcError(L.ECUDA, self._lib.sfxc_gpu_global_error().decode())
        self._keep = []
        # recordings and phase-cal folds made on this context, held here so
        # that closing the context closes them first, whatever order the
        # objects are collected in (the library wants them destroyed before
        # their context)
        self._dependents = []

    def _adopt(self, obj):
        self._dependents = [d for d in self._dependents if d._h] + [obj]

    def close(self):
        if self._h:
            for obj in self._dependents:
                obj.close()
            self._dependents = []
            self._lib.sfxc_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc < 0:
            raise L.SfxcError(rc, self._lib.sfxc_gpu_last_error(self._h).decode())
        return rc

    # ------------------------------------------------------------------
    def set_parameters(self, job):
        """job: dict with the keys of oracle/jobs.correlate (the same dicts
        drive the reference checker, the C restatement and this library)."""
        p, keep = correlation_params(job)
        self._check(self._lib.sfxc_gpu_set_parameters(self._h, C.byref(p)))
        self._keep = keep
        self.nstreams = len(job["streams"])
        self.job = job

    def push_protocol(self, stream, data):
        """data: bytes, or a contiguous uint8 numpy array (passed without a copy)."""
        if isinstance(data, np.ndarray) and data.dtype == np.uint8 and data.flags.c_contiguous:
            self._check(self._lib.sfxc_gpu_push_protocol(self._h, stream, C.c_void_p(data.ctypes.data), data.size))
            return
        buf = _bytes_ptr(data)
        self._check(self._lib.sfxc_gpu_push_protocol(self._h, stream, buf, len(data)))

    def set_uvw(self, uvw):
        """u, v, w per stream and phase centre (array [n_streams][centres][3])
        for the timeslice headers of the next integrations."""
        u = np.ascontiguousarray(uvw, dtype=np.float64)
        self._check(self._lib.sfxc_gpu_set_uvw(self._h, u.ctypes.data, u.size))

    def run_integration(self):
        """Returns (output bytes (bytes or bytearray), [tsys record bytes per stream])."""
        out, tsys = [], []

        def sink(user, kind, data, n):
            # the copy is a foreign call (ctypes.memmove), so other threads
            # driving other contexts keep the interpreter meanwhile
            b = bytearray(n)
            if n:
                C.memmove((C.c_char * n).from_buffer(b), data, n)
            (out if kind == 0 else tsys).append(bytes(b) if kind else b)
            return 0

        cb = L.SINK(sink)
        self._check(self._lib.sfxc_gpu_run_integration(self._h, cb, None))
        return (out[0] if len(out) == 1 else b"".join(out)), tsys

    def correlate(self, job):
        """Run every integration of a job dict; returns (cor bytes, tsys bytes)."""
        self.set_parameters(job)
        cor, tsys = [], []
        for it in range(int(job["n_integrations"])):
            if job.get("uvw") is not None:  # [integration][stream][centre][3]
                self.set_uvw(job["uvw"][it])
            for k in range(self.nstreams):
                self.push_protocol(k, job["protocols"][k][it])
            o, t = self.run_integration()
            cor.append(o)
            tsys += t
        return b"".join(cor), b"".join(tsys)

    def unpacked(self, stream, n):
        out = np.empty(n, dtype=np.float32)
        self._check(self._lib.sfxc_gpu_copy_unpacked(self._h, stream, out.ctypes.data, n))
        return out

    def spectra(self, stream, nrows, nchan):
        out = np.empty((nrows, nchan + 1), dtype=np.complex64)
        self._check(self._lib.sfxc_gpu_copy_spectra(self._h, stream, out.ctypes.data, out.size * 2))
        return out

    def autotune(self, trials=3):
        """Tune the F-step launch shapes on the last integration (sfxc_gpu_autotune);
        returns the number of shapes tuned."""
        return self._check(self._lib.sfxc_gpu_autotune(self._h, trials))

    def pulsar_bins(self, nrows, nchan):
        """Pulsar bin of every FFT row and channel of the last integration:
        int32 [nrows][nchan + 1] (0 off-pulse)."""
        out = np.zeros((nrows, nchan + 1), dtype=np.int32)
        self._check(self._lib.sfxc_gpu_copy_pulsar_bins(self._h, out.ctypes.data, out.size))
        return out

    def spectra_noalloc(self, stream, nrows, nchan):
        """spectra() through the allocation-free entry point (static device scratch)."""
        out = np.empty((nrows, nchan + 1), dtype=np.complex64)
        self._check(self._lib.sfxc_gpu_copy_spectra_noalloc(self._h, stream, out.ctypes.data, out.size * 2))
        return out

    def timings(self):
        t = (C.c_float * 7)()
        self._check(self._lib.sfxc_gpu_last_timings_n(self._h, t, 7))
        # stage times overlap where the X-step runs beside the next chunk's
        # F-step: each is its own kernels' elapsed time
        return {"unpack_fringe_ms": t[0], "window_fft_ms": t[1], "xstep_ms": t[2], "normalise_ms": t[3],
                "bitstat_ms": t[6], "total_ms": t[4], "launches": int(t[5])}

    def extract_block(self, block, word_bytes, bits, tracks):
        """One reader block (read_recording's dict) through the channel
        extractor: ([bytes per subband], invalid runs in subband bytes)."""
        nsub, fan_out = len(tracks), len(tracks[0])
        flat = (C.c_int32 * (nsub * fan_out))(*[t for tr in tracks for t in tr])
        data = np.frombuffer(block["data"], dtype=np.uint8)
        inv = (C.c_int32 * max(1, 2 * len(block["invalid"])))(*[v for r in block["invalid"] for v in r])
        b = L.ReaderBlock(data.ctypes.data_as(C.POINTER(C.c_uint8)), data.size, block["channel"],
                          block["start_ticks"], len(block["invalid"]), inv)
        per = data.size // word_bytes * fan_out // 8
        out = np.empty(nsub * per, dtype=np.uint8)
        oinv = (C.c_int32 * max(1, 2 * len(block["invalid"])))()
        self._check(self._lib.sfxc_gpu_extract_block(self._h, C.byref(b), word_bytes, bits, nsub, fan_out, flat,
                                                     out.ctypes.data, oinv))
        runs = [(oinv[2 * k], oinv[2 * k + 1]) for k in range(len(block["invalid"]))]
        return [out[i * per:(i + 1) * per].tobytes() for i in range(nsub)], runs

    def extract_channels(self, words, word_bytes, bits, tracks):
        """Channel_extractor semantics on the GPU.  tracks: list per subband."""
        nsub, fan_out = len(tracks), len(tracks[0])
        flat = (C.c_int32 * (nsub * fan_out))(*[t for tr in tracks for t in tr])
        w = np.ascontiguousarray(np.frombuffer(bytes(words), dtype=np.uint8))
        nwords = w.size // word_bytes
        out = np.empty(nsub * (nwords * fan_out // 8), dtype=np.uint8)
        self._check(self._lib.sfxc_gpu_extract_channels(self._h, w.ctypes.data, nwords, word_bytes, bits, nsub,
                                                        fan_out, flat, out.ctypes.data))
        per = nwords * fan_out // 8
        return [out[i * per:(i + 1) * per].tobytes() for i in range(nsub)]


def _slices(slices):
    keep = []
    sl = (L.Slice * max(1, len(slices)))()
    for i, (s0, s1, ns, dl) in enumerate(slices):
        tk = (C.c_int64 * len(dl))(*[d[0] for d in dl])
        by = (C.c_int32 * len(dl))(*[d[1] for d in dl])
        rm = (C.c_int32 * len(dl))(*[d[2] for d in dl])
        keep += [tk, by, rm]
        sl[i] = L.Slice(s0, s1, ns, len(dl), tk, by, rm)
    return sl, keep


class DeviceRecording:
    """A station recording read, channel-extracted and turned into the
    input-node protocol on the GPU of `node` (sfxc_gpu_recording_*): the same
    blocks as read_recording, channels as extract_block / thread_channel_blocks,
    protocol bytes as write_protocol.  recording: bytes / uint8 array (host),
    or a CUDA uint8 torch tensor on the node's device (used in place)."""

    def __init__(self, node, recording, fmt, *, ref_ticks, offset_ticks=0, track_bit_rate, frame_size=0, n_tracks,
                 bits, channel_tracks):
        self._lib, self._node = node._lib, node
        firsts = (C.c_int32 * len(channel_tracks))(*[int(t[0]) for t in channel_tracks])
        p = L.ReaderParams(L.FORMAT_VDIF if fmt == "vdif" else L.FORMAT_MARK5B, int(ref_ticks), int(offset_ticks),
                           int(track_bit_rate), int(frame_size), int(n_tracks), int(bits), len(channel_tracks[0]),
                           len(channel_tracks), firsts)
        if hasattr(recording, "data_ptr"):
            self._rec = recording  # kept alive: the library reads it in place
            ptr, n, on_dev = recording.data_ptr(), recording.numel(), 1
        elif isinstance(recording, np.ndarray) and recording.dtype == np.uint8 and recording.flags.c_contiguous:
            self._rec = recording  # host memory (pinned or not), copied to the device by the library
            ptr, n, on_dev = (recording.ctypes.data if recording.size else None), recording.size, 0
        else:
            self._rec = np.ascontiguousarray(np.frombuffer(bytes(recording), dtype=np.uint8))
            ptr, n, on_dev = (self._rec.ctypes.data if self._rec.size else None), self._rec.size, 0
        self._h = self._lib.sfxc_gpu_recording_create(node._h, C.byref(p), ptr, n, on_dev)
        if not self._h:
            raise L.SfxcError(L.EINVAL, self._lib.sfxc_gpu_last_error(node._h).decode())
        node._adopt(self)
        self._nch = 0

    def close(self):
        if self._h:
            self._lib.sfxc_gpu_recording_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        return self._node._check(rc)

    def schedule(self, intervals):
        """The reader tasklet's blocks for time intervals [(start, stop, leave)
        ticks] instead of the reader's (sfxc_gpu_recording_schedule)."""
        flat = (C.c_int64 * max(1, 3 * len(intervals)))(*[int(v) for iv in intervals for v in iv])
        self._check(self._lib.sfxc_gpu_recording_schedule(self._h, len(intervals), flat))

    def n_blocks(self):
        return self._lib.sfxc_gpu_recording_n_blocks(self._h)

    def block_start(self, i):
        """Start time (ticks) of reader block i."""
        b = L.ReaderBlock()
        self._check(self._lib.sfxc_gpu_recording_block(self._h, i, C.byref(b), None))
        return b.start_ticks

    def blocks(self, data=True):
        """[{channel, start_ticks, data (None unless data), invalid}] per reader block."""
        out = []
        b = L.ReaderBlock()
        for i in range(self._lib.sfxc_gpu_recording_n_blocks(self._h)):
            self._check(self._lib.sfxc_gpu_recording_block(self._h, i, C.byref(b), None))
            buf = np.empty(b.size, dtype=np.uint8) if data else None
            if data:
                self._check(self._lib.sfxc_gpu_recording_block(self._h, i, C.byref(b), buf.ctypes.data))
            out.append({"channel": b.channel, "start_ticks": b.start_ticks,
                        "data": buf.tobytes() if data else None,
                        "invalid": [(b.invalid[2 * k], b.invalid[2 * k + 1]) for k in range(b.n_invalid)]})
        return out

    def extract(self, word_bytes, bits, tracks):
        """Subbands of every block (tracks: list per subband, as extract_block)."""
        nsub, fan_out = len(tracks), len(tracks[0])
        flat = (C.c_int32 * (nsub * fan_out))(*[t for tr in tracks for t in tr])
        self._check(self._lib.sfxc_gpu_recording_extract(self._h, word_bytes, bits, nsub, fan_out, flat))
        self._nch = nsub

    def extract_threads(self, n_channels):
        """One channel per VDIF thread, blocks as they are (thread_channel_blocks)."""
        self._check(self._lib.sfxc_gpu_recording_extract(self._h, 0, 0, n_channels, 0, None))
        self._nch = n_channels

    def channel(self, c):
        """Channel c's blocks [(start_ticks, bytes, [(begin, n)])], as write_protocol takes them."""
        nb = self._check(self._lib.sfxc_gpu_recording_channel(self._h, c, 0, None, None))
        cb = (L.ChannelBlock * max(1, nb))()
        total = 0
        self._check(self._lib.sfxc_gpu_recording_channel(self._h, c, nb, cb, None))
        total = sum(cb[i].size for i in range(nb))
        data = np.empty(max(1, total), dtype=np.uint8)
        self._check(self._lib.sfxc_gpu_recording_channel(self._h, c, nb, cb, data.ctypes.data))
        out, off = [], 0
        for i in range(nb):
            out.append((cb[i].start_ticks, data[off:off + cb[i].size].tobytes(),
                        [(cb[i].invalid[2 * k], cb[i].invalid[2 * k + 1]) for k in range(cb[i].n_invalid)]))
            off += cb[i].size
        return out

    def protocol(self, c, slices, sample_rate, bits, integration_time_us, copy=True):
        """Channel c's protocol for `slices` ([(start, stop, nr_samples, delays)])
        assembled on the device; with copy, the bytes of each slice."""
        sl, keep = _slices(slices)
        offs = (C.c_int64 * (len(slices) + 1))()
        need = self._lib.sfxc_gpu_recording_protocol(self._h, c, len(slices), sl, sample_rate, bits,
                                                     integration_time_us, None, 0, offs)
        self._check(need)
        if not copy:
            return None
        out = np.empty(max(1, int(need)), dtype=np.uint8)
        self._check(self._lib.sfxc_gpu_recording_protocol(self._h, c, len(slices), sl, sample_rate, bits,
                                                          integration_time_us, out.ctypes.data, need, offs))
        return [out[offs[i]:offs[i + 1]].tobytes() for i in range(len(slices))]

    def push(self, c, slice_index, node, stream):
        """Slice `slice_index` of channel c's last protocol into a correlator node's stream, device to device."""
        node._check(self._lib.sfxc_gpu_recording_push(self._h, c, slice_index, node._h, stream))


class UvwModel:
    """A station's UVW model from its .del bytes (sfxc_gpu_uvw_*): get(pc,
    ticks) -> (u, v, w) in metres, as the reference's Uvw_model::get_uvw."""

    def __init__(self, del_bytes):
        self._lib = L.load()
        self._buf = bytes(del_bytes)
        self._h = self._lib.sfxc_gpu_uvw_create(self._buf, len(self._buf))
        if not self._h:
            raise L.SfxcError(L.EINVAL, self._lib.sfxc_gpu_global_error().decode())

    def get(self, phase_center, ticks):
        out = (C.c_double * 3)()
        rc = self._lib.sfxc_gpu_uvw_get(self._h, phase_center, int(ticks), out)
        if rc < 0:
            raise L.SfxcError(rc, self._lib.sfxc_gpu_global_error().decode())
        return out[0], out[1], out[2]

    def close(self):
        if self._h:
            self._lib.sfxc_gpu_uvw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PhaseCal:
    """Phase-cal extraction of one channel on a CorrelatorNode's GPU
    (Input_node_data_writer::do_phasecal, sfxc/src/input_node_data_writer.cc:230-312).
    push(blocks) takes the channel blocks the input node's writer takes up,
    [(start_ticks, bytes, [(invalid_begin, n), ...])], and returns the packed
    phase-cal messages of the integrations they finish."""

    def __init__(self, node, sample_rate, bits, integration_ticks, station=0, frequency_number=0, sideband=1,
                 polarisation=0):
        self._node = node
        self._lib = node._lib
        p = L.PhasecalParams(sample_rate, bits, integration_ticks, station, frequency_number, sideband, polarisation)
        self._h = self._lib.sfxc_gpu_phasecal_create(node._h, C.byref(p))
        if not self._h:
            raise L.SfxcError(L.EINVAL, self._lib.sfxc_gpu_last_error(node._h).decode())
        node._adopt(self)

    def close(self):
        if self._h:
            self._lib.sfxc_gpu_phasecal_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def push(self, blocks):
        stream = b"".join(bytes(b[1]) for b in blocks)
        keep = []
        cb = (L.ChannelBlock * max(1, len(blocks)))()
        for i, (st, data, inv) in enumerate(blocks):
            arr = (C.c_int32 * max(1, 2 * len(inv)))(*[x for pr in inv for x in pr])
            keep.append(arr)
            cb[i] = L.ChannelBlock(st, len(data), len(inv), arr)
        msgs = []

        def sink(user, kind, data, n):
            if kind != 2:
                return 1
            msgs.append(C.string_at(data, n))
            return 0

        self._node._check(self._lib.sfxc_gpu_phasecal_push(self._h, _bytes_ptr(stream), len(blocks), cb,
                                                            L.SINK(sink), None))
        return msgs


def delay_list(del_bytes, start_ticks, stop_ticks, sample_rate, bits, clock=(0.0, 0.0, 0), capacity=1 << 20):
    lib = L.load()
    buf = _bytes_ptr(del_bytes)
    t = L.DelayTable(C.cast(buf, C.POINTER(C.c_uint8)), len(del_bytes), clock[0], clock[1], clock[2])
    ticks = (C.c_int64 * capacity)()
    by = (C.c_int32 * capacity)()
    rem = (C.c_int32 * capacity)()
    n = lib.sfxc_gpu_delay_list(C.byref(t), start_ticks, stop_ticks, sample_rate, bits, ticks, by, rem, capacity)
    if n < 0:
        raise L.SfxcError(n, lib.sfxc_gpu_global_error().decode())
    return [(ticks[i], by[i], rem[i]) for i in range(n)]


_BLOCK_DTYPE = np.dtype([("start", "<i8"), ("size", "<i4"), ("ninv", "<i4"), ("inv", "<u8")])


def write_protocol_stream(stream, block_bytes, block_starts, slices, sample_rate, bits, integration_time_us,
                          alloc=None):
    """write_protocol for a whole channel stream held in one array (blocks of
    `block_bytes` back to back, starting at `block_starts`, no invalid runs).
    `alloc(n)` may supply the output buffer (e.g. pinned memory); returns one
    uint8 array view per slice."""
    lib = L.load()
    stream = np.ascontiguousarray(stream, dtype=np.uint8)
    nb = len(block_starts)
    cb = np.zeros(nb, dtype=_BLOCK_DTYPE)
    cb["start"] = block_starts
    cb["size"] = block_bytes
    keep = []
    sl = (L.Slice * len(slices))()
    for i, (s0, s1, ns, dl) in enumerate(slices):
        tk = (C.c_int64 * len(dl))(*[d[0] for d in dl])
        by = (C.c_int32 * len(dl))(*[d[1] for d in dl])
        rm = (C.c_int32 * len(dl))(*[d[2] for d in dl])
        keep += [tk, by, rm]
        sl[i] = L.Slice(s0, s1, ns, len(dl), tk, by, rm)
    offs = (C.c_int64 * (len(slices) + 1))()
    cbp = C.cast(cb.ctypes.data, C.POINTER(L.ChannelBlock))
    need = lib.sfxc_gpu_write_protocol(stream.ctypes.data, nb, cbp, len(slices), sl, sample_rate, bits,
                                       integration_time_us, None, 0, offs)
    if need < 0:
        raise L.SfxcError(int(need), lib.sfxc_gpu_global_error().decode())
    out = alloc(int(need)) if alloc else np.empty(int(need), dtype=np.uint8)
    n = lib.sfxc_gpu_write_protocol(stream.ctypes.data, nb, cbp, len(slices), sl, sample_rate, bits,
                                    integration_time_us, out.ctypes.data, need, offs)
    if n < 0:
        raise L.SfxcError(int(n), lib.sfxc_gpu_global_error().decode())
    return [out[offs[i]:offs[i + 1]] for i in range(len(slices))]


def write_protocol(blocks, slices, sample_rate, bits, integration_time_us):
    """blocks: [(start_ticks, bytes, [(begin, n), ...])]; slices: [(start, stop, nr_samples, delays)].
    Returns the protocol bytes of each slice."""
    lib = L.load()
    stream = b"".join(bytes(b[1]) for b in blocks)
    keep = []
    cb = (L.ChannelBlock * len(blocks))()
    for i, (st, data, inv) in enumerate(blocks):
        arr = (C.c_int32 * max(1, 2 * len(inv)))(*[x for pr in inv for x in pr])
        keep.append(arr)
        cb[i] = L.ChannelBlock(st, len(data), len(inv), arr)
    sl = (L.Slice * len(slices))()
    for i, (s0, s1, ns, dl) in enumerate(slices):
        tk = (C.c_int64 * len(dl))(*[d[0] for d in dl])
        by = (C.c_int32 * len(dl))(*[d[1] for d in dl])
        rm = (C.c_int32 * len(dl))(*[d[2] for d in dl])
        keep += [tk, by, rm]
        sl[i] = L.Slice(s0, s1, ns, len(dl), tk, by, rm)
    sbuf = _bytes_ptr(stream)
    offs = (C.c_int64 * (len(slices) + 1))()
    need = lib.sfxc_gpu_write_protocol(sbuf, len(blocks), cb, len(slices), sl, sample_rate, bits,
                                       integration_time_us, None, 0, offs)
    if need < 0:
        raise L.SfxcError(int(need), lib.sfxc_gpu_global_error().decode())
    out = (C.c_uint8 * max(1, need))()
    n = lib.sfxc_gpu_write_protocol(sbuf, len(blocks), cb, len(slices), sl, sample_rate, bits,
                                    integration_time_us, out, need, offs)
    if n < 0:
        raise L.SfxcError(int(n), lib.sfxc_gpu_global_error().decode())
    raw = bytes(out)[:n]
    return [raw[offs[i]:offs[i + 1]] for i in range(len(slices))]


def plan_cache():
    """The autotuner's plan cache: [(kernel, shape..., variant)]."""
    lib = L.load()
    n = lib.sfxc_gpu_plan_cache(None, 0)
    out = (C.c_int32 * (5 * max(n, 1)))()
    n = lib.sfxc_gpu_plan_cache(out, n)
    return [tuple(out[5 * i:5 * i + 5]) for i in range(n)]


class Batch:
    """Several correlator nodes' jobs (one timeslice: any mix of stream
    counts, rates, bit depths, FFT lengths and integration times) correlated
    together, one CUDA graph per integration (sfxc_gpu_batch_*).  Each node
    needs its parameters set and its input pushed before run()."""

    def __init__(self, nodes):
        self._lib = L.load()
        self.nodes = list(nodes)
        arr = (C.c_void_p * len(self.nodes))(*[n._h for n in self.nodes])
        self._h = self._lib.sfxc_gpu_batch_create(arr, len(self.nodes))
        if not self._h:
            raise L.SfxcError(L.EINVAL, self._lib.sfxc_gpu_global_error().decode())

    def run(self, counts=None):
        """The next integration (or counts[i] integrations) of every node:
        [(output bytes (bytes or bytearray), [tsys records])] in node order."""
        outs = [([], []) for _ in self.nodes]

        def sink(user, kind, data, n):
            b = bytearray(n)
            if n:
                C.memmove((C.c_char * n).from_buffer(b), data, n)
            o = outs[user or 0]
            (o[0] if kind == 0 else o[1]).append(b)
            return 0

        cb = L.SINK(sink)
        users = (C.c_void_p * len(self.nodes))(*range(len(self.nodes)))
        if counts is None:
            rc = self._lib.sfxc_gpu_batch_run(self._h, cb, users)
        else:
            cnt = (C.c_int32 * len(self.nodes))(*counts)
            rc = self._lib.sfxc_gpu_batch_run_counts(self._h, cnt, cb, users)
        if rc < 0:
            raise L.SfxcError(rc, self._lib.sfxc_gpu_global_error().decode())
        # one output buffer is passed on as it is (bytearray); several are joined
        return [(o[0] if len(o) == 1 else b"".join(o), [bytes(x) for x in t]) for o, t in outs]

    def last_ms(self):
        return float(self._lib.sfxc_gpu_batch_last_ms(self._h))

    def last_host_ms(self):
        """Host wall time of the last run's phases: planning, graph capture and
        update, launch to completion, outputs (sfxc_gpu_batch_last_host_ms)."""
        out = (C.c_float * 4)()
        self._lib.sfxc_gpu_batch_last_host_ms(self._h, out)
        return {"plan_ms": out[0], "graph_ms": out[1], "run_ms": out[2], "outputs_ms": out[3]}

    def correlate(self, jobs, per_run=None, setup_lock=None):
        """Every integration of the jobs (one per node; any integration
        counts): per_run[i] integrations of job i in each graph (default: all
        of them in one).  Returns [(cor (bytes or bytearray), tsys)] per job.
        setup_lock (a threading.Lock), when given, is held while the jobs are
        set up and their inputs pushed before each graph: consecutive
        timeslices correlated from several threads on other batches then set
        up one at a time, each beside the others' graphs, instead of all at
        once with the GPU idle."""
        import contextlib
        guard = setup_lock if setup_lock is not None else contextlib.nullcontext()
        pool = ThreadPoolExecutor(max_workers=len(self.nodes))
        left = [int(j["n_integrations"]) for j in jobs]
        step = per_run or left
        done = [0] * len(jobs)
        cor = [[] for _ in jobs]
        tsys = [[] for _ in jobs]

        def push(n, j, d, c):
            for it in range(d, d + c):
                for k in range(n.nstreams):
                    n.push_protocol(k, j["protocols"][k][it])

        first = True
        try:
            while any(left):
                counts = [min(s, l) for s, l in zip(step, left)]
                with guard:
                    if first:
                        # each node's set-up and pushes from its own thread: the host
                        # work and the copies of different contexts run at the same
                        # time (the library calls drop the GIL)
                        for f in [pool.submit(n.set_parameters, j) for n, j in zip(self.nodes, jobs)]:
                            f.result()
                        first = False
                    for f in [pool.submit(push, n, j, d, c) for n, j, d, c in zip(self.nodes, jobs, done, counts)]:
                        f.result()
                for q, (o, t) in enumerate(self.run(counts)):
                    cor[q].append(o)
                    tsys[q] += t
                done = [d + c for d, c in zip(done, counts)]
                left = [l - c for l, c in zip(left, counts)]
        finally:
            pool.shutdown()  # after a failed call too: no worker threads left behind
        return [(c[0] if len(c) == 1 else b"".join(c), b"".join(t)) for c, t in zip(cor, tsys)]

    def close(self):
        if self._h:
            self._lib.sfxc_gpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OutputFiles:
    """The output node (Output_node, sfxc/src/output_node.cc:68-214) into
    in-memory files: `files[f]` holds file f's bytes, starting with the global
    header.  global_fields: experiment, start_year, start_day, start_time,
    number_channels, integration_time_us, correlator_version,
    polarisation_type, correlator_branch, job_nr, subjob_nr.  refuse_files:
    file indices whose writes the sink refuses after the global header (a
    full disk, say).  Host only."""

    def __init__(self, n_files, refuse_files=(), **global_fields):
        self._lib = L.load()
        g = L.OutputGlobal()
        sizes = {"experiment": 32, "correlator_branch": 15}
        for k, v in global_fields.items():
            setattr(g, k, v.encode()[:sizes[k]] if isinstance(v, str) else v)
        self.files = [bytearray() for _ in range(n_files)]

        refuse = set(refuse_files)

        def sink(user, kind, data, n):
            if kind in refuse and len(self.files[kind]) > 0:
                return 1
            self.files[kind] += C.string_at(data, n)
            return 0

        self._sink = L.SINK(sink)  # kept alive with the object
        self._h = self._lib.sfxc_gpu_output_create(C.byref(g), n_files, self._sink, None)
        if not self._h:
            raise L.SfxcError(L.EINVAL, self._lib.sfxc_gpu_global_error().decode())

    def put_slice(self, slice_nr, data, n_bins=1):
        buf = _bytes_ptr(bytes(data))
        rc = self._lib.sfxc_gpu_output_put_slice(self._h, slice_nr, buf, len(data), n_bins)
        if rc < 0:
            raise L.SfxcError(rc, self._lib.sfxc_gpu_global_error().decode())

    def finish(self):
        rc = self._lib.sfxc_gpu_output_finish(self._h)
        if rc < 0:
            raise L.SfxcError(rc, self._lib.sfxc_gpu_global_error().decode())
        return [bytes(f) for f in self.files]

    def close(self):
        if self._h:
            self._lib.sfxc_gpu_output_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def split_output(data, nchan):
    """Output bytes of run_integration (Correlation_core::integration_write
    layout) split into (header bytes, [complex64 visibilities of each baseline
    header, nchan + 1 values]) in file order: per output an int32 file index,
    the 16-byte timeslice header, 32 bytes per UVW entry, 24 per statistics
    entry, then per baseline its 8-byte header and visibilities."""
    hdr, vis, p = bytearray(), [], 0
    data = bytes(data)
    while p < len(data):
        hdr += data[p:p + 20]
        _, nbl, nuvw, nstat = np.frombuffer(data[p + 4:p + 20], dtype=np.int32)
        p += 20
        n = int(nuvw) * 32 + int(nstat) * 24
        hdr += data[p:p + n]
        p += n
        for _ in range(int(nbl)):
            hdr += data[p:p + 8]
            p += 8
            vis.append(np.frombuffer(data[p:p + (nchan + 1) * 8], dtype=np.complex64).copy())
            p += (nchan + 1) * 8
    return bytes(hdr), vis


def thread_channel_blocks(blocks, n_channels):
    """The VDIF path with one channel per thread (Channel_extractor_tasklet_VDIF::
    do_task, sfxc/src/channel_extractor_tasklet_vdif.cc:25-49): no extraction,
    each reader block (read_recording's dicts) is its channel's next block as it
    is, invalid runs included.  Returns, per channel, [(start_ticks, bytes,
    [(invalid_begin, n), ...])] as write_protocol takes them."""
    out = [[] for _ in range(n_channels)]
    for b in blocks:
        if not 0 <= b["channel"] < n_channels:
            raise ValueError("block of channel %d outside the %d channels" % (b["channel"], n_channels))
        out[b["channel"]].append((b["start_ticks"], b["data"], [tuple(r) for r in b["invalid"]]))
    return out


def read_recording(recording, fmt, *, ref_ticks, offset_ticks=0, track_bit_rate, frame_size=0, n_tracks, bits,
                   channel_tracks, max_blocks=None):
    """Reader blocks of a VDIF or Mark5B recording (fmt "vdif" / "mark5b"):
    dicts {channel, start_ticks, data, invalid [(begin, n)]}, as the input
    node's reader produces them.  channel_tracks: the track list of each
    channel (its first track is the VDIF thread id when n_tracks == 0)."""
    lib = L.load()
    data = np.frombuffer(bytes(recording), dtype=np.uint8)
    firsts = (C.c_int32 * len(channel_tracks))(*[int(t[0]) for t in channel_tracks])
    p = L.ReaderParams(L.FORMAT_VDIF if fmt == "vdif" else L.FORMAT_MARK5B, int(ref_ticks), int(offset_ticks),
                       int(track_bit_rate), int(frame_size), int(n_tracks), int(bits), len(channel_tracks[0]),
                       len(channel_tracks), firsts)
    h = lib.sfxc_gpu_reader_create(C.byref(p), data.ctypes.data if data.size else None, data.size)
    if not h:
        raise L.SfxcError(L.EINVAL, lib.sfxc_gpu_global_error().decode())
    blocks = []
    try:
        b = L.ReaderBlock()
        while max_blocks is None or len(blocks) < max_blocks:
            rc = lib.sfxc_gpu_reader_next(h, C.byref(b))
            if rc < 0:
                raise L.SfxcError(rc, "reader failed")
            if rc == 0:
                break
            inv = [(b.invalid[2 * k], b.invalid[2 * k + 1]) for k in range(b.n_invalid)]
            blocks.append({"channel": b.channel, "start_ticks": b.start_ticks, "data": C.string_at(b.data, b.size),
                           "invalid": inv})
    finally:
        lib.sfxc_gpu_reader_destroy(h)
    return blocks

