// Station recording formats on the host: VDIF and Mark5B frame readers that
// turn a recording (bytes in memory) into the reader blocks of the input
// node -- payload bytes, start time, channel, invalid byte runs -- with the
// block, skip, restart and resync rules of the reference's readers
// (VDIF_reader, sfxc/src/vdif_reader.cc; Mark5b_reader,
// sfxc/src/mark5b_reader.cc; fill-pattern search,
// sfxc/src/input_data_format_reader.cc:20-72).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include "frames.hpp"

namespace sfxc {

enum { FORMAT_VDIF = 0, FORMAT_MARK5B = 1 };

struct ReaderParams {
  int format = FORMAT_VDIF;
  int64_t ref_ticks = 0;      // reference time; its day is the reader's reference MJD
  int64_t offset_ticks = 0;   // Input_node_parameters::offset, subtracted from every time
  int track_bit_rate = 0;     // samples/s per track
  int frame_size = 0;         // VDIF payload bytes per frame
  int n_tracks = 0;           // VDIF: 0 = one thread per channel; Mark5B: bitstreams
  int bits_per_sample = 2;
  int tracks_per_channel = 2;
  std::vector<int> first_track;  // per channel: its first track (the VDIF thread id when n_tracks == 0)
};

struct ReaderBlock {
  std::vector<uint8_t> data;
  int channel = -1;
  int64_t start_ticks = 0;
  std::vector<int32_t> invalid;  // (begin, n) byte pairs
};

// Reads the recording bytes[0, n) (not copied: they must outlive the reader).
class FormatReader {
 public:
  virtual ~FormatReader() {}
  // The next block; false at the end of the data (or when no valid block can
  // be found within the readers' search limits).
  virtual bool next(ReaderBlock &out) = 0;
  static std::unique_ptr<FormatReader> create(const ReaderParams &p, const uint8_t *bytes, size_t n);
};

// Modified Julian Day of a Gregorian date (day count from 1858-11-17).
int mjd_of_date(int day, int month, int year);

// ---- The same readers over a recording that stays where it is (device
// memory): the block, skip, restart and resync rules run on decoded frame
// headers, and each block comes out as the recording offsets of its frames'
// payloads instead of copied bytes.

// What the walker reads of a recording it does not hold.
class FrameSource {
 public:
  virtual ~FrameSource() {}
  virtual int64_t size() const = 0;
  // decoded headers (decode_vdif / decode_mk5b of 16 bytes) of the frames at
  // pos0 + k * stride, k < count; every such pos + 16 <= size()
  virtual void decode(int format, int64_t pos0, int64_t stride, int64_t count, FrameInfo *out) = 0;
  // raw bytes [pos, pos + len), within size(): only the Mark5B sync search reads them
  virtual void fetch(int64_t pos, int64_t len, uint8_t *dst) = 0;
};

// One reader block: the reader's data bytes are the payloads of its
// nframes frames, frame_bytes each at block offsets 0, frame_bytes, ...,
// then zeros up to size.  invalid: the VDIF invalid-frame runs; Mark5B
// blocks take their fill-pattern runs (fill_pattern_runs over the block
// bytes) afterwards.
struct FrameBlock {
  int channel = -1;
  int64_t start_ticks = 0;
  int32_t size = 0;
  int32_t frame_bytes = 0;
  int64_t first = 0;  // index of its first frame in FrameWalk::frames
  int32_t nframes = 0;
  std::vector<int32_t> invalid;
};
// One read_new_block call of the reader: the block it returned (an index
// into FrameWalk::blocks) or -1 when it failed, whether the data ran out,
// and the reader's get_current_time() after it, as it reads once the reader
// is open.
struct ReadEvent {
  int32_t block;
  bool eof;
  int64_t time;
};
struct FrameWalk {
  std::vector<FrameBlock> blocks;
  std::vector<int64_t> frames;  // payload offsets in the recording, block after block
  std::vector<ReadEvent> reads;  // every read until the data runs out (the last one)
};

// The reader's successive read_new_block calls over the whole recording:
// the blocks are those FormatReader::create(p, ...)->next() returns, in
// order, and a failed read (more than 256 frames skipped, a Mark5B resync
// that found nothing) is followed by the reads after it, as the reader
// continues.  Differences from the reader: where a truncated Mark5B
// recording ends inside a resync, the reader may still return one block
// whose bytes are partly left over from the previous block (the walk ends
// before it); where the data ends inside a frame header, the reader mixes
// the partial header into its current one, so its time after that read (the
// walk keeps the last whole header's) is not defined by the data.
FrameWalk walk_frames(const ReaderParams &p, FrameSource &src);

// ---- The reader tasklet (Input_data_format_reader_tasklet,
// sfxc/src/input_data_format_reader_tasklet.cc:33-260) over a walk: for
// each time interval (start, stop, leave), the blocks it pushes to the
// channel extractor, with the blocks of missing frames, of data that ended
// or of streams that fell behind filled in as wholly invalid blocks.
struct TimeInterval {
  int64_t start, stop, leave;
};
struct ScheduledBlock {
  int64_t start_ticks;
  int channel;
  int32_t block;       // the walk block whose bytes it carries (index into FrameWalk::blocks), or -1
  bool whole_invalid;  // filled in, or its bytes are not a block's (a read failed into them)
  // VDIF: its invalid runs, as the reader appended them to the tasklet's
  // frame (a frame read again by goto_time keeps the runs it had), after
  // (0, size) when whole_invalid; Mark5B: empty, the block's fill-pattern
  // runs apply
  std::vector<int32_t> invalid;
};
// The reads the tasklet makes (walk: its blocks and reads, which with
// Mark5B's skips to a later time are not all of the recording's) and the
// blocks it pushes.  Throws std::runtime_error where the reference asserts
// (a block off its channel's time grid) or would not finish.
struct Schedule {
  FrameWalk walk;
  std::vector<ScheduledBlock> blocks;
};
Schedule schedule_blocks(const ReaderParams &p, FrameSource &src, const std::vector<TimeInterval> &intervals);
// the reader's time between block headers (time_between_headers), in ticks
int64_t reader_tbh(const ReaderParams &p);

}  // namespace sfxc
