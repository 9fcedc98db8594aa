// VDIF and Mark5B readers (formats.hpp).  Every rule below restates the
// reference's reader behaviour; the file:line cites are the reference's.
#include "formats.hpp"

#include "frames.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>

namespace sfxc {
namespace {

constexpr double kClockRate = 512000000.0;  // Time ticks per second (sfxc/include/utils.h:36)
constexpr int kReferenceMjd = 51544;        // sfxc/include/correlator_time.h:9

// ---- Time, as the reference's Time class rounds (sfxc/include/correlator_time.h:76-141)
int64_t ticks_of(int mjd, double sec) {
  return (int64_t)((mjd - kReferenceMjd) * 86400 * kClockRate) + (int64_t)std::round(sec * kClockRate);
}
int64_t ticks_of_usec(double usec) { return (int64_t)std::round(usec * (kClockRate / 1000000)); }
double mjd_of_ticks(int64_t t) {  // Time::get_mjd (sfxc/src/correlator_time.cc:49-54)
  const int64_t per_day = (int64_t)(86400 * kClockRate);
  const int ndays = (int)(t / per_day);
  return kReferenceMjd + ndays + (t % per_day) / kClockRate / 86400;
}

// ---- a recording in memory read like Data_reader_file through
// Data_reader_blocking::get_bytes_s (sfxc/src/data_reader_file.cc,
// sfxc/src/data_reader_blocking.cc:12-33): a read past the end delivers what
// is left and sets end-of-file; a skip moves the position and never does.
class Source {
 public:
  Source(const uint8_t *p, size_t n) : p_(p), n_(n) {}
  bool eof() const { return eof_; }
  size_t get(size_t want, void *dst) {
    if (eof_ || want == 0) return 0;
    if (!dst) {
      pos_ += want;
      return want;
    }
    size_t have = pos_ < n_ ? n_ - pos_ : 0;
    size_t k = std::min(want, have);
    if (k) std::memcpy(dst, p_ + pos_, k);
    pos_ += k;
    if (k < want) eof_ = true;
    return k;
  }

 private:
  const uint8_t *p_;
  size_t n_, pos_ = 0;
  bool eof_ = false;
};

uint32_t word_at(const uint8_t *b, int i) {
  uint32_t w;
  std::memcpy(&w, b + 4 * i, 4);
  return w;
}

// ---- VDIF (sfxc/src/vdif_reader.cc, header sfxc/include/vdif_reader.h:36-61)
struct VdifHeader {
  uint8_t b[32] = {};
  FrameInfo f() const { return decode_vdif(b); }
  uint32_t sec_from_epoch() const { return f().seconds; }
  int legacy() const { return (f().flags & FRAME_LEGACY) ? 1 : 0; }
  int invalid() const { return (f().flags & FRAME_INVALID) ? 1 : 0; }
  uint32_t frame_in_second() const { return f().frame_nr; }
  int log2_nchan() const { return f().log2_nchan; }
  int thread_id() const { return f().thread; }
  int bits_minus_one() const { return f().bits_m1; }
  int data_size() const { return f().data_size; }
  int jday_epoch() const { return f().epoch_mjd; }
  bool fill() const { return (f().flags & FRAME_FILL) != 0; }
};

class VdifReader : public FormatReader {
 public:
  VdifReader(const ReaderParams &p, const uint8_t *bytes, size_t n) : src_(bytes, n) {
    if (p.frame_size <= 0) throw std::invalid_argument("VDIF frame size must be positive");
    ref_jday_ = (int)mjd_of_ticks(p.ref_ticks);
    // set_parameters (vdif_reader.cc:202-226)
    sample_rate_ = (double)p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
    offset_ = p.offset_ticks;
    frame_size_ = p.frame_size;
    if (p.n_tracks == 0) {
      for (size_t i = 0; i < p.first_track.size(); i++) thread_map_[p.first_track[i]] = (int)i;
      frames_per_block_ = 1;
    } else {
      frames_per_block_ = std::max(1, 32128 / frame_size_);  // VDIF_FRAME_BUFFER_SIZE
    }
  }

  bool next(ReaderBlock &out) override {
    if (!open_) {  // open_input_stream (vdif_reader.cc:19-36)
      out.invalid.clear();
      if (!read_block(out)) return false;
      open_ = true;
      out.start_ticks = current_time();
      return true;
    }
    out.invalid.clear();
    return read_block(out);
  }

 private:
  Source src_;
  int ref_jday_ = 0, frame_size_ = 0, frames_per_block_ = 1;
  double sample_rate_ = 0;
  int64_t offset_ = 0;
  bool open_ = false, first_seen_ = false;
  VdifHeader first_, cur_;
  std::map<int, int> thread_map_;

  // get_current_time (vdif_reader.cc:63-75)
  int64_t current_time() const {
    int64_t t = 0;
    if (open_) {
      const double seconds = (double)cur_.sec_from_epoch() - (ref_jday_ - cur_.jday_epoch()) * 24 * 60 * 60;
      double subsec = 0;
      if (sample_rate_ > 0) {
        const int spf = 8 * frame_size_ / ((first_.bits_minus_one() + 1) * (1 << first_.log2_nchan()));
        subsec = (double)cur_.frame_in_second() * spf / sample_rate_;
      }
      t = ticks_of(ref_jday_, seconds + subsec);
    }
    return t - offset_;
  }

  // read_new_block (vdif_reader.cc:77-190)
  bool read_block(ReaderBlock &out) {
    int restarts = 0;
    for (;;) {
      if (!first_seen_) {
        src_.get(16, cur_.b);
        if (src_.eof()) return false;
        if (cur_.fill()) {  // no frame size from the header yet: skip a non-legacy frame
          src_.get((size_t)frame_size_ + 16, nullptr);
          if (++restarts > 256) return false;
          continue;
        }
        std::memcpy(first_.b, cur_.b, 16);
        first_seen_ = true;
        if (first_.legacy() == 0) {
          src_.get(16, cur_.b + 16);
          if (src_.eof()) return false;
        }
      } else {
        src_.get(first_.legacy() == 0 ? 32 : 16, cur_.b);
        if (src_.eof()) return false;
      }
      // size_data_block(); never smaller than the frames read into it (a
      // header whose frame length disagrees with the frame size would
      // overrun the reference's buffer)
      if (out.data.empty())
        out.data.assign((size_t)frames_per_block_ * std::max(first_.data_size(), frame_size_), 0);
      if (cur_.fill() || cur_.frame_in_second() % (uint32_t)frames_per_block_ != 0) {
        src_.get((size_t)frame_size_, nullptr);
        if (++restarts > 256) return false;
        continue;
      }
      src_.get((size_t)frame_size_, out.data.data());
      if (src_.eof()) return false;
      if (cur_.invalid()) {
        out.invalid.push_back(0);
        out.invalid.push_back(frame_size_);
        auto it = thread_map_.find(cur_.thread_id());
        out.channel = it != thread_map_.end() ? it->second : 0;
      } else {
        auto it = thread_map_.find(cur_.thread_id());
        if (it == thread_map_.end()) {
          if (thread_map_.empty()) {  // a single thread: its id comes from the data
            thread_map_[cur_.thread_id()] = 0;
          } else {
            if (++restarts > 256) return false;
            continue;
          }
        }
        out.channel = thread_map_[cur_.thread_id()];
      }
      for (int i = 1; i < frames_per_block_; i++) {
        VdifHeader h;
        src_.get(first_.legacy() == 0 ? 32 : 16, h.b);
        if (src_.eof()) return false;
        src_.get((size_t)frame_size_, out.data.data() + (size_t)i * frame_size_);
        if (src_.eof()) return false;
        if (h.invalid()) {
          out.invalid.push_back(i * frame_size_);
          out.invalid.push_back(frame_size_);
        }
      }
      out.start_ticks = current_time();
      return true;
    }
  }
};

// ---- Mark5B (sfxc/src/mark5b_reader.cc, header sfxc/include/mark5b_reader.h:33-55)
constexpr int kMk5bFrame = 2500 * 4;   // SIZE_MK5B_FRAME words of SIZE_MK5B_WORD bytes
constexpr int kMk5bHeader = 4 * 4;     // SIZE_MK5B_HEADER words
constexpr int kMk5bBlockFrames = 8;    // N_MK5B_BLOCKS_TO_READ
constexpr int kMk5bBlock = kMk5bBlockFrames * kMk5bFrame;

struct Mk5bHeader {
  uint8_t b[16] = {};
  FrameInfo f() const { return decode_mk5b(b); }
  int frame_nr() const { return (int)f().frame_nr; }
  int64_t seconds() const { return f().seconds; }
  int64_t microseconds() const { return 1000000 * seconds() + f().epoch_mjd; }
  int julian_day() const { return f().thread; }
};

class Mark5bReader : public FormatReader {
 public:
  Mark5bReader(const ReaderParams &p, const uint8_t *bytes, size_t n) : src_(bytes, n) {
    current_jday_ = (int)mjd_of_ticks(p.ref_ticks);
    // set_parameters (mark5b_reader.cc:241-252)
    bitstreams_ = p.n_tracks;
    const int word = bitstreams_ <= 32 ? 4 : 8;
    const int tbr = p.track_bit_rate;
    if (tbr <= 0 || tbr % 1000000) throw std::invalid_argument("Mark5B track bit rate must be whole Mb/s");
    tbh_ = ticks_of_usec((double)kMk5bBlock / (word * tbr / 1000000));
    sample_rate_ = p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
    offset_ = p.offset_ticks;
  }

  bool next(ReaderBlock &out) override {
    if (!open_) {  // open_input_stream (mark5b_reader.cc:23-38)
      if (!read_block(out)) return false;
      open_ = true;
      out.start_ticks = current_time();
      return true;
    }
    return read_block(out);
  }

 private:
  Source src_;
  int current_jday_ = 0, bitstreams_ = 0, sample_rate_ = 0, frame_nr_ = -1;
  int64_t tbh_ = 0, offset_ = 0;
  bool open_ = false, frame_nr_valid_ = true;
  Mk5bHeader cur_, tmp_, prev_;

  // check_header (mark5b_reader.cc:195-239), decoded as the device decodes it
  static bool check(const Mk5bHeader &h) { return (h.f().flags & FRAME_CHECK) != 0; }

  // get_current_time (mark5b_reader.cc:84-105)
  int64_t current_time() {
    if (!open_) return 0;
    const double rate = (double)sample_rate_ * bitstreams_;
    const double subsec = (double)((uint64_t)(int64_t)frame_nr_ * (8 * kMk5bFrame)) / rate;
    if (subsec > 1 && frame_nr_valid_) frame_nr_valid_ = false;
    int64_t t;
    if (frame_nr_valid_) {
      t = ticks_of(current_jday_, (double)cur_.seconds() + subsec);
    } else {  // VLBA time stamp, rounded to whole frames
      const int64_t second = ticks_of(current_jday_, (double)cur_.seconds());
      const int64_t sub = ticks_of_usec((double)(cur_.microseconds() - cur_.seconds() * 1000000));
      const int nframes = (int)std::round((double)sub / tbh_);
      t = second + (int64_t)std::round((double)tbh_ * nframes);
    }
    return t - offset_;
  }

  void frame_nr_update() {
    // frame numbers wrap within a second at 64 bitstreams (mark5b_reader.cc:127-131)
    if (bitstreams_ == 64 && cur_.seconds() == prev_.seconds() && frame_nr_ > cur_.frame_nr())
      frame_nr_ = cur_.frame_nr() + 32768;
    else
      frame_nr_ = cur_.frame_nr();
  }

  void finish_block(ReaderBlock &out) {
    out.start_ticks = current_time();
    out.invalid.clear();
    find_fill_pattern(out);
  }

  // read_new_block (mark5b_reader.cc:111-162)
  bool read_block(ReaderBlock &out) {
    if (out.data.size() != (size_t)kMk5bBlock) out.data.assign(kMk5bBlock, 0);
    uint8_t *blk = out.data.data();
    for (int i = 0; i < kMk5bBlockFrames; i++) {
      src_.get(sizeof(tmp_.b), tmp_.b);
      if (i == 0) {
        if (!check(tmp_) || (tmp_.frame_nr() % kMk5bBlockFrames != 0 && frame_nr_valid_)) return resync(out);
        prev_ = cur_;
        cur_ = tmp_;
        frame_nr_update();
      }
      src_.get(kMk5bFrame, blk + (size_t)i * kMk5bFrame);
    }
    if (src_.eof()) return false;
    if (cur_.julian_day() != current_jday_ % 1000) current_jday_++;
    finish_block(out);
    return true;
  }

  // resync_header (mark5b_reader.cc:254-327): scan 4-byte aligned windows
  // for the sync word; note that once a sync word has been seen the flag
  // stays set, so later windows without one take their last 16 bytes as the
  // candidate header.
  bool resync(ReaderBlock &out) {
    const int max_read = 16 * kMk5bBlock;  // RESYNC_MAX_DATA_FRAMES blocks
    uint8_t *buf = out.data.data();
    int total = 0;
    bool found = false;
    src_.get(kMk5bHeader, buf);
    while (total < max_read) {
      int got = (int)src_.get(kMk5bFrame - kMk5bHeader, buf + kMk5bHeader);
      total += got;
      if (got <= 0) return false;
      int pos;
      for (pos = 0; pos < kMk5bFrame - kMk5bHeader; pos += 4) {
        if (word_at(buf + pos, 0) == 0xABADDEEDu) {
          found = true;
          break;
        }
      }
      if (!found) {
        std::memcpy(buf, buf + kMk5bFrame - kMk5bHeader, kMk5bHeader);
        continue;
      }
      const int in_buf = std::min((int)sizeof(tmp_.b), kMk5bFrame - pos);
      int start = 0;
      std::memcpy(tmp_.b, buf + pos, in_buf);
      if (in_buf < (int)sizeof(tmp_.b)) {
        src_.get(sizeof(tmp_.b) - in_buf, tmp_.b + in_buf);
      } else {
        const int frame_start = pos + (int)sizeof(tmp_.b);
        std::memmove(buf, buf + frame_start, kMk5bFrame - frame_start);
        start = kMk5bFrame - frame_start;
      }
      total += (int)src_.get(kMk5bFrame - start, buf + start);
      if (check(tmp_) && tmp_.frame_nr() % kMk5bBlockFrames == 0) {
        prev_ = cur_;
        cur_ = tmp_;
        for (int i = 1; i < kMk5bBlockFrames; i++) {
          total += (int)src_.get(sizeof(tmp_.b), tmp_.b);
          total += (int)src_.get(kMk5bFrame, buf + (size_t)i * kMk5bFrame);
        }
        if (cur_.julian_day() != current_jday_ % 1000) current_jday_++;
        frame_nr_update();
        finish_block(out);
        return true;
      }
    }
    return false;
  }

  // Input_data_format_reader::find_fill_pattern (input_data_format_reader.cc:20-72)
  static void find_fill_pattern(ReaderBlock &out) {
    const uint8_t *d = out.data.data();
    auto w = [d](int i) { return word_at(d, i); };
    auto emit = [&out](int begin, int n) {
      out.invalid.push_back(begin);
      out.invalid.push_back(n);
    };
    fill_pattern_runs(w, (int)(out.data.size() / 4), emit);
  }
};

}  // namespace

int mjd_of_date(int day, int month, int year) { return mjd_from_date(day, month, year); }

// ---- The readers over decoded headers (walk_frames).  Each rule below is
// the corresponding reader's rule above, restated on header records and
// recording offsets: a header "read" at offset q is the 16 bytes there
// (q + header size <= size, else end of data), a payload read likewise.
namespace {

FrameWalk walk_vdif(const ReaderParams &p, FrameSource &src) {
  if (p.frame_size <= 0) throw std::invalid_argument("VDIF frame size must be positive");
  const int64_t n = src.size();
  const int fs = p.frame_size;
  const int ref_jday = (int)mjd_of_ticks(p.ref_ticks);
  const double sample_rate = (double)p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
  std::map<int, int> thread_map;
  int fpb = std::max(1, 32128 / fs);
  if (p.n_tracks == 0) {
    for (size_t i = 0; i < p.first_track.size(); i++) thread_map[p.first_track[i]] = (int)i;
    fpb = 1;
  }
  FrameWalk out;
  // before the first header: 16-byte candidates, a fill header skips a
  // non-legacy frame (vdif_reader.cc:84-100)
  const int64_t cstride = (int64_t)fs + 32;
  int64_t ncand = 0;
  while (ncand <= 256 && ncand * cstride + 16 <= n) ncand++;
  std::vector<FrameInfo> cand((size_t)ncand);
  if (ncand) src.decode(FORMAT_VDIF, 0, cstride, ncand, cand.data());
  int restarts = 0;
  int64_t k = 0;
  for (;; k++) {
    if (k >= ncand) return out;
    if (!(cand[k].flags & FRAME_FILL)) break;
    if (++restarts > 256) return out;
  }
  const FrameInfo first = cand[k];
  const int64_t p0 = k * cstride;
  const int hs = (first.flags & FRAME_LEGACY) ? 16 : 32;
  if (p0 + hs > n) return out;
  // after it, frames at a fixed stride
  const int64_t stride = hs + fs;
  const int64_t nf = (n - p0 - 16) / stride + 1;
  std::vector<FrameInfo> hdr((size_t)nf);
  src.decode(FORMAT_VDIF, p0, stride, nf, hdr.data());
  const int32_t block_size = fpb * std::max(first.data_size, fs);
  auto time_of = [&](const FrameInfo &h) {  // get_current_time (vdif_reader.cc:63-75)
    const double seconds = (double)h.seconds - (ref_jday - h.epoch_mjd) * 24 * 60 * 60;
    double subsec = 0;
    if (sample_rate > 0) {
      const int spf = 8 * fs / ((first.bits_m1 + 1) * (1 << first.log2_nchan));
      subsec = (double)h.frame_nr * spf / sample_rate;
    }
    return ticks_of(ref_jday, seconds + subsec) - p.offset_ticks;
  };
  auto header_in = [&](int64_t j) { return j < nf && p0 + j * stride + hs <= n; };
  int64_t j = 0;
  bool have = true;  // the first header has been read
  for (;;) {         // read_new_block (vdif_reader.cc:77-190)
    FrameBlock b;
    b.first = (int64_t)out.frames.size();
    for (;;) {
      if (!have && !header_in(j)) {
        out.frames.resize((size_t)b.first);
        return out;
      }
      have = false;
      const FrameInfo &h = hdr[(size_t)j];
      const int64_t pos = p0 + j * stride;
      if ((h.flags & FRAME_FILL) || h.frame_nr % (uint32_t)fpb != 0) {
        j++;
        if (++restarts > 256) return out;
        continue;
      }
      if (pos + hs + fs > n) return out;
      auto it = thread_map.find(h.thread);
      if (h.flags & FRAME_INVALID) {
        b.invalid.push_back(0);
        b.invalid.push_back(fs);
        b.channel = it != thread_map.end() ? it->second : 0;
      } else {
        if (it == thread_map.end()) {
          if (thread_map.empty()) {
            thread_map[h.thread] = 0;
          } else {
            j++;
            if (++restarts > 256) return out;
            continue;
          }
        }
        b.channel = thread_map[h.thread];
      }
      out.frames.push_back(pos + hs);
      j++;
      for (int i = 1; i < fpb; i++, j++) {
        const int64_t q = p0 + j * stride;
        if (!header_in(j) || q + hs + fs > n) {
          out.frames.resize((size_t)b.first);
          return out;
        }
        out.frames.push_back(q + hs);
        if (hdr[(size_t)j].flags & FRAME_INVALID) {
          b.invalid.push_back(i * fs);
          b.invalid.push_back(fs);
        }
      }
      b.start_ticks = time_of(h);
      b.size = block_size;
      b.frame_bytes = fs;
      b.nframes = fpb;
      out.blocks.push_back(std::move(b));
      restarts = 0;
      break;
    }
  }
}

// Reads of the bytes fetched for one Mark5B resync, with Source's
// end-of-data rule; any short read ends the walk.
struct FetchedBytes {
  std::vector<uint8_t> b;
  int64_t base = 0, pos = 0, n = 0;  // recording offset of b[0], read position (recording), recording size
  bool short_read = false;
  void get(int64_t want, uint8_t *dst) {
    if (short_read) return;
    if (pos + want > n) {
      short_read = true;
      return;
    }
    if (pos + want > base + (int64_t)b.size()) throw std::logic_error("Mark5B resync read beyond the fetched span");
    if (dst) std::memcpy(dst, b.data() + (pos - base), (size_t)want);
    pos += want;
  }
};

FrameWalk walk_mk5b(const ReaderParams &p, FrameSource &src) {
  const int64_t n = src.size();
  int current_jday = (int)mjd_of_ticks(p.ref_ticks);
  const int bitstreams = p.n_tracks;
  const int word = bitstreams <= 32 ? 4 : 8;
  const int tbr = p.track_bit_rate;
  if (tbr <= 0 || tbr % 1000000) throw std::invalid_argument("Mark5B track bit rate must be whole Mb/s");
  const int64_t tbh = ticks_of_usec((double)kMk5bBlock / (word * tbr / 1000000));
  const int sample_rate = p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
  const int64_t fstride = kMk5bHeader + kMk5bFrame, bstride = kMk5bBlockFrames * fstride;
  const uint8_t zero[16] = {};
  FrameInfo cur = decode_mk5b(zero), prev = cur;
  int frame_nr = -1;
  bool frame_nr_valid = true;
  FrameWalk out;
  auto frame_nr_update = [&]() {  // mark5b_reader.cc:127-131
    if (bitstreams == 64 && cur.seconds == prev.seconds && frame_nr > (int)cur.frame_nr)
      frame_nr = (int)cur.frame_nr + 32768;
    else
      frame_nr = (int)cur.frame_nr;
  };
  auto finish = [&](const int64_t *frames) {  // jday, then get_current_time (mark5b_reader.cc:84-105)
    if (cur.thread != current_jday % 1000) current_jday++;
    const double rate = (double)sample_rate * bitstreams;
    const double subsec = (double)((uint64_t)(int64_t)frame_nr * (8 * kMk5bFrame)) / rate;
    if (subsec > 1 && frame_nr_valid) frame_nr_valid = false;
    int64_t t;
    if (frame_nr_valid) {
      t = ticks_of(current_jday, (double)cur.seconds + subsec);
    } else {
      const int64_t second = ticks_of(current_jday, (double)cur.seconds);
      const int64_t sub = ticks_of_usec((double)cur.epoch_mjd);
      const int nframes = (int)std::round((double)sub / tbh);
      t = second + (int64_t)std::round((double)tbh * nframes);
    }
    FrameBlock b;
    b.start_ticks = t - p.offset_ticks;
    b.size = kMk5bBlock;
    b.frame_bytes = kMk5bFrame;
    b.first = (int64_t)out.frames.size();
    b.nframes = kMk5bBlockFrames;
    out.frames.insert(out.frames.end(), frames, frames + kMk5bBlockFrames);
    out.blocks.push_back(std::move(b));
  };
  // block-start headers on the grid g0 + k * bstride
  int64_t g0 = -1;
  std::vector<FrameInfo> grid;
  int64_t P = 0;
  for (;;) {  // read_new_block (mark5b_reader.cc:111-162)
    if (P + kMk5bHeader > n) return out;
    if (g0 < 0 || P < g0 || (P - g0) % bstride || (P - g0) / bstride >= (int64_t)grid.size()) {
      g0 = P;
      grid.assign((size_t)((n - P - kMk5bHeader) / bstride + 1), FrameInfo{});
      src.decode(FORMAT_MARK5B, g0, bstride, (int64_t)grid.size(), grid.data());
    }
    const FrameInfo h = grid[(size_t)((P - g0) / bstride)];
    if ((h.flags & FRAME_CHECK) && !(h.frame_nr % kMk5bBlockFrames != 0 && frame_nr_valid)) {
      prev = cur;
      cur = h;
      frame_nr_update();
      if (P + bstride > n) return out;
      int64_t frames[kMk5bBlockFrames];
      for (int i = 0; i < kMk5bBlockFrames; i++) frames[i] = P + i * fstride + kMk5bHeader;
      P += bstride;
      finish(frames);
      continue;
    }
    // resync_header (mark5b_reader.cc:254-327) on the bytes that follow the
    // header, fetched once: the scan reads at most 16 blocks plus one frame
    // before it gives up, and a found block's eight frames after that
    const int max_read = 16 * kMk5bBlock;
    FetchedBytes r;
    r.n = n;
    r.base = r.pos = P + kMk5bHeader;
    const int64_t span = std::min<int64_t>(n - r.base, 16 + max_read + 2 * kMk5bFrame + bstride);
    r.b.resize((size_t)std::max<int64_t>(span, 0));
    if (span > 0) src.fetch(r.base, span, r.b.data());
    std::vector<uint8_t> buf(kMk5bFrame, 0);
    int total = 0;
    bool found = false, resynced = false;
    r.get(kMk5bHeader, buf.data());
    while (total < max_read && !r.short_read) {
      const int64_t bstart = r.pos;  // recording offset of buf[16]
      r.get(kMk5bFrame - kMk5bHeader, buf.data() + kMk5bHeader);
      if (r.short_read) break;
      total += kMk5bFrame - kMk5bHeader;
      int pos;
      for (pos = 0; pos < kMk5bFrame - kMk5bHeader; pos += 4)
        if (word_at(buf.data() + pos, 0) == kMk5bSync) {
          found = true;
          break;
        }
      if (!found) {
        std::memcpy(buf.data(), buf.data() + kMk5bFrame - kMk5bHeader, kMk5bHeader);
        continue;
      }
      // the candidate header is buf[pos, pos + 16); the frame after it is
      // the rest of the window and the bytes that follow it
      const FrameInfo t = decode_mk5b(buf.data() + pos);
      const int frame_start = pos + kMk5bHeader;
      const int64_t frame0 = bstart + pos;
      std::memmove(buf.data(), buf.data() + frame_start, kMk5bFrame - frame_start);
      r.get(frame_start, buf.data() + kMk5bFrame - frame_start);
      if (r.short_read) break;
      total += frame_start;
      if ((t.flags & FRAME_CHECK) && t.frame_nr % kMk5bBlockFrames == 0) {
        prev = cur;
        cur = t;
        int64_t frames[kMk5bBlockFrames] = {frame0};
        for (int i = 1; i < kMk5bBlockFrames; i++) {
          r.get(kMk5bHeader, nullptr);
          frames[i] = r.pos;
          r.get(kMk5bFrame, nullptr);
        }
        if (r.short_read) break;
        frame_nr_update();
        P = r.pos;
        finish(frames);
        resynced = true;
        break;
      }
    }
    if (!resynced) return out;
  }
}

}  // namespace

FrameWalk walk_frames(const ReaderParams &p, FrameSource &src) {
  if (p.bits_per_sample != 1 && p.bits_per_sample != 2) throw std::invalid_argument("bits per sample must be 1 or 2");
  if (p.tracks_per_channel < p.bits_per_sample) throw std::invalid_argument("fewer tracks than bits per sample");
  if (p.track_bit_rate <= 0) throw std::invalid_argument("track bit rate must be positive");
  if (p.format == FORMAT_VDIF) return walk_vdif(p, src);
  if (p.format == FORMAT_MARK5B) return walk_mk5b(p, src);
  throw std::invalid_argument("unknown recording format");
}

std::unique_ptr<FormatReader> FormatReader::create(const ReaderParams &p, const uint8_t *bytes, size_t n) {
  if (p.bits_per_sample != 1 && p.bits_per_sample != 2) throw std::invalid_argument("bits per sample must be 1 or 2");
  if (p.tracks_per_channel < p.bits_per_sample) throw std::invalid_argument("fewer tracks than bits per sample");
  if (p.track_bit_rate <= 0) throw std::invalid_argument("track bit rate must be positive");
  if (p.format == FORMAT_VDIF) return std::unique_ptr<FormatReader>(new VdifReader(p, bytes, n));
  if (p.format == FORMAT_MARK5B) return std::unique_ptr<FormatReader>(new Mark5bReader(p, bytes, n));
  throw std::invalid_argument("unknown recording format");
}

}  // namespace sfxc
