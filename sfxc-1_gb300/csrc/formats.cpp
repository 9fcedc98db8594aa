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

// One reader: read() is one read_new_block call, appending its ReadEvent
// (and its block) to out.
class Walker {
 public:
  virtual ~Walker() {}
  virtual void read() = 0;
  // get_current_time() as when the reader is open; `apply`: with the side
  // effect the reader's call has (Mark5B: the switch to VLBA time stamps)
  virtual int64_t now(bool apply) = 0;
  bool ended() const { return ended_; }
  FrameWalk out;

 protected:
  bool ended_ = false;
  void event(int32_t block, bool eof) {
    if (eof) ended_ = true;
    out.reads.push_back(ReadEvent{block, eof, now(false)});
  }
};

class VdifWalker : public Walker {
 public:
  VdifWalker(const ReaderParams &p, FrameSource &src) : p_(p), src_(src) {
    if (p.frame_size <= 0) throw std::invalid_argument("VDIF frame size must be positive");
    n_ = src.size();
    fs_ = p.frame_size;
    ref_jday_ = (int)mjd_of_ticks(p.ref_ticks);
    sample_rate_ = (double)p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
    fpb_ = std::max(1, 32128 / fs_);
    if (p.n_tracks == 0) {
      for (size_t i = 0; i < p.first_track.size(); i++) thread_map_[p.first_track[i]] = (int)i;
      fpb_ = 1;
    }
    cstride_ = (int64_t)fs_ + 32;
  }

  int64_t now(bool) override {  // get_current_time (vdif_reader.cc:63-75)
    const double seconds = (double)cur_.seconds - (ref_jday_ - cur_.epoch_mjd) * 24 * 60 * 60;
    double subsec = 0;
    if (sample_rate_ > 0) {
      const int spf = 8 * fs_ / ((first_.bits_m1 + 1) * (1 << first_.log2_nchan));
      subsec = (double)cur_.frame_nr * spf / sample_rate_;
    }
    return ticks_of(ref_jday_, seconds + subsec) - p_.offset_ticks;
  }

  void read() override {  // read_new_block (vdif_reader.cc:77-190)
    if (ended_) return event(-1, true);
    int restarts = 0;
    for (;;) {
      int64_t pos;
      if (!first_seen_) {
        // before the first header: 16-byte candidates fs + 32 apart (a fill
        // header skips a non-legacy frame, vdif_reader.cc:84-100)
        pos = k_ * cstride_;
        if (pos + 16 > n_) return event(-1, true);
        cur_ = candidate(k_);
        if (cur_.flags & FRAME_FILL) {
          k_++;
          if (++restarts > 256) return event(-1, false);
          continue;
        }
        first_ = cur_;
        first_seen_ = true;
        p0_ = pos;
        hs_ = (first_.flags & FRAME_LEGACY) ? 16 : 32;
        if (p0_ + hs_ > n_) return event(-1, true);
        // after it, frames at a fixed stride
        stride_ = hs_ + fs_;
        nf_ = (n_ - p0_ - 16) / stride_ + 1;
        hdr_.resize((size_t)nf_);
        src_.decode(FORMAT_VDIF, p0_, stride_, nf_, hdr_.data());
        block_size_ = fpb_ * std::max(first_.data_size, fs_);
        j_ = 0;
      } else {
        if (!header_in(j_)) return event(-1, true);
        pos = p0_ + j_ * stride_;
        cur_ = hdr_[(size_t)j_];
      }
      const FrameInfo h = cur_;
      if ((h.flags & FRAME_FILL) || h.frame_nr % (uint32_t)fpb_ != 0) {
        j_++;
        if (++restarts > 256) return event(-1, false);
        continue;
      }
      if (pos + hs_ + fs_ > n_) return event(-1, true);
      FrameBlock b;
      auto it = thread_map_.find(h.thread);
      if (h.flags & FRAME_INVALID) {
        b.invalid.push_back(0);
        b.invalid.push_back(fs_);
        b.channel = it != thread_map_.end() ? it->second : 0;
      } else {
        if (it == thread_map_.end()) {
          if (thread_map_.empty()) {  // a single thread: its id comes from the data
            thread_map_[h.thread] = 0;
          } else {
            j_++;
            if (++restarts > 256) return event(-1, false);
            continue;
          }
        }
        b.channel = thread_map_[h.thread];
      }
      b.first = (int64_t)out.frames.size();
      out.frames.push_back(pos + hs_);
      j_++;
      for (int i = 1; i < fpb_; i++, j_++) {
        const int64_t q = p0_ + j_ * stride_;
        if (!header_in(j_) || q + hs_ + fs_ > n_) {
          out.frames.resize((size_t)b.first);
          return event(-1, true);
        }
        out.frames.push_back(q + hs_);
        if (hdr_[(size_t)j_].flags & FRAME_INVALID) {
          b.invalid.push_back(i * fs_);
          b.invalid.push_back(fs_);
        }
      }
      b.start_ticks = now(false);
      b.size = block_size_;
      b.frame_bytes = fs_;
      b.nframes = fpb_;
      out.blocks.push_back(std::move(b));
      return event((int32_t)out.blocks.size() - 1, false);
    }
  }

 private:
  const ReaderParams &p_;
  FrameSource &src_;
  int64_t n_ = 0, cstride_ = 0, k_ = 0, p0_ = 0, stride_ = 0, nf_ = 0, j_ = 0;
  int fs_ = 0, ref_jday_ = 0, fpb_ = 1, hs_ = 32;
  int32_t block_size_ = 0;
  double sample_rate_ = 0;
  bool first_seen_ = false;
  FrameInfo first_{}, cur_{};  // the first header (zero before it); the header the reader holds as current
  std::map<int, int> thread_map_;
  std::vector<FrameInfo> cand_, hdr_;

  bool header_in(int64_t j) const { return j < nf_ && p0_ + j * stride_ + hs_ <= n_; }
  FrameInfo candidate(int64_t k) {  // decoded as needed
    while ((int64_t)cand_.size() <= k) {
      const int64_t k0 = (int64_t)cand_.size();
      int64_t cnt = 0;
      while (cnt < 1024 && (k0 + cnt) * cstride_ + 16 <= n_) cnt++;
      if (cnt == 0) throw std::logic_error("VDIF candidate header past the end");
      cand_.resize((size_t)(k0 + cnt));
      src_.decode(FORMAT_VDIF, k0 * cstride_, cstride_, cnt, cand_.data() + k0);
    }
    return cand_[(size_t)k];
  }
};

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

class Mk5bWalker : public Walker {
 public:
  Mk5bWalker(const ReaderParams &p, FrameSource &src) : p_(p), src_(src) {
    n_ = src.size();
    current_jday_ = (int)mjd_of_ticks(p.ref_ticks);
    bitstreams_ = p.n_tracks;
    const int word = bitstreams_ <= 32 ? 4 : 8;
    const int tbr = p.track_bit_rate;
    if (tbr <= 0 || tbr % 1000000) throw std::invalid_argument("Mark5B track bit rate must be whole Mb/s");
    tbh_ = ticks_of_usec((double)kMk5bBlock / (word * tbr / 1000000));
    sample_rate_ = p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
    const uint8_t zero[16] = {};
    cur_ = prev_ = decode_mk5b(zero);
  }

  int64_t now(bool apply) override {  // get_current_time (mark5b_reader.cc:84-105)
    bool valid = frame_nr_valid_;
    const double rate = (double)sample_rate_ * bitstreams_;
    const double subsec = (double)((uint64_t)(int64_t)frame_nr_ * (8 * kMk5bFrame)) / rate;
    if (subsec > 1 && valid) valid = false;
    if (apply) frame_nr_valid_ = valid;
    int64_t t;
    if (valid) {
      t = ticks_of(current_jday_, (double)cur_.seconds + subsec);
    } else {  // VLBA time stamp, rounded to whole blocks
      const int64_t second = ticks_of(current_jday_, (double)cur_.seconds);
      const int64_t sub = ticks_of_usec((double)cur_.epoch_mjd);
      const int nframes = (int)std::round((double)sub / tbh_);
      t = second + (int64_t)std::round((double)tbh_ * nframes);
    }
    return t - p_.offset_ticks;
  }

  void read() override {  // read_new_block (mark5b_reader.cc:111-162)
    if (ended_) return event(-1, true);
    if (P_ + kMk5bHeader > n_) return event(-1, true);
    if (g0_ < 0 || P_ < g0_ || (P_ - g0_) % kBStride || (P_ - g0_) / kBStride >= (int64_t)grid_.size()) {
      g0_ = P_;  // block-start headers on the grid g0 + k * (8 frames)
      grid_.assign((size_t)((n_ - P_ - kMk5bHeader) / kBStride + 1), FrameInfo{});
      src_.decode(FORMAT_MARK5B, g0_, kBStride, (int64_t)grid_.size(), grid_.data());
    }
    const FrameInfo h = grid_[(size_t)((P_ - g0_) / kBStride)];
    if ((h.flags & FRAME_CHECK) && !(h.frame_nr % kMk5bBlockFrames != 0 && frame_nr_valid_)) {
      prev_ = cur_;
      cur_ = h;
      frame_nr_update();
      if (P_ + kBStride > n_) return event(-1, true);
      int64_t frames[kMk5bBlockFrames];
      for (int i = 0; i < kMk5bBlockFrames; i++) frames[i] = P_ + i * kFStride + kMk5bHeader;
      P_ += kBStride;
      return finish(frames);
    }
    resync(P_ + kMk5bHeader);
  }

  // get_bytes_s without a buffer on a file: nothing once the data has run
  // out, else the whole skip (a seek may pass the end)
  int64_t skip(int64_t bytes) {
    if (ended_) return 0;
    P_ += bytes;
    return bytes;
  }
  int frame_nr() const { return (int)cur_.frame_nr; }
  int64_t position() const { return P_; }

  // resync_header (mark5b_reader.cc:254-327) from recording offset q, on the
  // bytes that follow, fetched once: the scan reads at most 16 blocks plus
  // one frame before it gives up, and a found block's eight frames after
  // that.  Returns whether it found a block.
  bool resync(int64_t q) {
    const int max_read = 16 * kMk5bBlock;
    FetchedBytes r;
    r.n = n_;
    r.base = r.pos = q;
    const int64_t span = std::min<int64_t>(n_ - r.base, 16 + max_read + 2 * kMk5bFrame + kBStride);
    r.b.resize((size_t)std::max<int64_t>(span, 0));
    if (span > 0) src_.fetch(r.base, span, r.b.data());
    std::vector<uint8_t> buf(kMk5bFrame, 0);
    int total = 0;
    bool found = false;
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
        prev_ = cur_;
        cur_ = t;
        int64_t frames[kMk5bBlockFrames] = {frame0};
        for (int i = 1; i < kMk5bBlockFrames; i++) {
          r.get(kMk5bHeader, nullptr);
          frames[i] = r.pos;
          r.get(kMk5bFrame, nullptr);
        }
        if (r.short_read) break;
        frame_nr_update();
        P_ = r.pos;
        finish(frames);
        return true;
      }
    }
    if (r.short_read) {
      event(-1, true);
      return false;
    }
    P_ = r.pos;  // no block within the search limit; the next read starts where this one stopped
    event(-1, false);
    return false;
  }

 private:
  static constexpr int64_t kFStride = kMk5bHeader + kMk5bFrame, kBStride = kMk5bBlockFrames * kFStride;
  const ReaderParams &p_;
  FrameSource &src_;
  int64_t n_ = 0, tbh_ = 0, P_ = 0, g0_ = -1;
  int current_jday_ = 0, bitstreams_ = 0, sample_rate_ = 0, frame_nr_ = -1;
  bool frame_nr_valid_ = true;
  FrameInfo cur_{}, prev_{};
  std::vector<FrameInfo> grid_;

  void frame_nr_update() {  // mark5b_reader.cc:127-131
    if (bitstreams_ == 64 && cur_.seconds == prev_.seconds && frame_nr_ > (int)cur_.frame_nr)
      frame_nr_ = (int)cur_.frame_nr + 32768;
    else
      frame_nr_ = (int)cur_.frame_nr;
  }
  void finish(const int64_t *frames) {  // the julian-day step, then the block's time
    if (cur_.thread != current_jday_ % 1000) current_jday_++;
    FrameBlock b;
    b.start_ticks = now(true);
    b.size = kMk5bBlock;
    b.frame_bytes = kMk5bFrame;
    b.first = (int64_t)out.frames.size();
    b.nframes = kMk5bBlockFrames;
    out.frames.insert(out.frames.end(), frames, frames + kMk5bBlockFrames);
    out.blocks.push_back(std::move(b));
    event((int32_t)out.blocks.size() - 1, false);
  }
};

std::unique_ptr<Walker> make_walker(const ReaderParams &p, FrameSource &src) {
  if (p.bits_per_sample != 1 && p.bits_per_sample != 2) throw std::invalid_argument("bits per sample must be 1 or 2");
  if (p.tracks_per_channel < p.bits_per_sample) throw std::invalid_argument("fewer tracks than bits per sample");
  if (p.track_bit_rate <= 0) throw std::invalid_argument("track bit rate must be positive");
  if (p.format == FORMAT_VDIF) return std::unique_ptr<Walker>(new VdifWalker(p, src));
  if (p.format == FORMAT_MARK5B) return std::unique_ptr<Walker>(new Mk5bWalker(p, src));
  throw std::invalid_argument("unknown recording format");
}

}  // namespace

FrameWalk walk_frames(const ReaderParams &p, FrameSource &src) {
  std::unique_ptr<Walker> w = make_walker(p, src);
  while (!w->ended()) w->read();
  return std::move(w->out);
}

// ---- Input_data_format_reader_tasklet over a walker
int64_t reader_tbh(const ReaderParams &p) {
  // time_between_headers (vdif_reader.cc:211-222, mark5b_reader.cc:245-247), as Time(usec) rounds it
  const double sample_rate = (double)p.track_bit_rate * (p.tracks_per_channel / p.bits_per_sample);
  double usec;
  if (p.format == FORMAT_VDIF) {
    if (p.n_tracks == 0)
      usec = p.frame_size * 8.e6 / (sample_rate * p.bits_per_sample);
    else
      usec = std::max(1, 32128 / p.frame_size) * p.frame_size * 8.e6 / (sample_rate * p.n_tracks);
  } else {
    const int word = p.n_tracks <= 32 ? 4 : 8;
    usec = (double)kMk5bBlock / (word * p.track_bit_rate / 1000000);
  }
  return ticks_of_usec(usec);
}

namespace {
constexpr int kSkipFrames = 16;   // NSKIP (input_data_format_reader_tasklet.cc:2)
constexpr int kSkewFrames = 128;  // NSKEW (input_data_format_reader_tasklet.cc:3)

// The tasklet's current frame (input_element_): the walk block last read
// into its buffer, its invalid runs, and whether its bytes are not a
// block's (a new buffer, or a read that failed into it: the reference pushes
// such bytes as they are, here they go out wholly invalid).
struct Element {
  int64_t start = 0;
  int channel = 0;
  int32_t block = -1;
  bool stale = true, whole = false;
  std::vector<int32_t> runs;
};

class Tasklet {
 public:
  Tasklet(const ReaderParams &p, Walker &w) : w_(w), tbh_(reader_tbh(p)) {
    if (tbh_ <= 0) throw std::invalid_argument("no time between frame headers");
    mk5b_ = p.format == FORMAT_MARK5B;
    not_open_time_ = mk5b_ ? 0 : -p.offset_ticks;
    thread_mode_ = p.format == FORMAT_VDIF && p.n_tracks == 0;
    // set_parameters (input_data_format_reader_tasklet.cc:262-297)
    const int nt = thread_mode_ ? (int)p.first_track.size() : 1;
    current_.assign(nt, 0);
    left_.assign(nt, 0);
    dup_.assign(nt, {});
    if (thread_mode_)
      for (int i = 0; i < nt; i++)
        for (int j = 0; j < nt; j++)
          if (j != i && p.first_track[j] == p.first_track[i]) dup_[i].push_back(j);
  }

  std::vector<ScheduledBlock> run(const std::vector<TimeInterval> &intervals) {
    // do_execute (33-47): an empty interval (stop <= start) ends it
    size_t next = 0;
    auto fetch = [&]() -> bool {
      if (next >= intervals.size() || intervals[next].stop <= intervals[next].start) return false;
      fetch_interval(intervals[next++]);
      return true;
    };
    if (!fetch()) return out_;
    // every step pushes a block, reads one or takes the next interval; steps
    // that do none of these in a row mean the reference would not finish
    int idle = 0;
    for (;;) {
      const size_t pushed = out_.size(), reads = w_.out.reads.size();
      if (*std::min_element(current_.begin(), current_.end()) < iv_.stop) {
        do_task();
        idle = (out_.size() == pushed && w_.out.reads.size() == reads) ? idle + 1 : 0;
        if (idle > 1000) throw std::runtime_error("reader tasklet makes no progress in its interval");
      } else if (!fetch()) {
        return out_;
      }
    }
  }

 private:
  Walker &w_;
  int64_t tbh_, not_open_time_ = 0;
  bool mk5b_ = false, thread_mode_ = false, open_ = false;
  TimeInterval iv_{};
  std::vector<int64_t> current_;
  std::vector<int> left_;
  int min_left_ = 0;
  std::vector<std::vector<int>> dup_;
  Element e_;
  std::vector<ScheduledBlock> out_;

  int64_t times(int64_t nframes) const { return (int64_t)std::round((double)tbh_ * (double)nframes); }
  int frames_between(int64_t a, int64_t b) const { return (int)((double)(b - a) / (double)tbh_); }
  int64_t reader_now(bool apply = false) { return open_ ? w_.now(apply) : not_open_time_; }

  // read_new_block into the element: VDIF appends the block's invalid runs
  // to the frame's, Mark5B replaces them (mark5b_reader.cc:157-160)
  bool read() {
    w_.read();
    const ReadEvent &ev = w_.out.reads.back();
    if (ev.block < 0) {
      e_.stale = true;
      return false;
    }
    const FrameBlock &b = w_.out.blocks[(size_t)ev.block];
    e_.block = ev.block;
    e_.stale = false;
    e_.start = open_ ? b.start_ticks : not_open_time_;
    e_.channel = thread_mode_ ? b.channel : 0;
    if (mk5b_) {
      e_.whole = false;
      e_.runs.clear();
    } else {
      e_.runs.insert(e_.runs.end(), b.invalid.begin(), b.invalid.end());
    }
    return true;
  }
  void randomize() {  // randomize_block (342-370): the frame wholly invalid
    e_.whole = true;
    e_.runs.clear();
  }
  bool open_stream() {  // open_input_stream
    if (!read()) return false;
    open_ = true;
    e_.start = w_.out.blocks[(size_t)e_.block].start_ticks;
    return true;
  }
  int64_t goto_time(int64_t t) {
    if (!mk5b_) {  // VDIF_reader::goto_time (vdif_reader.cc:51-57)
      while (t > reader_now())
        if (!read()) break;
      return reader_now();
    }
    // Mark5b_reader::goto_time on a file (mark5b_reader.cc:44-84): skip a
    // second's blocks at a time, then the rest, reading the last block of each step
    Mk5bWalker &m = static_cast<Mk5bWalker &>(w_);
    const int64_t one_sec = 512000000;
    if (t > reader_now(true)) {
      int64_t delta = t - reader_now(true);
      while (delta >= one_sec) {
        const int64_t nb = (int64_t)((double)one_sec / (double)tbh_);
        const int64_t bytes = (nb - 1) * kMk5bBlockFrames * (kMk5bHeader + kMk5bFrame);
        if (m.skip(bytes) != bytes) return reader_now(true);
        read();
        delta = t - reader_now(true);
      }
      const int nb = (int)std::round((double)delta / (double)tbh_);
      if (nb > 0) {
        const int64_t bytes = (int64_t)(nb - 1) * kMk5bBlockFrames * (kMk5bHeader + kMk5bFrame);
        if (m.skip(bytes) != bytes) return reader_now(true);
        read();
        if (m.frame_nr() % kMk5bBlockFrames != 0) {
          // the reader returns resync_header's result as a time: 0 or 1 microsecond
          const size_t before = w_.out.blocks.size();
          const bool ok = m.resync(m.position());
          if (ok && w_.out.blocks.size() > before) e_.block = (int32_t)before;
          return ok ? ticks_of_usec(1.0) : 0;
        }
      }
    }
    return reader_now(true);
  }

  void push() {  // push_element (324-337)
    const int c = e_.channel;
    // a filled-in frame keeps the runs reads appended to it after (0, size)
    const bool whole = e_.whole || e_.stale || e_.block < 0;
    out_.push_back(ScheduledBlock{e_.start, c, e_.block, whole,
                                  (whole && (e_.stale || !e_.whole)) ? std::vector<int32_t>() : e_.runs});
    current_[c] += tbh_;
    left_[c]--;
    if (left_[c] < min_left_) min_left_ = left_[c];
  }
  void push_random(int n, int c) {  // push_random_blocks (230-240)
    for (int i = 0; i < n; i++) {
      randomize();
      e_.start = current_[c];
      e_.channel = c;
      push();
    }
  }

  // fetch_next_time_interval (175-228)
  void fetch_interval(const TimeInterval &iv) {
    iv_ = iv;
    if (!open_ && !open_stream()) {
      for (size_t i = 0; i < current_.size(); i++) {
        current_[i] = iv.start;
        left_[i] = frames_between(current_[i], iv.stop);
      }
      min_left_ = left_[0];
      return;
    }
    int64_t t;
    if (iv.start <= e_.start) {
      t = iv.start + times((int64_t)std::round((double)(e_.start - iv.start) / (double)tbh_));
    } else {
      e_.start = goto_time(iv.start);  // the element takes the reader's time
      t = iv.start + times((int64_t)std::round((double)(e_.start - iv.start) / (double)tbh_));
      if (t < iv.start) t = iv.start;
    }
    if (t > iv.stop) {
      t = iv.stop - tbh_;
      randomize();
      e_.start = t;
      e_.channel = 0;
    }
    for (size_t i = 0; i < current_.size(); i++) {
      current_[i] = t;
      left_[i] = frames_between(current_[i], iv.stop);
    }
    min_left_ = left_[0];
    push();
  }

  // do_task (49-160)
  void do_task() {
    e_ = Element();  // allocate_element
    if (w_.ended()) {  // the data reader is at its end
      for (size_t i = 0; i < current_.size(); i++)
        if (current_[i] < iv_.stop) push_random(1, (int)i);
      return;
    }
    for (size_t i = 0; i < current_.size(); i++) {
      const int skew = std::max(0, std::min(2 * kSkewFrames, left_[i] - 1));
      if (left_[i] > min_left_ + skew) {
        push_random((left_[i] - min_left_) - skew, (int)i);
        return;
      }
    }
    if (!read()) {
      push_random(std::min(kSkipFrames, left_[0]), 0);
      return;
    }
    const int c = e_.channel;
    if (c < 0 || c >= (int)current_.size()) throw std::runtime_error("block of a channel outside the channel list");
    if (current_[c] >= iv_.leave) {
      push_random(std::min(kSkipFrames, left_[0]), c);
      return;
    }
    const int64_t expected = current_[c];
    if (e_.start != expected) {
      int64_t missing = (int64_t)((double)(e_.start - expected) / (double)tbh_);
      missing = std::min(missing, (int64_t)left_[c]);
      // (the reference also drops a frame from more than 5 s after the host's
      // clock, a causality check on live data; recorded data is in the past)
      if (missing > 0) {
        const Element keep = e_;
        push_random((int)missing, c);
        e_ = keep;
      } else if (missing < 0) {
        return;  // data from the past: dropped
      }
      if (missing >= left_[c]) return;
    }
    if (e_.start != current_[c]) throw std::runtime_error("reader block off its channel's time grid");
    push();
    for (int j : dup_[c]) {
      e_.channel = j;
      push();
    }
  }
};
}  // namespace

Schedule schedule_blocks(const ReaderParams &p, FrameSource &src, const std::vector<TimeInterval> &intervals) {
  std::unique_ptr<Walker> w = make_walker(p, src);
  Tasklet t(p, *w);
  Schedule s;
  s.blocks = t.run(intervals);
  s.walk = std::move(w->out);
  return s;
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
