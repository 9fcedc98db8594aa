// VDIF and Mark5B readers (formats.hpp).  Every rule below restates the
// reference's reader behaviour; the file:line cites are the reference's.
#include "formats.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>

namespace sfxc {
namespace {

constexpr double kClockRate = 512000000.0;  // Time ticks per second (sfxc/include/utils.h:36)
constexpr int kReferenceMjd = 51544;        // sfxc/include/correlator_time.h:9
constexpr uint32_t kFill = 0x11223344u;     // MARK5_FILLPATTERN (sfxc/include/utils.h:45)
constexpr int kFillWords = 65528 / 4;       // MARK5_FILLPATTERN_NWORDS (utils.h:47)

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
  uint32_t w(int i) const { return word_at(b, i); }
  uint32_t sec_from_epoch() const { return w(0) & 0x3FFFFFFFu; }
  int legacy() const { return (w(0) >> 30) & 1; }
  int invalid() const { return (w(0) >> 31) & 1; }
  uint32_t frame_in_second() const { return w(1) & 0xFFFFFFu; }
  int ref_epoch() const { return (w(1) >> 24) & 0x3F; }
  uint32_t frame_length8() const { return w(2) & 0xFFFFFFu; }
  int log2_nchan() const { return (w(2) >> 24) & 0x1F; }
  int thread_id() const { return (w(3) >> 16) & 0x3FF; }
  int bits_minus_one() const { return (w(3) >> 26) & 0x1F; }
  int header_size() const { return 16 + 16 * (1 - legacy()); }
  int data_size() const { return 8 * (int)frame_length8() - header_size(); }
  int jday_epoch() const { return mjd_of_date(1, 1 + 6 * (ref_epoch() % 2), 2000 + ref_epoch() / 2); }
  bool fill() const {
    return w(0) == kFill || w(1) == kFill || w(2) == kFill || w(3) == kFill;
  }
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
  uint32_t sync() const { return word_at(b, 0); }
  int frame_nr() const { return (int)(word_at(b, 1) & 0x7FFF); }
  int nib(int byte, int high) const { return high ? b[byte] >> 4 : b[byte] & 0xF; }
  // BCD fields: word 2 = JJJSSSSS, word 3 = .SSSS (high half) and the CRC
  int64_t seconds() const {
    return ((((int64_t)nib(10, 0) * 10 + nib(9, 1)) * 10 + nib(9, 0)) * 10 + nib(8, 1)) * 10 + nib(8, 0);
  }
  int64_t microseconds() const {
    const int64_t sub = ((((int64_t)nib(15, 1) * 10 + nib(15, 0)) * 10 + nib(14, 1)) * 10 + nib(14, 0)) * 100;
    return 1000000 * seconds() + sub;
  }
  int julian_day() const { return (nib(11, 1) * 10 + nib(11, 0)) * 10 + nib(10, 1); }
  uint16_t crc() const { return (uint16_t)(b[12] | (b[13] << 8)); }
  bool subsec_zero() const { return b[14] == 0 && b[15] == 0; }
};

class Mark5bReader : public FormatReader {
 public:
  Mark5bReader(const ReaderParams &p, const uint8_t *bytes, size_t n) : src_(bytes, n) {
    // CRC-16 table, polynomial 0x8005, 16-bit register (mark5b_reader.cc:195-209)
    for (int i = 0; i < 256; i++) {
      uint16_t c = (uint16_t)(i << 8);
      for (int j = 0; j < 8; j++) c = (c & 0x8000) ? (uint16_t)((c << 1) ^ 0x8005) : (uint16_t)(c << 1);
      crc_table_[i] = c;
    }
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
  uint16_t crc_table_[256];
  int current_jday_ = 0, bitstreams_ = 0, sample_rate_ = 0, frame_nr_ = -1;
  int64_t tbh_ = 0, offset_ = 0;
  bool open_ = false, frame_nr_valid_ = true;
  Mk5bHeader cur_, tmp_, prev_;

  // check_header (mark5b_reader.cc:211-239): the register is a 32-bit
  // unsigned that is never masked to 16 bits
  bool check(const Mk5bHeader &h) const {
    if (h.sync() != 0xABADDEEDu) return false;
    if (h.crc() == 0) return true;
    if (h.subsec_zero() && h.frame_nr() != 0) return true;
    uint32_t crc = 0;
    for (int word = 2; word <= 3; word++)
      for (int i = 3; i >= 0; i--) {
        crc ^= (uint32_t)h.b[word * 4 + i] << 8;
        crc = (crc << 8) ^ crc_table_[(crc >> 8) & 0xff];
      }
    return crc == 0;
  }

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

  // Input_data_format_reader::find_fill_pattern (input_data_format_reader.cc:20-72):
  // galloping search for runs of the fill word, 4-byte granularity
  static void find_fill_pattern(ReaderBlock &out) {
    const int nw = (int)(out.data.size() / 4);
    auto w = [&](int i) { return word_at(out.data.data(), i); };
    int start = 0;
    while (start < nw) {
      if (w(start) != kFill) {
        int step = std::min(kFillWords, nw - start - 1);
        while (step > 0) {
          if (w(start + step) != kFill) {
            start += step;
            step = std::min(step, nw - start - 1);
          } else {
            step /= 2;
          }
        }
        start += 1;
      }
      if (start >= nw) break;
      int end = start;
      int step = std::min(kFillWords, nw - end - 1);
      while (step > 0) {
        if (w(end + step) == kFill) {
          end += step;
          step = std::min(step, nw - end - 1);
        } else {
          step /= 2;
        }
      }
      out.invalid.push_back(start * 4);
      out.invalid.push_back((end - start + 1) * 4);
      start = end + 1;
    }
  }
};

}  // namespace

int mjd_of_date(int day, int month, int year) {
  // days since 0000-03-01 of the proleptic Gregorian calendar, less the
  // count for 1858-11-17
  const int y = year - (month <= 2 ? 1 : 0);
  const int era = (y >= 0 ? y : y - 399) / 400;
  const int yoe = y - era * 400;
  const int mp = (month + 9) % 12;
  const int doy = (153 * mp + 2) / 5 + day - 1;
  const int doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 678881;
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
