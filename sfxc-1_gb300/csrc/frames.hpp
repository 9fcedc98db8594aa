// Frame headers of station recordings, decoded the same way on the host and
// on the device: VDIF headers (sfxc/include/vdif_reader.h:36-61, fields as
// VDIF_reader uses them in sfxc/src/vdif_reader.cc:19-226) and Mark5B headers
// (sfxc/include/mark5b_reader.h:33-55, with Mark5b_reader::check_header's
// CRC, sfxc/src/mark5b_reader.cc:195-239), plus the fill-pattern run search
// of Input_data_format_reader::find_fill_pattern
// (sfxc/src/input_data_format_reader.cc:20-72).  Plain integer code, compiled
// both for the host reader and for the device decode kernels.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define SFXC_HD __host__ __device__ __forceinline__
#else
#define SFXC_HD inline
#endif

namespace sfxc {

constexpr uint32_t kFillWord = 0x11223344u;  // MARK5_FILLPATTERN (sfxc/include/utils.h:45)
constexpr int kFillRunWords = 65528 / 4;     // MARK5_FILLPATTERN_NWORDS (sfxc/include/utils.h:47)
constexpr uint32_t kMk5bSync = 0xABADDEEDu;
constexpr int kMk5bFrame = 2500 * 4;  // payload bytes: SIZE_MK5B_FRAME words of SIZE_MK5B_WORD bytes
constexpr int kMk5bHeader = 4 * 4;    // SIZE_MK5B_HEADER words
constexpr int kMk5bBlockFrames = 8;   // N_MK5B_BLOCKS_TO_READ
constexpr int kMk5bBlock = kMk5bBlockFrames * kMk5bFrame;

enum : uint32_t {
  FRAME_FILL = 1,     // VDIF: one of header words 0-3 is the fill word
  FRAME_INVALID = 2,  // VDIF: the invalid bit of word 0
  FRAME_LEGACY = 4,   // VDIF: the legacy bit (16-byte header)
  FRAME_SYNC = 8,     // Mark5B: word 0 is the sync word
  FRAME_CHECK = 16,   // Mark5B: check_header passes (sync, then zero CRC field, or the CRC rule)
};

// One decoded frame header (32 bytes).  VDIF / Mark5B meaning per field.
struct FrameInfo {
  uint32_t flags;       // FRAME_*
  uint32_t seconds;     // seconds from the reference epoch / BCD seconds of the day (5 digits)
  uint32_t frame_nr;    // frame within the second (24 bits) / frame number (15 bits)
  int32_t thread;       // thread id / julian day (3 BCD digits)
  int32_t epoch_mjd;    // MJD of the reference epoch / sub-second in microseconds (BCD .SSSS x 100)
  int32_t bits_m1;      // bits per sample - 1 / 0
  int32_t log2_nchan;   // log2 channels / 0
  int32_t data_size;    // 8 x frame length - header size / 0
};

SFXC_HD uint32_t le32(const uint8_t *b) {
  return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}

// Modified Julian Day of a Gregorian date (days since 0000-03-01 of the
// proleptic Gregorian calendar, less the count for 1858-11-17).
SFXC_HD int mjd_from_date(int day, int month, int year) {
  const int y = year - (month <= 2 ? 1 : 0);
  const int era = (y >= 0 ? y : y - 399) / 400;
  const int yoe = y - era * 400;
  const int mp = (month + 9) % 12;
  const int doy = (153 * mp + 2) / 5 + day - 1;
  const int doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 678881;
}

// The first 16 header bytes of a VDIF frame.
SFXC_HD FrameInfo decode_vdif(const uint8_t *h) {
  const uint32_t w0 = le32(h), w1 = le32(h + 4), w2 = le32(h + 8), w3 = le32(h + 12);
  FrameInfo f;
  const int legacy = (w0 >> 30) & 1;
  f.flags = ((w0 == kFillWord || w1 == kFillWord || w2 == kFillWord || w3 == kFillWord) ? FRAME_FILL : 0u) |
            (((w0 >> 31) & 1) ? FRAME_INVALID : 0u) | (legacy ? FRAME_LEGACY : 0u);
  f.seconds = w0 & 0x3FFFFFFFu;
  f.frame_nr = w1 & 0xFFFFFFu;
  f.thread = (int32_t)((w3 >> 16) & 0x3FF);
  const int epoch = (int)((w1 >> 24) & 0x3F);  // half-years since 2000
  f.epoch_mjd = mjd_from_date(1, 1 + 6 * (epoch % 2), 2000 + epoch / 2);
  f.bits_m1 = (int32_t)((w3 >> 26) & 0x1F);
  f.log2_nchan = (int32_t)((w2 >> 24) & 0x1F);
  f.data_size = 8 * (int32_t)(w2 & 0xFFFFFFu) - (16 + 16 * (1 - legacy));
  return f;
}

// CRC-16 table entry, polynomial 0x8005, 16-bit register.
SFXC_HD uint32_t crc16_entry(uint32_t i) {
  uint32_t c = (i << 8) & 0xFFFFu;
  for (int j = 0; j < 8; j++) c = (c & 0x8000u) ? (((c << 1) ^ 0x8005u) & 0xFFFFu) : ((c << 1) & 0xFFFFu);
  return c;
}

// The 16 header bytes of a Mark5B frame.  Words 2-3 hold BCD JJJSSSSS and
// .SSSS (high half of word 3) and the CRC (low half).
SFXC_HD FrameInfo decode_mk5b(const uint8_t *h) {
  auto nib = [h](int byte, int high) -> int { return high ? h[byte] >> 4 : h[byte] & 0xF; };
  FrameInfo f;
  const uint32_t sync = le32(h);
  const int frame_nr = (int)(le32(h + 4) & 0x7FFF);
  const int secs = (((nib(10, 0) * 10 + nib(9, 1)) * 10 + nib(9, 0)) * 10 + nib(8, 1)) * 10 + nib(8, 0);
  const int sub = (((nib(15, 1) * 10 + nib(15, 0)) * 10 + nib(14, 1)) * 10 + nib(14, 0)) * 100;
  const uint32_t crc_field = (uint32_t)h[12] | ((uint32_t)h[13] << 8);
  bool ok = false;
  if (sync == kMk5bSync) {
    if (crc_field == 0) {
      ok = true;
    } else if (h[14] == 0 && h[15] == 0 && frame_nr != 0) {
      ok = true;
    } else {
      // the reader's register is a 32-bit unsigned that is never masked to 16 bits
      uint32_t crc = 0;
      for (int word = 2; word <= 3; word++)
        for (int i = 3; i >= 0; i--) {
          crc ^= (uint32_t)h[word * 4 + i] << 8;
          crc = (crc << 8) ^ crc16_entry((crc >> 8) & 0xff);
        }
      ok = crc == 0;
    }
  }
  f.flags = (sync == kMk5bSync ? FRAME_SYNC : 0u) | (ok ? FRAME_CHECK : 0u);
  f.seconds = (uint32_t)secs;
  f.frame_nr = (uint32_t)frame_nr;
  f.thread = (nib(11, 1) * 10 + nib(11, 0)) * 10 + nib(10, 1);
  f.epoch_mjd = sub;
  f.bits_m1 = 0;
  f.log2_nchan = 0;
  f.data_size = 0;
  return f;
}

// Fill-pattern runs of a block of nw 32-bit words, as the reader's galloping
// search finds them (4-byte granularity; runs shorter than the probe step
// between two non-fill probes are not seen, as in the reader).  w(i) is word
// i; emit(begin_byte, n_bytes) takes each run.
template <class W, class E>
SFXC_HD void fill_pattern_runs(const W &w, int nw, E &emit) {
  auto lo = [](int a, int b) { return a < b ? a : b; };
  int start = 0;
  while (start < nw) {
    if (w(start) != kFillWord) {
      int step = lo(kFillRunWords, nw - start - 1);
      while (step > 0) {
        if (w(start + step) != kFillWord) {
          start += step;
          step = lo(step, nw - start - 1);
        } else {
          step /= 2;
        }
      }
      start += 1;
    }
    if (start >= nw) break;
    int end = start;
    int step = lo(kFillRunWords, nw - end - 1);
    while (step > 0) {
      if (w(end + step) == kFillWord) {
        end += step;
        step = lo(step, nw - end - 1);
      } else {
        step /= 2;
      }
    }
    emit(start * 4, (end - start + 1) * 4);
    start = end + 1;
  }
}

}  // namespace sfxc
