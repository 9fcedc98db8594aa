// Test driver (CPU): runs the library's frame walker (formats.cpp's
// walk_frames, the readers restated on decoded headers) over a recording
// held in host memory, with the headers decoded by the same functions the
// device decode kernel runs (frames.hpp), and assembles each block's bytes
// from its frame offsets, Mark5B blocks with their fill-pattern runs, so
// that the walk can be checked against the reference readers' blocks
// without a GPU.
//
// With time intervals, the blocks the reader tasklet pushes instead
// (schedule_blocks): wholly invalid blocks have no bytes in the output.
//
// usage: walk_driver <recording> <block bytes out> <format 0 vdif / 1 mark5b>
//                    <ref_ticks> <offset_ticks> <track_bit_rate> <frame_size>
//                    <n_tracks> <bits> <tracks_per_channel>
//                    <n_intervals> <start stop leave>... <first_track...>
// stdout: one line per block: channel start_ticks size n_runs begin n ...
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <vector>

#include "formats.hpp"

using namespace sfxc;

struct HostFrames : FrameSource {
  std::vector<uint8_t> b;
  int64_t size() const override { return (int64_t)b.size(); }
  void decode(int format, int64_t pos0, int64_t stride, int64_t count, FrameInfo *out) override {
    for (int64_t k = 0; k < count; k++) {
      const uint8_t *h = b.data() + pos0 + k * stride;
      out[k] = format == FORMAT_VDIF ? decode_vdif(h) : decode_mk5b(h);
    }
  }
  void fetch(int64_t pos, int64_t len, uint8_t *dst) override { std::memcpy(dst, b.data() + pos, (size_t)len); }
};

int main(int argc, char **argv) {
  if (argc < 12) return 2;
  HostFrames src;
  std::ifstream in(argv[1], std::ios::binary);
  src.b.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
  ReaderParams p;
  p.format = std::atoi(argv[3]);
  p.ref_ticks = std::atoll(argv[4]);
  p.offset_ticks = std::atoll(argv[5]);
  p.track_bit_rate = std::atoi(argv[6]);
  p.frame_size = std::atoi(argv[7]);
  p.n_tracks = std::atoi(argv[8]);
  p.bits_per_sample = std::atoi(argv[9]);
  p.tracks_per_channel = std::atoi(argv[10]);
  const int niv = std::atoi(argv[11]);
  std::vector<TimeInterval> iv;
  for (int k = 0; k < niv; k++)
    iv.push_back(TimeInterval{std::atoll(argv[12 + 3 * k]), std::atoll(argv[13 + 3 * k]), std::atoll(argv[14 + 3 * k])});
  for (int i = 12 + 3 * niv; i < argc; i++) p.first_track.push_back(std::atoi(argv[i]));
  FrameWalk walk;
  std::ofstream out(argv[2], std::ios::binary);
  std::vector<ScheduledBlock> sched;
  if (niv) {
    Schedule s = schedule_blocks(p, src, iv);
    walk = std::move(s.walk);
    sched = std::move(s.blocks);
  } else {
    walk = walk_frames(p, src);
    for (size_t b = 0; b < walk.blocks.size(); b++)
      sched.push_back(
          ScheduledBlock{walk.blocks[b].start_ticks, walk.blocks[b].channel, (int32_t)b, false, walk.blocks[b].invalid});
  }
  const int32_t size = walk.blocks.empty() ? 0 : walk.blocks[0].size;
  for (const ScheduledBlock &sb : sched) {
    if (sb.whole_invalid) {  // a wholly invalid block: no bytes
      std::printf("%d %lld %d %d 0 %d", sb.channel, (long long)sb.start_ticks, size, 1 + (int)sb.invalid.size() / 2,
                  size);
      for (int32_t v : sb.invalid) std::printf(" %d", v);
      std::printf("\n");
      continue;
    }
    FrameBlock blk = walk.blocks[(size_t)sb.block];
    blk.channel = sb.channel;
    blk.start_ticks = sb.start_ticks;
    blk.invalid = sb.invalid;
    std::vector<uint8_t> data((size_t)blk.size, 0);
    for (int i = 0; i < blk.nframes; i++)
      std::memcpy(data.data() + (size_t)i * blk.frame_bytes, src.b.data() + walk.frames[(size_t)(blk.first + i)],
                  (size_t)blk.frame_bytes);
    if (p.format == FORMAT_MARK5B) {
      const uint8_t *d = data.data();
      auto w = [d](int i) {
        uint32_t v;
        std::memcpy(&v, d + 4 * i, 4);
        return v;
      };
      auto emit = [&blk](int begin, int n) {
        blk.invalid.push_back(begin);
        blk.invalid.push_back(n);
      };
      fill_pattern_runs(w, blk.size / 4, emit);
    }
    bool whole = false;
    for (size_t k = 0; k + 1 < blk.invalid.size(); k += 2)
      if (blk.invalid[k] == 0 && blk.invalid[k + 1] >= blk.size) whole = true;
    if (!niv || !whole) out.write((const char *)data.data(), (std::streamsize)data.size());
    std::printf("%d %lld %d %d", blk.channel, (long long)blk.start_ticks, blk.size, (int)blk.invalid.size() / 2);
    for (int32_t v : blk.invalid) std::printf(" %d", v);
    std::printf("\n");
  }
  return 0;
}
