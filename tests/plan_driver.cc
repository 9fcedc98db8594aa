// Test driver (CPU): runs the library's host-side unpack plan (host.cpp's
// plan_unpack, the Bit2float_worker replica) over consecutive integrations of
// one stream's protocol and decodes the planned samples, so that the plan can
// be checked against the reference's unpacked-sample digests without a GPU.
// Also prints the counted-byte histogram and the invalid runs.
//
// usage: plan_driver <protocol file: per integration u64 length + bytes>
//                    <n_integrations> <n_blocks> <nfft_max> <bits> <sample_rate>
//                    <tsys_freq> <delay_at_start per integration...> <out prefix>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "host.hpp"

using namespace sfxc;

int main(int argc, char **argv) {
  if (argc < 9) return 2;
  std::ifstream in(argv[1], std::ios::binary);
  std::vector<uint8_t> all((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  const int nint = std::atoi(argv[2]), n_blocks = std::atoi(argv[3]), nfft_max = std::atoi(argv[4]);
  const int bits = std::atoi(argv[5]), sr = std::atoi(argv[6]), tsys_freq = std::atoi(argv[7]);
  if (argc != 8 + nint + 1) return 2;
  const std::string prefix = argv[8 + nint];
  StreamUnpackState st;
  std::vector<Record> recs;
  size_t pos = 0;
  const float lut2[4] = {-7, -2, 2, 7}, lut1[2] = {-5, 5};
  try {
    for (int it = 0; it < nint; it++) {
      uint64_t len;
      std::memcpy(&len, &all[pos], 8);
      pos += 8;
      const uint8_t *chunk = &all[pos];
      std::vector<Record> next(recs.begin() + (long)st.rec, recs.end());
      std::vector<Record> fresh = parse_protocol(chunk, len, 0);
      next.insert(next.end(), fresh.begin(), fresh.end());
      recs.swap(next);
      st.rec = 0;
      UnpackPlan p = plan_unpack(recs, st, n_blocks, nfft_max, 256, bits, sr, tsys_freq, std::atof(argv[8 + it]));
      std::vector<float> out((size_t)n_blocks * 256, 0.0f);
      for (const Segment &g : p.segs) {
        if (g.src_bit < 0) continue;
        for (int k = 0; k < g.n; k++) {
          const int64_t bit = g.src_bit + (int64_t)k * bits;
          const int code = (chunk[bit >> 3] >> (bit & 7)) & ((1 << bits) - 1);
          out[(size_t)g.out0 + k] = bits == 2 ? lut2[code] : lut1[code];
        }
      }
      FILE *f = std::fopen((prefix + "_u" + std::to_string(it) + ".f32").c_str(), "wb");
      std::fwrite(out.data(), 4, out.size(), f);
      std::fclose(f);
      // histogram of counted bytes with the cal-diode split
      std::vector<long long> h(512, 0);
      for (const StatRange &r : p.stats)
        for (int j = 0; j < r.n; j++) {
          const long long c = (long long)r.cidx + j;
          int on = p.tsys.two_bit ? p.tsys.on0 : 1;
          if (p.tsys.two_bit && p.tsys.t0 > 0 && c >= p.tsys.t0)
            on ^= (int)((p.tsys.period > 0 ? 1 + (c - p.tsys.t0) / p.tsys.period : 1) & 1);
          h[(on ? 0 : 256) + chunk[r.src_byte + j]]++;
        }
      f = std::fopen((prefix + "_h" + std::to_string(it) + ".txt").c_str(), "w");
      for (int k = 0; k < 512; k++) std::fprintf(f, "%lld\n", h[k]);
      std::fprintf(f, "%lld\n", (long long)p.n_invalid);
      for (const InvalidRun &r : p.invalid) std::fprintf(f, "I %d %d\n", r.begin, r.n);
      std::fclose(f);
      pos += len;
    }
  } catch (const Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
