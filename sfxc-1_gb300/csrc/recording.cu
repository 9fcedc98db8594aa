// The input node's front end on a recording in device memory: frame-header
// decode (VDIF_reader / Mark5b_reader headers, sfxc/src/vdif_reader.cc,
// sfxc/src/mark5b_reader.cc), the fill-pattern run search of
// Input_data_format_reader::find_fill_pattern
// (sfxc/src/input_data_format_reader.cc:20-72), the channel extractor
// reading each block's frames where they lie (Channel_extractor_5,
// sfxc/src/channel_extractor_5.cc:67-99), and the input-node writer's byte
// protocol assembled from its records (Input_node_data_writer::do_task,
// sfxc/src/input_node_data_writer.cc:107-229; record bytes of
// sfxc/include/correlator_node_types.h:14-31).  All of it is byte work
// bound by memory traffic; the block, skip and resync decisions run on the
// host over the decoded headers (formats.cpp, walk_frames).
#include <algorithm>

#include "frames.hpp"
#include "kernels.hpp"

namespace sfxc {
namespace {

// One thread per frame: the 16 header bytes at pos0 + k * stride.
__global__ void decode_frames_kernel(const uint8_t *__restrict__ rec, int64_t pos0, int64_t stride, int64_t count,
                                     int mk5b, FrameInfo *__restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint8_t *p = rec + pos0 + k * stride;
  uint8_t h[16];
  if (((uintptr_t)p & 15) == 0) {
    const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    for (int i = 0; i < 16; i++) h[i] = (uint8_t)(w[i >> 2] >> (8 * (i & 3)));
  } else {
    for (int i = 0; i < 16; i++) h[i] = p[i];
  }
  out[k] = mk5b ? decode_mk5b(h) : decode_vdif(h);
}

// The 32-bit words of one reader block: nf frames of wpf words at the
// recording offsets frames[0..nf), zeros after them.
struct BlockWords {
  const uint8_t *rec;
  const int64_t *frames;
  int nf, wpf;
  __device__ uint32_t operator()(int i) const {
    const int f = i / wpf;
    return f < nf ? le32(rec + frames[f] + 4 * (i - f * wpf)) : 0u;
  }
};

// One thread per block: the fill-pattern runs of its nw words.  Pass 1
// counts them, pass 2 writes (begin, n) byte pairs at 2 * offsets[b].
template <bool WRITE>
__global__ void fill_runs_kernel(const uint8_t *__restrict__ rec, const int64_t *__restrict__ frames, int nf,
                                 int wpf, int nw, int nblocks, int32_t *__restrict__ counts,
                                 const int64_t *__restrict__ offsets, int32_t *__restrict__ runs) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  const BlockWords w{rec, frames + (int64_t)b * nf, nf, wpf};
  int c = 0;
  int32_t *o = WRITE ? runs + 2 * offsets[b] : nullptr;
  auto emit = [&](int begin, int n) {
    if (WRITE) {
      o[2 * c] = begin;
      o[2 * c + 1] = n;
    }
    c++;
  };
  fill_pattern_runs(w, nw, emit);
  if (!WRITE) counts[b] = c;
}

// The listed blocks' bytes back to back: byte j of list entry e is byte
// j % block_size of block list[e]: its frame (j % block_size) / fb, or zero
// past the frames.
__global__ void gather_blocks_kernel(const uint8_t *__restrict__ rec, const int64_t *__restrict__ frames, int nf,
                                     int fb, int block_size, const int32_t *__restrict__ list, int64_t total,
                                     uint8_t *__restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = j / block_size;
    const int r = (int)(j - e * block_size);
    const int f = r / fb;
    out[j] = f < nf ? rec[frames[(int64_t)list[e] * nf + f] + (r - f * fb)] : (uint8_t)0;
  }
}

// Channel extraction of every block at once: output byte ob of subband
// blockIdx.y is byte r = ob % opb of block ob / opb, made from the spb words
// at block byte r * spb * N, which lie in one frame (fb is a multiple of
// spb * N) or past the frames (zero words).
__global__ void extract_frames_kernel(const uint8_t *__restrict__ rec, const int64_t *__restrict__ frames, int nf,
                                      int fb, int64_t opb, int64_t nout, int N, int bits, int fan_out,
                                      const int *__restrict__ tracks, uint8_t *__restrict__ out) {
  const int64_t ob = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int sb = blockIdx.y;
  if (ob >= nout) return;
  const int64_t b = ob / opb;
  const int64_t byte = (ob - b * opb) * (8 / fan_out) * N;
  const int64_t f = byte / fb;
  uint8_t v = 0;
  if (f < nf)
    v = extract_byte(rec + frames[b * nf + f] + (byte - f * fb), N, bits, fan_out, tracks + sb * fan_out);
  out[(int64_t)sb * nout + ob] = v;
}

// One warp per record: the header bytes, then a DATA record's payload from
// the channel stream.
__global__ void serialize_protocol_kernel(const ProtoRecord *__restrict__ recs, int nrec,
                                          const uint8_t *__restrict__ stream, uint8_t *__restrict__ out) {
  const int r = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= nrec) return;
  const ProtoRecord q = recs[r];
  uint8_t *o = out + q.out;
  if (lane == 0) {
    o[0] = q.type;
    if (q.type == 2) {  // HEADER_DELAY
      o[1] = (uint8_t)q.rem;
    } else if (q.type == 0 || q.type == 1) {  // HEADER_DATA / HEADER_INVALID: int16 count, little endian
      const int16_t k = (int16_t)q.n;
      o[1] = (uint8_t)(k & 0xff);
      o[2] = (uint8_t)((k >> 8) & 0xff);
    }
  }
  if (q.type == 0)
    for (int j = lane; j < q.n; j += 32) o[3 + j] = stream[q.src + j];
}

unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void launch_decode_frames(const uint8_t *rec, int64_t pos0, int64_t stride, int64_t count, int mk5b, FrameInfo *out,
                          cudaStream_t st) {
  if (count <= 0) return;
  decode_frames_kernel<<<blocks_for(count, 256), 256, 0, st>>>(rec, pos0, stride, count, mk5b, out);
}

void launch_fill_runs(const uint8_t *rec, const int64_t *frames, int nf, int wpf, int nw, int nblocks,
                      int32_t *counts, const int64_t *offsets, int32_t *runs, cudaStream_t st) {
  if (nblocks <= 0) return;
  if (!runs)
    fill_runs_kernel<false><<<blocks_for(nblocks, 128), 128, 0, st>>>(rec, frames, nf, wpf, nw, nblocks, counts,
                                                                      nullptr, nullptr);
  else
    fill_runs_kernel<true><<<blocks_for(nblocks, 128), 128, 0, st>>>(rec, frames, nf, wpf, nw, nblocks, nullptr,
                                                                     offsets, runs);
}

void launch_gather_blocks(const uint8_t *rec, const int64_t *frames, int nf, int fb, int block_size,
                          const int32_t *list, int nlist, uint8_t *out, cudaStream_t st) {
  const int64_t total = (int64_t)nlist * block_size;
  if (total <= 0) return;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
    nsm = 1;
  const unsigned grid = (unsigned)std::min<int64_t>(blocks_for(total, 256), (int64_t)nsm * 8);
  gather_blocks_kernel<<<grid, 256, 0, st>>>(rec, frames, nf, fb, block_size, list, total, out);
}

void launch_extract_frames(const uint8_t *rec, const int64_t *frames, int nf, int fb, int64_t opb, int64_t nout,
                           int N, int bits, int nsub, int fan_out, const int *tracks, uint8_t *out,
                           cudaStream_t st) {
  if (nout <= 0) return;
  extract_frames_kernel<<<dim3(blocks_for(nout, 256), nsub), 256, 0, st>>>(rec, frames, nf, fb, opb, nout, N, bits,
                                                                           fan_out, tracks, out);
}

void launch_serialize_protocol(const ProtoRecord *recs, int nrec, const uint8_t *stream, uint8_t *out,
                               cudaStream_t st) {
  if (nrec <= 0) return;
  serialize_protocol_kernel<<<blocks_for((int64_t)nrec * 32, 256), 256, 0, st>>>(recs, nrec, stream, out);
}

}  // namespace sfxc
