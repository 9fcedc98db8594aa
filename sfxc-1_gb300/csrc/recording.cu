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
// recording offsets frames[0..nf), zeros after them.  (A frame offset of -1,
// a block filled in for missing data, reads as zeros in every kernel here.)
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
    const int64_t off = f < nf ? frames[(int64_t)list[e] * nf + f] : -1;
    out[j] = off >= 0 ? rec[off + (r - f * fb)] : (uint8_t)0;
  }
}

// Channel extraction of every block at once: thread ob takes output byte r
// = ob % opb of block ob / opb in every subband, from the SPB = 8 / fan_out
// words at block byte r * SPB * N (read once, held as 64-bit values), each
// in its frame (fb is a multiple of N) or past the frames (zero words).  Bit placement as extract_byte: track t of a sample lands at
// low_bit << ((t + 1) % BITS), low_bit starting at 1 << (8 - fan_out) and
// advancing by BITS per complete sample; earlier samples sit lower.
constexpr int kMaxExtractTracks = 1024;
template <int SPB, int BITS>
__global__ void __launch_bounds__(256) extract_frames_kernel(const uint8_t *__restrict__ rec,
                                                             const int64_t *__restrict__ frames, int nf, int fb,
                                                             int64_t opb, int64_t nout, int N, int nsub,
                                                             const int *__restrict__ tracks,
                                                             uint8_t *__restrict__ out) {
  constexpr int FAN = 8 / SPB;
  __shared__ int str[kMaxExtractTracks];
  for (int i = threadIdx.x; i < nsub * FAN; i += blockDim.x) str[i] = tracks[i];
  __syncthreads();
  const int64_t ob = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ob >= nout) return;
  const int64_t b = ob / opb;
  const int64_t byte = (ob - b * opb) * SPB * N;
  const int64_t f = byte / fb, f_last = (byte + (SPB - 1) * N) / fb;
  uint64_t w[SPB];
#pragma unroll
  for (int j = 0; j < SPB; j++) w[j] = 0;
  const int64_t off = f < nf ? frames[b * nf + f] : -1;
  const uint8_t *p = off >= 0 ? rec + off + (byte - f * fb) : nullptr;
  if (SPB == 4 && N == 4 && f == f_last && p && ((uintptr_t)p & 15) == 0) {
    const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
    w[0] = v.x;
    w[1 % SPB] = v.y;
    w[2 % SPB] = v.z;
    w[3 % SPB] = v.w;
  } else {
    // word by word: the SPB words of an output byte may span two frames
#pragma unroll
    for (int j = 0; j < SPB; j++) {
      const int64_t wb = byte + j * N, fj = wb / fb;
      const int64_t offj = fj < nf ? frames[b * nf + fj] : -1;
      if (offj >= 0) {
        const uint8_t *q = rec + offj + (wb - fj * fb);
        for (int i = 0; i < N; i++) w[j] |= (uint64_t)q[i] << (8 * i);
      }
    }
  }
  for (int sb = 0; sb < nsub; sb++) {
    int tr[FAN];
#pragma unroll
    for (int t = 0; t < FAN; t++) tr[t] = str[sb * FAN + t];
    unsigned out_byte = 0;
#pragma unroll
    for (int j = 0; j < SPB; j++) {
      unsigned v = 0, low_bit = 1u << (8 - FAN);
#pragma unroll
      for (int t = 0; t < FAN; t++) {
        v |= (unsigned)((w[j] >> tr[t]) & 1u) * (low_bit << ((t + 1) % BITS));
        if ((t + 1) % BITS == 0) low_bit <<= BITS;
      }
      out_byte |= (v >> ((SPB - 1 - j) * FAN)) & 0xffu;
    }
    out[(int64_t)sb * nout + ob] = (uint8_t)out_byte;
  }
}

// The usual track layouts: every subband's tracks are one bit field of the
// word, in the order the extractor places them (bits b0 .. b0 + fan_out - 1
// of sample j land on output bits j * fan_out .. ; for 2-bit samples the
// extractor swaps each track pair, so tracks {b0 + 1, b0} are the field).
// Then output byte = OR_j ((word_j >> b0) & mask) << (j * fan_out).  Each
// thread makes G consecutive output bytes of every subband from G * SPB
// words (G = 4: 64 bytes for 32-bit words and 2-bit pairs, stored as one
// 32-bit word per subband; G = 1 where a frame is not a multiple of four
// output bytes).  T: the word type (uint32_t for words of up to 4 bytes).
template <int SPB, class T, int G>
__global__ void __launch_bounds__(256) extract_fields_kernel(const uint8_t *__restrict__ rec,
                                                             const int64_t *__restrict__ frames, int nf, int fb,
                                                             int64_t opb, int64_t nout, int N, int nsub,
                                                             const int *__restrict__ bases,
                                                             uint8_t *__restrict__ out) {
  constexpr int FAN = 8 / SPB;
  constexpr unsigned MASK = (1u << FAN) - 1u;
  constexpr int NW = G * SPB;
  __shared__ int sb0[kMaxExtractTracks];
  for (int i = threadIdx.x; i < nsub; i += blockDim.x) sb0[i] = bases[i];
  __syncthreads();
  const int64_t ob = G * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  if (ob >= nout) return;
  const int64_t b = ob / opb;
  const int64_t byte = (ob - b * opb) * SPB * N;
  const int64_t f = byte / fb;
  T w[NW];
#pragma unroll
  for (int j = 0; j < NW; j++) w[j] = 0;
  const int64_t off = f < nf ? frames[b * nf + f] : -1;
  if (off >= 0) {
    const uint8_t *p = rec + off + (byte - f * fb);
    if (sizeof(T) == 4 && N == 4 && NW % 4 == 0 && ((uintptr_t)p & 15) == 0) {
#pragma unroll
      for (int v = 0; v < NW / 4; v++) {
        const uint4 q = __ldg(reinterpret_cast<const uint4 *>(p) + v);
        w[4 * v] = q.x;
        w[4 * v + 1] = q.y;
        w[4 * v + 2] = q.z;
        w[4 * v + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < NW; j++)
        for (int i = 0; i < N; i++) w[j] |= (T)p[j * N + i] << (8 * i);
    }
  }
  for (int sb = 0; sb < nsub; sb++) {
    const int b0 = sb0[sb];
    unsigned o = 0;
#pragma unroll
    for (int k = 0; k < G; k++)
#pragma unroll
      for (int j = 0; j < SPB; j++) o |= ((unsigned)(w[k * SPB + j] >> b0) & MASK) << (8 * k + j * FAN);
    if (G == 4)
      *reinterpret_cast<unsigned *>(out + (int64_t)sb * nout + ob) = o;
    else
      out[(int64_t)sb * nout + ob] = (uint8_t)o;
  }
}

// Words wider than 8 bytes: one thread per output byte and subband
// (extract_byte on the words where they lie; frames a whole number of output bytes).
__global__ void extract_frames_wide_kernel(const uint8_t *__restrict__ rec, const int64_t *__restrict__ frames,
                                           int nf, int fb, int64_t opb, int64_t nout, int N, int bits, int fan_out,
                                           const int *__restrict__ tracks, uint8_t *__restrict__ out) {
  const int64_t ob = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int sb = blockIdx.y;
  if (ob >= nout) return;
  const int64_t b = ob / opb;
  const int64_t byte = (ob - b * opb) * (8 / fan_out) * N;
  const int64_t f = byte / fb;
  uint8_t v = 0;
  const int64_t off = f < nf ? frames[b * nf + f] : -1;
  if (off >= 0) v = extract_byte(rec + off + (byte - f * fb), N, bits, fan_out, tracks + sb * fan_out);
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

bool launch_extract_frames(const uint8_t *rec, const int64_t *frames, int nf, int fb, int64_t opb, int64_t nout,
                           int N, int bits, int nsub, int fan_out, const int *tracks, uint8_t *out,
                           cudaStream_t st) {
  if (nout <= 0) return true;
  const unsigned g = blocks_for(nout, 256);
  if (N > 8) {
    if (fb % ((8 / fan_out) * N)) return false;
    extract_frames_wide_kernel<<<dim3(g, nsub), 256, 0, st>>>(rec, frames, nf, fb, opb, nout, N, bits, fan_out,
                                                              tracks, out);
    return true;
  }
  if (nsub * fan_out > kMaxExtractTracks) return false;
#define SFXC_EXTRACT(SPB, BITS) \
  extract_frames_kernel<SPB, BITS><<<g, 256, 0, st>>>(rec, frames, nf, fb, opb, nout, N, nsub, tracks, out)
  if (fan_out == 1 && bits == 1) SFXC_EXTRACT(8, 1);
  else if (fan_out == 2 && bits == 1) SFXC_EXTRACT(4, 1);
  else if (fan_out == 2 && bits == 2) SFXC_EXTRACT(4, 2);
  else if (fan_out == 4 && bits == 1) SFXC_EXTRACT(2, 1);
  else if (fan_out == 4 && bits == 2) SFXC_EXTRACT(2, 2);
  else if (fan_out == 8 && bits == 1) SFXC_EXTRACT(1, 1);
  else if (fan_out == 8 && bits == 2) SFXC_EXTRACT(1, 2);
  else return false;
#undef SFXC_EXTRACT
  return true;
}

bool launch_extract_fields(const uint8_t *rec, const int64_t *frames, int nf, int fb, int64_t opb, int64_t nout,
                           int N, int fan_out, int nsub, const int *bases, uint8_t *out, cudaStream_t st) {
  if (N > 8 || nsub > kMaxExtractTracks || fb % ((8 / fan_out) * N)) return false;
  if (nout <= 0) return true;
  const bool quad = nout % 4 == 0 && opb % 4 == 0 && fb % (4 * (8 / fan_out) * N) == 0;
  const unsigned g = blocks_for(quad ? nout / 4 : nout, 256);
#define SFXC_FIELDS(SPB, T)                                                                                    \
  do {                                                                                                         \
    if (quad)                                                                                                  \
      extract_fields_kernel<SPB, T, 4><<<g, 256, 0, st>>>(rec, frames, nf, fb, opb, nout, N, nsub, bases, out); \
    else                                                                                                       \
      extract_fields_kernel<SPB, T, 1><<<g, 256, 0, st>>>(rec, frames, nf, fb, opb, nout, N, nsub, bases, out); \
  } while (0)
  if (N <= 4) {
    if (fan_out == 1) SFXC_FIELDS(8, uint32_t);
    else if (fan_out == 2) SFXC_FIELDS(4, uint32_t);
    else if (fan_out == 4) SFXC_FIELDS(2, uint32_t);
    else if (fan_out == 8) SFXC_FIELDS(1, uint32_t);
    else return false;
  } else {
    if (fan_out == 1) SFXC_FIELDS(8, uint64_t);
    else if (fan_out == 2) SFXC_FIELDS(4, uint64_t);
    else if (fan_out == 4) SFXC_FIELDS(2, uint64_t);
    else if (fan_out == 8) SFXC_FIELDS(1, uint64_t);
    else return false;
  }
#undef SFXC_FIELDS
  return true;
}

void launch_serialize_protocol(const ProtoRecord *recs, int nrec, const uint8_t *stream, uint8_t *out,
                               cudaStream_t st) {
  if (nrec <= 0) return;
  serialize_protocol_kernel<<<blocks_for((int64_t)nrec * 32, 256), 256, 0, st>>>(recs, nrec, stream, out);
}

}  // namespace sfxc
