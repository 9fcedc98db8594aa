// Launch wrappers of the correlator-node kernels (kernels.cu, xcorr_tc.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "frames.hpp"

namespace sfxc {

// block stage: per-block parameters (block_params_kernel), then the
// transforms (fstep_block_kernel); launch_fstep_block runs both in order
void launch_fstep_block(const StreamDev *d_streams, int nstreams, int max_blocks, const float2 *tw256_128,
                        cudaStream_t st);
// ctas_per_sm > 0: at most that many CTAs per SM in all (each striding over its stream's blocks)
void launch_block_params(const StreamDev *d_streams, int nstreams, int max_blocks, cudaStream_t st,
                         int ctas_per_sm = 0);
// ctas_per_sm: grid of the block stage, CTAs per SM over all streams (0: the default, 12)
void launch_fstep(const StreamDev *d_streams, int nstreams, int max_blocks, const float2 *tw256, cudaStream_t st,
                  int ctas_per_sm = 0);
void launch_unpack(const StreamDev *d_streams, int nstreams, int max_blocks, float *out, cudaStream_t st);
void launch_extract(const uint8_t *in, int64_t nout, int N, int bits, int nsub, int fan_out, const int *tracks,
                    uint8_t *out, cudaStream_t st);
// tc_slots: slots per (row, channel) of the TC layout (32 or 64); 0 writes the FP32 layout
// waves: resident-CTA waves the runs of rows are cut into (0: the default, 2)
void launch_window_fft(const StreamDev *d_streams, int nstreams, int row0, int nrows, int nrows_total,
                       const float *window, const float2 *tw_rot, int rot, int nper, int M, int kpad, void *spec,
                       int tc_slots, float tc_scale, cudaStream_t st, int waves = 0);
void launch_bitstat(const StreamDev *d_streams, const int4 *d_items, int nitems, cudaStream_t st);
// FP32 X-step (xcorr_f32_kernel): launch arguments and work split
constexpr int kF32Stages = 4;         // cp.async ring depth
constexpr int kF32StageBytes = 32768;  // rows x streams x 32 channels staged per step, at most
struct F32Args {
  const float2 *spec;  // [stream][row][kpad] complex64
  int nrows_total, kpad, nstreams, npad, r0, r1, K;
  const int *tiles;    // (I, J) per 4x4 stream-pair tile
  int ntiles, tiles_per_part, nparts, rblock, R;
  const int *blmap;
  int nbl;
  const int16_t *bins;  // binned (pulsar): [channel][row] with row stride bins_rows, row 0 = r0; else NULL
  int bins_rows;
  float2 *acc;          // [bin][baseline][kpad]
  float2 *part;         // non-NULL: each row block's partial sums [block][baseline][kpad], added later in order
};
struct F32Plan {
  int nparts = 0, tiles_per_part = 0, tpw = 0, warps = 0, R = 0;
  size_t smem = 0;
};
// tpw == 0: the streams do not fit (npad x 256 B over 128 KB of staging)
F32Plan xcorr_f32_plan(int ntiles, int npad);
// Scratch the unbinned FP32 X-step wants for its row blocks' partial sums
// (0: one block); with less, it runs the rows as one block.
size_t xcorr_f32_scratch_bytes(int ntiles, int npad, int K, int nrows, int nbl, int kpad);
// rows [r0, r1) of spec into acc; bins != NULL: binned, acc[bins[k][r - r0]].
// Deterministic: every accumulator entry has one writer, partial sums are
// added in a fixed order.
void launch_xcorr_f32(const float2 *spec, int nrows_total, int kpad, int nstreams, int npad, int r0, int r1, int K,
                      const int *tiles, int ntiles, const int *blmap, int nbl, const int16_t *bins, int bins_rows,
                      float2 *acc, float2 *scratch, size_t scratch_bytes, cudaStream_t st);
// pulsar bin of every (row, channel), FP64 in the reference's order: bins[k * nrows + r]
void launch_pulsar_bins(int nrows, int K, double start_phase, double rate_term, double fft_duration,
                        const double *offsets, double g0, double g1, int nbins, int16_t *bins, cudaStream_t st);
// rows of each channel sorted stably by bin, each bin's run padded with -1 to a
// multiple of 16: rowlist[ch * list_len + e], segs[ch * nbins + bin] = (first, entries)
void launch_pulsar_sort(const int16_t *bins, int nrows, int K, int nbins, int list_len, int *rowlist, int2 *segs,
                        cudaStream_t st);
size_t xcorr_tc_smem_bytes();
// TC spectra: per row, channels x 32 stream slots of 4 FP16 (hi.re, hi.im, lo.re, lo.im), in the
// line-complete order of tc_index.
cudaError_t launch_xcorr_tc(const void *spec, int nrows, int kpad, int K, const int *blmap, int npad,
                            float inv_scale2, float2 *acc, int *err, cudaStream_t st);
// Row-gathered tensor-core X-step over TC spectra with `slots` (32 or 64)
// slots: rowlist == NULL: rows 0..nrows-1 in order into acc (jobs of up to 64
// streams); else per channel the rows of rowlist, segment (channel, bin) of
// segs into acc[bin] (pulsar binning).  Rows need no zero padding.
cudaError_t launch_xcorr_tc_gather(const void *spec, int slots, int nrows, int kpad, int K, int nstreams,
                                   const int *blmap, int npad, int nbl, int nbins, const int *rowlist, int list_len,
                                   const int2 *segs, float inv_scale2, float2 *acc, int *err, cudaStream_t st);
void launch_normalize(const float2 *acc, int kpad, int M, int nstreams, int nbl, const int *bl, double *norms,
                      const double *flagfac, float2 *out, cudaStream_t st);
// Sub-integration dump with extra phase centres: acc[b][k] (b < nbl, k < K,
// rows kpad apart) added to every centre's accumulator pcacc[c][b][k], rotated
// for c >= 1 on cross baselines (b >= nstreams) by uvp[(c - 1) nbl + b] =
// {phase, phase step per channel, amplitude}, then cleared.
void launch_pc_dump(float2 *acc, float2 *pcacc, const UvShift *uvp, int nstreams, int nbl, int kpad, int K, int npc,
                    cudaStream_t st);
// Phased array: acc[(r0 + r) / nsub][k] += spec[i][r][k] over the chunk's rows
// r < nrows and streams i < nstreams, in that order (FP32 spectra layout,
// nrows_total rows per stream slot, kpad apart).
void launch_phased(const float2 *spec, int nrows_total, int kpad, int nstreams, int r0, int nrows, int K, int nsub,
                   float2 *acc, cudaStream_t st);
// Spectral reduction of nspec normalised spectra of M + 1 channels to nch + 1
// channels (M, nch powers of two, nch < M); mask: M + 1 values, lag_window:
// 2 nch values, tw2M: exp(-2 pi i k / 2M) for k < 2M.
cudaError_t launch_reduce(const float2 *in, int nspec, int M, int nch, const float *mask, const float *lag_window,
                          int normalize, const float2 *tw2M, float2 *out, cudaStream_t st);
// Phase-cal folding: run k adds the samples of its bytes data[off, off + n)
// to accumulator row `row` (pb * (8 / bits) int32 bins), byte j to byte-bin
// (bin0 + j) mod pb.
struct PcalRun {
  int64_t off;
  int32_t n, bin0, row, pad;
};
void launch_phasecal(const uint8_t *data, const PcalRun *runs, int nruns, int pb, int bits, int32_t *acc,
                     cudaStream_t st);

// Recordings in device memory (recording.cu)
// one protocol record as the input-node writer emits it, with its byte offset in the output
struct ProtoRecord {
  int64_t src;  // HEADER_DATA: payload offset in the channel stream
  int64_t out;  // offset of the record's first byte in the protocol bytes
  int32_t n;    // HEADER_DATA bytes / HEADER_INVALID samples
  uint8_t type; // HEADER_*
  int8_t rem;   // HEADER_DELAY
  uint16_t pad;
};
void launch_decode_frames(const uint8_t *rec, int64_t pos0, int64_t stride, int64_t count, int mk5b, FrameInfo *out,
                          cudaStream_t st);
// runs == NULL: counts[b] = number of runs of block b; else runs at 2 * offsets[b]
void launch_fill_runs(const uint8_t *rec, const int64_t *frames, int nf, int wpf, int nw, int nblocks,
                      int32_t *counts, const int64_t *offsets, int32_t *runs, cudaStream_t st);
void launch_gather_blocks(const uint8_t *rec, const int64_t *frames, int nf, int fb, int block_size,
                          const int32_t *list, int nlist, uint8_t *out, cudaStream_t st);
// false: more than 1024 tracks in all for words of up to 8 bytes, or words
// over 8 bytes in frames that are not a whole number of output bytes (the
// caller checked fan_out, bits and that frames are whole words)
bool launch_extract_frames(const uint8_t *rec, const int64_t *frames, int nf, int fb, int64_t opb, int64_t nout,
                           int N, int bits, int nsub, int fan_out, const int *tracks, uint8_t *out,
                           cudaStream_t st);
// subbands whose tracks are bit fields (bases[s] = the field's lowest bit);
// false for words over 8 bytes, more than 1024 subbands or frames that are
// not a whole number of output bytes: use launch_extract_frames
bool launch_extract_fields(const uint8_t *rec, const int64_t *frames, int nf, int fb, int64_t opb, int64_t nout,
                           int N, int fan_out, int nsub, const int *bases, uint8_t *out, cudaStream_t st);
void launch_serialize_protocol(const ProtoRecord *recs, int nrec, const uint8_t *stream, uint8_t *out,
                               cudaStream_t st);

}  // namespace sfxc
