// Kernel parameter blocks and launchers of the FDAS hot path.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fdas {

constexpr int kTile = 2048;          // FFT / tile size (gen_info.h:33, 42)
constexpr int kMaxPlanes = 16;       // harmonic planes supported by the kernels
constexpr int kHsBins = 256;         // bins per harmonic-summing work item
constexpr int kSortCap = 8192;       // boundary records one CTA ranks in shared memory
constexpr int kMaxCompat = 2048;     // entries per plane of the fixed-size list
constexpr int kSelBuckets = 2048;    // power buckets of the top-K selection (float bits 30..20)

// device status bits (per buffer set)
constexpr int kStatusHsumTimeout = 1;
constexpr int kStatusRecheckOverflow = 2;
constexpr int kStatusCandidateOverflow = 4;
constexpr int kStatusSelectionOverflow = 8;
constexpr int kStatusFtcTimeout = 16;

// Device-side waits.  kWaitNs is the default bound after which a wait is
// reported as timed out (FtcParams / HsumParams::timeout_ns may lower it);
// kDrainNs bounds the wait for a kernel's own copies in flight before it
// exits after a timeout, so no CTA ends with a copy into its shared memory
// still pending.
constexpr long long kWaitNs = 2000000000LL;
constexpr long long kDrainNs = 2000000000LL;

// Candidate record key: plane << 48 | row << 32 | bin.  Ascending key order is
// (harmonic, template, bin) -- the order of hsum.py's list.
__host__ __device__ inline unsigned long long cand_key(int plane, int row, int bin) {
  return ((unsigned long long)(unsigned)plane << 48) | ((unsigned long long)(unsigned)row << 32) | (unsigned)bin;
}

// ---- (a) overlap-save tiling + forward FFT (tile_input.cl.mako, fft_4p.cl)
// One trial of a batched search: its tiles are the global tiles
// [tile_begin, next trial's tile_begin), its spectrum starts at input_offset of
// the batch input, its FOP (n_templates rows of `stride` floats) at fop_offset.
struct BatchTrial {
  long long tile_begin;
  long long input_offset;
  long long fop_offset;
  long long stride;
  int n_bins;
  int pad_;
};

// trial of global tile `tile` (trials sorted by tile_begin; binary search)
__device__ __forceinline__ int batch_trial_of(const BatchTrial *tr, int n, long long tile) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tr[mid].tile_begin <= tile) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct TileParams {
  const float2 *input;    // N spectrum bins
  int n_bins;
  int n_tiles;
  int overlap;            // O
  int payload;            // P = 2048 - O
  float2 *tiles;          // n_tiles x 2048, natural bin order
  const float2 *twiddle;  // e^(+2 pi i j / 2048), j < 2048
  const BatchTrial *trials = nullptr;  // batched search: n_tiles spans all trials
  int n_trials = 0;
};

// ---- (c) template multiply + inverse FFT + |.|^2 + discard (mux_and_mult,
//      square_and_discard)
struct FtcParams {
  const float2 *tiles;    // n_tiles x 2048
  const float2 *tmpl;     // n_templates x 2048 spectra, natural order, scaled by 2^-11
  float *fop;             // n_templates x stride
  long long fop_stride;
  int n_bins;
  int n_tiles;
  int overlap;
  int payload;
  int row_begin;          // first FOP row of the part
  int n_rows;             // rows of the part
  const float2 *twiddle;
  int *status;
  long long timeout_ns;
  int ctas_per_sm;        // persistent CTAs per SM (1 leaves room for harmonic summing)
  int variant = 0;        // FFT split: 0 default, 1 one warp per item (64 x 32), 2 a warp pair (32 x 64);
                          // 3 / 4: tensor-core DFT factors with split BF16 / FP16 operands
  const BatchTrial *trials = nullptr;  // batched search: tiles of all trials, FOPs per trial
  int n_trials = 0;
  long long tile_begin = 0;  // batched search: global index of the launch's first tile
  int inject_stall = 0;      // test hook: each warp pair's first template copy is announced on its
                             // barrier but not issued, so that wait runs out (nothing is in flight)
  // forward transform of the tiles on the tensor cores (precision form):
  // items are tiles, read from `input` (n_bins spectrum values) and written
  // to `tiles_out` as complex spectra
  const float2 *input = nullptr;
  float2 *tiles_out = nullptr;
};

// ---- (d) harmonic summing + thresholds + candidate compaction (preload,
//      delay, detect, store_cands; hms_baseline.cl.mako)
struct HsumParams {
  const float *fop;
  long long stride;
  int n_bins;
  int half;               // n_templates / 2: row of template t is half + t
  int n_planes;
  int tlo[2];             // first |t| of the negative / positive half; > half disables it
  float trig[kMaxPlanes]; // fast-path trigger: a cell needs a closer look if HP >= trig
  float hi[kMaxPlanes];   // candidate if HP > hi
  float lo[kMaxPlanes];   // recheck if lo <= HP <= hi (lo = +inf: never)
  // staging boxes: plane 1 is 128 bins x 4 NW rows; plane j >= 2 is bw[j] bins
  // (from (f0/j) rounded down to 4) x bh[j] rows (trunc(t/j) of the half)
  int bw[kMaxPlanes + 1];
  int bh[kMaxPlanes + 1];
  int soff[kMaxPlanes + 1]; // float offset of plane j's box in a stage (128-byte aligned)
  int stage_floats;         // floats per pipeline stage
  unsigned stage_bytes;     // bytes the TMA copies deliver per stage
  unsigned *item_counter;   // dynamic work distribution
  unsigned long long *cand_key;  // [cap] records, any order
  float *cand_pwr;               // [cap]
  unsigned *cand_total;          // records appended (may exceed cap)
  unsigned *cand_count;          // [plane] hits per plane
  int cand_cap;
  uint4 *rc_list;         // recheck entries (plane, row, bin, 0)
  unsigned *rc_count;
  int rc_cap;
  int *status;
  long long timeout_ns;   // bound on every wait
  int lean;               // 1: 3 stages and <= 80 registers (shares an SM with the FT convolution)
  int inject_stall = 0;   // test hook: the first stage of every CTA is announced on its barriers
                          // but its copies are not issued, so the consumers' waits run out
};

// 2-D tensor maps of the FOP (rows x stride floats), one box shape per plane
struct HsumMaps {
  CUtensorMap map[kMaxPlanes + 1];
};

// ---- FP64 recheck of near-threshold cells
struct RecheckParams {
  const float2 *input;    // the spectrum the FOP was computed from
  int n_bins;
  int half;
  const float4 *taps;     // n_templates x tap_pitch time-domain taps as float pairs
                          // (re hi, im hi, re lo, im lo): tap = hi + lo to 2^-48
  const int *tap_len;     // taps per template
  int tap_pitch;
  double thr[kMaxPlanes];
  const uint4 *rc_list;
  const unsigned *rc_count;
  int rc_cap;
  unsigned long long *cand_key;
  float *cand_pwr;
  unsigned *cand_total;
  unsigned *cand_count;
  int cand_cap;
  int *status;
};

// ---- deterministic top-K per plane + fixed-size list
struct SelectParams {
  const unsigned long long *cand_key;
  const float *cand_pwr;
  const unsigned *cand_total;
  const unsigned *cand_count;   // [plane]
  int cand_cap;
  int n_planes;
  int per_plane;          // K: entries per plane in the fixed-size list
  unsigned *hist;         // [plane][kSelBuckets], left zeroed after use
  unsigned *ticket;       // last-block detection of the histogram kernel
  int *sel_bucket;        // [plane] boundary bucket (-1: take every hit)
  unsigned *sure_count;   // [plane] records above the boundary bucket
  unsigned *bound_count;  // [plane] records in the boundary bucket
  unsigned long long *sel_key;  // [plane][2][kSortCap]: sure list, boundary list
  float *sel_pwr;
  uint32_t *compat_loc;   // [plane][per_plane]
  float *compat_pwr;
  uint32_t invalid_location;
  int *status;
};

// ---- template spectra / taps in FP64
struct SpectraParams {
  const double2 *taps;    // n_templates x tap_pitch
  const int *tap_len;
  int tap_pitch;
  int n_templates;
  const double2 *twiddle64;  // e^(-2 pi i j / 2048)
  float2 *spectra;        // n_templates x 2048, natural, scaled by 2^-11
};

struct TapsParams {
  const float2 *spectra;  // n_templates x 2048 natural, unscaled
  int n_templates;
  int n_taps;             // taps to recover per template
  const double2 *twiddle64;
  double2 *taps;          // n_templates x tap_pitch
  int *tap_len;
  int tap_pitch;
};

// ---- upstream: spectrum of a real series (ft_conv.py:134-143)
struct SeriesParams {
  float2 *z;              // N complex: the 2N samples on entry, the N-bin spectrum on exit
  float2 *scratch;        // N complex
  const float2 *tw;       // e^(-i pi x / N), x < N
  int n;                  // N
  float scale;            // applied to every output bin (1 / (2N) in ft_conv.py)
};
// radix sequence of an N-point mixed-radix FFT (8, 4, 2, 3, 5, 7); -1 if N has another factor
int series_radices(int n, int *radix, int max_passes);
cudaError_t launch_series_twiddles(float2 *tw, int n, cudaStream_t s);
cudaError_t launch_series_spectrum(const SeriesParams &p, cudaStream_t s);

cudaError_t launch_tile_fft(const TileParams &p, cudaStream_t s);
cudaError_t launch_ftc(const FtcParams &p, cudaStream_t s);
// precision form: inverse DFT on tcgen05 with split FP16 (f16) or BF16 operands
cudaError_t launch_ftc_tc(const FtcParams &p, bool f16, cudaStream_t s);
// precision form: tiling + forward DFT of the tiles on tcgen05, the same DFT
// factors conjugated; status / timeout as for the FT convolution
cudaError_t launch_tile_tc(const TileParams &p, bool f16, int *status, long long timeout_ns, cudaStream_t s);
cudaError_t launch_hsum(const HsumParams &p, const HsumMaps &m, cudaStream_t s);
// consumer warps of the harmonic-summing kernel for `half` (4 templates each)
int hsum_warps(int half);
cudaError_t launch_recheck(const RecheckParams &p, cudaStream_t s);
cudaError_t launch_split_taps(double2 *taps, long long n, cudaStream_t s);
cudaError_t launch_select(const SelectParams &p, cudaStream_t s);
cudaError_t launch_spectra(const SpectraParams &p, cudaStream_t s);
cudaError_t launch_taps(const TapsParams &p, cudaStream_t s);

// SM count of the current device, queried on every call (a process may drive
// GPUs with different SM counts; the query costs well under a microsecond)
int current_sm_count();

// shared memory bytes needed by launch_hsum for a given plane geometry
int hsum_smem_bytes(const HsumParams &p);
constexpr int kStatusHsumSetup = 32;

}  // namespace fdas
