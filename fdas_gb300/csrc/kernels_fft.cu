// (a) overlap-save tiling + forward FFT, (c) fused template multiply,
// inverse FFT, power and overlap discard, and the FP64 template precompute.
#include <climits>
#include <cstdlib>
#include <cstring>

#include "fft2048.cuh"
#include "kernels.cuh"

namespace fdas {

constexpr int kWarpsPerCta = 8;

// One warp per tile.  Tile i covers spectrum bins [i P - O, i P + P): bins
// below 0 (the first tile's overlap) and from N on (the last tile's padding)
// read as zero -- tile_input.cl.mako:42-94 / ft_conv.py:165-180.
// Three warps per CTA and three CTAs per SM (at most 224 registers): 9 warps
// per SM, so the 1289 tiles of a 2^21-bin search run in a single wave
// (1368 warp slots) instead of 1216 + 73.
constexpr int kTileWarps = 3;
template <bool BATCH>
__global__ void __launch_bounds__(32 * kTileWarps, 3) tile_fft_kernel(TileParams p) {
  extern __shared__ float4 smem_f4[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * kTileWarps + warp;
  if (tile >= p.n_tiles) return;
  float *ex = reinterpret_cast<float *>(smem_f4) + warp * kExFloats;
  const TwiddleBases tb = load_twiddle_bases<-1>(p.twiddle, lane);
  float2 v[64];
  const float2 *input = p.input;
  int n_bins = p.n_bins;
  long long local = tile;
  if constexpr (BATCH) {  // batched: the trial's own spectrum and tile numbering
    const BatchTrial &tr = p.trials[batch_trial_of(p.trials, p.n_trials, tile)];
    input += tr.input_offset;
    n_bins = tr.n_bins;
    local = tile - tr.tile_begin;
  }
  const long long start = local * p.payload - p.overlap;
  sfor<2>([&](auto C) {
    constexpr int c = decltype(C)::value;
    sfor<32>([&](auto D) {
      constexpr int d = decltype(D)::value;
      const long long b = start + lane + 32 * c + 64 * d;
      v[32 * c + d] = (b >= 0 && b < n_bins) ? __ldg(input + b) : make_float2(0.f, 0.f);
    });
  });
  fft2048_core(v, tb, ex, lane);
  float2 *out = p.tiles + (long long)tile * kTile;
  sfor<64>([&](auto K) {
    constexpr int k = decltype(K)::value;
    out[32 * k + lane] = v[pos64(k)];
  });
}

// ------------------------------------------------------------ TMA helpers
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long timeout_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  while (!mbar_try_wait(bar, parity))
    if ((long long)(gtimer() - t0) > timeout_ns) return false;
  return true;
}
// 16 KB template spectrum -> this warp's exchange buffer (async proxy)
__device__ __forceinline__ void prefetch_template(float *ex, const float2 *src, uint64_t *bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_arrive_expect_tx(bar, kTile * 8);
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(ex)),
      "l"(src), "r"((uint32_t)(kTile * 8)), "r"(smem_addr(bar))
      : "memory");
}

// Where the outputs of (global tile, FOP row) go: the row's start, the bin of
// the tile's first output (before the discard) and the row length.
struct FopTarget {
  float *out;
  long long base;
  int n_bins;
};
// The trial of a warp's (or pair's) current item in the batched search, its
// fields held in registers.  A warp's items only move forward (item += grid
// size), so after one binary search at the first item the trial is found by
// walking forward from the previous one -- usually no step at all -- instead
// of a dependent chain of loads per item.
struct TrialCursor {
  long long next_begin;  // first global tile of the next trial
  long long tile_begin;  // first global tile of this trial
  long long fop_offset;
  long long stride;
  int t;
  int n_bins;
};
__device__ __forceinline__ void cursor_load(const FtcParams &p, TrialCursor &c) {
  const BatchTrial &tr = p.trials[c.t];
  c.tile_begin = tr.tile_begin;
  c.fop_offset = tr.fop_offset;
  c.stride = tr.stride;
  c.n_bins = tr.n_bins;
  c.next_begin = c.t + 1 < p.n_trials ? p.trials[c.t + 1].tile_begin : LLONG_MAX;
}
template <bool BATCH>
__device__ __forceinline__ void cursor_start(const FtcParams &p, int tile, TrialCursor &c) {
  if constexpr (BATCH) {
    c.t = batch_trial_of(p.trials, p.n_trials, p.tile_begin + tile);  // the launch may cover a range of tiles
    cursor_load(p, c);
  }
}
template <bool BATCH>
__device__ __forceinline__ void cursor_seek(const FtcParams &p, int tile, TrialCursor &c) {
  if constexpr (BATCH) {
    while (p.tile_begin + tile >= c.next_begin) {
      ++c.t;
      cursor_load(p, c);
    }
  }
}
template <bool BATCH>
__device__ __forceinline__ FopTarget fop_target(const FtcParams &p, int tile, int row, const TrialCursor &c) {
  if constexpr (!BATCH)
    return FopTarget{p.fop + (long long)row * p.fop_stride, (long long)tile * p.payload - p.overlap, p.n_bins};
  return FopTarget{p.fop + c.fop_offset + (long long)row * c.stride,
                   (p.tile_begin + tile - c.tile_begin) * p.payload - p.overlap, c.n_bins};
}

template <bool BATCH>
__global__ void __launch_bounds__(256, 1) ftc_kernel(FtcParams p) {
  extern __shared__ float4 smem_f4[];
  __shared__ uint64_t bars[kWarpsPerCta];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *ex = reinterpret_cast<float *>(smem_f4) + warp * kExFloats;
  uint64_t *bar = &bars[warp];
  const int n_items = p.n_tiles * p.n_rows;
  const int stride = gridDim.x * kWarpsPerCta;
  int item = blockIdx.x * kWarpsPerCta + warp;
  if (lane == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const TwiddleBases tb = load_twiddle_bases<+1>(p.twiddle, lane);
  if (item < n_items && lane == 0)
    prefetch_template(ex, p.tmpl + (long long)(p.row_begin + item % p.n_rows) * kTile, bar);
  uint32_t parity = 0;
  TrialCursor cur;
  if (item < n_items) cursor_start<BATCH>(p, item / p.n_rows, cur);
  for (; item < n_items; item += stride) {
    const int tile = item / p.n_rows;
    const int row = p.row_begin + (item - tile * p.n_rows);
    cursor_seek<BATCH>(p, tile, cur);
    const float2 *s = p.tiles + (long long)tile * kTile + lane;
    float2 v[64];
    sfor<64>([&](auto K) {
      constexpr int k = decltype(K)::value;
      v[k] = __ldg(s + 32 * k);
    });
    if (!mbar_wait(bar, parity, p.timeout_ns)) {
      if (lane == 0) atomicOr(p.status, kStatusFtcTimeout);
      mbar_wait(bar, parity, kDrainNs);  // bounded: let the copy land before exiting
      return;
    }
    parity ^= 1u;
    const float2 *t = reinterpret_cast<const float2 *>(ex) + lane;
    sfor<64>([&](auto K) {
      constexpr int k = decltype(K)::value;
      v[k] = cmul(v[k], t[32 * k]);
    });
    const int next = item + stride;
    ifft2048_core(v, tb, ex, lane, [&]() {
      if (next < n_items && lane == 0)
        prefetch_template(ex, p.tmpl + (long long)(p.row_begin + next % p.n_rows) * kTile, bar);
    });
    const FopTarget tg = fop_target<BATCH>(p, tile, row, cur);
    sfor<2>([&](auto C) {
      constexpr int c = decltype(C)::value;
      sfor<32>([&](auto D) {
        constexpr int d = decltype(D)::value;
        const int n = lane + 32 * c + 64 * d;
        const long long b = tg.base + n;
        const float2 y = v[32 * c + pos32(d)];
        if (n >= p.overlap && b < tg.n_bins) tg.out[b] = fmaf(y.x, y.x, y.y * y.y);
      });
    });
  }
}

// ---------------------------------------------------------------------------
// Two-warp variant: one warp pair per (tile, template) item, 32 values per
// thread (<= 128 registers, two CTAs of 4 pairs per SM).  The pair buffer
// (16.9 KB) holds the TMA-prefetched template spectrum of the item, then the
// pass-1 exchange; the next item's template is prefetched into it as soon as
// both warps have read the exchange back.
constexpr int kPairsPerCta = 4;

__device__ __forceinline__ void pair_sync(int pair) {
  asm volatile("bar.sync %0, %1;" ::"r"(pair + 1), "r"(64) : "memory");
}
// barrier over the pair that also ANDs a predicate across its 64 threads
__device__ __forceinline__ bool pair_and(int pair, bool v) {
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((unsigned)v), "r"(pair + 1), "r"(64)
      : "memory");
  return r != 0;
}

template <bool BATCH>
__global__ void __launch_bounds__(256, 2) ftc2_kernel(FtcParams p) {
  extern __shared__ float4 smem_f4[];
  __shared__ uint64_t bars[kPairsPerCta];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pair = warp >> 1, h = warp & 1;
  const int tp = 32 * h + lane;  // thread of the pair
  float *buf_f = reinterpret_cast<float *>(smem_f4) + pair * kEx2Floats;
  float2 *twt = reinterpret_cast<float2 *>(reinterpret_cast<float *>(smem_f4) + kPairsPerCta * kEx2Floats);
  float2 *buf = reinterpret_cast<float2 *>(buf_f);
  uint64_t *bar = &bars[pair];
  const int n_items = p.n_tiles * p.n_rows;
  const int stride = gridDim.x * kPairsPerCta;
  int item = blockIdx.x * kPairsPerCta + pair;
  if (tp == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fill_twiddle2(twt, p.twiddle);
  __syncthreads();
  if (item < n_items && tp == 0) {
    if (p.inject_stall) mbar_arrive_expect_tx(bar, kTile * 8);  // test hook: a copy that never comes
    else prefetch_template(buf_f, p.tmpl + (long long)(p.row_begin + item % p.n_rows) * kTile, bar);
  }
  uint32_t parity = 0;
  const int m = 16 * h + (lane & 15);
  const int g = lane >> 4;
  // (tile, row) of the item, advanced by the grid stride without divisions
  const int st_tiles = stride / p.n_rows, st_rows = stride - st_tiles * p.n_rows;
  int tile = item / p.n_rows, rr = item - tile * p.n_rows;
  TrialCursor cur;
  if (item < n_items) cursor_start<BATCH>(p, tile, cur);
  for (; item < n_items; item += stride) {
    const int row = p.row_begin + rr;
    int next_tile = tile + st_tiles, next_rr = rr + st_rows;
    if (next_rr >= p.n_rows) {
      next_rr -= p.n_rows;
      ++next_tile;
    }
    cursor_seek<BATCH>(p, tile, cur);
    const float2 *s = p.tiles + (long long)tile * kTile + tp;
    float2 v[32];
    sfor<32>([&](auto A) {
      constexpr int a = decltype(A)::value;
      v[a] = __ldg(s + 64 * a);
    });
    // the decision to go on is made uniform over the pair
    if (!pair_and(pair, mbar_wait(bar, parity, p.timeout_ns))) {
      if (tp == 0) atomicOr(p.status, kStatusFtcTimeout);
      // bounded: let the copy land before exiting (the test hook issued none)
      if (!p.inject_stall) mbar_wait(bar, parity, kDrainNs);
      return;
    }
    parity ^= 1u;
    sfor<32>([&](auto A) {
      constexpr int a = decltype(A)::value;
      v[a] = cmul(v[a], buf[64 * a + tp]);
    });
    pair_sync(pair);  // template read by both warps: the buffer takes the exchange
    ifft2_pass1(v, twt, buf, tp);
    pair_sync(pair);  // exchange written
    const int next = item + stride;
    float pw[32];
    ifft2_pass2(buf, h, lane, pw, [&]() {
      pair_sync(pair);  // exchange read by both warps: prefetch the next template
      if (next < n_items && tp == 0)
        prefetch_template(buf_f, p.tmpl + (long long)(p.row_begin + next_rr) * kTile, bar);
    });
    // output n = m + 128 g + c, c = 32 r + 256 d2 known at compile time: the
    // discard (n >= O) and the row end (bin < n_bins) become two 32-bit
    // limits on c per thread and item
    const FopTarget tg = fop_target<BATCH>(p, tile, row, cur);
    const int mb = m + 128 * g;
    const long long first = tg.base + mb;  // bin of c = 0 (negative in the first tile)
    const long long room = (long long)tg.n_bins - first;
    const int lo = p.overlap - mb, hi = room < kTile ? (int)room : kTile;
    const unsigned long long dst =
        reinterpret_cast<unsigned long long>(tg.out) + 4ull * static_cast<unsigned long long>(first);
    sfor<4>([&](auto R) {
      constexpr int r = decltype(R)::value;
      sfor<8>([&](auto D2) {
        constexpr int d2 = decltype(D2)::value;
        constexpr int c = 32 * r + 256 * d2;
        if (c >= lo && c < hi) *reinterpret_cast<float *>(dst + 4ull * c) = pw[8 * r + d2];
      });
    });
    tile = next_tile;
    rr = next_rr;
  }
}

// FP64 DFT of the time-domain taps -> float spectra scaled by 2^-11.
__global__ void spectra_kernel(SpectraParams p) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (k >= kTile || r >= p.n_templates) return;
  const double2 *h = p.taps + (long long)r * p.tap_pitch;
  const int len = p.tap_len[r];
  double re = 0.0, im = 0.0;
  for (int q = 0; q < len; ++q) {
    const double2 w = p.twiddle64[(q * k) & (kTile - 1)];
    const double2 x = h[q];
    re += x.x * w.x - x.y * w.y;
    im += x.x * w.y + x.y * w.x;
  }
  const double scale = 1.0 / 2048.0;
  p.spectra[(long long)r * kTile + k] = make_float2((float)(re * scale), (float)(im * scale));
}

// FP64 inverse DFT of float spectra -> the first n_taps time-domain taps.
__global__ void taps_kernel(TapsParams p) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (r >= p.n_templates) return;
  if (q == 0) p.tap_len[r] = p.n_taps;
  if (q >= p.n_taps) return;
  const float2 *sp = p.spectra + (long long)r * kTile;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < kTile; ++k) {
    const double2 w = p.twiddle64[(q * k) & (kTile - 1)];  // e^(-i..): use conjugate
    const float2 x = sp[k];
    re += (double)x.x * w.x + (double)x.y * w.y;
    im += (double)x.y * w.x - (double)x.x * w.y;
  }
  p.taps[(long long)r * p.tap_pitch + q] = make_double2(re / 2048.0, im / 2048.0);
}

int current_sm_count() {
  int dev = 0, n_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n_sm <= 0) {
    cudaGetLastError();
    return 1;
  }
  return n_sm;
}

static int ex_smem_bytes() { return kWarpsPerCta * kExFloats * (int)sizeof(float); }

cudaError_t launch_tile_fft(const TileParams &p, cudaStream_t s) {
  const int smem = kTileWarps * kExFloats * (int)sizeof(float);
  auto kern = p.trials ? tile_fft_kernel<true> : tile_fft_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  dim3 grid((p.n_tiles + kTileWarps - 1) / kTileWarps);
  kern<<<grid, 32 * kTileWarps, smem, s>>>(p);
  return cudaGetLastError();
}

// FFT variant of the FT convolution: the two-warp form (default) or the
// one-warp form; FDAS_FTC_VARIANT=1warp selects the latter.
static int ftc_variant() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("FDAS_FTC_VARIANT");
    v = (e && strcmp(e, "1warp") == 0) ? 1 : 2;
  }
  return v;
}

cudaError_t launch_ftc(const FtcParams &p, cudaStream_t s) {
  if (p.n_rows <= 0 || p.n_tiles <= 0) return cudaSuccess;
  const int n_sm = current_sm_count();
  if ((p.variant == 3 || p.variant == 4) && !p.trials) return launch_ftc_tc(p, p.variant == 4, s);
  const long long items = (long long)p.n_tiles * p.n_rows;
  if ((p.variant ? p.variant : ftc_variant()) == 1 && !p.inject_stall) {  // the test hook is the pair form's
    const int smem = ex_smem_bytes();
    auto kern = p.trials ? ftc_kernel<true> : ftc_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const long long ctas = (items + kWarpsPerCta - 1) / kWarpsPerCta;
    kern<<<(int)(ctas < n_sm ? ctas : n_sm), 256, smem, s>>>(p);
  } else {
    const int smem = (kPairsPerCta * kEx2Floats + kTw2Floats) * (int)sizeof(float);
    auto kern = p.trials ? ftc2_kernel<true> : ftc2_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const long long ctas = (items + kPairsPerCta - 1) / kPairsPerCta;
    const long long per_sm = p.ctas_per_sm >= 1 && p.ctas_per_sm <= 2 ? p.ctas_per_sm : 2;
    kern<<<(int)(ctas < per_sm * n_sm ? ctas : per_sm * n_sm), 256, smem, s>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_spectra(const SpectraParams &p, cudaStream_t s) {
  dim3 grid(kTile / 128, p.n_templates);
  spectra_kernel<<<grid, 128, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_taps(const TapsParams &p, cudaStream_t s) {
  dim3 grid((p.n_taps + 127) / 128, p.n_templates);
  taps_kernel<<<grid, 128, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace fdas
