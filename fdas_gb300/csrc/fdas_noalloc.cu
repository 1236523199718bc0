// FT convolution without allocation: overlap-save tiling + forward FFT and the
// fused template multiply / inverse FFT / power / discard, run on a spectrum
// and into a FOP that the caller holds in device memory, with every
// intermediate array in a fixed static device scratch area.
//
// Who needs it: a caller that cannot allocate device memory at call time --
// a pipeline whose device memory is all owned by its own pool allocator with a
// fixed budget, a real-time search that must not meet an out-of-memory error
// in the middle of an observation, or a caller on a path where cudaMalloc /
// cudaFree would synchronise the device and stall its other streams.  The
// handle-based path (fdas_initialise_accelerator) allocates its buffers once
// per handle; this entry point allocates nothing, ever: the scratch is a
// file-scope __device__ array that exists for as long as the library's module
// is loaded, and the only per-device setup is looking up its address.
//
// The kernels are the ones of fdas_perform_input_tiling +
// fdas_perform_ft_convolution (kernels_fft.cu), with the same twiddle table and
// the same 2^-11-scaled template spectra, so the FOP equals the handle path's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "fdas_gb300.h"
#include "kernels.cuh"

using namespace fdas;

namespace {

// Scratch layout (float2 elements): tile spectra | template spectra | twiddles,
// then one int status word.  Only the status word has to start at zero (the
// FT convolution ORs error bits into it); static __device__ storage is zeroed
// when the module loads and nothing ever sets it except a timed-out kernel.
// The other regions are fully written by every call before they are read.
constexpr size_t kTileElems = (size_t)FDAS_NOALLOC_MAX_TILES * kTile;
constexpr size_t kTmplElems = (size_t)FDAS_NOALLOC_MAX_TEMPLATES * kTile;
constexpr size_t kTwElems = kTile;
constexpr size_t kScratchElems = kTileElems + kTmplElems + kTwElems + 32;  // + status word (padded)

__device__ __align__(256) float2 g_noalloc_scratch[kScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float2 *g_scratch_ptr[kMaxDevices] = {};

// e^(+2 pi i j / 2048), computed in double precision and rounded to float, as
// for the handle's table; a static host array, so setup allocates nothing.
float2 g_twiddle_host[kTile];
bool g_twiddle_host_ready = false;

// p4 position 4 s + j holds natural bin bitrev2(j) * 512 + s
// (tmpl-gen.py:145-153); natural bin k therefore sits at p4 position
// 4 (k mod 512) + bitrev2(k / 512).  Spectra are scaled by 2^-11 (the inverse
// transform's 1/2048, exact in float) as the handle does at upload.
__global__ void noalloc_templates_kernel(const float2 *__restrict__ src, float2 *__restrict__ dst, int n_templates,
                                         int p4) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (k >= kTile || r >= n_templates) return;
  int q = k;
  if (p4) {
    const int b = k >> 9;
    q = 4 * (k & 511) + (((b & 1) << 1) | ((b >> 1) & 1));
  }
  const float2 v = src[(size_t)r * kTile + q];
  dst[(size_t)r * kTile + k] = make_float2(v.x * (1.0f / 2048.0f), v.y * (1.0f / 2048.0f));
}

// Address of this device's scratch; on the first call for a device (with that
// device current) it is looked up and the twiddle table is written into it.
fdas_status scratch_for_current_device(float2 **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return FDAS_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= kMaxDevices) return FDAS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev]) {
    *out = g_scratch_ptr[dev];
    return FDAS_OK;
  }
  if (!g_twiddle_host_ready) {
    for (int j = 0; j < kTile; ++j) {
      const double a = 2.0 * M_PI * (double)j / (double)kTile;
      g_twiddle_host[j] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    g_twiddle_host_ready = true;
  }
  void *addr = nullptr;
  if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) {
    cudaGetLastError();
    return FDAS_ERR_CUDA;
  }
  if (cudaMemcpyToSymbol(g_noalloc_scratch, g_twiddle_host, sizeof(g_twiddle_host),
                         sizeof(float2) * (kTileElems + kTmplElems), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    return FDAS_ERR_CUDA;
  }
  g_scratch_ptr[dev] = static_cast<float2 *>(addr);
  *out = g_scratch_ptr[dev];
  return FDAS_OK;
}

}  // namespace

extern "C" fdas_status fdas_ft_convolution_noalloc(const fdas_complex *d_spectrum, uint32_t n_bins,
                                                   const fdas_complex *d_templates, fdas_template_layout layout,
                                                   uint32_t n_templates, uint32_t tile_overlap, fdas_fop_part which,
                                                   float *d_fop, uint64_t fop_stride, int32_t *d_status,
                                                   void *stream) {
  // ---- arguments (no CUDA call before these pass)
  if (!d_spectrum || !d_templates || !d_fop) return FDAS_ERR_INVALID_ARG;
  // odd template counts only: row n_templates / 2 is template 0 (as for the handle)
  if (n_bins == 0 || n_templates % 2 == 0 || fop_stride < n_bins) return FDAS_ERR_INVALID_ARG;
  if (tile_overlap >= (uint32_t)kTile) return FDAS_ERR_INVALID_ARG;
  if (which != FDAS_NEGATIVE_ACCELERATIONS && which != FDAS_POSITIVE_ACCELERATIONS &&
      which != FDAS_ALL_ACCELERATIONS)
    return FDAS_ERR_INVALID_ARG;
  if (layout == FDAS_TEMPLATES_TIME_DOMAIN) return FDAS_ERR_UNSUPPORTED;
  if (layout != FDAS_TEMPLATES_FFT_P4 && layout != FDAS_TEMPLATES_FFT_NATURAL) return FDAS_ERR_INVALID_ARG;
  if ((reinterpret_cast<uintptr_t>(d_spectrum) | reinterpret_cast<uintptr_t>(d_templates)) % 8 ||
      reinterpret_cast<uintptr_t>(d_fop) % 4 || reinterpret_cast<uintptr_t>(d_status) % 4)
    return FDAS_ERR_INVALID_ARG;
  const uint32_t payload = (uint32_t)kTile - tile_overlap;
  const uint64_t n_tiles = ((uint64_t)n_bins + payload - 1) / payload;
  // sizes beyond the static scratch are refused, never truncated
  if (n_tiles > FDAS_NOALLOC_MAX_TILES || n_templates > FDAS_NOALLOC_MAX_TEMPLATES) return FDAS_ERR_CAPACITY;

  float2 *scratch = nullptr;
  fdas_status st = scratch_for_current_device(&scratch);
  if (st != FDAS_OK) return st;
  float2 *tiles = scratch;
  float2 *tmpl = scratch + kTileElems;
  float2 *twiddle = tmpl + kTmplElems;
  int *status_word = reinterpret_cast<int *>(twiddle + kTwElems);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  noalloc_templates_kernel<<<dim3(kTile / 256, n_templates), 256, 0, s>>>(
      reinterpret_cast<const float2 *>(d_templates), tmpl, (int)n_templates, layout == FDAS_TEMPLATES_FFT_P4);
  if (cudaGetLastError() != cudaSuccess) return FDAS_ERR_CUDA;

  TileParams tp{};
  tp.input = reinterpret_cast<const float2 *>(d_spectrum);
  tp.n_bins = (int)n_bins;
  tp.n_tiles = (int)n_tiles;
  tp.overlap = (int)tile_overlap;
  tp.payload = (int)payload;
  tp.tiles = tiles;
  tp.twiddle = twiddle;
  if (launch_tile_fft(tp, s) != cudaSuccess) {
    cudaGetLastError();
    return FDAS_ERR_CUDA;
  }

  const int T = (int)n_templates, H = T / 2;
  FtcParams fp{};
  fp.tiles = tiles;
  fp.tmpl = tmpl;
  fp.fop = d_fop;
  fp.fop_stride = (long long)fop_stride;
  fp.n_bins = (int)n_bins;
  fp.n_tiles = (int)n_tiles;
  fp.overlap = (int)tile_overlap;
  fp.payload = (int)payload;
  if (which == FDAS_NEGATIVE_ACCELERATIONS) { fp.row_begin = 0; fp.n_rows = H + 1; }
  else if (which == FDAS_POSITIVE_ACCELERATIONS) { fp.row_begin = H; fp.n_rows = H + 1; }
  else { fp.row_begin = 0; fp.n_rows = T; }
  fp.twiddle = twiddle;
  fp.status = d_status ? reinterpret_cast<int *>(d_status) : status_word;
  fp.timeout_ns = 2000000000LL;  // 2 s
  fp.ctas_per_sm = 2;
  if (launch_ftc(fp, s) != cudaSuccess) {
    cudaGetLastError();
    return FDAS_ERR_CUDA;
  }
  return FDAS_OK;
}
