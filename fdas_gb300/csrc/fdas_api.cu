// Host orchestration behind the C ABI (include/fdas_gb300.h).
//
// Mirrors the reference's host class FDAS (fdas/src/host/FDAS.cpp): two buffer
// sets A/B, each with its own CUDA stream in place of the OpenCL command
// queues, CUDA events in place of cl::Event for the stage timings, and the
// same enqueue order: input copy -> tiling -> FT convolution -> harmonic
// summing -> candidate download.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fdas_gb300.h"
#include "kernels.cuh"

using namespace fdas;

namespace {

thread_local std::string g_init_error;

// device control words of a buffer set (zeroed before every harmonic summing)
constexpr int kCtrlStatus = 0;
constexpr int kCtrlRecheckCount = 1;
constexpr int kCtrlTotal = 2;                       // records appended
constexpr int kCtrlCount = 3;                       // + plane: hits per plane
constexpr int kCtrlSelCount = kCtrlCount + kMaxPlanes;
constexpr int kCtrlSelLo = kCtrlSelCount + kMaxPlanes;
constexpr int kCtrlItems = kCtrlSelLo + kMaxPlanes;  // harmonic-summing work counter
constexpr int kCtrlBound = kCtrlItems + 1;           // + plane: boundary records of the selection
constexpr int kCtrlWords = kCtrlBound + kMaxPlanes;   // zeroed before every harmonic summing
constexpr int kCtrlFtcStatus = kCtrlWords;           // FT-convolution status, zeroed before each FT convolution
constexpr int kCtrlTileStatus = kCtrlWords + 1;      // tiling status (tensor-core form), zeroed before each tiling
constexpr int kCtrlStride = kCtrlWords + 2;          // control words per buffer set
constexpr uint32_t kDefaultCapacity = 1u << 22;     // candidate records per buffer set
constexpr uint32_t kMaxCapacity = 1u << 27;
constexpr int kRecheckCap = 65536;
constexpr int kNumEvents = 6;  // start, input, tiling, ftc, hsum, done

struct BufferSet {
  cudaStream_t stream = nullptr;
  float2 *d_input = nullptr;
  const float2 *cur_input = nullptr;
  float2 *d_tiles = nullptr;
  float2 *d_tmpl = nullptr;
  double2 *d_taps = nullptr;  // FP64 taps while templates are uploaded, then float pairs (split_taps)
  int *d_taplen = nullptr;
  float *d_fop = nullptr;
  unsigned long long *d_key = nullptr;
  float *d_pwr = nullptr;
  unsigned *d_ctrl = nullptr;
  unsigned *h_ctrl = nullptr;  // pinned mirror of d_ctrl
  uint4 *d_rc = nullptr;
  unsigned *d_hist = nullptr;
  unsigned *d_ticket = nullptr;
  unsigned long long *d_sel_key = nullptr;
  float *d_sel_pwr = nullptr;
  uint32_t *d_cloc = nullptr;
  float *d_cpwr = nullptr;
  cudaEvent_t ev[kNumEvents] = {};
  HsumMaps maps;  // TMA descriptors of this set's FOP
  bool have_templates = false;
  bool have_taps = false;
  bool have_input = false;
  bool series_spectrum = false;  // d_input holds a spectrum made by fdas_series_to_spectrum
  std::vector<int> taplen;       // non-zero taps per uploaded template row (host copy)
  bool fop_from_input = false;
  bool launched = false;
  bool ctrl_valid = false;
  std::vector<float> thresholds;
  // harmonic summing held back by sync_pipeline
  bool pending = false;
  std::vector<float> p_thr;
  fdas_fop_part p_which = FDAS_ALL_ACCELERATIONS;
  uint32_t *p_loc = nullptr;
  float *p_pwr = nullptr;
  bool ev_ftc_recorded = false;
  bool ftc_unchecked = false;  // an FT convolution ran whose status word has not been checked
  bool tile_unchecked = false; // a tensor-core tiling ran whose status word has not been checked
  cudaEvent_t ev_hsum = nullptr;  // end of this set's last harmonic-summing kernel
  bool ev_hsum_recorded = false;
  bool input_from_host = false;   // the current spectrum was copied in from host memory
};

}  // namespace

struct fdas_handle {
  fdas_config cfg{};
  int N = 0, T = 0, H = 0, L = 0, O = 0, payload = 0, n_tiles = 0, P = 0, cap = 0, per_plane = 0;
  long long stride = 0;
  int tap_pitch = 0;
  std::string err;
  fdas_log_fn log_fn = nullptr;
  void *log_user = nullptr;
  float2 *d_twiddle = nullptr;
  double2 *d_twiddle64 = nullptr;
  float2 *d_series_tw = nullptr;  // e^(-i pi x / N), made on first use
  // fdas_reshape: first template row in use, and the sizes the buffers were allocated for
  int row0 = 0;
  int rc_cap = kRecheckCap;  // entries of the near-threshold recheck list
  int alloc_N = 0, alloc_T = 0, alloc_P = 0, alloc_tiles = 0;
  size_t alloc_fop_floats = 0;
  BufferSet set[2];
  long long wait_timeout_ns = kWaitNs;  // bound on the kernels' waits (fdas_set_wait_timeout)
  uint32_t inject = 0;                   // fdas_set_fault_injection flags
  // print_stats / print_events bookkeeping: device event times are placed on
  // the host's steady clock through an anchor event recorded (and waited for)
  // at initialisation
  cudaEvent_t anchor = nullptr;
  long long anchor_ns = 0;       // steady-clock time of the anchor event
  long long pipeline_start_ns = 0;
  long long pipeline_accum_ns = 0;
  unsigned pipeline_launches = 0;
};

namespace {

void logf(fdas_handle *h, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h && h->log_fn) h->log_fn(buf, h->log_user);
  else fprintf(stderr, "%s\n", buf);
}

fdas_status fail(fdas_handle *h, fdas_status st, const std::string &msg) {
  if (h) h->err = msg;
  else g_init_error = msg;
  return st;
}

fdas_status cuda_fail(fdas_handle *h, cudaError_t e, const char *what, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA call failed with %s (%s): %s [%s:%d]", cudaGetErrorName(e),
           cudaGetErrorString(e), what, file, line);
  if (h) logf(h, "[ERROR] %s", buf);
  return fail(h, e == cudaErrorMemoryAllocation ? FDAS_ERR_OUT_OF_MEMORY : FDAS_ERR_CUDA, buf);
}

#define CK(h, expr)                                                  \
  do {                                                               \
    cudaError_t e_ = (expr);                                         \
    if (e_ != cudaSuccess) return cuda_fail((h), e_, #expr, __FILE__, __LINE__); \
  } while (0)

bool valid_set(fdas_buffer_set ab) { return ab == FDAS_SET_A || ab == FDAS_SET_B; }

long long steady_ns() {
  return (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
long long system_ns() {
  return (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::system_clock::now().time_since_epoch())
      .count();
}
bool valid_part(fdas_fop_part w) {
  return w == FDAS_NEGATIVE_ACCELERATIONS || w == FDAS_POSITIVE_ACCELERATIONS || w == FDAS_ALL_ACCELERATIONS;
}

#define CHECK_HANDLE(h)                                                              \
  do {                                                                               \
    if (!(h)) return fail(nullptr, FDAS_ERR_INVALID_ARG, "null handle");             \
  } while (0)
#define CHECK_SET(h, ab)                                                             \
  do {                                                                               \
    if (!valid_set(ab)) return fail((h), FDAS_ERR_INVALID_ARG, "invalid buffer set"); \
  } while (0)

int bitrev2(int x) { return ((x & 1) << 1) | ((x >> 1) & 1); }

// p4 position 4 s + j holds natural bin bitrev2(j) * 512 + s (tmpl-gen.py:145-153)
void p4_to_natural(const fdas_complex *p4, fdas_complex *nat) {
  for (int s = 0; s < 512; ++s)
    for (int j = 0; j < 4; ++j) nat[bitrev2(j) * 512 + s] = p4[4 * s + j];
}
void natural_to_p4(const float2 *nat, fdas_complex *p4) {
  for (int s = 0; s < 512; ++s)
    for (int j = 0; j < 4; ++j) {
      const float2 v = nat[bitrev2(j) * 512 + s];
      p4[4 * s + j] = fdas_complex{v.x, v.y};
    }
}

void rows_of(const fdas_handle *h, fdas_fop_part w, int *row_begin, int *n_rows) {
  if (w == FDAS_NEGATIVE_ACCELERATIONS) { *row_begin = 0; *n_rows = h->H + 1; }
  else if (w == FDAS_POSITIVE_ACCELERATIONS) { *row_begin = h->H; *n_rows = h->H + 1; }
  else { *row_begin = 0; *n_rows = h->T; }
}

// ------------------------------------------------- harmonic-summing geometry
// Box shapes of the per-item staging (see hsum_kernel): plane 1 is 128 bins x
// 4 NW rows, plane j >= 2 covers bins [(f0/j) & ~3, ...) of the rows
// trunc(|t|/j), |t| < 4 NW, with one spare row and column for the 2 x 2 windows.
void hsum_geometry(const fdas_handle *h, HsumParams &p) {
  const int nw = hsum_warps(h->H);
  p.bw[1] = kHsBins;
  p.bh[1] = 4 * nw;
  int off = 0;
  p.soff[1] = off;
  off += p.bw[1] * p.bh[1];
  unsigned bytes = (unsigned)(p.bw[1] * p.bh[1] * 4);
  for (int j = 2; j <= h->P; ++j) {
    p.bw[j] = ((kHsBins - 1) / j + 6 + 3) & ~3;
    p.bh[j] = (4 * nw - 1) / j + 2;
    off = (off + 31) & ~31;  // 128-byte aligned TMA destinations
    p.soff[j] = off;
    off += p.bw[j] * p.bh[j];
    bytes += (unsigned)(p.bw[j] * p.bh[j] * 4);
  }
  p.stage_floats = (off + 255) & ~255;  // 1 KB aligned stages
  p.stage_bytes = bytes;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

fdas_status make_hsum_maps(fdas_handle *h, BufferSet &S) {
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return fail(h, FDAS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    encode = reinterpret_cast<EncodeTiledFn>(fn);
  }
  HsumParams g{};
  hsum_geometry(h, g);
  std::memset(&S.maps, 0, sizeof(S.maps));
  for (int j = 1; j <= h->P; ++j) {
    const cuuint64_t dims[2] = {(cuuint64_t)h->stride, (cuuint64_t)h->T};
    const cuuint64_t strides[1] = {(cuuint64_t)h->stride * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)g.bw[j], (cuuint32_t)g.bh[j]};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&S.maps.map[j], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, S.d_fop, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      char msg[128];
      snprintf(msg, sizeof(msg), "cuTensorMapEncodeTiled failed (%d) for plane %d", (int)r, j);
      return fail(h, FDAS_ERR_CUDA, msg);
    }
  }
  return FDAS_OK;
}

// ---------------------------------------------------------------- stages
fdas_status enqueue_input(fdas_handle *h, int ab, const fdas_complex *input, bool device_ptr) {
  BufferSet &S = h->set[ab];
  // NULL: the spectrum that fdas_series_to_spectrum left in this set
  if (!input && !(S.series_spectrum && !device_ptr))
    return fail(h, FDAS_ERR_INVALID_ARG, "input is NULL and no spectrum was made on this buffer set");
  CK(h, cudaEventRecord(S.ev[0], S.stream));
  if (h->cfg.sync_pipeline && h->set[1 - ab].ev_ftc_recorded)
    CK(h, cudaStreamWaitEvent(S.stream, h->set[1 - ab].ev[3], 0));  // FDAS.cpp:287-288
  S.input_from_host = false;
  if (!input) {
    S.cur_input = S.d_input;
  } else if (device_ptr) {
    S.cur_input = reinterpret_cast<const float2 *>(input);
  } else {
    CK(h, cudaMemcpyAsync(S.d_input, input, sizeof(float2) * (size_t)h->N, cudaMemcpyHostToDevice, S.stream));
    S.cur_input = S.d_input;
    S.series_spectrum = false;
    S.input_from_host = true;
  }
  CK(h, cudaEventRecord(S.ev[1], S.stream));
  S.have_input = true;
  return FDAS_OK;
}

fdas_status enqueue_tiling(fdas_handle *h, int ab) {
  BufferSet &S = h->set[ab];
  TileParams p{};
  p.input = S.cur_input;
  p.n_bins = h->N;
  p.n_tiles = h->n_tiles;
  p.overlap = h->O;
  p.payload = h->payload;
  p.tiles = S.d_tiles;
  p.twiddle = h->d_twiddle;
  S.ctrl_valid = false;  // the host copy of the control words predates this stage
  if (h->cfg.precision) {  // precision form: the forward DFT on the tensor cores too
    CK(h, cudaMemsetAsync(S.d_ctrl + kCtrlTileStatus, 0, sizeof(unsigned), S.stream));
    CK(h, launch_tile_tc(p, h->cfg.precision == 2, reinterpret_cast<int *>(S.d_ctrl + kCtrlTileStatus),
                         h->wait_timeout_ns, S.stream));
    S.tile_unchecked = true;
  } else {
    CK(h, launch_tile_fft(p, S.stream));
  }
  CK(h, cudaEventRecord(S.ev[2], S.stream));
  return FDAS_OK;
}

fdas_status enqueue_ftc(fdas_handle *h, int ab, fdas_fop_part which) {
  BufferSet &S = h->set[ab];
  if (!S.have_templates) return fail(h, FDAS_ERR_STATE, "templates not uploaded for this buffer set");
  if (!S.have_input) return fail(h, FDAS_ERR_STATE, "no input tiled on this buffer set");
  FtcParams p{};
  p.tiles = S.d_tiles;
  p.tmpl = S.d_tmpl + (size_t)h->row0 * kTile;
  p.fop = S.d_fop;
  p.fop_stride = h->stride;
  p.n_bins = h->N;
  p.n_tiles = h->n_tiles;
  p.overlap = h->O;
  p.payload = h->payload;
  rows_of(h, which, &p.row_begin, &p.n_rows);
  p.twiddle = h->d_twiddle;
  p.status = reinterpret_cast<int *>(S.d_ctrl + kCtrlFtcStatus);
  p.timeout_ns = h->wait_timeout_ns;
  p.ctas_per_sm = h->cfg.overlap ? 1 : 2;
  p.variant = h->cfg.precision == 1 ? 3 : h->cfg.precision == 2 ? 4 : 0;
  if (h->inject & FDAS_INJECT_FTC_STALL) {
    p.inject_stall = 1;
    p.variant = 2;  // the hook lives in the warp-pair FFT kernel
  }
  S.ctrl_valid = false;  // the host copy of the control words predates this stage
  // A search whose spectrum was copied from host memory starts its FT
  // convolution only once the other set's harmonic-summing kernel has ended.
  // Otherwise that harmonic summing finds every SM held by this FT convolution
  // (two CTAs of 128 registers x 256 threads fill an SM's register file), both
  // searches end together, and with launch(A) / wait(B) the next launch -- its
  // 16 MB copy and tiling -- starts on an empty GPU every second search.
  // Device-resident searches queued ahead keep the unordered form, where the
  // two harmonic summings run side by side after both FT convolutions.
  if (S.input_from_host && !h->cfg.overlap && !h->cfg.sync_pipeline && h->set[1 - ab].ev_hsum_recorded)
    CK(h, cudaStreamWaitEvent(S.stream, h->set[1 - ab].ev_hsum, 0));
  CK(h, cudaMemsetAsync(S.d_ctrl + kCtrlFtcStatus, 0, sizeof(unsigned), S.stream));
  CK(h, launch_ftc(p, S.stream));
  CK(h, cudaEventRecord(S.ev[3], S.stream));
  S.ftc_unchecked = true;
  S.ev_ftc_recorded = true;
  S.fop_from_input = true;
  return FDAS_OK;
}

fdas_status enqueue_hsum(fdas_handle *h, int ab, const float *thr_in, fdas_fop_part which) {
  BufferSet &S = h->set[ab];
  const float *thr = thr_in;
  if (!thr) {
    if (S.thresholds.empty()) return fail(h, FDAS_ERR_STATE, "no thresholds given or uploaded");
    thr = S.thresholds.data();
  }
  const int P = h->P;
  const bool recheck = h->cfg.recheck && S.fop_from_input && S.have_taps && S.cur_input;
  const float band_rel = h->cfg.recheck_band > 0.f ? h->cfg.recheck_band : 1e-4f;

  HsumParams p{};
  p.fop = S.d_fop;
  p.stride = h->stride;
  p.n_bins = h->N;
  p.half = h->H;
  p.n_planes = P;
  const int H = h->H;
  if (which == FDAS_NEGATIVE_ACCELERATIONS) { p.tlo[0] = 0; p.tlo[1] = H + 1; }
  else if (which == FDAS_POSITIVE_ACCELERATIONS) { p.tlo[0] = H + 1; p.tlo[1] = 0; }
  else { p.tlo[0] = 1; p.tlo[1] = 0; }
  for (int j = 0; j < kMaxPlanes; ++j) {
    const float t = j < P ? thr[j] : INFINITY;
    if (recheck) {
      const float band = band_rel * std::fabs(t);
      p.hi[j] = t + band;
      p.lo[j] = t - band;
      p.trig[j] = p.lo[j];
    } else {
      p.hi[j] = t;
      p.lo[j] = INFINITY;
      p.trig[j] = t;
    }
  }
  hsum_geometry(h, p);
  p.item_counter = S.d_ctrl + kCtrlItems;
  p.lean = h->cfg.overlap && P <= 8 && hsum_warps(H) == 11 ? 1 : 0;
  p.inject_stall = (h->inject & FDAS_INJECT_HSUM_STALL) ? 1 : 0;
  p.cand_key = S.d_key;
  p.cand_pwr = S.d_pwr;
  p.cand_total = S.d_ctrl + kCtrlTotal;
  p.cand_count = S.d_ctrl + kCtrlCount;
  p.cand_cap = h->cap;
  p.rc_list = S.d_rc;
  p.rc_count = S.d_ctrl + kCtrlRecheckCount;
  p.rc_cap = h->rc_cap;
  p.status = reinterpret_cast<int *>(S.d_ctrl + kCtrlStatus);
  p.timeout_ns = h->wait_timeout_ns;

  if (hsum_smem_bytes(p) > 227 * 1024)
    return fail(h, FDAS_ERR_UNSUPPORTED, "harmonic summing staging exceeds shared memory (too many templates x planes)");
  CK(h, cudaMemsetAsync(S.d_ctrl, 0, sizeof(unsigned) * kCtrlWords, S.stream));
  CK(h, launch_hsum(p, S.maps, S.stream));
  if (S.ev_hsum) {  // (the batched form's per-trial views have none)
    CK(h, cudaEventRecord(S.ev_hsum, S.stream));
    S.ev_hsum_recorded = true;
  }
  if (recheck) {
    RecheckParams r{};
    r.input = S.cur_input;
    r.n_bins = h->N;
    r.half = H;
    r.taps = reinterpret_cast<const float4 *>(S.d_taps + (size_t)h->row0 * h->tap_pitch);
    r.tap_len = S.d_taplen + h->row0;
    r.tap_pitch = h->tap_pitch;
    for (int j = 0; j < kMaxPlanes; ++j) r.thr[j] = j < P ? (double)thr[j] : INFINITY;
    r.rc_list = S.d_rc;
    r.rc_count = S.d_ctrl + kCtrlRecheckCount;
    r.rc_cap = h->rc_cap;
    r.cand_key = S.d_key;
    r.cand_pwr = S.d_pwr;
    r.cand_total = S.d_ctrl + kCtrlTotal;
    r.cand_count = S.d_ctrl + kCtrlCount;
    r.cand_cap = h->cap;
    r.status = p.status;
    CK(h, launch_recheck(r, S.stream));
  }
  SelectParams f{};
  f.cand_key = S.d_key;
  f.cand_pwr = S.d_pwr;
  f.cand_total = S.d_ctrl + kCtrlTotal;
  f.cand_count = S.d_ctrl + kCtrlCount;
  f.cand_cap = h->cap;
  f.n_planes = P;
  f.per_plane = h->per_plane;
  f.hist = S.d_hist;
  f.ticket = S.d_ticket;
  f.sel_bucket = reinterpret_cast<int *>(S.d_ctrl + kCtrlSelLo);
  f.sure_count = S.d_ctrl + kCtrlSelCount;
  f.bound_count = S.d_ctrl + kCtrlBound;
  f.sel_key = S.d_sel_key;
  f.sel_pwr = S.d_sel_pwr;
  f.compat_loc = S.d_cloc;
  f.compat_pwr = S.d_cpwr;
  f.invalid_location = (uint32_t)((h->H + 1 + h->H) & 0x7f) << 22;  // encode(1, H+1, 0), gen_info.h:69
  f.status = p.status;
  CK(h, launch_select(f, S.stream));
  CK(h, cudaMemcpyAsync(S.h_ctrl, S.d_ctrl, sizeof(unsigned) * kCtrlStride, cudaMemcpyDeviceToHost, S.stream));
  CK(h, cudaEventRecord(S.ev[4], S.stream));
  S.ctrl_valid = true;
  return FDAS_OK;
}

fdas_status enqueue_download(fdas_handle *h, int ab, uint32_t *loc, float *pwr) {
  BufferSet &S = h->set[ab];
  const size_t n = (size_t)h->P * h->per_plane;
  if (loc) CK(h, cudaMemcpyAsync(loc, S.d_cloc, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, S.stream));
  if (pwr) CK(h, cudaMemcpyAsync(pwr, S.d_cpwr, sizeof(float) * n, cudaMemcpyDeviceToHost, S.stream));
  CK(h, cudaEventRecord(S.ev[5], S.stream));
  S.launched = true;
  return FDAS_OK;
}

fdas_status release_pending(fdas_handle *h, int ab) {
  BufferSet &S = h->set[ab];
  if (!S.pending) return FDAS_OK;
  S.pending = false;
  fdas_status st = enqueue_hsum(h, ab, S.p_thr.data(), S.p_which);
  if (st != FDAS_OK) return st;
  return enqueue_download(h, ab, S.p_loc, S.p_pwr);
}

// Device-side timeouts of the last search on set `ab`, once its stream has
// completed: the status words come back with the candidate counters; an FT
// convolution run without harmonic summing has its word read here.
fdas_status check_timeouts(fdas_handle *h, int ab) {
  BufferSet &S = h->set[ab];
  unsigned word[2] = {0u, 0u};  // FT convolution, tiling
  if (S.ftc_unchecked || S.tile_unchecked) {
    if (S.ctrl_valid) {
      word[0] = S.h_ctrl[kCtrlFtcStatus];
      word[1] = S.h_ctrl[kCtrlTileStatus];
    } else {
      CK(h, cudaMemcpy(word, S.d_ctrl + kCtrlFtcStatus, sizeof(word), cudaMemcpyDeviceToHost));
    }
  }
  if (word[1] & kStatusFtcTimeout) return fail(h, FDAS_ERR_TIMEOUT, "tiling: tensor-core wait timed out");
  if (word[0] & kStatusFtcTimeout) return fail(h, FDAS_ERR_TIMEOUT, "FT convolution: template staging timed out");
  if (S.ctrl_valid && (S.h_ctrl[kCtrlStatus] & kStatusHsumTimeout))
    return fail(h, FDAS_ERR_TIMEOUT, "harmonic summing: shared-memory staging timed out");
  return FDAS_OK;
}

fdas_status sync_set(fdas_handle *h, int ab) {
  BufferSet &S = h->set[ab];
  CK(h, cudaStreamSynchronize(S.stream));
  return check_timeouts(h, ab);
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return -1.f;
  }
  return ms;
}

void free_set(BufferSet &S) {
  if (S.stream) cudaStreamSynchronize(S.stream);
  cudaFree(S.d_input);
  cudaFree(S.d_tiles);
  cudaFree(S.d_tmpl);
  cudaFree(S.d_taps);
  cudaFree(S.d_taplen);
  cudaFree(S.d_fop);
  cudaFree(S.d_key);
  cudaFree(S.d_pwr);
  cudaFree(S.d_ctrl);
  cudaFree(S.d_rc);
  cudaFree(S.d_hist);
  cudaFree(S.d_ticket);
  cudaFree(S.d_sel_key);
  cudaFree(S.d_sel_pwr);
  cudaFree(S.d_cloc);
  cudaFree(S.d_cpwr);
  if (S.h_ctrl) cudaFreeHost(S.h_ctrl);
  for (auto &e : S.ev)
    if (e) cudaEventDestroy(e);
  if (S.ev_hsum) cudaEventDestroy(S.ev_hsum);
  if (S.stream) cudaStreamDestroy(S.stream);
  S = BufferSet();
}

}  // namespace

// ===================================================================== C ABI
extern "C" {

const char *fdas_version(void) { return "fdas_gb300 0.1 (sm_103a)"; }

void fdas_default_config(fdas_config *cfg, uint32_t n_frequency_bins) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->n_frequency_bins = n_frequency_bins;
  cfg->n_templates = 85;
  cfg->max_template_len = 421;
  cfg->tile_overlap = 0;
  cfg->n_planes = 8;
  cfg->candidate_capacity = 0;
  cfg->candidates_per_plane_compat = 0;
  cfg->device = 0;
  cfg->buffer_mode = FDAS_MODE_PER_SET;
  cfg->sync_pipeline = 0;
  cfg->recheck = 1;
  cfg->recheck_band = 0.f;
}

const char *fdas_last_error(const fdas_handle *h) { return h ? h->err.c_str() : g_init_error.c_str(); }

fdas_status fdas_initialise_accelerator(const fdas_config *cfg_in, fdas_handle **out) {
  if (!out) return fail(nullptr, FDAS_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!cfg_in) return fail(nullptr, FDAS_ERR_INVALID_ARG, "config is NULL");
  fdas_config cfg = *cfg_in;
  if (cfg.n_frequency_bins == 0) return fail(nullptr, FDAS_ERR_INVALID_ARG, "n_frequency_bins must be > 0");
  if (cfg.n_frequency_bins > (1u << 30)) return fail(nullptr, FDAS_ERR_INVALID_ARG, "n_frequency_bins too large");
  if (cfg.n_templates == 0 || cfg.n_templates % 2 == 0 || cfg.n_templates > 127)
    return fail(nullptr, FDAS_ERR_INVALID_ARG, "n_templates must be odd and at most 127");
  if (cfg.n_planes < 1 || cfg.n_planes > (uint32_t)kMaxPlanes)
    return fail(nullptr, FDAS_ERR_INVALID_ARG, "n_planes must be in 1..16");
  if (cfg.max_template_len < 1) return fail(nullptr, FDAS_ERR_INVALID_ARG, "max_template_len must be >= 1");
  uint32_t O = cfg.tile_overlap ? cfg.tile_overlap : ((cfg.max_template_len - 1 + 3) / 4) * 4;
  if (O + 1 < cfg.max_template_len)
    return fail(nullptr, FDAS_ERR_INVALID_ARG, "tile_overlap must be >= max_template_len - 1 (overlap-save)");
  if (O >= (uint32_t)kTile) return fail(nullptr, FDAS_ERR_INVALID_ARG, "tile_overlap must be < 2048");
  uint32_t cap = cfg.candidate_capacity ? cfg.candidate_capacity : kDefaultCapacity;
  if (cap > kMaxCapacity) return fail(nullptr, FDAS_ERR_INVALID_ARG, "candidate_capacity must be <= 2^27");
  uint32_t pc = cfg.candidates_per_plane_compat ? cfg.candidates_per_plane_compat : 512u;
  if (pc > (uint32_t)kMaxCompat)
    return fail(nullptr, FDAS_ERR_INVALID_ARG, "candidates_per_plane_compat must be <= 2048");
  if (cfg.precision > 2) return fail(nullptr, FDAS_ERR_INVALID_ARG, "precision must be 0, 1 or 2");

  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(nullptr, FDAS_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (cfg.device < 0 || cfg.device >= ndev) return fail(nullptr, FDAS_ERR_INVALID_ARG, "invalid device ordinal");
  e = cudaSetDevice(cfg.device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice", __FILE__, __LINE__);

  fdas_handle *h = new fdas_handle();
  h->log_fn = cfg.log_fn;
  h->log_user = cfg.log_user;
  // FDAS.cpp:60-63: wall-clock and steady-clock times, to map the steady-clock
  // times of the "%%%" and "@@@" lines onto wall-clock time
  logf(h, "^^^,%lld,%lld", system_ns(), steady_ns());
  h->cfg = cfg;
  h->cfg.tile_overlap = O;
  h->cfg.candidate_capacity = cap;
  h->cfg.candidates_per_plane_compat = pc;
  h->N = (int)cfg.n_frequency_bins;
  h->T = (int)cfg.n_templates;
  h->H = h->T / 2;
  h->L = (int)cfg.max_template_len;
  h->O = (int)O;
  h->payload = kTile - h->O;
  h->n_tiles = (h->N + h->payload - 1) / h->payload;  // FDAS.cpp:177-183
  h->P = (int)cfg.n_planes;
  h->cap = (int)cap;
  h->per_plane = (int)pc;
  h->stride = ((long long)h->N + kHsBins - 1) / kHsBins * kHsBins;
  h->tap_pitch = std::max(h->L, h->O + 1);

  auto bail = [&](fdas_status st) {
    g_init_error = h->err;
    if (h->anchor) cudaEventDestroy(h->anchor);
    for (auto &S : h->set) free_set(S);
    cudaFree(h->d_twiddle);
    cudaFree(h->d_twiddle64);
    delete h;
    return st;
  };

  // twiddle tables, computed on the host in double precision
  {
    std::vector<float2> tw(kTile);
    std::vector<double2> tw64(kTile);
    for (int j = 0; j < kTile; ++j) {
      const double a = 2.0 * M_PI * (double)j / (double)kTile;
      tw[j] = make_float2((float)std::cos(a), (float)std::sin(a));
      tw64[j] = make_double2(std::cos(a), -std::sin(a));
    }
    if ((e = cudaMalloc(&h->d_twiddle, sizeof(float2) * kTile)) != cudaSuccess ||
        (e = cudaMalloc(&h->d_twiddle64, sizeof(double2) * kTile)) != cudaSuccess ||
        (e = cudaMemcpy(h->d_twiddle, tw.data(), sizeof(float2) * kTile, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(h->d_twiddle64, tw64.data(), sizeof(double2) * kTile, cudaMemcpyHostToDevice)) !=
            cudaSuccess) {
      cuda_fail(h, e, "twiddle tables", __FILE__, __LINE__);
      return bail(e == cudaErrorMemoryAllocation ? FDAS_ERR_OUT_OF_MEMORY : FDAS_ERR_CUDA);
    }
  }

  const size_t fop_floats = (size_t)h->T * (size_t)h->stride + 4096;
  h->alloc_N = h->N;
  h->alloc_T = h->T;
  h->alloc_P = h->P;
  h->alloc_tiles = h->n_tiles;
  h->alloc_fop_floats = fop_floats;
  for (int ab = 0; ab < 2; ++ab) {
    BufferSet &S = h->set[ab];
    struct A {
      void **p;
      size_t bytes;
    } allocs[] = {
        {(void **)&S.d_input, sizeof(float2) * ((size_t)h->N + 64)},
        {(void **)&S.d_tiles, sizeof(float2) * (size_t)h->n_tiles * kTile},
        {(void **)&S.d_tmpl, sizeof(float2) * (size_t)h->T * kTile},
        {(void **)&S.d_taps, sizeof(double2) * (size_t)h->T * h->tap_pitch},
        {(void **)&S.d_taplen, sizeof(int) * (size_t)h->T},
        {(void **)&S.d_fop, sizeof(float) * fop_floats},
        {(void **)&S.d_key, sizeof(unsigned long long) * (size_t)h->cap},
        {(void **)&S.d_pwr, sizeof(float) * (size_t)h->cap},
        {(void **)&S.d_ctrl, sizeof(unsigned) * kCtrlStride},
        {(void **)&S.d_rc, sizeof(uint4) * kRecheckCap},
        {(void **)&S.d_hist, sizeof(unsigned) * (size_t)h->P * kSelBuckets},
        {(void **)&S.d_ticket, sizeof(unsigned)},
        {(void **)&S.d_sel_key, sizeof(unsigned long long) * (size_t)h->P * 2 * kSortCap},
        {(void **)&S.d_sel_pwr, sizeof(float) * (size_t)h->P * 2 * kSortCap},
        {(void **)&S.d_cloc, sizeof(uint32_t) * (size_t)h->P * h->per_plane},
        {(void **)&S.d_cpwr, sizeof(float) * (size_t)h->P * h->per_plane},
    };
    for (auto &a : allocs) {
      if ((e = cudaMalloc(a.p, a.bytes)) != cudaSuccess) {
        char msg[160];
        snprintf(msg, sizeof(msg), "device allocation of %zu bytes", a.bytes);
        cuda_fail(h, e, msg, __FILE__, __LINE__);
        return bail(FDAS_ERR_OUT_OF_MEMORY);
      }
    }
    if ((e = cudaMemset(S.d_fop, 0, sizeof(float) * fop_floats)) != cudaSuccess ||
        (e = cudaMemset(S.d_hist, 0, sizeof(unsigned) * (size_t)h->P * kSelBuckets)) != cudaSuccess ||
        (e = cudaMemset(S.d_ticket, 0, sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemset(S.d_ctrl, 0, sizeof(unsigned) * kCtrlStride)) != cudaSuccess ||
        (e = cudaHostAlloc((void **)&S.h_ctrl, sizeof(unsigned) * kCtrlStride, cudaHostAllocDefault)) !=
            cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&S.stream, cudaStreamNonBlocking, h->cfg.stream_priority)) != cudaSuccess) {
      cuda_fail(h, e, "buffer set initialisation", __FILE__, __LINE__);
      return bail(FDAS_ERR_CUDA);
    }
    std::memset(S.h_ctrl, 0, sizeof(unsigned) * kCtrlStride);
    if (make_hsum_maps(h, S) != FDAS_OK) return bail(FDAS_ERR_CUDA);
    for (auto &ev : S.ev) {
      if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
        cuda_fail(h, e, "cudaEventCreate", __FILE__, __LINE__);
        return bail(FDAS_ERR_CUDA);
      }
    }
    if ((e = cudaEventCreateWithFlags(&S.ev_hsum, cudaEventDisableTiming)) != cudaSuccess) {
      cuda_fail(h, e, "cudaEventCreate", __FILE__, __LINE__);
      return bail(FDAS_ERR_CUDA);
    }
  }
  // the anchor placing device events on the host's steady clock
  if ((e = cudaEventCreate(&h->anchor)) != cudaSuccess ||
      (e = cudaEventRecord(h->anchor, h->set[0].stream)) != cudaSuccess ||
      (e = cudaEventSynchronize(h->anchor)) != cudaSuccess) {
    cuda_fail(h, e, "anchor event", __FILE__, __LINE__);
    return bail(FDAS_ERR_CUDA);
  }
  h->anchor_ns = steady_ns();
  logf(h, "[INFO] Device %d: %d bins, %d templates, %d tiles (overlap %d), %d planes", cfg.device, h->N, h->T,
       h->n_tiles, h->O, h->P);
  *out = h;
  return FDAS_OK;
}

void fdas_destroy(fdas_handle *h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  for (auto &S : h->set) free_set(S);
  cudaFree(h->d_twiddle);
  cudaFree(h->d_twiddle64);
  cudaFree(h->d_series_tw);
  if (h->anchor) cudaEventDestroy(h->anchor);
  delete h;
}

fdas_status fdas_reshape(fdas_handle *h, uint32_t n_frequency_bins, uint32_t template_row_begin,
                         uint32_t n_templates, uint32_t tile_overlap, uint32_t n_planes) {
  CHECK_HANDLE(h);
  if (n_frequency_bins == 0 || n_frequency_bins > (uint32_t)h->alloc_N)
    return fail(h, FDAS_ERR_INVALID_ARG, "n_frequency_bins must be 1 .. the initialised size");
  if (n_templates == 0 || n_templates % 2 == 0 || template_row_begin + n_templates > (uint32_t)h->alloc_T)
    return fail(h, FDAS_ERR_INVALID_ARG, "template rows must be an odd count within the initialised bank");
  if (n_planes == 0 || n_planes > (uint32_t)h->alloc_P)
    return fail(h, FDAS_ERR_INVALID_ARG, "n_planes must be 1 .. the initialised count");
  // longest template of the range, from the uploaded banks
  int longest = 0;
  for (auto &S : h->set)
    for (uint32_t r = template_row_begin; r < template_row_begin + n_templates && r < S.taplen.size(); ++r)
      longest = std::max(longest, S.taplen[r]);
  uint32_t O = tile_overlap ? tile_overlap : (longest > 0 ? ((uint32_t)longest - 1 + 3) / 4 * 4 : (uint32_t)h->O);
  if (O >= (uint32_t)kTile) return fail(h, FDAS_ERR_INVALID_ARG, "tile_overlap must be < 2048");
  if ((int)O + 1 < longest)
    return fail(h, FDAS_ERR_INVALID_ARG, "tile_overlap is shorter than a template of the range (overlap-save)");
  const int payload = kTile - (int)O;
  const int n_tiles = ((int)n_frequency_bins + payload - 1) / payload;
  const long long stride = ((long long)n_frequency_bins + kHsBins - 1) / kHsBins * kHsBins;
  if (n_tiles > h->alloc_tiles || (size_t)n_templates * (size_t)stride + 4096 > h->alloc_fop_floats)
    return fail(h, FDAS_ERR_CAPACITY, "shape does not fit the buffers the handle was initialised with");
  for (auto &S : h->set)
    if (S.pending) return fail(h, FDAS_ERR_STATE, "a buffer set holds a pending harmonic summing");
  CK(h, cudaSetDevice(h->cfg.device));
  for (auto &S : h->set) CK(h, cudaStreamSynchronize(S.stream));
  h->N = (int)n_frequency_bins;
  h->row0 = (int)template_row_begin;
  h->T = (int)n_templates;
  h->H = h->T / 2;
  h->O = (int)O;
  h->payload = payload;
  h->n_tiles = n_tiles;
  h->P = (int)n_planes;
  h->stride = stride;
  h->cfg.n_frequency_bins = n_frequency_bins;
  h->cfg.n_templates = n_templates;
  h->cfg.tile_overlap = O;
  h->cfg.n_planes = n_planes;
  for (auto &S : h->set) {
    S.have_input = S.fop_from_input = S.launched = S.ctrl_valid = S.series_spectrum = false;
    S.ev_ftc_recorded = false;
    S.thresholds.clear();
    fdas_status st = make_hsum_maps(h, S);
    if (st != FDAS_OK) return st;
  }
  return FDAS_OK;
}

fdas_status fdas_upload_templates(fdas_handle *h, const fdas_complex *templates, fdas_template_layout layout,
                                  fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!templates) return fail(h, FDAS_ERR_INVALID_ARG, "templates is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  BufferSet &S = h->set[ab];
  const int T = h->T;
  // rows [row0, row0 + T) of the set's template buffers (row0 = 0 unless reshaped)
  float2 *d_tmpl = S.d_tmpl + (size_t)h->row0 * kTile;
  double2 *d_taps = S.d_taps + (size_t)h->row0 * h->tap_pitch;
  int *d_taplen = S.d_taplen + h->row0;
  std::vector<int> len(T, 0);
  if (layout == FDAS_TEMPLATES_TIME_DOMAIN) {
    // ft_conv.py:203 convolves with the non-zero taps of each row
    std::vector<double2> taps((size_t)T * h->tap_pitch, make_double2(0.0, 0.0));
    for (int r = 0; r < T; ++r) {
      int n = 0;
      for (int q = 0; q < h->L; ++q) {
        const fdas_complex c = templates[(size_t)r * h->L + q];
        if (c.re != 0.f || c.im != 0.f) taps[(size_t)r * h->tap_pitch + n++] = make_double2(c.re, c.im);
      }
      if (n > h->O + 1)
        return fail(h, FDAS_ERR_INVALID_ARG, "template has more non-zero taps than tile_overlap + 1");
      len[r] = n;
    }
    CK(h, cudaMemcpy(d_taps, taps.data(), sizeof(double2) * taps.size(), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(d_taplen, len.data(), sizeof(int) * T, cudaMemcpyHostToDevice));
    SpectraParams p{};
    p.taps = d_taps;
    p.tap_len = d_taplen;
    p.tap_pitch = h->tap_pitch;
    p.n_templates = T;
    p.twiddle64 = h->d_twiddle64;
    p.spectra = d_tmpl;
    CK(h, launch_spectra(p, S.stream));
    CK(h, cudaStreamSynchronize(S.stream));
  } else if (layout == FDAS_TEMPLATES_FFT_P4 || layout == FDAS_TEMPLATES_FFT_NATURAL) {
    std::vector<fdas_complex> nat((size_t)T * kTile);
    for (int r = 0; r < T; ++r) {
      if (layout == FDAS_TEMPLATES_FFT_P4) p4_to_natural(templates + (size_t)r * kTile, nat.data() + (size_t)r * kTile);
      else std::memcpy(nat.data() + (size_t)r * kTile, templates + (size_t)r * kTile, sizeof(fdas_complex) * kTile);
    }
    // unscaled spectra -> FP64 taps for the recheck (via the tiles buffer as scratch
    // would clash with a tiled input; use the template buffer before scaling)
    CK(h, cudaMemcpy(d_tmpl, nat.data(), sizeof(float2) * nat.size(), cudaMemcpyHostToDevice));
    TapsParams tp{};
    tp.spectra = d_tmpl;
    tp.n_templates = T;
    tp.n_taps = h->O + 1;
    tp.twiddle64 = h->d_twiddle64;
    tp.taps = d_taps;
    tp.tap_len = d_taplen;
    tp.tap_pitch = h->tap_pitch;
    CK(h, launch_taps(tp, S.stream));
    CK(h, cudaStreamSynchronize(S.stream));
    CK(h, cudaMemcpy(len.data(), d_taplen, sizeof(int) * T, cudaMemcpyDeviceToHost));
    // 1/2048 of the inverse transform folded into the template spectra (exact)
    for (auto &c : nat) {
      c.re *= 1.0f / 2048.0f;
      c.im *= 1.0f / 2048.0f;
    }
    CK(h, cudaMemcpy(d_tmpl, nat.data(), sizeof(float2) * nat.size(), cudaMemcpyHostToDevice));
  } else {
    return fail(h, FDAS_ERR_INVALID_ARG, "unknown template layout");
  }
  // the recheck reads the taps as hi + lo float pairs (FP32-pipe products)
  CK(h, launch_split_taps(d_taps, (long long)T * h->tap_pitch, S.stream));
  CK(h, cudaStreamSynchronize(S.stream));
  S.have_templates = true;
  S.have_taps = true;
  if (S.taplen.size() < (size_t)h->alloc_T) S.taplen.assign(h->alloc_T, 0);
  std::copy(len.begin(), len.end(), S.taplen.begin() + h->row0);
  logf(h, "[INFO] Uploaded template coefficients");
  return FDAS_OK;
}

fdas_status fdas_upload_thresholds(fdas_handle *h, const float *thresholds, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!thresholds) return fail(h, FDAS_ERR_INVALID_ARG, "thresholds is NULL");
  h->set[ab].thresholds.assign(thresholds, thresholds + h->P);
  logf(h, "[INFO] Uploaded thresholds");
  return FDAS_OK;
}

fdas_status fdas_perform_input_tiling(fdas_handle *h, const fdas_complex *input, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = enqueue_input(h, ab, input, false);
  if (st != FDAS_OK) return st;
  if ((st = enqueue_tiling(h, ab)) != FDAS_OK) return st;
  if ((st = sync_set(h, ab)) != FDAS_OK) return st;
  logf(h, "[INFO] Preparation duration: %.3f ms", elapsed(h->set[ab].ev[1], h->set[ab].ev[2]));
  return FDAS_OK;
}

fdas_status fdas_perform_ft_convolution(fdas_handle *h, fdas_fop_part which, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!valid_part(which)) return fail(h, FDAS_ERR_INVALID_ARG, "invalid FOP part");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = enqueue_ftc(h, ab, which);
  if (st != FDAS_OK) return st;
  if ((st = sync_set(h, ab)) != FDAS_OK) return st;
  logf(h, "[INFO] FT convolution and IFFT duration: %.3f ms", elapsed(h->set[ab].ev[2], h->set[ab].ev[3]));
  return FDAS_OK;
}

fdas_status fdas_perform_harmonic_summing(fdas_handle *h, const float *thresholds, fdas_fop_part which,
                                          fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!valid_part(which)) return fail(h, FDAS_ERR_INVALID_ARG, "invalid FOP part");
  CK(h, cudaSetDevice(h->cfg.device));
  BufferSet &S = h->set[ab];
  CK(h, cudaEventRecord(S.ev[3], S.stream));
  fdas_status st = enqueue_hsum(h, ab, thresholds, which);
  if (st != FDAS_OK) return st;
  if ((st = sync_set(h, ab)) != FDAS_OK) return st;
  logf(h, "[INFO] Harmonic summing duration: %.3f ms", elapsed(S.ev[3], S.ev[4]));
  return FDAS_OK;
}

fdas_status fdas_series_to_spectrum(fdas_handle *h, const float *samples, uint64_t n_samples, int samples_on_device,
                                    float scale, fdas_complex *spectrum, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!samples) return fail(h, FDAS_ERR_INVALID_ARG, "samples is NULL");
  // ft_conv.py:125-132: at least 2 N samples; extra samples are ignored
  if (n_samples < 2 * (uint64_t)h->N)
    return fail(h, FDAS_ERR_INVALID_ARG, "the series needs at least 2 x n_frequency_bins samples");
  int radix[64];
  if (series_radices(h->N, radix, 64) < 0)
    return fail(h, FDAS_ERR_UNSUPPORTED, "n_frequency_bins must factor into 2, 3, 5 and 7 for the series FFT");
  BufferSet &S = h->set[ab];
  if (S.pending)
    return fail(h, FDAS_ERR_STATE, "buffer set holds a pending harmonic summing (sync_pipeline); end the pipeline first");
  CK(h, cudaSetDevice(h->cfg.device));
  if (!h->d_series_tw) {
    CK(h, cudaMalloc(&h->d_series_tw, sizeof(float2) * (size_t)h->N));
    CK(h, launch_series_twiddles(h->d_series_tw, h->N, S.stream));
  }
  CK(h, cudaMemcpyAsync(S.d_input, samples, sizeof(float) * 2 * (size_t)h->N,
                        samples_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, S.stream));
  SeriesParams p{};
  p.z = S.d_input;
  p.scratch = S.d_tiles;  // n_tiles x 2048 >= N complex
  p.tw = h->d_series_tw;
  p.n = h->N;
  p.scale = scale;
  CK(h, launch_series_spectrum(p, S.stream));
  if (spectrum)
    CK(h, cudaMemcpyAsync(spectrum, S.d_input, sizeof(float2) * (size_t)h->N, cudaMemcpyDeviceToHost, S.stream));
  CK(h, cudaStreamSynchronize(S.stream));
  S.series_spectrum = true;
  S.have_input = false;  // the tiles buffer was used as scratch
  logf(h, "[INFO] Spectrum of %llu samples -> %d bins", (unsigned long long)(2 * (uint64_t)h->N), h->N);
  return FDAS_OK;
}

fdas_status fdas_launch(fdas_handle *h, const fdas_complex *input, const float *thresholds,
                        uint32_t *detection_location, float *detection_power, fdas_fop_part which,
                        fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!valid_part(which)) return fail(h, FDAS_ERR_INVALID_ARG, "invalid FOP part");
  if (!thresholds && h->set[ab].thresholds.empty())
    return fail(h, FDAS_ERR_STATE, "no thresholds given or uploaded");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st;
  // FDAS.cpp:549-550: launching releases the other set's held-back stage
  if (h->cfg.sync_pipeline && (st = release_pending(h, 1 - ab)) != FDAS_OK) return st;
  long long t[5];  // steady-clock times around the enqueue steps (FDAS.cpp:556-566)
  t[0] = steady_ns();
  if ((st = enqueue_input(h, ab, input, false)) != FDAS_OK) return st;
  if ((st = enqueue_tiling(h, ab)) != FDAS_OK) return st;
  t[1] = steady_ns();
  if ((st = enqueue_ftc(h, ab, which)) != FDAS_OK) return st;
  t[2] = steady_ns();
  BufferSet &S = h->set[ab];
  if (h->cfg.sync_pipeline) {
    S.pending = true;
    const float *thr = thresholds ? thresholds : S.thresholds.data();
    S.p_thr.assign(thr, thr + h->P);
    S.p_which = which;
    S.p_loc = detection_location;
    S.p_pwr = detection_power;
    S.launched = true;
    t[3] = t[4] = steady_ns();  // harmonic summing and download are enqueued later
  } else {
    if ((st = enqueue_hsum(h, ab, thresholds, which)) != FDAS_OK) return st;
    t[3] = steady_ns();
    if ((st = enqueue_download(h, ab, detection_location, detection_power)) != FDAS_OK) return st;
    t[4] = steady_ns();
  }
  if (h->cfg.trace_enqueue) {
    // FDAS.cpp:567-575: whole milliseconds of the enqueue steps, then the raw times
    const char c = ab == FDAS_SET_A ? 'A' : 'B';
    logf(h, "[INFO] Enqueueing: %c\n       %lldms\n       %lldms\n       %lldms\n       %lldms\n       %lldms", c,
         (t[4] - t[0]) / 1000000, (t[1] - t[0]) / 1000000, (t[2] - t[1]) / 1000000, (t[3] - t[2]) / 1000000,
         (t[4] - t[3]) / 1000000);
    logf(h, "%%%%%%,%c,%lld,%lld,%lld,%lld,%lld,", c, t[0], t[1], t[2], t[3], t[4]);
  }
  return FDAS_OK;
}

fdas_status fdas_enqueue_search_device(fdas_handle *h, const fdas_complex *d_input, const float *thresholds,
                                       fdas_fop_part which, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!valid_part(which)) return fail(h, FDAS_ERR_INVALID_ARG, "invalid FOP part");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st;
  if ((st = enqueue_input(h, ab, d_input, true)) != FDAS_OK) return st;
  if ((st = enqueue_tiling(h, ab)) != FDAS_OK) return st;
  if ((st = enqueue_ftc(h, ab, which)) != FDAS_OK) return st;
  if ((st = enqueue_hsum(h, ab, thresholds, which)) != FDAS_OK) return st;
  return enqueue_download(h, ab, nullptr, nullptr);
}

fdas_status fdas_synchronize(fdas_handle *h, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  CK(h, cudaSetDevice(h->cfg.device));
  return sync_set(h, ab);
}

void *fdas_get_stream(fdas_handle *h, fdas_buffer_set ab) {
  if (!h || !valid_set(ab)) return nullptr;
  return (void *)h->set[ab].stream;
}

fdas_status fdas_wait(fdas_handle *h, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  BufferSet &S = h->set[ab];
  if (S.pending)
    return fail(h, FDAS_ERR_STATE,
                "harmonic summing of this set is held back by sync_pipeline: launch the other set or call "
                "end_pipeline first");
  if (!S.launched) return fail(h, FDAS_ERR_STATE, "nothing launched on this buffer set");
  CK(h, cudaSetDevice(h->cfg.device));
  CK(h, cudaEventSynchronize(S.ev[5]));
  return check_timeouts(h, ab);
}

fdas_status fdas_end_pipeline(fdas_handle *h, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  CK(h, cudaSetDevice(h->cfg.device));
  return release_pending(h, 1 - ab);
}

fdas_status fdas_retrieve_tiles(fdas_handle *h, fdas_complex *tiles, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!tiles) return fail(h, FDAS_ERR_INVALID_ARG, "tiles is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = sync_set(h, ab);
  if (st != FDAS_OK) return st;
  std::vector<float2> nat((size_t)h->n_tiles * kTile);
  CK(h, cudaMemcpy(nat.data(), h->set[ab].d_tiles, sizeof(float2) * nat.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < h->n_tiles; ++i) natural_to_p4(nat.data() + (size_t)i * kTile, tiles + (size_t)i * kTile);
  return FDAS_OK;
}

fdas_status fdas_retrieve_fop(fdas_handle *h, float *fop, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!fop) return fail(h, FDAS_ERR_INVALID_ARG, "fop is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = sync_set(h, ab);
  if (st != FDAS_OK) return st;
  CK(h, cudaMemcpy2D(fop, sizeof(float) * h->N, h->set[ab].d_fop, sizeof(float) * h->stride, sizeof(float) * h->N,
                     h->T, cudaMemcpyDeviceToHost));
  return FDAS_OK;
}

fdas_status fdas_inject_fop(fdas_handle *h, const float *fop, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!fop) return fail(h, FDAS_ERR_INVALID_ARG, "fop is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  BufferSet &S = h->set[ab];
  CK(h, cudaStreamSynchronize(S.stream));
  CK(h, cudaMemcpy2D(S.d_fop, sizeof(float) * h->stride, fop, sizeof(float) * h->N, sizeof(float) * h->N, h->T,
                     cudaMemcpyHostToDevice));
  S.fop_from_input = false;
  return FDAS_OK;
}

fdas_status fdas_retrieve_candidates(fdas_handle *h, uint32_t *detection_location, float *detection_power,
                                     fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!detection_location || !detection_power) return fail(h, FDAS_ERR_INVALID_ARG, "output is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = sync_set(h, ab);
  if (st != FDAS_OK) return st;
  const size_t n = (size_t)h->P * h->per_plane;
  CK(h, cudaMemcpy(detection_location, h->set[ab].d_cloc, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
  CK(h, cudaMemcpy(detection_power, h->set[ab].d_cpwr, sizeof(float) * n, cudaMemcpyDeviceToHost));
  return FDAS_OK;
}

fdas_status fdas_retrieve_candidate_list(fdas_handle *h, fdas_candidate *out, uint32_t capacity, uint32_t *n_total,
                                         uint32_t *n_dropped, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!out && capacity > 0) return fail(h, FDAS_ERR_INVALID_ARG, "out is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = sync_set(h, ab);
  if (st != FDAS_OK) return st;
  BufferSet &S = h->set[ab];
  unsigned ctrl[kCtrlWords];
  CK(h, cudaMemcpy(ctrl, S.d_ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost));
  uint32_t total = 0;
  for (int pl = 0; pl < h->P; ++pl) total += ctrl[kCtrlCount + pl];
  const uint32_t stored = std::min(ctrl[kCtrlTotal], (unsigned)h->cap);
  if (capacity == 0) {  // counts only
    if (n_total) *n_total = total;
    if (n_dropped) *n_dropped = total - stored;
    return FDAS_OK;
  }
  std::vector<unsigned long long> keys(stored);
  std::vector<float> pwrs(stored);
  if (stored) {
    CK(h, cudaMemcpy(keys.data(), S.d_key, sizeof(unsigned long long) * stored, cudaMemcpyDeviceToHost));
    CK(h, cudaMemcpy(pwrs.data(), S.d_pwr, sizeof(float) * stored, cudaMemcpyDeviceToHost));
  }
  // (harmonic, template, bin) order, as hsum.py lists its detections
  std::vector<uint32_t> idx(stored);
  std::iota(idx.begin(), idx.end(), 0u);
  std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  const uint32_t n = std::min(stored, capacity);
  for (uint32_t i = 0; i < n; ++i) {
    const unsigned long long k = keys[idx[i]];
    fdas_candidate &c = out[i];
    c.harmonic = (uint32_t)(k >> 48) + 1;
    c.template_num = (int32_t)((k >> 32) & 0xffffu) - h->H;
    c.bin = (uint32_t)(k & 0xffffffffu);
    c.power = pwrs[idx[i]];
  }
  if (n_total) *n_total = total;
  if (n_dropped) *n_dropped = total - stored;
  return FDAS_OK;
}

fdas_status fdas_retrieve_candidates_ring(fdas_handle *h, uint32_t *detection_location, float *detection_power,
                                          fdas_fop_part which, fdas_buffer_set ab) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!detection_location || !detection_power) return fail(h, FDAS_ERR_INVALID_ARG, "output is NULL");
  if (which != FDAS_NEGATIVE_ACCELERATIONS && which != FDAS_POSITIVE_ACCELERATIONS)
    return fail(h, FDAS_ERR_UNSUPPORTED, "the FPGA candidate ring covers one sign half (FDAS.cpp:447-450)");
  CK(h, cudaSetDevice(h->cfg.device));
  fdas_status st = sync_set(h, ab);
  if (st != FDAS_OK) return st;
  BufferSet &S = h->set[ab];
  unsigned ctrl[kCtrlWords];
  CK(h, cudaMemcpy(ctrl, S.d_ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost));
  const uint32_t stored = std::min(ctrl[kCtrlTotal], (unsigned)h->cap);
  std::vector<unsigned long long> keys(stored);
  std::vector<float> pwrs(stored);
  if (stored) {
    CK(h, cudaMemcpy(keys.data(), S.d_key, sizeof(unsigned long long) * stored, cudaMemcpyDeviceToHost));
    CK(h, cudaMemcpy(pwrs.data(), S.d_pwr, sizeof(float) * stored, cudaMemcpyDeviceToHost));
  }
  // FPGA geometry of the shipped design: groups of 4 templates, bundles of 2
  // bins, 64 slots of 8 lanes per plane (gen_info.h:47-54)
  constexpr int kGroup = 4, kBundle = 2, kSlots = 64, kLanes = 8;
  const uint32_t invalid = (uint32_t)((h->H + 1 + h->H) & 0x7f) << 22;
  const size_t n_out = (size_t)h->P * kSlots * kLanes;
  for (size_t i = 0; i < n_out; ++i) {
    detection_location[i] = invalid;
    detection_power[i] = -1.0f;
  }
  struct Hit {
    unsigned long long ev;  // scan order: group-major, then bundle
    int lane;
    uint32_t loc;
    float pwr;
  };
  std::vector<std::vector<Hit>> per_plane(h->P);
  for (uint32_t i = 0; i < stored; ++i) {
    const int plane = (int)(keys[i] >> 48);
    const int row = (int)((keys[i] >> 32) & 0xffffu);
    const uint32_t bin = (uint32_t)(keys[i] & 0xffffffffu);
    const int t = row - h->H;
    if ((which == FDAS_NEGATIVE_ACCELERATIONS && t > 0) || (which == FDAS_POSITIVE_ACCELERATIONS && t < 0)) continue;
    const int at = t < 0 ? -t : t;
    Hit x;
    x.ev = ((unsigned long long)(at / kGroup) << 32) | (bin / kBundle);
    x.lane = (at % kGroup) * kBundle + (int)(bin % kBundle);
    x.loc = (((unsigned)plane & 7u) << 29) | (((unsigned)row & 0x7fu) << 22) | (bin & 0x3fffffu);
    x.pwr = pwrs[i];
    per_plane[plane].push_back(x);
  }
  for (int pl = 0; pl < h->P; ++pl) {
    auto &v = per_plane[pl];
    std::sort(v.begin(), v.end(), [](const Hit &a, const Hit &b) { return a.ev < b.ev || (a.ev == b.ev && a.lane < b.lane); });
    // events in scan order; the last kSlots survive, slot = event index mod kSlots
    size_t n_ev = 0;
    for (size_t i = 0; i < v.size(); ++i)
      if (i == 0 || v[i].ev != v[i - 1].ev) ++n_ev;
    size_t rank = 0;
    for (size_t i = 0; i < v.size(); ++i) {
      if (i > 0 && v[i].ev != v[i - 1].ev) ++rank;
      if (rank + kSlots < n_ev) continue;
      const size_t o = ((size_t)pl * kSlots + rank % kSlots) * kLanes + v[i].lane;
      detection_location[o] = v[i].loc;
      detection_power[o] = v[i].pwr;
    }
  }
  return FDAS_OK;
}

fdas_status fdas_get_stage_times(fdas_handle *h, fdas_buffer_set ab, float *ms6) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!ms6) return fail(h, FDAS_ERR_INVALID_ARG, "ms6 is NULL");
  BufferSet &S = h->set[ab];
  CK(h, cudaSetDevice(h->cfg.device));
  CK(h, cudaEventSynchronize(S.ev[5]));
  ms6[0] = elapsed(S.ev[0], S.ev[1]);
  ms6[1] = elapsed(S.ev[1], S.ev[2]);
  ms6[2] = elapsed(S.ev[2], S.ev[3]);
  ms6[3] = elapsed(S.ev[3], S.ev[4]);
  ms6[4] = elapsed(S.ev[4], S.ev[5]);
  ms6[5] = elapsed(S.ev[0], S.ev[5]);
  return FDAS_OK;
}

fdas_status fdas_get_counters(fdas_handle *h, fdas_buffer_set ab, uint32_t *out, uint32_t n) {
  CHECK_HANDLE(h);
  CHECK_SET(h, ab);
  if (!out && n) return fail(h, FDAS_ERR_INVALID_ARG, "out is NULL");
  CK(h, cudaSetDevice(h->cfg.device));
  CK(h, cudaStreamSynchronize(h->set[ab].stream));
  unsigned ctrl[kCtrlStride];
  CK(h, cudaMemcpy(ctrl, h->set[ab].d_ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost));
  ctrl[kCtrlStatus] |= ctrl[kCtrlFtcStatus] | ctrl[kCtrlTileStatus];
  for (uint32_t i = 0; i < n && i < (uint32_t)kCtrlSelLo; ++i) out[i] = ctrl[i];
  return FDAS_OK;
}

// time of a completed event on the host's steady clock (ns), through the
// handle's anchor event
static long long event_ns(const fdas_handle *h, cudaEvent_t e) {
  return h->anchor_ns + (long long)llround(1e6 * (double)elapsed(h->anchor, e));
}

void fdas_print_stats(fdas_handle *h, fdas_buffer_set ab, int reset) {
  if (!h || !valid_set(ab)) return;
  BufferSet &S = h->set[ab];
  if (!S.launched || cudaEventSynchronize(S.ev[5]) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  // FDAS.cpp:643-666: the series starts at the input transfer of the launch
  // printed with `reset`; "complete @" is the end of this launch's candidate
  // transfer, "II" the increase since the previous print
  if (reset || !h->pipeline_launches) {
    h->pipeline_start_ns = event_ns(h, S.ev[0]);
    h->pipeline_accum_ns = 0;
    h->pipeline_launches = 1;
  } else {
    ++h->pipeline_launches;
  }
  const long long acc = event_ns(h, S.ev[5]) - h->pipeline_start_ns;
  const char set_c = ab == FDAS_SET_A ? 'A' : 'B';
  logf(h, "[INFO] Launch  #%u%c complete @ %.3f ms II ~ %.3f ms", h->pipeline_launches, set_c, acc * 1e-6,
       (acc - h->pipeline_accum_ns) * 1e-6);
  logf(h, "[INFO]   Preparation duration: %.3f ms", elapsed(S.ev[1], S.ev[2]));
  logf(h, "[INFO]   FT convolution and IFFT duration: %.3f ms", elapsed(S.ev[2], S.ev[3]));
  logf(h, "[INFO]   Harmonic summing duration: %.3f ms", elapsed(S.ev[3], S.ev[4]));
  logf(h, "[INFO]   Total duration: %.3f ms", elapsed(S.ev[0], S.ev[5]));
  h->pipeline_accum_ns = acc;
}

void fdas_print_events(fdas_handle *h, fdas_buffer_set ab) {
  if (!h || !valid_set(ab)) return;
  BufferSet &S = h->set[ab];
  if (!S.launched || cudaEventSynchronize(S.ev[5]) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  // FDAS.cpp:668-686: start and end of the input transfer, tiling, FT
  // convolution, harmonic summing and candidate transfer; each stage starts
  // where the one before it ends on the set's stream
  long long t[6];
  for (int i = 0; i < 6; ++i) t[i] = event_ns(h, S.ev[i]);
  logf(h, "@@@,%c,%lld,%lld,%lld,%lld,%lld,%lld,%lld,%lld,%lld,%lld", ab == FDAS_SET_A ? 'A' : 'B', t[0], t[1], t[1],
       t[2], t[2], t[3], t[3], t[4], t[4], t[5]);
}

fdas_status fdas_set_fault_injection(fdas_handle *h, uint32_t flags) {
  CHECK_HANDLE(h);
  if (flags & ~(uint32_t)(FDAS_INJECT_FTC_STALL | FDAS_INJECT_HSUM_STALL))
    return fail(h, FDAS_ERR_INVALID_ARG, "unknown injection flag");
  h->inject = flags;
  return FDAS_OK;
}

fdas_status fdas_set_wait_timeout(fdas_handle *h, int64_t ns) {
  CHECK_HANDLE(h);
  h->wait_timeout_ns = ns > 0 ? (long long)ns : kWaitNs;
  return FDAS_OK;
}

void fdas_set_log(fdas_handle *h, fdas_log_fn fn, void *user) {
  if (!h) return;
  h->log_fn = fn;
  h->log_user = user;
}

uint32_t fdas_get_input_sz(const fdas_handle *h) { return h ? (uint32_t)h->N : 0; }
uint32_t fdas_get_tiles_sz(const fdas_handle *h) { return h ? (uint32_t)(h->n_tiles * kTile) : 0; }
uint32_t fdas_get_templates_sz(const fdas_handle *h) { return h ? (uint32_t)(h->T * kTile) : 0; }
uint32_t fdas_get_thresholds_sz(const fdas_handle *h) { return h ? (uint32_t)h->P : 0; }
uint32_t fdas_get_fop_sz(const fdas_handle *h) { return h ? (uint32_t)((size_t)h->T * h->N) : 0; }
uint32_t fdas_get_candidate_list_sz(const fdas_handle *h) { return h ? (uint32_t)(h->P * h->per_plane) : 0; }

fdas_status fdas_host_alloc(void **ptr, size_t bytes) {
  if (!ptr) return fail(nullptr, FDAS_ERR_INVALID_ARG, "ptr is NULL");
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaHostAlloc", __FILE__, __LINE__);
  return FDAS_OK;
}
void fdas_host_free(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
}
fdas_status fdas_host_register(void *ptr, size_t bytes) {
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaHostRegister", __FILE__, __LINE__);
  return FDAS_OK;
}
fdas_status fdas_host_unregister(void *ptr) {
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaHostUnregister", __FILE__, __LINE__);
  return FDAS_OK;
}

}  // extern "C"

// ===========================================================================
// Batched search (fdas_batch_*): many trials of uneven length in one pass.
//
// All trials' tiles are transformed by one tiling launch and the (trial, tile,
// template) items by a few persistent FT-convolution launches over consecutive
// groups of trials (the trial of a global tile is found from a table of tile
// ranges), into one FOP arena with each trial's FOP at its own offset.
// Harmonic summing, FP64 recheck and candidate selection run per trial --
// through "views", FDAS handles that borrow the batch's buffers -- on branch
// streams, each group's as soon as its FOPs are written, alongside the next
// group's FT convolution.  The whole sequence
// is captured once into a CUDA graph and replayed; before capture an
// autotuner times the FFT split of the FT convolution (one warp, 64 x 32, or a
// warp pair, 32 x 64), its CTAs per SM, and the harmonic-summing pipeline
// depth on the batch itself and keeps the fastest.
struct fdas_batch {
  fdas_batch_config cfg{};
  fdas_handle *owner = nullptr;  // holds the bank (spectra, FP64 taps) and the twiddle tables
  int n_trials = 0;
  int T = 0, O = 0, payload = 0, P = 0;
  std::vector<BatchTrial> trials;
  long long total_tiles = 0, total_bins = 0;
  size_t fop_floats = 0;
  float2 *d_input = nullptr, *d_tiles = nullptr;
  float *d_fop = nullptr;
  BatchTrial *d_trials = nullptr;
  int *d_status = nullptr, *h_status = nullptr;
  unsigned long long *d_key = nullptr, *d_sel_key = nullptr;
  float *d_pwr = nullptr, *d_sel_pwr = nullptr, *d_cpwr = nullptr;
  unsigned *d_ctrl = nullptr, *h_ctrl = nullptr, *d_hist = nullptr, *d_ticket = nullptr;
  uint4 *d_rc = nullptr;
  uint32_t *d_cloc = nullptr;
  std::vector<fdas_handle *> views;
  cudaStream_t main = nullptr;
  std::vector<cudaStream_t> branch;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> forks;  // end of each group's FT convolution
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t exec = nullptr;
  std::vector<float> graph_thr;
  int ftc_variant = 2, ftc_ctas = 2, hsum_lean = 0;
  int groups = 16;  // FT-convolution launches (1: the whole (trial, tile, template) queue in one)
  bool tuned = false;
  std::vector<float> tune_ms;
  std::string err;
};

namespace {

constexpr int kBatchBranches = 8;  // streams for the per-trial harmonic summing
// The FT convolution runs as this many launches over consecutive groups of
// trials; a group's harmonic summing starts on the branch streams as soon as
// its FOPs are written, while the next group's FT convolution runs.
constexpr int kBatchGroups = 16;
constexpr int kBatchRecheckCap = 8192;

fdas_status bfail(fdas_batch *b, fdas_status st, const std::string &msg) {
  if (b) b->err = msg;
  else g_init_error = msg;
  return st;
}

#define BCK(b, expr)                                                                        \
  do {                                                                                      \
    cudaError_t e_ = (expr);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      char m_[256];                                                                         \
      snprintf(m_, sizeof(m_), "CUDA call failed with %s: %s", cudaGetErrorName(e_), #expr); \
      return bfail((b), e_ == cudaErrorMemoryAllocation ? FDAS_ERR_OUT_OF_MEMORY : FDAS_ERR_CUDA, m_); \
    }                                                                                       \
  } while (0)

void batch_free(fdas_batch *b) {
  if (b->main) cudaStreamSynchronize(b->main);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (auto *v : b->views) {
    for (auto &ev : v->set[0].ev)
      if (ev) cudaEventDestroy(ev);
    delete v;  // borrowed buffers: nothing else to free
  }
  void *dev[] = {b->d_input, b->d_tiles, b->d_fop, b->d_trials, b->d_status, b->d_key, b->d_sel_key, b->d_pwr,
                 b->d_sel_pwr, b->d_cpwr, b->d_ctrl, b->d_hist, b->d_ticket, b->d_rc, b->d_cloc};
  for (void *p : dev) cudaFree(p);
  cudaFreeHost(b->h_ctrl);
  cudaFreeHost(b->h_status);
  for (auto s : b->branch) cudaStreamDestroy(s);
  for (auto e : b->joins) cudaEventDestroy(e);
  for (auto e : b->forks) cudaEventDestroy(e);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  if (b->main) cudaStreamDestroy(b->main);
  if (b->owner) fdas_destroy(b->owner);
  delete b;
}

// Enqueue the whole batched search on b->main (capturable).
fdas_status batch_enqueue(fdas_batch *b, const float *thr) {
  BCK(b, cudaMemsetAsync(b->d_status, 0, sizeof(int), b->main));
  TileParams tp{};
  tp.input = b->d_input;
  tp.n_tiles = (int)b->total_tiles;
  tp.overlap = b->O;
  tp.payload = b->payload;
  tp.tiles = b->d_tiles;
  tp.twiddle = b->owner->d_twiddle;
  tp.trials = b->d_trials;
  tp.n_trials = b->n_trials;
  BCK(b, launch_tile_fft(tp, b->main));
  FtcParams fp{};
  fp.tiles = b->d_tiles;
  fp.tmpl = b->owner->set[0].d_tmpl;
  fp.fop = b->d_fop;
  fp.n_tiles = (int)b->total_tiles;
  fp.overlap = b->O;
  fp.payload = b->payload;
  fp.row_begin = 0;
  fp.n_rows = b->T;
  fp.twiddle = b->owner->d_twiddle;
  fp.status = b->d_status;
  fp.timeout_ns = 2000000000LL;
  fp.ctas_per_sm = b->ftc_ctas;
  fp.variant = b->ftc_variant;
  fp.trials = b->d_trials;
  fp.n_trials = b->n_trials;
  // groups of consecutive trials with about equal numbers of tiles
  int i0 = 0;
  const int n_groups = std::max(1, std::min(b->groups, (int)b->forks.size()));
  for (int g = 0; g < n_groups && i0 < b->n_trials; ++g) {
    const long long target = b->total_tiles * (g + 1) / (long long)n_groups;
    int i1 = i0 + 1;
    while (i1 < b->n_trials && (g + 1 == n_groups || b->trials[i1].tile_begin < target)) ++i1;
    const long long t_lo = b->trials[i0].tile_begin;
    const long long t_hi = i1 < b->n_trials ? b->trials[i1].tile_begin : b->total_tiles;
    FtcParams gp = fp;
    gp.tiles = b->d_tiles + (size_t)t_lo * kTile;
    gp.n_tiles = (int)(t_hi - t_lo);
    gp.tile_begin = t_lo;
    BCK(b, launch_ftc(gp, b->main));
    BCK(b, cudaEventRecord(b->forks[g], b->main));
    for (auto s : b->branch) BCK(b, cudaStreamWaitEvent(s, b->forks[g], 0));
    for (int i = i0; i < i1; ++i) {
      fdas_handle *v = b->views[i];
      v->cfg.overlap = (uint32_t)b->hsum_lean;  // the lean harmonic-summing kernel
      fdas_status st = enqueue_hsum(v, 0, thr, FDAS_ALL_ACCELERATIONS);
      if (st != FDAS_OK) return bfail(b, st, v->err);
    }
    i0 = i1;
  }
  for (size_t k = 0; k < b->branch.size(); ++k) {
    BCK(b, cudaEventRecord(b->joins[k], b->branch[k]));
    BCK(b, cudaStreamWaitEvent(b->main, b->joins[k], 0));
  }
  BCK(b, cudaMemcpyAsync(b->h_status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, b->main));
  return FDAS_OK;
}

fdas_status batch_capture(fdas_batch *b, const float *thr) {
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  cudaGraph_t g = nullptr;
  BCK(b, cudaStreamBeginCapture(b->main, cudaStreamCaptureModeRelaxed));
  fdas_status st = batch_enqueue(b, thr);
  cudaError_t e = cudaStreamEndCapture(b->main, &g);
  if (st != FDAS_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  BCK(b, e);
  e = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  BCK(b, e);
  b->graph_thr.assign(thr, thr + b->P);
  return FDAS_OK;
}

// Time one configuration: two direct runs after a warm-up run.
fdas_status batch_time(fdas_batch *b, const float *thr, float *ms) {
  for (int rep = 0; rep < 3; ++rep) {
    if (rep == 1) BCK(b, cudaEventRecord(b->t0, b->main));
    fdas_status st = batch_enqueue(b, thr);
    if (st != FDAS_OK) return st;
  }
  BCK(b, cudaEventRecord(b->t1, b->main));
  BCK(b, cudaEventSynchronize(b->t1));
  BCK(b, cudaEventElapsedTime(ms, b->t0, b->t1));
  *ms *= 0.5f;
  return FDAS_OK;
}

fdas_status batch_autotune(fdas_batch *b, const float *thr) {
  // FFT split (radix 32 x 64 over a warp pair, or 64 x 32 in one warp),
  // FT-convolution CTAs per SM (templates in flight per SM: 4 per CTA),
  // harmonic-summing depth, and the grouping of the FT convolution: 16
  // launches, 4, or one persistent launch over the whole (trial, tile,
  // template) queue
  struct Cfg {
    int variant, ctas, lean, groups;
  };
  const Cfg cands[] = {{2, 2, 0, 16}, {2, 1, 0, 16}, {1, 1, 0, 16}, {2, 2, 1, 16},
                       {2, 1, 1, 16}, {1, 1, 1, 16}, {2, 2, 0, 4},  {2, 2, 0, 1}};
  float best = 1e30f;
  Cfg pick = cands[0];
  b->tune_ms.clear();
  for (const Cfg &c : cands) {
    b->ftc_variant = c.variant;
    b->ftc_ctas = c.ctas;
    b->hsum_lean = c.lean;
    b->groups = c.groups;
    float ms = 0.f;
    fdas_status st = batch_time(b, thr, &ms);
    if (st != FDAS_OK) return st;
    b->tune_ms.push_back(ms);
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  b->ftc_variant = pick.variant;
  b->ftc_ctas = pick.ctas;
  b->hsum_lean = pick.lean;
  b->groups = pick.groups;
  b->tuned = true;
  return FDAS_OK;
}

}  // namespace

extern "C" {

void fdas_batch_default_config(fdas_batch_config *c) {
  std::memset(c, 0, sizeof(*c));
  c->device = 0;
  c->n_planes = 8;
  c->candidate_capacity = 1u << 18;
  c->candidates_per_plane_compat = 512;
  c->autotune = 1;
  c->recheck = 1;
}

fdas_status fdas_batch_create(const fdas_batch_config *cfg, const fdas_complex *bank, fdas_template_layout layout,
                              uint32_t bank_rows, uint32_t bank_len, uint32_t n_trials, const uint32_t *n_bins,
                              fdas_batch **out) {
  if (!cfg || !bank || !n_bins || !out || n_trials == 0) return bfail(nullptr, FDAS_ERR_INVALID_ARG, "invalid argument");
  if (cfg->n_planes == 0 || cfg->n_planes > (uint32_t)kMaxPlanes)
    return bfail(nullptr, FDAS_ERR_INVALID_ARG, "n_planes must be 1..16");
  for (uint32_t i = 0; i < n_trials; ++i)
    if (n_bins[i] == 0) return bfail(nullptr, FDAS_ERR_INVALID_ARG, "a trial has no bins");
  *out = nullptr;
  fdas_batch *b = new fdas_batch();
  b->cfg = *cfg;
  fdas_config c;
  fdas_default_config(&c, kTile);
  c.device = cfg->device;
  c.n_templates = bank_rows;
  if (layout == FDAS_TEMPLATES_TIME_DOMAIN) c.max_template_len = bank_len;
  c.n_planes = cfg->n_planes;
  c.candidate_capacity = 1024;
  c.recheck = cfg->recheck;
  fdas_status st = fdas_initialise_accelerator(&c, &b->owner);
  if (st != FDAS_OK) {
    delete b;
    return st;
  }
  if ((st = fdas_upload_templates(b->owner, bank, layout, FDAS_SET_A)) != FDAS_OK) {
    g_init_error = b->owner->err;
    batch_free(b);
    return st;
  }
  fdas_handle *o = b->owner;
  b->n_trials = (int)n_trials;
  b->T = o->T;
  b->O = o->O;
  b->payload = o->payload;
  b->P = o->P;
  const int cap = (int)(cfg->candidate_capacity ? cfg->candidate_capacity : (1u << 18));
  const int per_plane = (int)(cfg->candidates_per_plane_compat ? cfg->candidates_per_plane_compat : 512);
  if (per_plane > kMaxCompat) {
    batch_free(b);
    return bfail(nullptr, FDAS_ERR_INVALID_ARG, "candidates_per_plane_compat must be <= 2048");
  }
  // trial table: tile ranges, input and FOP offsets (FOP rows 256-float aligned)
  b->trials.resize(n_trials);
  long long tile = 0, in = 0;
  size_t fop = 0;
  for (uint32_t i = 0; i < n_trials; ++i) {
    BatchTrial &t = b->trials[i];
    t.tile_begin = tile;
    t.input_offset = in;
    t.fop_offset = (long long)fop;
    t.stride = ((long long)n_bins[i] + kHsBins - 1) / kHsBins * kHsBins;
    t.n_bins = (int)n_bins[i];
    t.pad_ = 0;
    tile += ((long long)n_bins[i] + b->payload - 1) / b->payload;
    in += n_bins[i];
    fop += (size_t)b->T * (size_t)t.stride;
  }
  b->total_tiles = tile;
  b->total_bins = in;
  b->fop_floats = fop + 4096;
  if ((long long)b->total_tiles * b->T >= (1ll << 31)) {
    batch_free(b);
    return bfail(nullptr, FDAS_ERR_CAPACITY, "too many (tile, template) items for one batch");
  }
  const size_t n = n_trials;
  const size_t P = (size_t)b->P;
#define BALLOC(ptr, bytes)                                                          \
  if (cudaMalloc((void **)&(ptr), (bytes)) != cudaSuccess) {                         \
    cudaGetLastError();                                                             \
    batch_free(b);                                                                  \
    return bfail(nullptr, FDAS_ERR_OUT_OF_MEMORY, "batch device allocation failed"); \
  }
  BALLOC(b->d_input, sizeof(float2) * (size_t)(b->total_bins + 64));
  BALLOC(b->d_tiles, sizeof(float2) * (size_t)b->total_tiles * kTile);
  BALLOC(b->d_fop, sizeof(float) * b->fop_floats);
  BALLOC(b->d_trials, sizeof(BatchTrial) * n);
  BALLOC(b->d_status, sizeof(int));
  BALLOC(b->d_key, sizeof(unsigned long long) * n * cap);
  BALLOC(b->d_pwr, sizeof(float) * n * cap);
  BALLOC(b->d_ctrl, sizeof(unsigned) * n * kCtrlStride);
  BALLOC(b->d_rc, sizeof(uint4) * n * kBatchRecheckCap);
  BALLOC(b->d_hist, sizeof(unsigned) * n * P * kSelBuckets);
  BALLOC(b->d_ticket, sizeof(unsigned) * n);
  BALLOC(b->d_sel_key, sizeof(unsigned long long) * n * P * 2 * kSortCap);
  BALLOC(b->d_sel_pwr, sizeof(float) * n * P * 2 * kSortCap);
  BALLOC(b->d_cloc, sizeof(uint32_t) * n * P * per_plane);
  BALLOC(b->d_cpwr, sizeof(float) * n * P * per_plane);
#undef BALLOC
  cudaError_t e;
  if ((e = cudaMemcpy(b->d_trials, b->trials.data(), sizeof(BatchTrial) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(b->d_fop, 0, sizeof(float) * b->fop_floats)) != cudaSuccess ||
      (e = cudaMemset(b->d_hist, 0, sizeof(unsigned) * n * P * kSelBuckets)) != cudaSuccess ||
      (e = cudaMemset(b->d_ticket, 0, sizeof(unsigned) * n)) != cudaSuccess ||
      (e = cudaMemset(b->d_ctrl, 0, sizeof(unsigned) * n * kCtrlStride)) != cudaSuccess ||
      (e = cudaHostAlloc((void **)&b->h_ctrl, sizeof(unsigned) * n * kCtrlStride, cudaHostAllocDefault)) != cudaSuccess ||
      (e = cudaHostAlloc((void **)&b->h_status, sizeof(int), cudaHostAllocDefault)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&b->t0)) != cudaSuccess || (e = cudaEventCreate(&b->t1)) != cudaSuccess) {
    batch_free(b);
    return bfail(nullptr, FDAS_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
  }
  *b->h_status = 0;
  for (int g = 0; g < kBatchGroups; ++g) {
    cudaEvent_t ev = nullptr;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      batch_free(b);
      return bfail(nullptr, FDAS_ERR_CUDA, "batch events");
    }
    b->forks.push_back(ev);
  }
  for (int k = 0; k < kBatchBranches; ++k) {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      batch_free(b);
      return bfail(nullptr, FDAS_ERR_CUDA, "batch streams");
    }
    b->branch.push_back(s);
    b->joins.push_back(ev);
  }
  // views: one handle per trial over the batch buffers
  const BufferSet &OS = o->set[0];
  for (uint32_t i = 0; i < n_trials; ++i) {
    const BatchTrial &t = b->trials[i];
    fdas_handle *v = new fdas_handle();
    b->views.push_back(v);
    v->cfg = o->cfg;
    v->cfg.n_frequency_bins = (uint32_t)t.n_bins;
    v->cfg.candidate_capacity = (uint32_t)cap;
    v->cfg.candidates_per_plane_compat = (uint32_t)per_plane;
    v->N = t.n_bins;
    v->T = o->T;
    v->H = o->H;
    v->L = o->L;
    v->O = o->O;
    v->payload = o->payload;
    v->n_tiles = (int)(((long long)t.n_bins + o->payload - 1) / o->payload);
    v->P = o->P;
    v->cap = cap;
    v->per_plane = per_plane;
    v->stride = t.stride;
    v->tap_pitch = o->tap_pitch;
    v->rc_cap = kBatchRecheckCap;
    v->d_twiddle = o->d_twiddle;
    v->d_twiddle64 = o->d_twiddle64;
    v->alloc_N = v->N;
    v->alloc_T = v->T;
    v->alloc_P = v->P;
    v->alloc_tiles = v->n_tiles;
    BufferSet &S = v->set[0];
    S.stream = b->branch[i % kBatchBranches];
    S.d_input = b->d_input + t.input_offset;
    S.cur_input = S.d_input;
    S.d_tiles = b->d_tiles + (size_t)t.tile_begin * kTile;
    S.d_tmpl = OS.d_tmpl;
    S.d_taps = OS.d_taps;
    S.d_taplen = OS.d_taplen;
    S.taplen = OS.taplen;
    S.d_fop = b->d_fop + t.fop_offset;
    S.d_key = b->d_key + (size_t)i * cap;
    S.d_pwr = b->d_pwr + (size_t)i * cap;
    S.d_ctrl = b->d_ctrl + (size_t)i * kCtrlStride;
    S.h_ctrl = b->h_ctrl + (size_t)i * kCtrlStride;
    S.d_rc = b->d_rc + (size_t)i * kBatchRecheckCap;
    S.d_hist = b->d_hist + (size_t)i * P * kSelBuckets;
    S.d_ticket = b->d_ticket + i;
    S.d_sel_key = b->d_sel_key + (size_t)i * P * 2 * kSortCap;
    S.d_sel_pwr = b->d_sel_pwr + (size_t)i * P * 2 * kSortCap;
    S.d_cloc = b->d_cloc + (size_t)i * P * per_plane;
    S.d_cpwr = b->d_cpwr + (size_t)i * P * per_plane;
    S.have_templates = S.have_taps = S.have_input = S.fop_from_input = true;
    for (auto &ev : S.ev)
      if (cudaEventCreate(&ev) != cudaSuccess) {
        batch_free(b);
        return bfail(nullptr, FDAS_ERR_CUDA, "batch events");
      }
    if ((st = make_hsum_maps(v, S)) != FDAS_OK) {
      g_init_error = v->err;
      batch_free(b);
      return st;
    }
  }
  *out = b;
  return FDAS_OK;
}

fdas_status fdas_batch_set_inputs(fdas_batch *b, const fdas_complex *spectra, int on_device) {
  if (!b || !spectra) return bfail(b, FDAS_ERR_INVALID_ARG, "spectra is NULL");
  BCK(b, cudaSetDevice(b->cfg.device));
  BCK(b, cudaMemcpyAsync(b->d_input, spectra, sizeof(float2) * (size_t)b->total_bins,
                         on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->main));
  return FDAS_OK;
}

fdas_complex *fdas_batch_input(fdas_batch *b) { return b ? reinterpret_cast<fdas_complex *>(b->d_input) : nullptr; }

fdas_status fdas_batch_run(fdas_batch *b, const float *thresholds, int wait) {
  if (!b || !thresholds) return bfail(b, FDAS_ERR_INVALID_ARG, "thresholds is NULL");
  BCK(b, cudaSetDevice(b->cfg.device));
  const bool same = b->exec && std::equal(thresholds, thresholds + b->P, b->graph_thr.begin());
  if (!same) {
    if (b->cfg.autotune && !b->tuned) {
      fdas_status st = batch_autotune(b, thresholds);
      if (st != FDAS_OK) return st;
    }
    fdas_status st = batch_capture(b, thresholds);
    if (st != FDAS_OK) return st;
  }
  BCK(b, cudaGraphLaunch(b->exec, b->main));
  for (auto *v : b->views) v->set[0].launched = true;
  if (!wait) return FDAS_OK;
  return fdas_batch_wait(b);
}

fdas_status fdas_batch_wait(fdas_batch *b) {
  if (!b) return bfail(b, FDAS_ERR_INVALID_ARG, "null batch");
  BCK(b, cudaStreamSynchronize(b->main));
  if (*b->h_status & kStatusFtcTimeout) return bfail(b, FDAS_ERR_TIMEOUT, "FT convolution wait timed out");
  for (auto *v : b->views)
    if (v->set[0].h_ctrl[kCtrlStatus] & kStatusHsumTimeout)
      return bfail(b, FDAS_ERR_TIMEOUT, "harmonic summing: shared-memory staging timed out");
  return FDAS_OK;
}

fdas_handle *fdas_batch_trial(fdas_batch *b, uint32_t trial) {
  return (b && trial < (uint32_t)b->n_trials) ? b->views[trial] : nullptr;
}

fdas_status fdas_batch_info(fdas_batch *b, int32_t *out, uint32_t n, float *tune_ms, uint32_t n_ms) {
  if (!b) return FDAS_ERR_INVALID_ARG;
  const int32_t v[7] = {b->ftc_variant, b->ftc_ctas, b->hsum_lean, b->tuned ? 1 : 0, (int32_t)b->total_tiles,
                        (int32_t)b->tune_ms.size(), b->groups};
  for (uint32_t i = 0; out && i < n && i < 7; ++i) out[i] = v[i];
  for (uint32_t i = 0; tune_ms && i < n_ms && i < b->tune_ms.size(); ++i) tune_ms[i] = b->tune_ms[i];
  return FDAS_OK;
}

fdas_status fdas_batch_set_tuning(fdas_batch *b, int32_t ftc_variant, int32_t ftc_ctas_per_sm, int32_t hsum_lean) {
  if (!b || ftc_variant < 1 || ftc_variant > 2 || ftc_ctas_per_sm < 1 || ftc_ctas_per_sm > 2)
    return bfail(b, FDAS_ERR_INVALID_ARG, "invalid tuning");
  b->ftc_variant = ftc_variant;
  b->ftc_ctas = ftc_ctas_per_sm;
  b->hsum_lean = hsum_lean ? 1 : 0;
  b->tuned = true;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return FDAS_OK;
}

fdas_status fdas_batch_set_groups(fdas_batch *b, int32_t groups) {
  if (!b || groups < 1 || groups > kBatchGroups) return bfail(b, FDAS_ERR_INVALID_ARG, "groups must be 1..16");
  b->groups = groups;
  b->tuned = true;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return FDAS_OK;
}

const char *fdas_batch_last_error(const fdas_batch *b) { return b ? b->err.c_str() : g_init_error.c_str(); }

void fdas_batch_destroy(fdas_batch *b) {
  if (!b) return;
  cudaSetDevice(b->cfg.device);
  batch_free(b);
}

}  // extern "C"
