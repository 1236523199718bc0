/*
 * fdas_gb300 -- C ABI of the GB300-native FDAS hot path.
 *
 * Each entry point replaces one method of the reference's host class
 * `FDAS` (fdas/src/host/FDAS.h:36-187 in UOA-PARC-SKA/FDAS) and keeps its call
 * sequence: template upload, threshold upload, input tiling, FT convolution,
 * harmonic summing, candidate retrieval, with `launch` / `wait` enqueueing the
 * whole pipeline asynchronously on one of two buffer sets (A/B).
 *
 * Differences from the reference, by design:
 *  - errors are returned as `fdas_status` (never abort); a message is kept per
 *    handle and returned by `fdas_last_error` (the reference logs and returns
 *    `false`, FDAS.cpp:34-52);
 *  - sizes (bins, templates, overlap, planes, candidate capacity) are runtime
 *    configuration instead of the generated constants of gen_info.h;
 *  - `FDAS_ALL_ACCELERATIONS` is supported by harmonic summing (the reference's
 *    systolic detector rejects it, FDAS.cpp:447-450); template 0 is then
 *    reported once;
 *  - the candidate list is deterministic: every hit is kept (up to a
 *    capacity), the 4096-entry reference-format list holds per plane the
 *    strongest `candidates_per_plane_compat` hits in location order.
 *
 * A handle is single-threaded: calls on one handle must not run concurrently.
 * Several handles may share a device.
 */
#ifndef FDAS_GB300_H
#define FDAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fdas_handle fdas_handle;

/* A complex single-precision value, layout-compatible with cl_float2 and
 * std::complex<float>. */
typedef struct {
  float re;
  float im;
} fdas_complex;

typedef enum {
  FDAS_OK = 0,
  FDAS_ERR_INVALID_ARG = 1,
  FDAS_ERR_OUT_OF_MEMORY = 2,
  FDAS_ERR_CUDA = 3,
  FDAS_ERR_TIMEOUT = 4,
  FDAS_ERR_UNSUPPORTED = 5,
  FDAS_ERR_CAPACITY = 6,
  FDAS_ERR_STATE = 7,
  FDAS_ERR_NO_DEVICE = 8
} fdas_status;

/* FDAS::FOPPart (FDAS.h:38) */
typedef enum {
  FDAS_NEGATIVE_ACCELERATIONS = 0,
  FDAS_POSITIVE_ACCELERATIONS = 1,
  FDAS_ALL_ACCELERATIONS = 2
} fdas_fop_part;

/* FDAS::BufferSet (FDAS.h:39) */
typedef enum { FDAS_SET_A = 0, FDAS_SET_B = 1 } fdas_buffer_set;

/* FDAS::BufferMode (FDAS.h:40).  DDR bank placement on the FPGA board; on a
 * GB300 all buffers live in the same HBM, so the modes are accepted and only
 * recorded. */
typedef enum { FDAS_MODE_PER_SET = 0, FDAS_MODE_PER_STAGE = 1, FDAS_MODE_CROSSED = 2 } fdas_buffer_mode;

/* Layout of the array given to fdas_upload_templates. */
typedef enum {
  /* n_templates x 2048 spectra in the reference's "FFT order" with 4 parallel
   * inputs (fdas_templates_85_350_ft_p4.npy, tmpl-gen.py:145-153) */
  FDAS_TEMPLATES_FFT_P4 = 0,
  /* n_templates x 2048 spectra in natural bin order */
  FDAS_TEMPLATES_FFT_NATURAL = 1,
  /* n_templates x max_template_len time-domain taps, left aligned and zero
   * padded (fdas_templates_85_350.npy); spectra are computed on the device in
   * FP64 and the taps are kept for the FP64 recheck */
  FDAS_TEMPLATES_TIME_DOMAIN = 2
} fdas_template_layout;

/* A log sink: receives one line at a time, without the newline.  The
 * reference writes these lines to the std::ostream given to its constructor
 * (FDAS.h:42). */
typedef void (*fdas_log_fn)(const char *line, void *user);

typedef struct {
  uint32_t n_frequency_bins;   /* N, the input size (FDAS::initialise_accelerator input_sz) */
  uint32_t n_templates;        /* odd; 85 in the reference (gen_info.h:27) */
  uint32_t max_template_len;   /* 421 in the reference (gen_info.h:28) */
  uint32_t tile_overlap;       /* 0 = ceil((max_template_len - 1) / 4) * 4 (cl_codegen.py:99) */
  uint32_t n_planes;           /* harmonic planes, 1..16 (8 in the reference) */
  uint32_t candidate_capacity; /* hit records kept per buffer set; 0 = 2^22 (max 2^27) */
  uint32_t candidates_per_plane_compat; /* entries per plane in the fixed list; 0 = 512 */
  int32_t device;              /* CUDA device ordinal */
  uint32_t buffer_mode;        /* fdas_buffer_mode */
  uint32_t sync_pipeline;      /* FDAS::initialise_accelerator sync_pipeline */
  uint32_t recheck;            /* 1 = FP64-grade recheck of near-threshold cells (default) */
  float recheck_band;          /* relative band around each threshold; 0 = 1e-4 */
  uint32_t overlap;            /* 1 = size the kernels so that the FT convolution of one
                                  buffer set and the harmonic summing of the other run
                                  concurrently on every SM (for pipelined A/B searches) */
  uint32_t precision;          /* the forward DFT of the tiles and the inverse DFT of the
                                  FT convolution: 0 = FP32 FFTs on the CUDA cores
                                  (default); 1 / 2 = DFT-64 x DFT-32 factor products on
                                  the tensor cores (tcgen05) with split (hi + lo) BF16 /
                                  FP16 operands, FP32 accumulation */
  uint32_t trace_enqueue;      /* 1 = fdas_launch logs the reference's per-launch host trace:
                                  "[INFO] Enqueueing: A" with the enqueue times of its
                                  stages in ms, and "%%%,A,t0,t1,t2,t3,t4," with the
                                  steady-clock times (ns) around them (FDAS.cpp:556-575).
                                  0 (default) = off: at a thousand launches per second the
                                  log sink would become part of the launch cost */
  fdas_log_fn log_fn;          /* log sink from initialisation on (NULL = stderr): the
                                  "^^^" clock-sync line and the "[INFO] Device ..." line
                                  of fdas_initialise_accelerator go here, like every later
                                  line of the handle (fdas_set_log changes it) */
  void *log_user;              /* passed to log_fn */
  int32_t stream_priority;     /* CUDA priority of the buffer sets' streams: 0 (default) the
                                  default priority, negative values higher ones (the range is
                                  cudaDeviceGetStreamPriorityRange's; CUDA clamps others) */
} fdas_config;

/* Fill `cfg` with the reference's defaults for `n_frequency_bins` bins. */
void fdas_default_config(fdas_config *cfg, uint32_t n_frequency_bins);

/* FDAS::FDAS + FDAS::initialise_accelerator (FDAS.h:42-49, FDAS.cpp:54-261).
 * Allocates both buffer sets on `cfg->device`.  On failure *out is NULL and the
 * message is available from fdas_last_error(NULL).  Logs first, like
 * FDAS.cpp:60-63, the line "^^^,<system clock>,<steady clock>" (both in ns
 * since their epochs) that lets a log reader map the steady-clock times of
 * "%%%" and "@@@" lines onto wall-clock time. */
fdas_status fdas_initialise_accelerator(const fdas_config *cfg, fdas_handle **out);

/* Releases all device resources of the handle. */
void fdas_destroy(fdas_handle *h);

/* Last error message of `h` (or of the last failed initialisation if h is NULL). */
const char *fdas_last_error(const fdas_handle *h);

/* Re-size an idle handle within the sizes it was initialised with (no
 * counterpart in the reference; lets one handle serve searches of different
 * lengths and banks without reallocating): N' <= N bins, the template rows
 * [template_row_begin, template_row_begin + n_templates) of the uploaded bank
 * (an odd count; 21 + 43 rows of the 85-row bank is the z = -21..+21 half
 * bank), n_planes' <= n_planes, and tile_overlap (0 = from the longest
 * template of the range).  Template spectra stay on the device; uploaded
 * thresholds, inputs and FOP contents are dropped.  FDAS_ERR_CAPACITY if the
 * tiles or the FOP of the new shape do not fit. */
fdas_status fdas_reshape(fdas_handle *h, uint32_t n_frequency_bins, uint32_t template_row_begin,
                         uint32_t n_templates, uint32_t tile_overlap, uint32_t n_planes);

/* FDAS::upload_templates (FDAS.h:51, FDAS.cpp:263-269).  `templates` is a host
 * array of n_templates x 2048 complex values (FFT layouts) or n_templates x
 * max_template_len taps (FDAS_TEMPLATES_TIME_DOMAIN).  Blocking. */
fdas_status fdas_upload_templates(fdas_handle *h, const fdas_complex *templates, fdas_template_layout layout,
                                  fdas_buffer_set ab);

/* FDAS::upload_thresholds (FDAS.h:53, FDAS.cpp:271-280): n_planes floats,
 * used when fdas_perform_harmonic_summing / fdas_launch get thresholds == NULL. */
fdas_status fdas_upload_thresholds(fdas_handle *h, const float *thresholds, fdas_buffer_set ab);

/* FDAS::perform_input_tiling (FDAS.h:55, FDAS.cpp:319-328): copy the N-bin
 * spectrum to the device, build the overlap-save tiles and transform them.
 * `input` NULL: use the spectrum fdas_series_to_spectrum made on this set.
 * Blocking. */
fdas_status fdas_perform_input_tiling(fdas_handle *h, const fdas_complex *input, fdas_buffer_set ab);

/* FDAS::perform_ft_convolution (FDAS.h:57, FDAS.cpp:396-405): template
 * multiply + inverse FFT + |.|^2 + overlap discard into the FOP rows of `which`.
 * Blocking. */
fdas_status fdas_perform_ft_convolution(fdas_handle *h, fdas_fop_part which, fdas_buffer_set ab);

/* FDAS::perform_harmonic_summing (FDAS.h:59, FDAS.cpp:533-546).  Blocking. */
fdas_status fdas_perform_harmonic_summing(fdas_handle *h, const float *thresholds, fdas_fop_part which,
                                          fdas_buffer_set ab);

/* FDAS::launch (FDAS.h:61, FDAS.cpp:548-583): enqueue tiling, FT convolution,
 * harmonic summing and the candidate download into the caller's
 * `detection_location` / `detection_power` (get_candidate_list_sz() entries
 * each).  `input` NULL: search the spectrum fdas_series_to_spectrum made on
 * this set.  Returns without waiting; use fdas_wait. */
fdas_status fdas_launch(fdas_handle *h, const fdas_complex *input, const float *thresholds,
                        uint32_t *detection_location, float *detection_power, fdas_fop_part which,
                        fdas_buffer_set ab);

/* FDAS::wait (FDAS.h:63, FDAS.cpp:585-588): block until the last launch on
 * `ab` has delivered its candidates.  Returns FDAS_ERR_STATE if that launch's
 * harmonic summing is still held back by sync_pipeline (the reference would
 * block forever there). */
fdas_status fdas_wait(fdas_handle *h, fdas_buffer_set ab);

/* FDAS::end_pipeline (FDAS.h:65, FDAS.cpp:590-594): release the held-back
 * stage of the other set (sync_pipeline mode). */
fdas_status fdas_end_pipeline(fdas_handle *h, fdas_buffer_set ab);

/* FDAS::retrieve_tiles (FDAS.h:67, FDAS.cpp:596-599): n_tiles x 2048 tile
 * spectra in the reference's p4 FFT order.  Blocking. */
fdas_status fdas_retrieve_tiles(fdas_handle *h, fdas_complex *tiles, fdas_buffer_set ab);

/* FDAS::retrieve_FOP (FDAS.h:69, FDAS.cpp:601-604): n_templates x N floats,
 * row = template number + n_templates/2.  Blocking. */
fdas_status fdas_retrieve_fop(fdas_handle *h, float *fop, fdas_buffer_set ab);

/* FDAS::inject_FOP (FDAS.h:71, FDAS.cpp:628-632): replace the FOP of `ab`
 * (the stage seam for harmonic-summing-only tests).  Harmonic summing of an
 * injected FOP runs without the FP64 recheck, in plain FP32 like hsum.py. */
fdas_status fdas_inject_fop(fdas_handle *h, const float *fop, fdas_buffer_set ab);

/* FDAS::retrieve_candidates (FDAS.h:73, FDAS.cpp:619-626): the fixed-size
 * list (get_candidate_list_sz() entries) of the last harmonic summing on `ab`:
 * plane h occupies entries [h*P, (h+1)*P), P = candidates_per_plane_compat;
 * unused entries hold location encode(1, 43, 0) and power -1.  Blocking. */
fdas_status fdas_retrieve_candidates(fdas_handle *h, uint32_t *detection_location, float *detection_power,
                                     fdas_buffer_set ab);

/* Full candidate record (wide form; no 8-plane / 127-template / 2^22-bin limit). */
typedef struct {
  uint32_t harmonic;    /* 1..n_planes */
  int32_t template_num; /* -n_templates/2 .. n_templates/2 */
  uint32_t bin;         /* frequency bin */
  float power;          /* harmonic-plane power HP_harmonic(template, bin) */
} fdas_candidate;

/* Every hit of the last harmonic summing on `ab`, sorted by (harmonic,
 * template, bin) -- the order of hsum.py's list.  Writes min(total, capacity)
 * records; *n_total gets the number of hits found, *n_dropped the hits lost to
 * the device capacity (candidate_capacity records per set).  Blocking. */
fdas_status fdas_retrieve_candidate_list(fdas_handle *h, fdas_candidate *out, uint32_t capacity,
                                         uint32_t *n_total, uint32_t *n_dropped, fdas_buffer_set ab);

/* The reference FPGA's own candidate list for one sign half (which =
 * FDAS_NEGATIVE_ACCELERATIONS or FDAS_POSITIVE_ACCELERATIONS), reproduced from
 * the hits of the last harmonic summing on `ab`: per plane a 64-slot ring of
 * 8-lane events, scanned in template groups of 4 and bin bundles of 2, where
 * later events overwrite older ones (detect.cl.mako:32-216, store_cands.cl.mako:
 * 21-33).  n_planes x 64 x 8 entries, [plane][slot][lane]; empty entries hold
 * location encode(1, 43, 0) and power -1.  For side-by-side comparison with
 * FPGA logs.  Blocking. */
fdas_status fdas_retrieve_candidates_ring(fdas_handle *h, uint32_t *detection_location, float *detection_power,
                                          fdas_fop_part which, fdas_buffer_set ab);

/* FDAS::print_stats (FDAS.h:75, FDAS.cpp:643-666): after the last launch on
 * `ab` has completed, logs
 *   "[INFO] Launch  #<n><A|B> complete @ <X> ms II ~ <Y> ms"
 * where X is the time from the start of the input transfer of the launch
 * printed with reset != 0 (the start of the series) to the end of this
 * launch's candidate transfer, and Y the increase of X since the previous
 * print_stats, then the durations of preparation (tiling), FT convolution,
 * harmonic summing and the total, one "[INFO]   <phase> duration: <ms> ms"
 * line each.  The reference prints whole milliseconds; these lines carry three
 * decimals (a search here takes well under a millisecond). */
void fdas_print_stats(fdas_handle *h, fdas_buffer_set ab, int reset);
/* FDAS::print_events (FDAS.h:77, FDAS.cpp:668-686): logs
 *   "@@@,<A|B>,<input xfer start>,<input xfer end>,<tiling start>,<tiling end>,
 *    <FT convolution start>,<FT convolution end>,<harmonic summing start>,
 *    <harmonic summing end>,<candidate xfer start>,<candidate xfer end>"
 * for the last launch on `ab`: ten times in ns on the host's steady clock (the
 * reference gives OpenCL profiling times in ns).  The GPU's events are placed
 * on that clock through an event recorded and waited for at initialisation;
 * their spacing is exact to the event resolution (about 0.5 us), their offset
 * to within the few microseconds of that wait. */
void fdas_print_events(fdas_handle *h, fdas_buffer_set ab);

/* Redirect the handle's log lines ("[INFO] ...", "@@@,...") to a callback. */
void fdas_set_log(fdas_handle *h, fdas_log_fn fn, void *user);

/* Bound on every wait inside the kernels (a TMA copy or a tensor-core
 * product that has not landed), after which the search stops, its status
 * word gets the timeout bit and fdas_wait / fdas_synchronize return
 * FDAS_ERR_TIMEOUT.  ns <= 0 restores the default of 2 s.  A kernel that
 * times out still waits, bounded by 2 s, for its own copies in flight before
 * it exits, so a short bound only turns slow searches into reported errors:
 * the handle stays usable (no counterpart in the reference, whose OpenCL
 * waits have no bound). */
fdas_status fdas_set_wait_timeout(fdas_handle *h, int64_t ns);

/* Test hooks for the timeout paths (no counterpart in the reference).  With
 * FDAS_INJECT_FTC_STALL set, the FT convolution of later searches announces
 * each warp pair's first template copy on its barrier but never issues it, so
 * that wait cannot complete and runs out after the bound of
 * fdas_set_wait_timeout: the search stops with the FT-convolution timeout bit
 * and fdas_wait returns FDAS_ERR_TIMEOUT.  FDAS_INJECT_HSUM_STALL does the
 * same to the first staged item of every harmonic-summing CTA (status bit 1).
 * No memory access is made or left in flight by the hooks; 0 switches them
 * off. */
#define FDAS_INJECT_FTC_STALL 1u
#define FDAS_INJECT_HSUM_STALL 2u
fdas_status fdas_set_fault_injection(fdas_handle *h, uint32_t flags);

/* Stage times of the last completed launch on `ab`, in milliseconds:
 * [0] input copy, [1] tiling, [2] FT convolution, [3] harmonic summing,
 * [4] candidate download, [5] total. */
fdas_status fdas_get_stage_times(fdas_handle *h, fdas_buffer_set ab, float *ms6);

/* FDAS::get_*_sz (FDAS.h:79-89, FDAS.cpp:688-711) -- element counts. */
uint32_t fdas_get_input_sz(const fdas_handle *h);
uint32_t fdas_get_tiles_sz(const fdas_handle *h);
uint32_t fdas_get_templates_sz(const fdas_handle *h);
uint32_t fdas_get_thresholds_sz(const fdas_handle *h);
uint32_t fdas_get_fop_sz(const fdas_handle *h);
uint32_t fdas_get_candidate_list_sz(const fdas_handle *h);

/* Pinned host memory for the copy-in / copy-out buffers (replaces
 * AlignedBuffer, fdas/src/host/AlignedBuffer.h:26-52). */
fdas_status fdas_host_alloc(void **ptr, size_t bytes);
void fdas_host_free(void *ptr);
fdas_status fdas_host_register(void *ptr, size_t bytes);
fdas_status fdas_host_unregister(void *ptr);

/* Upstream step (ft_conv.py:134-143; no method of the reference's FDAS class):
 * the spectrum X[k] = scale * sum_n x[n] e^(-2 pi i n k / 2N), k < N, of the
 * first 2N samples of a real float32 series, N = n_frequency_bins.  The
 * reference's test-data script uses scale = 1 / (2N) (`fft(samples) / n_samp`)
 * and needs n_samples >= 2N (ft_conv.py:125-132).  `samples` is host memory,
 * or device memory when samples_on_device != 0.  The spectrum is left in the
 * set's input buffer -- fdas_perform_input_tiling / fdas_launch with input NULL
 * search it -- and, when `spectrum` is not NULL, copied to that host array of N
 * values.  N must factor into 2, 3, 5 and 7 (else FDAS_ERR_UNSUPPORTED).
 * Blocking. */
fdas_status fdas_series_to_spectrum(fdas_handle *h, const float *samples, uint64_t n_samples, int samples_on_device,
                                    float scale, fdas_complex *spectrum, fdas_buffer_set ab);

/* ------------------------------------------------------------------------
 * Device-resident entry points (no counterpart in the reference).  They let a
 * caller whose spectrum already sits in device memory run the same pipeline
 * without the host copy: `d_input` is a device pointer to N complex values.
 * The work is enqueued on the set's stream; candidates stay on the device
 * until fdas_retrieve_candidates / fdas_retrieve_candidate_list.
 * ---------------------------------------------------------------------- */
fdas_status fdas_enqueue_search_device(fdas_handle *h, const fdas_complex *d_input, const float *thresholds,
                                       fdas_fop_part which, fdas_buffer_set ab);
/* Block until all work enqueued on `ab` is done. */
fdas_status fdas_synchronize(fdas_handle *h, fdas_buffer_set ab);
/* The CUDA stream (cudaStream_t) of buffer set `ab`. */
void *fdas_get_stream(fdas_handle *h, fdas_buffer_set ab);

/* Device counters of the last search on `ab` (blocking), up to `n` words:
 * [0] status bits (1 staging timeout, 2 recheck list full, 4 candidate list
 * full, 8 selection buffer full, 16 FT-convolution timeout), [1] cells sent
 * to the FP64 recheck, [2] candidate records appended, [3 + p] hits of plane
 * p, [19 + p] hits of plane p certain to enter its fixed-size list (p < 16). */
fdas_status fdas_get_counters(fdas_handle *h, fdas_buffer_set ab, uint32_t *out, uint32_t n);

/* ------------------------------------------------------------------------
 * FT convolution that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory when they search: a pipeline
 * whose device memory all belongs to its own pool allocator with a fixed
 * budget, a real-time search that must not hit an out-of-memory error in the
 * middle of an observation, or code where cudaMalloc / cudaFree would
 * synchronise the device and stall the caller's other streams.  It does the
 * work of fdas_perform_input_tiling + fdas_perform_ft_convolution (same
 * kernels, same FOP values) on a spectrum and into a FOP that the caller holds
 * in device memory.  The tile spectra, the scaled template spectra and the
 * twiddle table live in a static device scratch array of the library (about
 * 8 MB, present while the library is loaded); no device or host memory is
 * allocated, by this call or by anything it calls.
 *
 *  d_spectrum  n_bins complex bins, device memory, 8-byte aligned
 *  d_templates n_templates x 2048 template spectra, device memory, in the
 *              p4 order of fdas_templates_85_350_ft_p4.npy (FFT_P4) or in
 *              natural order (FFT_NATURAL); TIME_DOMAIN is UNSUPPORTED here
 *  tile_overlap overlap-save overlap O (420 for the 421-tap bank); tiles of
 *              2048 bins advance by 2048 - O.  The caller must give at least
 *              the longest template's tap count minus 1: this call receives
 *              spectra, not taps, so it cannot check it, and a shorter overlap
 *              wraps the convolution around the tile (wrong FOP values,
 *              FDAS_OK); the handle path refuses such an overlap
 *  which       FOP rows computed (the other part's rows are left untouched)
 *  d_fop       n_templates x fop_stride floats, device memory, row = template
 *              + n_templates / 2; fop_stride >= n_bins
 *  d_status    NULL, or a device int32 that the caller has set to zero: a
 *              kernel wait that timed out (2 s) ORs 16 into it and leaves the
 *              FOP incomplete.  NULL means no timeout report at all: the call
 *              has returned FDAS_OK when the work is enqueued, and a timed-out
 *              wait then leaves an incomplete FOP that nothing flags
 *  stream      cudaStream_t (NULL: the default stream); the call only enqueues
 *
 * Limits: ceil(n_bins / (2048 - O)) <= FDAS_NOALLOC_MAX_TILES (2^19 bins and
 * more at O = 420) and n_templates <= FDAS_NOALLOC_MAX_TEMPLATES; larger sizes
 * return FDAS_ERR_CAPACITY before any work is enqueued.  Failures are reported
 * by the status only (no message is stored: storing one would allocate).
 *
 * The first call on a device, with that device current, is set-up: it looks
 * up the scratch address (cudaGetSymbolAddress) and copies the twiddle table
 * into it with a blocking copy.  With CUDA's default lazy module loading
 * (CUDA_MODULE_LOADING=LAZY) that first call may also be what loads the
 * library's device code onto the device, and loading allocates device memory
 * for the code and for the scratch array itself.  So make the first call on
 * each device at initialisation -- before the observation starts and before
 * any stream capture -- or set CUDA_MODULE_LOADING=EAGER so that the module
 * loads when the CUDA context is created; every later call allocates nothing
 * and does not block.  All calls
 * on one device share the one scratch area: two calls whose work overlaps on
 * the device (different streams with no ordering between them, or several
 * host threads) race and corrupt each other's FOP.  Order them on one stream.
 * ---------------------------------------------------------------------- */
#define FDAS_NOALLOC_MAX_TILES 384u
#define FDAS_NOALLOC_MAX_TEMPLATES 128u
fdas_status fdas_ft_convolution_noalloc(const fdas_complex *d_spectrum, uint32_t n_bins,
                                        const fdas_complex *d_templates, fdas_template_layout layout,
                                        uint32_t n_templates, uint32_t tile_overlap, fdas_fop_part which,
                                        float *d_fop, uint64_t fop_stride, int32_t *d_status, void *stream);

/* ------------------------------------------------------------------------
 * Request server (no counterpart in the reference; the served form of the
 * search).  One dispatcher thread runs queued requests on a pool of slots --
 * FDAS handles of power-of-two length classes with the template bank resident
 * on the device, reshaped per request -- each on its own stream, so requests
 * overlap on the device.  A request is admitted when a free slot of its class
 * exists or a new slot's device bytes (mostly its FOPs: 4 x templates x bins
 * per buffer set) fit the HBM budget; idle slots are released to make room.
 * A request's result does not depend on the other requests in flight.
 * ---------------------------------------------------------------------- */
typedef struct fdas_server fdas_server;
typedef struct {
  int32_t device;
  uint32_t max_bins;           /* longest request (2^21) */
  uint32_t min_class_bins;     /* smallest slot length class (2^15) */
  uint32_t max_planes;         /* planes a request may ask for, <= 16 */
  uint32_t max_slots;          /* searches in flight at most */
  uint64_t hbm_budget_bytes;   /* device bytes for slots; 0 = 90% of free HBM at creation */
  uint32_t candidate_capacity; /* hit records per slot (2^20) */
} fdas_server_config;

void fdas_server_default_config(fdas_server_config *cfg);
/* `bank`: bank_rows templates in `layout` (bank_len taps per row for
 * FDAS_TEMPLATES_TIME_DOMAIN, 2048 spectrum values otherwise). */
fdas_status fdas_server_create(const fdas_server_config *cfg, const fdas_complex *bank, fdas_template_layout layout,
                               uint32_t bank_rows, uint32_t bank_len, fdas_server **out);
/* Queue one search: n_bins spectrum values (host or device memory; copied
 * into the server's device memory before the call returns, so the caller may
 * reuse its buffer), the bank rows [template_row_begin, template_row_begin +
 * n_templates) (odd count), n_planes thresholds.  Returns with the request's
 * id; the search runs asynchronously. */
fdas_status fdas_server_submit(fdas_server *s, const fdas_complex *spectrum, uint32_t n_bins,
                               uint32_t template_row_begin, uint32_t n_templates, uint32_t n_planes,
                               const float *thresholds, uint64_t *request_id);
/* Wait up to timeout_ms (< 0: no limit; FDAS_ERR_TIMEOUT when it runs out)
 * for a request and collect its result: up to `capacity` wide candidate
 * records in the order of fdas_retrieve_candidate_list, the hit count, the
 * hits lost to the slot's capacity, and the submit-to-result latency.  A
 * collected request is forgotten, except when out is NULL and capacity 0
 * (counts only, to size the output).  Returns the request's own status. */
fdas_status fdas_server_wait(fdas_server *s, uint64_t request_id, int32_t timeout_ms, fdas_candidate *out,
                             uint32_t capacity, uint32_t *n_total, uint32_t *n_dropped, double *latency_ms);
/* [0] completed, [1] queued, [2] in flight, [3] slots, [4] slot device bytes,
 * [5] most requests in flight at once */
fdas_status fdas_server_stats(fdas_server *s, uint64_t *out, uint32_t n);
/* Message of the last failed request collected by fdas_server_wait. */
const char *fdas_server_last_error(fdas_server *s);
/* Stops the dispatcher (requests still queued are dropped) and frees the slots. */
void fdas_server_destroy(fdas_server *s);

/* ------------------------------------------------------------------------
 * Batched search (no counterpart in the reference; the batched form).  Many
 * trials (dedispersed spectra) of uneven length searched in one pass: one
 * tiling launch and persistent FT-convolution launches over the (trial, tile,
 * template) items of consecutive groups of trials, each group's harmonic
 * summing, FP64 recheck and candidate selection per trial on parallel branch
 * streams while the next group's FT convolution runs; the sequence is
 * captured once into a CUDA graph and replayed.  Before the capture an
 * autotuner (cfg->autotune) times the FT convolution's FFT split (one warp,
 * 64 x 32, or a warp pair, 32 x 64), its CTAs per SM and the harmonic-summing
 * pipeline depth on the batch itself and keeps the fastest.  Every trial gets
 * the candidates a plain search of it would give.
 * ---------------------------------------------------------------------- */
typedef struct fdas_batch fdas_batch;
typedef struct {
  int32_t device;
  uint32_t n_planes;                    /* 1..16 */
  uint32_t candidate_capacity;          /* hit records per trial (2^18) */
  uint32_t candidates_per_plane_compat; /* fixed-size list entries per plane (512) */
  uint32_t autotune;                    /* 1 = tune before the first capture */
  uint32_t recheck;                     /* 1 = FP64 recheck of near-threshold cells */
} fdas_batch_config;

void fdas_batch_default_config(fdas_batch_config *cfg);
/* Allocates for n_trials trials of n_bins[i] bins; the bank as for
 * fdas_upload_templates (bank_len taps per row for the time-domain layout). */
fdas_status fdas_batch_create(const fdas_batch_config *cfg, const fdas_complex *bank, fdas_template_layout layout,
                              uint32_t bank_rows, uint32_t bank_len, uint32_t n_trials, const uint32_t *n_bins,
                              fdas_batch **out);
/* The trials' spectra, concatenated (sum of n_bins values), from host or
 * device memory; enqueued before the next run. */
fdas_status fdas_batch_set_inputs(fdas_batch *b, const fdas_complex *spectra, int on_device);
/* Device address of the concatenated input spectra (for producers on the GPU). */
fdas_complex *fdas_batch_input(fdas_batch *b);
/* Search every trial with the n_planes thresholds (captures the graph on the
 * first call and when the thresholds change; autotunes before the first
 * capture).  wait != 0 blocks until done. */
fdas_status fdas_batch_run(fdas_batch *b, const float *thresholds, int wait);
fdas_status fdas_batch_wait(fdas_batch *b);
/* A handle viewing trial `trial` after a run: use it with
 * fdas_retrieve_candidate_list, fdas_retrieve_candidates, fdas_retrieve_fop
 * and fdas_get_counters (buffer set A).  Owned by the batch. */
fdas_handle *fdas_batch_trial(fdas_batch *b, uint32_t trial);
/* out: [0] FFT split (1 one warp, 2 warp pair), [1] FT-convolution CTAs per SM,
 * [2] lean harmonic summing, [3] tuned, [4] tiles of the batch, [5] configs
 * timed, [6] FT-convolution launches the trials are grouped into (1: one
 * persistent launch over the whole (trial, tile, template) queue); tune_ms:
 * the autotuner's time per configuration. */
fdas_status fdas_batch_info(fdas_batch *b, int32_t *out, uint32_t n, float *tune_ms, uint32_t n_ms);
/* Fix the tuning by hand (skips the autotuner; the graph is recaptured). */
fdas_status fdas_batch_set_tuning(fdas_batch *b, int32_t ftc_variant, int32_t ftc_ctas_per_sm, int32_t hsum_lean);
/* Fix the grouping by hand: the trials are split into `groups` (1..16) runs of
 * about equal tile counts, one FT-convolution launch each, whose harmonic
 * summing starts while the next run's FT convolution runs (1: one persistent
 * launch over the whole queue).  Skips the autotuner, like
 * fdas_batch_set_tuning; the graph is recaptured.  Results do not depend on
 * the grouping. */
fdas_status fdas_batch_set_groups(fdas_batch *b, int32_t groups);
const char *fdas_batch_last_error(const fdas_batch *b);
void fdas_batch_destroy(fdas_batch *b);

/* Library version string. */
const char *fdas_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FDAS_GB300_H */
