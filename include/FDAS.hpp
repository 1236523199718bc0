// C++ host class with the call sequence and method names of the reference's
// `FDAS` (fdas/src/host/FDAS.h:36-187), implemented over the C ABI of
// fdas_gb300.h.  A caller of the reference class switches by replacing
//   pipeline.initialise_accelerator(bitstream, platform_sel, device_sel, input_sz, mode, sync)
// with
//   pipeline.initialise_accelerator(device_ordinal, input_sz, mode, sync)
// and keeps every other call.  Methods return false and log "[ERROR] ..." on
// failure, like FDAS.cpp:34-52.  Header-only; link with -lfdas_gb300.
#ifndef FDAS_GB300_FDAS_HPP
#define FDAS_GB300_FDAS_HPP

#include <cstdint>
#include <ostream>
#include <string>

#include "fdas_gb300.h"

namespace fdas_gb300 {

class FDAS {
 public:
  enum FOPPart { NegativeAccelerations = FDAS_NEGATIVE_ACCELERATIONS,
                 PositiveAccelerations = FDAS_POSITIVE_ACCELERATIONS,
                 AllAccelerations = FDAS_ALL_ACCELERATIONS };
  enum BufferSet { A = FDAS_SET_A, B = FDAS_SET_B };
  enum BufferMode { PerSet = FDAS_MODE_PER_SET, PerStage = FDAS_MODE_PER_STAGE, Crossed = FDAS_MODE_CROSSED };

  explicit FDAS(std::ostream &log) : log(log) {}
  ~FDAS() { fdas_destroy(h); }
  FDAS(const FDAS &) = delete;
  FDAS &operator=(const FDAS &) = delete;

  // FDAS.h:44-49.  The bitstream / OpenCL selectors become a CUDA device ordinal;
  // `cfg` (optional) overrides the reference's generated constants.
  bool initialise_accelerator(int device, uint32_t input_sz, BufferMode mode = PerSet, bool sync_pipeline = false,
                              const fdas_config *cfg = nullptr) {
    fdas_config c;
    if (cfg) c = *cfg;
    else fdas_default_config(&c, input_sz);
    c.n_frequency_bins = input_sz;
    c.device = device;
    c.buffer_mode = (uint32_t)mode;
    c.sync_pipeline = sync_pipeline ? 1u : 0u;
    c.log_fn = &FDAS::forward_log;  // from the "^^^" line of initialisation on
    c.log_user = this;
    fdas_destroy(h);
    h = nullptr;
    fdas_status st = fdas_initialise_accelerator(&c, &h);
    if (st != FDAS_OK) return report(st, "initialise_accelerator");
    return true;
  }

  // FDAS.h:51 -- spectra in the reference's p4 FFT order (..._ft_p4.npy)
  bool upload_templates(const fdas_complex *templates, BufferSet ab) {
    return upload_templates(templates, FDAS_TEMPLATES_FFT_P4, ab);
  }
  bool upload_templates(const fdas_complex *templates, fdas_template_layout layout, BufferSet ab) {
    return check(fdas_upload_templates(h, templates, layout, (fdas_buffer_set)ab), "upload_templates");
  }
  bool upload_thresholds(const float *thresholds, BufferSet ab) {
    return check(fdas_upload_thresholds(h, thresholds, (fdas_buffer_set)ab), "upload_thresholds");
  }
  bool perform_input_tiling(const fdas_complex *input, BufferSet ab) {
    return check(fdas_perform_input_tiling(h, input, (fdas_buffer_set)ab), "perform_input_tiling");
  }
  bool perform_ft_convolution(FOPPart which, BufferSet ab) {
    return check(fdas_perform_ft_convolution(h, (fdas_fop_part)which, (fdas_buffer_set)ab), "perform_ft_convolution");
  }
  bool perform_harmonic_summing(const float *thresholds, FOPPart which, BufferSet ab) {
    return check(fdas_perform_harmonic_summing(h, thresholds, (fdas_fop_part)which, (fdas_buffer_set)ab),
                 "perform_harmonic_summing");
  }
  bool launch(const fdas_complex *input, const float *thresholds, uint32_t *detection_location,
              float *detection_power, FOPPart which, BufferSet ab) {
    return check(fdas_launch(h, input, thresholds, detection_location, detection_power, (fdas_fop_part)which,
                             (fdas_buffer_set)ab),
                 "launch");
  }
  bool wait(BufferSet ab) { return check(fdas_wait(h, (fdas_buffer_set)ab), "wait"); }
  bool end_pipeline(BufferSet ab) { return check(fdas_end_pipeline(h, (fdas_buffer_set)ab), "end_pipeline"); }
  bool retrieve_tiles(fdas_complex *tiles, BufferSet ab) {
    return check(fdas_retrieve_tiles(h, tiles, (fdas_buffer_set)ab), "retrieve_tiles");
  }
  bool retrieve_FOP(float *fop, BufferSet ab) { return check(fdas_retrieve_fop(h, fop, (fdas_buffer_set)ab), "retrieve_FOP"); }
  bool inject_FOP(const float *fop, BufferSet ab) {
    return check(fdas_inject_fop(h, fop, (fdas_buffer_set)ab), "inject_FOP");
  }
  bool retrieve_candidates(uint32_t *detection_location, float *detection_power, BufferSet ab) {
    return check(fdas_retrieve_candidates(h, detection_location, detection_power, (fdas_buffer_set)ab),
                 "retrieve_candidates");
  }
  void print_stats(BufferSet ab, bool reset = false) { fdas_print_stats(h, (fdas_buffer_set)ab, reset ? 1 : 0); }
  void print_events(BufferSet ab) { fdas_print_events(h, (fdas_buffer_set)ab); }

  uint32_t get_input_sz() const { return fdas_get_input_sz(h); }
  uint32_t get_tiles_sz() const { return fdas_get_tiles_sz(h); }
  uint32_t get_templates_sz() const { return fdas_get_templates_sz(h); }
  uint32_t get_thresholds_sz() const { return fdas_get_thresholds_sz(h); }
  uint32_t get_fop_sz() const { return fdas_get_fop_sz(h); }
  uint32_t get_candidate_list_sz() const { return fdas_get_candidate_list_sz(h); }

  fdas_handle *handle() { return h; }

 private:
  bool check(fdas_status st, const char *what) { return st == FDAS_OK ? true : report(st, what); }
  bool report(fdas_status st, const char *what) {
    log << "[ERROR] " << what << " failed with status " << (int)st << ": " << fdas_last_error(h) << std::endl;
    return false;
  }
  static void forward_log(const char *line, void *self) { static_cast<FDAS *>(self)->log << line << std::endl; }

  fdas_handle *h = nullptr;
  std::ostream &log;
};

}  // namespace fdas_gb300

#endif  // FDAS_GB300_FDAS_HPP
