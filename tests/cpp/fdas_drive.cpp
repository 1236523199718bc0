// C++ driver over include/FDAS.hpp mirroring the reference's gtest driver
// (fdas/src/host/main_gtest.cpp): FT_Convolution, Harmonic_Summing (injected
// FOP), FDAS_steps, drive_serially and drive_pipelined, with the same checks
// (tiles and FOP |d| < 1e-5, candidates a subset of the reference list with
// |d power| < 1e-5).
//
// Usage: fdas_drive <vector-dir> [n_runs]
// <vector-dir> holds raw little-endian files written by the pytest wrapper:
//   input.bin (complex64 x N), templates_p4.bin (complex64 x 85 x 2048),
//   thresholds.bin (float32 x 8), tiles_ref.bin (complex64 p4 tiles),
//   fop_ref.bin (float32 x 85 x N), det_loc_ref.bin (uint32), det_pwr_ref.bin
//   (float32).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "FDAS.hpp"

using fdas_gb300::FDAS;

static const float tolerance = 1e-5f;  // main_gtest.cpp:56
static int failures = 0;

#define EXPECT(cond)                                                        \
  do {                                                                      \
    if (!(cond)) {                                                          \
      std::cerr << "FAILED: " #cond " [" << __FILE__ << ":" << __LINE__ << "]\n"; \
      ++failures;                                                           \
      return;                                                               \
    }                                                                       \
  } while (0)

template <typename T>
static std::vector<T> load(const std::string &path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) {
    std::cerr << "cannot read " << path << "\n";
    return {};
  }
  size_t n = (size_t)f.tellg() / sizeof(T);
  f.seekg(0);
  std::vector<T> v(n);
  f.read(reinterpret_cast<char *>(v.data()), n * sizeof(T));
  return v;
}

struct Vectors {
  std::vector<fdas_complex> input, templates, tiles_ref;
  std::vector<float> thresholds, fop_ref, det_pwr_ref;
  std::vector<uint32_t> det_loc_ref;
};

static const uint32_t invalid_location = (uint32_t)((42 + 1 + 42) & 0x7f) << 22;  // gen_info.h:69

static void validate_harmonic_summing(std::vector<uint32_t> loc, std::vector<float> pwr, const Vectors &v) {
  std::vector<uint32_t> l;
  std::vector<float> p;
  for (size_t i = 0; i < loc.size(); ++i)
    if (loc[i] != invalid_location) l.push_back(loc[i]), p.push_back(pwr[i]);
  EXPECT(l.size() <= v.det_loc_ref.size());
  EXPECT(l.size() >= 1);
  int non_cands = 0;
  for (size_t i = 0; i < l.size(); ++i) {
    auto it = std::find(v.det_loc_ref.begin(), v.det_loc_ref.end(), l[i]);
    if (it == v.det_loc_ref.end()) {
      ++non_cands;
      continue;
    }
    float ref = v.det_pwr_ref[it - v.det_loc_ref.begin()];
    EXPECT(std::fabs(p[i] - ref) < tolerance * 8);
  }
  EXPECT(non_cands == 0);
}

static void test_ft_convolution(const Vectors &v) {
  FDAS pipeline(std::cerr);
  EXPECT(pipeline.initialise_accelerator(0, (uint32_t)v.input.size()));
  EXPECT(pipeline.upload_templates(v.templates.data(), FDAS::A));
  EXPECT(pipeline.perform_input_tiling(v.input.data(), FDAS::A));
  EXPECT(pipeline.perform_ft_convolution(FDAS::AllAccelerations, FDAS::A));
  std::vector<fdas_complex> tiles(pipeline.get_tiles_sz());
  EXPECT(pipeline.retrieve_tiles(tiles.data(), FDAS::A));
  EXPECT(tiles.size() == v.tiles_ref.size());
  for (size_t i = 0; i < tiles.size(); ++i)
    EXPECT(std::fabs(tiles[i].re - v.tiles_ref[i].re) < tolerance &&
           std::fabs(tiles[i].im - v.tiles_ref[i].im) < tolerance);
  std::vector<float> fop(pipeline.get_fop_sz());
  EXPECT(pipeline.retrieve_FOP(fop.data(), FDAS::A));
  EXPECT(fop.size() == v.fop_ref.size());
  for (size_t i = 0; i < fop.size(); ++i) EXPECT(std::fabs(fop[i] - v.fop_ref[i]) < tolerance);
  std::cout << "[ OK ] FT_Convolution\n";
}

static void test_harmonic_summing(const Vectors &v) {
  FDAS pipeline(std::cerr);
  EXPECT(pipeline.initialise_accelerator(0, (uint32_t)v.input.size()));
  EXPECT(pipeline.inject_FOP(v.fop_ref.data(), FDAS::A));
  EXPECT(pipeline.perform_harmonic_summing(v.thresholds.data(), FDAS::NegativeAccelerations, FDAS::A));
  std::vector<uint32_t> loc(pipeline.get_candidate_list_sz());
  std::vector<float> pwr(pipeline.get_candidate_list_sz());
  EXPECT(pipeline.retrieve_candidates(loc.data(), pwr.data(), FDAS::A));
  validate_harmonic_summing(loc, pwr, v);
  std::cout << "[ OK ] Harmonic_Summing\n";
}

static void test_steps(const Vectors &v) {
  FDAS pipeline(std::cerr);
  EXPECT(pipeline.initialise_accelerator(0, (uint32_t)v.input.size()));
  EXPECT(pipeline.upload_templates(v.templates.data(), FDAS::B));
  EXPECT(pipeline.upload_thresholds(v.thresholds.data(), FDAS::B));
  EXPECT(pipeline.perform_input_tiling(v.input.data(), FDAS::B));
  EXPECT(pipeline.perform_ft_convolution(FDAS::PositiveAccelerations, FDAS::B));
  EXPECT(pipeline.perform_harmonic_summing(v.thresholds.data(), FDAS::PositiveAccelerations, FDAS::B));
  std::vector<uint32_t> loc(pipeline.get_candidate_list_sz());
  std::vector<float> pwr(pipeline.get_candidate_list_sz());
  EXPECT(pipeline.retrieve_candidates(loc.data(), pwr.data(), FDAS::B));
  validate_harmonic_summing(loc, pwr, v);
  std::cout << "[ OK ] FDAS_steps\n";
}

static void drive_serially(const Vectors &v, FDAS::BufferMode mode, int n_runs) {
  FDAS pipeline(std::cerr);
  EXPECT(pipeline.initialise_accelerator(0, (uint32_t)v.input.size(), mode));
  EXPECT(pipeline.upload_templates(v.templates.data(), FDAS::A));
  std::vector<uint32_t> loc(pipeline.get_candidate_list_sz());
  std::vector<float> pwr(pipeline.get_candidate_list_sz());
  for (int i = 0; i < n_runs; ++i) {
    FDAS::FOPPart which = (i & 1) == 0 ? FDAS::PositiveAccelerations : FDAS::NegativeAccelerations;
    EXPECT(pipeline.launch(v.input.data(), v.thresholds.data(), loc.data(), pwr.data(), which, FDAS::A));
    EXPECT(pipeline.wait(FDAS::A));
    pipeline.print_stats(FDAS::A, i == 0);
    pipeline.print_events(FDAS::A);
  }
  validate_harmonic_summing(loc, pwr, v);
  std::cout << "[ OK ] FDAS_serial mode " << (int)mode << "\n";
}

static void drive_pipelined(const Vectors &v, FDAS::BufferMode mode, int n_runs) {
  FDAS pipeline(std::cerr);
  EXPECT(pipeline.initialise_accelerator(0, (uint32_t)v.input.size(), mode, true));
  EXPECT(pipeline.upload_templates(v.templates.data(), FDAS::A));
  EXPECT(pipeline.upload_templates(v.templates.data(), FDAS::B));
  std::vector<uint32_t> loc[2] = {std::vector<uint32_t>(pipeline.get_candidate_list_sz()),
                                  std::vector<uint32_t>(pipeline.get_candidate_list_sz())};
  std::vector<float> pwr[2] = {std::vector<float>(pipeline.get_candidate_list_sz()),
                               std::vector<float>(pipeline.get_candidate_list_sz())};
  FDAS::FOPPart which[2] = {FDAS::PositiveAccelerations, FDAS::NegativeAccelerations};
  for (int i = 0; i < n_runs + 1; ++i) {
    FDAS::BufferSet ab = (i & 1) == 0 ? FDAS::A : FDAS::B;
    FDAS::BufferSet prev = (i & 1) == 0 ? FDAS::B : FDAS::A;
    if (i < n_runs)
      EXPECT(pipeline.launch(v.input.data(), v.thresholds.data(), loc[ab].data(), pwr[ab].data(), which[ab], ab));
    else
      EXPECT(pipeline.end_pipeline(ab));
    if (i > 0) {
      EXPECT(pipeline.wait(prev));
      pipeline.print_stats(prev, i - 1 == 0);
      pipeline.print_events(prev);
    }
  }
  validate_harmonic_summing(loc[0], pwr[0], v);
  validate_harmonic_summing(loc[1], pwr[1], v);
  std::cout << "[ OK ] FDAS_pipelined mode " << (int)mode << "\n";
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::cerr << "usage: fdas_drive <vector-dir> [n_runs]\n";
    return 2;
  }
  std::string d = argv[1];
  int n_runs = argc > 2 ? std::stoi(argv[2]) : 10;
  Vectors v;
  v.input = load<fdas_complex>(d + "/input.bin");
  v.templates = load<fdas_complex>(d + "/templates_p4.bin");
  v.thresholds = load<float>(d + "/thresholds.bin");
  v.tiles_ref = load<fdas_complex>(d + "/tiles_ref.bin");
  v.fop_ref = load<float>(d + "/fop_ref.bin");
  v.det_loc_ref = load<uint32_t>(d + "/det_loc_ref.bin");
  v.det_pwr_ref = load<float>(d + "/det_pwr_ref.bin");
  if (v.input.empty() || v.templates.size() != 85u * 2048u || v.thresholds.size() != 8) {
    std::cerr << "bad test vectors in " << d << "\n";
    return 2;
  }
  test_ft_convolution(v);
  test_harmonic_summing(v);
  test_steps(v);
  for (auto mode : {FDAS::PerSet, FDAS::PerStage}) drive_serially(v, mode, n_runs);
  for (auto mode : {FDAS::PerSet, FDAS::PerStage, FDAS::Crossed}) drive_pipelined(v, mode, n_runs);
  std::cout << (failures ? "FAILED" : "PASSED") << " (" << failures << " failures)\n";
  return failures ? 1 : 0;
}
