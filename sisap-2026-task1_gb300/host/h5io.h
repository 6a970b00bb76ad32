// h5io.h -- dataset I/O of the knng_main CLI.
//
// The reference reads /train with the HDF5 C++ API and writes knns, dists and
// five root attributes (src/main.cpp:149-177, 459-480).  The CLI reads HDF5
// files (through the file-format reader in hdf5.h, no libhdf5 needed) and the
// knng container format (magic "KNNGH5S1"; layout documented in
// sisap-2026-task1_gb300/h5container.py), told apart by their signatures, and
// writes its result in either: HDF5 by default, as the reference does.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace knngio {

struct Matrix {
  std::vector<float> data;  // row-major
  int64_t rows = 0;
  int64_t cols = 0;
};

// Reads dataset `name` (leading '/' optional) of an HDF5 or container file as
// float32; other integer and floating-point types are converted.  Throws
// std::runtime_error on failure.
Matrix read_matrix(const std::string& path, const std::string& name);

struct Output {
  const int32_t* knns;
  const float* dists;
  int64_t rows;
  int64_t cols;
  std::string algo, task, params;
  float buildtime, querytime;
};

enum class Format { kHdf5, kContainer };

struct Result {
  std::vector<int32_t> knns;
  std::vector<float> dists;
  int64_t rows = 0;
  int64_t cols = 0;
  std::string algo, task, params;
  float buildtime = 0.0f, querytime = 0.0f;
};

// Reads a result file (knns, dists and the five attributes) of either format.
// Throws std::runtime_error on failure.
Result read_result(const std::string& path);

// Writes knns (i32), dists (f32) and the attributes algo, task, params
// (strings; variable-length in HDF5, as src/main.cpp:101-106 writes them),
// buildtime and querytime (f32).  Throws std::runtime_error on failure.
void write_result(const std::string& path, const Output& out, Format format = Format::kHdf5);

}  // namespace knngio
