// h5io.h -- dataset I/O of the knng_main CLI.
//
// The reference reads /train with the HDF5 C++ API and writes knns, dists and
// five root attributes (src/main.cpp:149-177, 459-480).  This image has no
// libhdf5, so the CLI reads and writes the knng container format (magic
// "KNNGH5S1"; layout documented in sisap-2026-task1_gb300/h5container.py),
// which carries the same dataset names, types, shapes and attributes.
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

// Reads dataset `name` (leading '/' optional) as float32; f16/i32/i8 are
// converted.  Throws std::runtime_error on failure.
Matrix read_matrix(const std::string& path, const std::string& name);

struct Output {
  const int32_t* knns;
  const float* dists;
  int64_t rows;
  int64_t cols;
  std::string algo, task, params;
  float buildtime, querytime;
};

// Writes knns (i32), dists (f32) and the attributes algo, task, buildtime,
// querytime, params.  Throws std::runtime_error on failure.
void write_result(const std::string& path, const Output& out);

}  // namespace knngio
