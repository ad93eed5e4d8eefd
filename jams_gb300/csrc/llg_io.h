// Host-side array files (HDF5 ".h5" or whitespace-separated text); see
// llg_io.cu for the formats.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace llgio {

struct Dataset {
  std::string name;      // dataset name in the root group (no '/')
  const double* data;    // rows x cols, row-major
  int64_t rows, cols;
};

// ".h5": one HDF5 file holding every dataset; otherwise one array as text
int write_array(const std::string& path, const std::vector<Dataset>& sets, std::string& err);
// ".h5": the named dataset (rows, cols from its dataspace; cols = 1 for a
// one-dimensional one); otherwise every number of the text file (rows =
// count, cols = 1)
int read_array(const std::string& path, const char* dataset, std::vector<double>& out, int64_t& rows,
               int64_t& cols, std::string& err);
// dataset path without leading '/'
std::string dataset_name(const char* name);

}  // namespace llgio
