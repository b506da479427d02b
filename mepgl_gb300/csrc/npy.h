// npy.h -- minimal reader / writer of NumPy .npy files (format 1.0 / 2.0).
//
// Replaces the reference's vendored cnpy for its only use, the input_data /
// output_data directories (mepgl/src/io.cu).  Unlike cnpy's data<T>() (a
// bare reinterpret_cast, cnpy.h:36-44), the reader checks the dtype and
// converts float32 / float64 / int32 / int64 / bool to the requested type.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace npy {

struct Array {
    std::vector<size_t> shape;
    std::string descr;            // e.g. "<f8"
    bool fortran = false;
    std::vector<char> bytes;
    size_t count() const;
};

// Read a file; throws std::runtime_error with the path on any problem.
Array read(const std::string &path);

// Values of a numeric array as doubles / int32 (C order as stored).
std::vector<double> as_double(const Array &a);
std::vector<int32_t> as_int32(const Array &a);

// Write a C-order array of doubles, floats or int32.
void write(const std::string &path, const double *data, const std::vector<size_t> &shape);
void write(const std::string &path, const float *data, const std::vector<size_t> &shape);
void write(const std::string &path, const int32_t *data, const std::vector<size_t> &shape);

}  // namespace npy
