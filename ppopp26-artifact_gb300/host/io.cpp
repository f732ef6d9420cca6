// io.cpp -- element files and Montgomery conversions over libppfr.so.
#include "io.h"

#include <cstdio>
#include <fstream>
#include <iostream>
#include <stdexcept>

#include "pp_ops.h"

void read_file(const char *filename, void *data) {
  std::ifstream file(filename, std::ios::binary | std::ios::ate);
  if (!file) {
    std::cerr << "Error opening file: " << filename << std::endl;
    return;
  }
  const std::streamsize bytes = file.tellg();
  file.seekg(0, std::ios::beg);
  if (!file.read(static_cast<char *>(data), bytes))
    std::cerr << "Error reading file: " << filename << std::endl;
}

void read_file_exact(const char *filename, void *data, size_t bytes) {
  std::ifstream file(filename, std::ios::binary);
  if (!file) throw std::runtime_error(std::string("Error opening file: ") + filename);
  if (!file.read(static_cast<char *>(data), (std::streamsize)bytes))
    throw std::runtime_error(std::string("Error reading file: ") + filename);
}

void writeToFile(const std::string &filename, uint64_t *array, uint64_t size) {
  std::ofstream out(filename);
  if (!out) {
    std::cerr << "Error opening file for writing: " << filename << std::endl;
    return;
  }
  for (uint64_t i = 0; i < size; ++i) out << array[i] << '\n';
  if (!out) std::cerr << "Error writing to file: " << filename << std::endl;
}

static SyncedMemory convert(SyncedMemory &input, cudaStream_t stream, bool to_mont_form,
                            const char *what) {
  if (input.size() % 32) throw pp::Error(PP_E_INVAL, std::string(what) + ": size is not a multiple of 32 bytes");
  SyncedMemory out(input.size());
  const uint64_t n = input.size() / 32;
  if (n == 0) return out;
  const void *in = input.mutable_gpu_data_async(stream);
  void *o = out.mutable_gpu_data_async(stream);
  pp::check(to_mont_form ? pp_to_mont(in, o, n, stream) : pp_to_base(in, o, n, stream), what);
  return out;
}

SyncedMemory to_mont(SyncedMemory input) { return convert(input, (cudaStream_t)0, true, "to_mont"); }

SyncedMemory to_base(SyncedMemory input, cudaStream_t stream) {
  return convert(input, stream, false, "to_base");
}
