// io.h -- the reference's element-file helpers and Montgomery conversions,
// same names and behaviour:
//
//   miss_ops.cu:8-24         read_file(filename, data): the whole file into data;
//                            prints an error and returns if it cannot be read
//   lde.cu:222-231           read_file_exact(filename, data, bytes): throws
//                            std::runtime_error on a missing or short file
//   PLONK/utils/function.cu:414-430  writeToFile(filename, array, size): the
//                            64-bit words as decimal text, one per line
//   PLONK/utils/function.cu:5-21     to_mont(input), to_base(input, stream):
//                            new buffers, converted on the GPU
//
// Element files are raw 32-byte little-endian Montgomery elements.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include "syncedmem.h"

void read_file(const char *filename, void *data);
void read_file_exact(const char *filename, void *data, size_t bytes);
void writeToFile(const std::string &filename, uint64_t *array, uint64_t size);

SyncedMemory to_mont(SyncedMemory input);
SyncedMemory to_base(SyncedMemory input, cudaStream_t stream = (cudaStream_t)0);
