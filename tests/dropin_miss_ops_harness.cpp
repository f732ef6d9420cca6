// dropin_miss_ops_harness.cpp -- linked with the reference's own miss_ops.cu
// (unmodified; compiled against ppopp26-artifact_gb300/host/ref_include with
// its main renamed) and this library's libppcompat.so / libppfr.so.  Every
// call below is resolved by this library except naive_gp / naive_div and one(),
// which are the reference's own code (miss_ops.cu:27-87) running on this
// library's cpu::BLS12_381_Fr_G1 and SyncedMemory.
//
//   dropin_miss_ops <lgN> <in.bin> <x.bin> <c.bin> <out-prefix>
// writes <prefix>.naive_gp, .naive_div (N-1 elements), .gp, .eval (1 element),
// .div, each raw 32-byte Montgomery elements.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "PLONK/utils/function.cuh"
#include "caffe/interface.hpp"

SyncedMemory naive_gp(int lg_N, SyncedMemory input);
SyncedMemory naive_div(int lg_N, SyncedMemory input, SyncedMemory divisor);
SyncedMemory one();

static SyncedMemory load(const char *path, size_t n) {
  SyncedMemory m(n * 32);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(m.mutable_cpu_data(), 32, n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return m;
}

static void save(const std::string &path, SyncedMemory m, size_t n) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(m.mutable_cpu_data(), 32, n, f) != n) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s lgN in x c out-prefix\n", argv[0]);
    return 2;
  }
  const int lg = std::atoi(argv[1]);
  const size_t n = size_t{1} << lg;
  const std::string out = argv[5];
  SyncedMemory x = load(argv[3], 1), c = load(argv[4], 1);

  SyncedMemory in = load(argv[2], n);
  save(out + ".naive_gp", naive_gp(lg, in), n);
  SyncedMemory divisor(64);  // [c, 1] = X + c, as miss_ops.cu:160-165 builds it
  std::memcpy(divisor.mutable_cpu_data(), c.mutable_cpu_data(), 32);
  std::memcpy(static_cast<char *>(divisor.mutable_cpu_data()) + 32, one().mutable_cpu_data(), 32);
  save(out + ".naive_div", naive_div(lg, in, divisor), n - 1);

  SyncedMemory g = load(argv[2], n);
  g.mutable_gpu_data();
  save(out + ".gp", accumulate_mul_poly(g), n);
  SyncedMemory e = load(argv[2], n);
  save(out + ".eval", evaluate(e, x), 1);
  SyncedMemory d = load(argv[2], n);
  save(out + ".div", poly_div_poly(d, c), n);
  std::printf("dropin ok\n");
  return 0;
}
