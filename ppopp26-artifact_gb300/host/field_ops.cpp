// field_ops.cpp -- the reference's element-wise field operators and buffer
// helpers (PLONK/utils/function.cu:23-280, zk_function.cu:3-21) over
// libppfr.so's pp_fr_* entry points.
#include <cstring>
#include <string>

#include "function.h"
#include "pp_ops.h"

namespace {

constexpr size_t kFr = 32;

size_t count(SyncedMemory &m, const char *what) {
  if (m.size() % kFr) throw pp::Error(PP_E_INVAL, std::string(what) + ": size is not a multiple of 32 bytes");
  return m.size() / kFr;
}

void need_scalar(SyncedMemory &s, const char *what) {
  if (s.size() < kFr) throw pp::Error(PP_E_INVAL, std::string(what) + ": scalar buffer holds no element");
}

// c = a op b (element-wise) into a new buffer or into a (in_place)
SyncedMemory binary(uint32_t op, SyncedMemory a, SyncedMemory b, cudaStream_t s, bool scalar,
                    bool in_place, const char *what) {
  const size_t n = count(a, what);
  if (scalar) need_scalar(b, what);
  else if (count(b, what) != n) throw pp::Error(PP_E_INVAL, std::string(what) + ": operand sizes differ");
  SyncedMemory c = in_place ? a : SyncedMemory(a.size());
  if (n == 0) return c;
  const void *da = a.mutable_gpu_data_async(s), *db = b.mutable_gpu_data_async(s);
  void *dc = in_place ? const_cast<void *>(da) : c.mutable_gpu_data_async(s);
  pp::check(pp_fr_binary(op, da, db, dc, n, scalar ? 1 : 0, s), what);
  return c;
}

SyncedMemory unary(uint32_t op, SyncedMemory a, const char *what) {
  const size_t n = count(a, what);
  SyncedMemory c(a.size());
  if (n == 0) return c;
  pp::check(pp_fr_unary(op, a.mutable_gpu_data(), c.mutable_gpu_data(), n, nullptr), what);
  return c;
}

}  // namespace

SyncedMemory neg_mod(SyncedMemory input) { return unary(PP_FR_NEG, input, "neg_mod"); }
SyncedMemory inv_mod(SyncedMemory input) { return unary(PP_FR_INV, input, "inv_mod"); }

SyncedMemory add_mod(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_ADD, a, b, s, false, false, "add_mod");
}
void add_mod_(SyncedMemory a, SyncedMemory b, cudaStream_t s) { binary(PP_FR_ADD, a, b, s, false, true, "add_mod_"); }
SyncedMemory sub_mod(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_SUB, a, b, s, false, false, "sub_mod");
}
void sub_mod_(SyncedMemory a, SyncedMemory b, cudaStream_t s) { binary(PP_FR_SUB, a, b, s, false, true, "sub_mod_"); }
SyncedMemory mul_mod(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_MUL, a, b, s, false, false, "mul_mod");
}
void mul_mod_(SyncedMemory a, SyncedMemory b, cudaStream_t s) { binary(PP_FR_MUL, a, b, s, false, true, "mul_mod_"); }
SyncedMemory div_mod(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_DIV, a, b, s, false, false, "div_mod");
}
void div_mod_(SyncedMemory a, SyncedMemory b, cudaStream_t s) { binary(PP_FR_DIV, a, b, s, false, true, "div_mod_"); }

SyncedMemory add_mod_scalar(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_ADD, a, b, s, true, false, "add_mod_scalar");
}
void add_mod_scalar_(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  binary(PP_FR_ADD, a, b, s, true, true, "add_mod_scalar_");
}
SyncedMemory sub_mod_scalar(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_SUB, a, b, s, true, false, "sub_mod_scalar");
}
void sub_mod_scalar_(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  binary(PP_FR_SUB, a, b, s, true, true, "sub_mod_scalar_");
}
SyncedMemory mul_mod_scalar(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_MUL, a, b, s, true, false, "mul_mod_scalar");
}
void mul_mod_scalar_(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  binary(PP_FR_MUL, a, b, s, true, true, "mul_mod_scalar_");
}
SyncedMemory div_mod_scalar(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  return binary(PP_FR_DIV, a, b, s, true, false, "div_mod_scalar");
}
void div_mod_scalar_(SyncedMemory a, SyncedMemory b, cudaStream_t s) {
  binary(PP_FR_DIV, a, b, s, true, true, "div_mod_scalar_");
}

SyncedMemory exp_mod(SyncedMemory input, int exp) {
  if (exp < 0) throw pp::Error(PP_E_INVAL, "exp_mod: negative exponent");
  const size_t n = count(input, "exp_mod");
  SyncedMemory c(input.size());
  if (n == 0) return c;
  pp::check(pp_fr_pow(input.mutable_gpu_data(), c.mutable_gpu_data(), n, (uint64_t)exp, nullptr), "exp_mod");
  return c;
}

void gen_sequence_(uint64_t N, SyncedMemory x, SyncedMemory y, cudaStream_t s) {
  need_scalar(x, "gen_sequence");
  if (y.size() < N * kFr) throw pp::Error(PP_E_INVAL, "gen_sequence_: output shorter than N elements");
  if (N == 0) return;
  pp::check(pp_fr_powers(x.mutable_gpu_data_async(s), y.mutable_gpu_data_async(s), N, s), "gen_sequence");
}

SyncedMemory gen_sequence(uint64_t N, SyncedMemory x, cudaStream_t s) {
  SyncedMemory y(N * kFr);
  gen_sequence_(N, x, y, s);
  return y;
}

void repeat_to_poly_(SyncedMemory x, SyncedMemory y, uint64_t N, cudaStream_t s) {
  need_scalar(x, "repeat_to_poly");
  if (y.size() < N * kFr) throw pp::Error(PP_E_INVAL, "repeat_to_poly_: output shorter than N elements");
  if (N == 0) return;
  pp::check(pp_fr_fill(x.mutable_gpu_data_async(s), y.mutable_gpu_data_async(s), N, s), "repeat_to_poly");
}

SyncedMemory repeat_to_poly(SyncedMemory x, uint64_t N, cudaStream_t s) {
  SyncedMemory y(N * kFr);
  repeat_to_poly_(x, y, N, s);
  return y;
}

void pad_poly_(SyncedMemory x, SyncedMemory out, uint64_t N, cudaStream_t s) {
  if (x.size() > N * kFr || out.size() < N * kFr)
    throw pp::Error(PP_E_INVAL, "pad_poly: input longer than N elements or output shorter");
  void *o = out.mutable_gpu_data_async(s);
  pp::check_cuda(cudaMemsetAsync(o, 0, N * kFr, s), "pad_poly");
  if (x.size())
    pp::check_cuda(cudaMemcpyAsync(o, x.mutable_gpu_data_async(s), x.size(), cudaMemcpyDeviceToDevice, s),
                   "pad_poly");
}

SyncedMemory pad_poly(SyncedMemory x, uint64_t N, cudaStream_t s) {
  SyncedMemory out(N * kFr);
  pad_poly_(x, out, N, s);
  return out;
}

SyncedMemory repeat_zero(uint64_t N) {
  SyncedMemory out(N * kFr);
  if (N) std::memset(out.mutable_cpu_data(), 0, out.size());
  return out;
}

SyncedMemory cat(SyncedMemory a, SyncedMemory b) {
  SyncedMemory res(a.size() + b.size());
  if (a.head() == SyncedMemory::HEAD_AT_CPU) {
    char *r = static_cast<char *>(res.mutable_cpu_data());
    if (a.size()) std::memcpy(r, a.mutable_cpu_data(), a.size());
    if (b.size()) std::memcpy(r + a.size(), b.mutable_cpu_data(), b.size());
  } else {
    char *r = static_cast<char *>(res.mutable_gpu_data());
    if (a.size()) pp::check_cuda(cudaMemcpy(r, a.mutable_gpu_data(), a.size(), cudaMemcpyDeviceToDevice), "cat");
    if (b.size())
      pp::check_cuda(cudaMemcpy(r + a.size(), b.mutable_gpu_data(), b.size(), cudaMemcpyDeviceToDevice), "cat");
  }
  return res;
}

SyncedMemory slice(SyncedMemory a, uint64_t len, bool forward) {
  const size_t bytes = len * kFr;
  if (bytes > a.size()) throw pp::Error(PP_E_INVAL, "slice: longer than the input");
  SyncedMemory res(bytes);
  if (!bytes) return res;
  const size_t off = forward ? 0 : a.size() - bytes;
  if (a.head() == SyncedMemory::HEAD_AT_CPU) {
    std::memcpy(res.mutable_cpu_data(), static_cast<char *>(a.mutable_cpu_data()) + off, bytes);
  } else {
    pp::check_cuda(cudaMemcpy(res.mutable_gpu_data(), static_cast<char *>(a.mutable_gpu_data()) + off,
                              bytes, cudaMemcpyDeviceToDevice),
                   "slice");
  }
  return res;
}

SyncedMemory make_tensor(SyncedMemory input, uint64_t pad_len) {
  const size_t words = input.size() / sizeof(uint64_t);
  if (words > pad_len) throw pp::Error(PP_E_INVAL, "make_tensor: more words than pad_len elements");
  SyncedMemory out(pad_len * kFr);
  if (!pad_len) return out;
  void *o = out.mutable_gpu_data();
  pp::check_cuda(cudaMemset(o, 0, out.size()), "make_tensor");
  if (words)  // word i -> the low limb of element i
    pp::check_cuda(cudaMemcpy2D(o, kFr, input.mutable_gpu_data(), sizeof(uint64_t), sizeof(uint64_t), words,
                                cudaMemcpyDeviceToDevice),
                   "make_tensor");
  return out;
}

bool gt_zkp(SyncedMemory a, SyncedMemory b) {
  const size_t na = a.size() / sizeof(uint64_t);
  if (b.size() / sizeof(uint64_t) < na) throw pp::Error(PP_E_INVAL, "gt_zkp: b shorter than a");
  const uint64_t *x = static_cast<const uint64_t *>(a.mutable_cpu_data());
  const uint64_t *y = static_cast<const uint64_t *>(b.mutable_cpu_data());
  for (size_t i = na; i-- > 0;) {
    if (x[i] != y[i]) return x[i] > y[i];
  }
  return false;
}
