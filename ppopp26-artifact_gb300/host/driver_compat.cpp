// driver_compat.cpp -- command-line driver over the reference-compatible host
// layer, in the shape of the reference's drivers (miss_ops.cu, ntt.cu
// --check-*, lde.cu --bench).  Inputs and outputs are raw files of 32-byte
// Montgomery elements, the format of the reference's input.bin.
//
//   pp_compat_driver miss_ops <lg_N> <in.bin> <outdir>
//       accumulate_mul_poly, accumulate_mul_poly_, evaluate, poly_div_poly on
//       the input (point and divisor constants of miss_ops.cu:133-135,
//       :180-183) -> <outdir>/{gp,gp_incl,eval,div}.bin
//   pp_compat_driver ntt <lg_N> <in.bin> <out.bin>
//       Ntt::forward -> out.bin; checks our_ntt and standard4_ntt against it
//       byte for byte and Intt::forward against the input (ntt.cu:1276-1351)
//   pp_compat_driver lde <lg_N> <lambda> <in.bin> <out.bin> [naive]
//       our_lde (or naive_lde) -> out.bin
//   pp_compat_driver quotient <n> <dir>
//       compute_quotient_identity_range_check_i, then ..._copy_... and
//       ..._term_check_one_i on one result buffer, as the prover calls them;
//       inputs <dir>/<argument name>.bin -> <dir>/quotient_out.bin
//   pp_compat_driver gate <n> <sbox_alpha> <dir>
//       compute_gate_constraint_allmerge_cuda -> <dir>/gate_out.bin
//   pp_compat_driver msm <n> <points.bin> <scalars.bin> <out.bin>
//       multi_scalar_mult -> out.bin (Jacobian x, y, 1)
//   pp_compat_driver convert <n> <in.bin> <outdir>
//       read_file, to_base -> base.bin and base.txt (writeToFile), to_mont of
//       that -> mont.bin (the input again)
//   pp_compat_driver fieldops <n> <dir>
//       add_mod ... make_tensor on <dir>/{a,b,s}.bin -> <dir>/<name>.bin, and
//       gt_zkp of (a, b) and (b, a) on stdout
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "function.h"
#include "io.h"
#include "zksnark.h"

static std::vector<unsigned char> read_file(const std::string &path, size_t bytes) {
  std::vector<unsigned char> v(bytes);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) throw pp::Error(1, "cannot open " + path);
  const size_t got = std::fread(v.data(), 1, bytes, f);
  std::fclose(f);
  if (got != bytes) throw pp::Error(1, "short read from " + path);
  return v;
}

static void write_file(const std::string &path, const void *p, size_t bytes) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw pp::Error(1, "cannot create " + path);
  std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}

static SyncedMemory load(const std::string &path, size_t n) {
  SyncedMemory m(n * 32);
  auto v = read_file(path, n * 32);
  std::memcpy(m.mutable_cpu_data(), v.data(), n * 32);
  return m;
}

static int miss_ops(int lg, const std::string &in, const std::string &outdir) {
  const size_t n = size_t{1} << lg;
  SyncedMemory gp = load(in, n);
  SyncedMemory incl(n * 32);
  SyncedMemory gp2 = load(in, n);
  accumulate_mul_poly(gp);
  accumulate_mul_poly_(gp2, incl);
  cudaDeviceSynchronize();
  if (std::memcmp(gp.mutable_cpu_data(), gp2.mutable_cpu_data(), n * 32) != 0) {
    std::printf("accumulate_mul_poly and accumulate_mul_poly_ disagree\n");
    return 2;
  }
  write_file(outdir + "/gp.bin", gp.mutable_cpu_data(), n * 32);
  write_file(outdir + "/gp_incl.bin", incl.mutable_cpu_data(), n * 32);

  SyncedMemory point(32);
  const uint64_t pt[4] = {123456789UL, 987654321UL, 1122334455UL, 6677889900UL};
  std::memcpy(point.mutable_cpu_data(), pt, 32);
  SyncedMemory poly = load(in, n);
  SyncedMemory y = evaluate(poly, point);
  write_file(outdir + "/eval.bin", y.mutable_cpu_data(), 32);

  SyncedMemory c(32);
  const uint64_t cv[4] = {123456789123456789UL, 987654321987654321UL, 1122334455667788UL,
                          1122334455667788UL};
  std::memcpy(c.mutable_cpu_data(), cv, 32);
  SyncedMemory div = load(in, n);
  poly_div_poly(div, c);
  write_file(outdir + "/div.bin", div.mutable_cpu_data(), n * 32);
  std::printf("miss_ops ok\n");
  return 0;
}

static int ntt_check(int lg, const std::string &in, const std::string &out) {
  const size_t n = size_t{1} << lg;
  Ntt ntt(32);
  Intt intt(32);
  SyncedMemory x = load(in, n);
  SyncedMemory expected = ntt.forward(x);
  cudaDeviceSynchronize();
  write_file(out, expected.mutable_cpu_data(), n * 32);
  SyncedMemory a = load(in, n), b = load(in, n);
  our_ntt(a, lg, lg / 2, lg - lg / 2, 2, 16, 16, ntt);
  standard4_ntt(b, lg, lg / 2, lg - lg / 2, 2, 16, ntt);
  const bool ok1 = std::memcmp(a.mutable_cpu_data(), expected.mutable_cpu_data(), n * 32) == 0;
  const bool ok2 = std::memcmp(b.mutable_cpu_data(), expected.mutable_cpu_data(), n * 32) == 0;
  SyncedMemory back = intt.forward(expected);
  cudaDeviceSynchronize();
  const bool ok3 = std::memcmp(back.mutable_cpu_data(), x.mutable_cpu_data(), n * 32) == 0;
  std::printf("check our_ntt: %s, standard4_ntt: %s, intt round trip: %s\n", ok1 ? "ok" : "MISMATCH",
              ok2 ? "ok" : "MISMATCH", ok3 ? "ok" : "MISMATCH");
  return ok1 && ok2 && ok3 ? 0 : 2;
}

static int lde(int lg, int lambda, const std::string &in, const std::string &out, bool naive) {
  const size_t n = size_t{1} << lg;
  auto v = read_file(in, n * 32);
  Ntt ntt(32);
  auto *p = reinterpret_cast<cpu::BLS12_381_Fr_G1 *>(v.data());
  const float ms = naive ? naive_lde(p, lg, lambda, 1, 16, 16, ntt) : our_lde(p, lg, lambda, 1, 16, 16, ntt);
  SyncedMemory o = last_lde_output();
  write_file(out, o.mutable_cpu_data(), o.size());
  std::printf("lde ok %.3f ms\n", ms);
  return 0;
}

static int quotient(size_t n, const std::string &dir) {
  auto V = [&](const char *name) { return load(dir + "/" + name + ".bin", n); };
  auto S = [&](const char *name) { return load(dir + "/" + name + ".bin", 1); };
  SyncedMemory result = V("result");
  cuda::compute_quotient_identity_range_check_i(V("x"), V("w_l"), V("w_r"), V("w_o"), V("w_4"),
                                                V("z"), S("alpha"), S("beta"), S("gamma"), S("k1"),
                                                S("k2"), S("k3"), result);
  cuda::compute_quotient_copy_range_check_i(V("left_sigma"), V("right_sigma"), V("out_sigma"),
                                            V("fourth_sigma"), V("mod"), V("w_l"), V("w_r"),
                                            V("w_o"), V("w_4"), V("z_next"), S("alpha"), S("beta"),
                                            S("gamma"), result);
  cuda::compute_quotient_term_check_one_i(V("z"), V("l1"), S("one"), result);
  cudaDeviceSynchronize();
  write_file(dir + "/quotient_out.bin", result.mutable_cpu_data(), n * 32);
  std::printf("quotient ok\n");
  return 0;
}

static int gate(size_t n, long long alpha, const std::string &dir) {
  auto V = [&](const char *name) { return load(dir + "/" + name + ".bin", n); };
  auto S = [&](const char *name) { return load(dir + "/" + name + ".bin", 1); };
  SyncedMemory out = cuda::compute_gate_constraint_allmerge_cuda(
      V("a_val"), V("b_val"), V("c_val"), V("d_val"), V("a_next_eval"), V("b_next_eval"),
      V("d_next_eval"), V("q_m"), V("q_l"), V("q_r"), V("q_o"), V("q_4"), V("q_c"), V("q_hl"),
      V("q_hr"), V("q_h4"), V("q_arith"), V("range"), V("logic"), V("fixed_group_add"),
      V("variable_group_add"), V("pi_eval_8n"), S("four"), S("one"), S("two"), S("three"),
      S("kappa_range"), S("kappa_sq_range"), S("kappa_cu_range"), S("range_challenge"), S("P_D"),
      S("nine"), S("kappa_cu_logic"), S("eighteen"), S("eightyone"), S("eightythree"),
      S("kappa_qu_logic"), S("logic_challenge"), S("P_A"), S("kappa_fb"), S("kappa_sq_fb"),
      S("kappa_cu_fb"), S("fb_challenge"), S("kappa_vb"), S("kappa_sq_vb"), S("vb_challenge"),
      alpha);
  cudaDeviceSynchronize();
  write_file(dir + "/gate_out.bin", out.mutable_cpu_data(), n * 32);
  std::printf("gate ok\n");
  return 0;
}

static int msm(size_t n, const std::string &pts, const std::string &scs, const std::string &out) {
  SyncedMemory p(n * 96), s(n * 32);
  auto pv = read_file(pts, n * 96), sv = read_file(scs, n * 32);
  std::memcpy(p.mutable_cpu_data(), pv.data(), n * 96);
  std::memcpy(s.mutable_cpu_data(), sv.data(), n * 32);
  SyncedMemory r = multi_scalar_mult(p, s);
  write_file(out, r.mutable_cpu_data(), 144);
  std::printf("msm ok\n");
  return 0;
}

static int convert(size_t n, const std::string &in, const std::string &outdir) {
  SyncedMemory x(n * 32);
  ::read_file(in.c_str(), x.mutable_cpu_data());
  SyncedMemory base = to_base(x);
  SyncedMemory mont = to_mont(base);
  cudaDeviceSynchronize();
  write_file(outdir + "/base.bin", base.mutable_cpu_data(), n * 32);
  writeToFile(outdir + "/base.txt", static_cast<uint64_t *>(base.mutable_cpu_data()), 4 * n);
  write_file(outdir + "/mont.bin", mont.mutable_cpu_data(), n * 32);
  std::printf("convert ok\n");
  return 0;
}

// element-wise operators and buffer helpers on a, b (n elements) and s (one)
static int fieldops(size_t n, const std::string &dir) {
  SyncedMemory a = load(dir + "/a.bin", n), b = load(dir + "/b.bin", n), s = load(dir + "/s.bin", 1);
  struct Out {
    const char *name;
    SyncedMemory m;
  };
  std::vector<Out> outs;
  outs.push_back({"add", add_mod(a, b)});
  outs.push_back({"sub", sub_mod(a, b)});
  outs.push_back({"mul", mul_mod(a, b)});
  outs.push_back({"div", div_mod(a, b)});
  SyncedMemory ip = load(dir + "/a.bin", n);
  div_mod_(ip, b);
  outs.push_back({"div_in_place", ip});
  outs.push_back({"add_scalar", add_mod_scalar(a, s)});
  outs.push_back({"div_scalar", div_mod_scalar(a, s)});
  SyncedMemory ms = load(dir + "/a.bin", n);
  mul_mod_scalar_(ms, s);
  outs.push_back({"mul_scalar_in_place", ms});
  outs.push_back({"neg", neg_mod(a)});
  outs.push_back({"inv", inv_mod(b)});
  outs.push_back({"exp5", exp_mod(a, 5)});
  outs.push_back({"seq", gen_sequence(n, s)});
  outs.push_back({"rep", repeat_to_poly(s, n)});
  outs.push_back({"pad", pad_poly(a, 2 * n)});
  outs.push_back({"cat", cat(a, b)});
  outs.push_back({"slice", slice(a, n / 2, false)});
  outs.push_back({"tensor", make_tensor(a, 4 * n)});
  cudaDeviceSynchronize();
  for (auto &o : outs) write_file(dir + "/" + o.name + ".bin", o.m.mutable_cpu_data(), o.m.size());
  std::printf("gt %d %d\n", gt_zkp(a, b) ? 1 : 0, gt_zkp(b, a) ? 1 : 0);
  std::printf("fieldops ok\n");
  return 0;
}

int main(int argc, char **argv) {
  try {
    if (argc >= 4 && std::string(argv[1]) == "fieldops")
      return fieldops(std::strtoull(argv[2], nullptr, 10), argv[3]);
    if (argc >= 5 && std::string(argv[1]) == "miss_ops") return miss_ops(std::atoi(argv[2]), argv[3], argv[4]);
    if (argc >= 5 && std::string(argv[1]) == "ntt") return ntt_check(std::atoi(argv[2]), argv[3], argv[4]);
    if (argc >= 4 && std::string(argv[1]) == "quotient")
      return quotient(std::strtoull(argv[2], nullptr, 10), argv[3]);
    if (argc >= 6 && std::string(argv[1]) == "msm")
      return msm(std::strtoull(argv[2], nullptr, 10), argv[3], argv[4], argv[5]);
    if (argc >= 5 && std::string(argv[1]) == "convert")
      return convert(std::strtoull(argv[2], nullptr, 10), argv[3], argv[4]);
    if (argc >= 5 && std::string(argv[1]) == "gate")
      return gate(std::strtoull(argv[2], nullptr, 10), std::atoll(argv[3]), argv[4]);
    if (argc >= 6 && std::string(argv[1]) == "lde")
      return lde(std::atoi(argv[2]), std::atoi(argv[3]), argv[4], argv[5],
                 argc >= 7 && std::string(argv[6]) == "naive");
  } catch (const pp::Error &e) {
    std::fprintf(stderr, "error (status %d): %s\n", e.status(), e.what());
    return 3;
  }
  std::fprintf(stderr, "usage: %s miss_ops|ntt|lde|quotient|gate|convert|msm|fieldops ...\n", argv[0]);
  return 1;
}
