// ref_gpu_driver.cu -- TEST INFRASTRUCTURE: runs the reference's own GPU
// operators on seeded inputs, to record golden outputs and timings.
//
// The oracle Makefile (target refgpu) compiles this file three times, each time
// around one of the reference's driver files, with that file's main renamed:
//   REF_UNIT_NTT  ntt.cu       Ntt::forward / Intt::forward
//                              (PLONK/utils/function.cu:280,330), our_ntt
//                              (ntt.cu:979-1037), standard4_ntt (ntt.cu:1039)
//   REF_UNIT_LDE  lde.cu       our_lde (lde.cu:1267-1365)
//   REF_UNIT_OPS  miss_ops.cu  accumulate_mul_poly, evaluate, poly_div_poly
//                              (PLONK/utils/function.cu:170-260 ->
//                              mont/cuda/mont_arithmetic.cu:507-550), and the
//                              blst CPU baselines naive_gp / naive_div
//                              (miss_ops.cu:34-87)
// It links against every PLONK/utils and caffe object of the reference, built
// with the reference's own flags.  Nothing in the product links or runs it.
//
// Commands (files hold raw 32-byte Montgomery elements, natural order):
//   ref_ntt fwd|inv <lgN> <in> <out>      Ntt(32).forward / Intt(32).forward (lgN >= 18)
//   ref_ntt split|std4 <lgN> <in> <out>   our_ntt / standard4_ntt with the
//                                         reference's configured split for lgN
//                                         (22, 24 or 26; ntt.cu:1193-1206)
//   ref_ntt time <lgN> <reps> <in>        CUDA-event times of the in-HBM forms
//   ref_lde lde <lgN> <lambda> <in> <out> our_lde with the configured chunking
//                                         (lde.cu:1550-1580); <in> = coefficients
//   ref_ops gp <lgN> <in> <out>           accumulate_mul_poly (in place)
//   ref_ops eval <lgN> <in> <x> <out>     evaluate (one element out)
//   ref_ops div <lgN> <in> <c> <out>      poly_div_poly by (X + c) (in place)
//   ref_ops time <lgN> <reps> <in> <x> <c> GPU ops (CUDA events) and the blst
//                                         CPU baselines (wall clock, 1 thread)
//   ref_ops msm <lgN> <reps> <points> <scalars> <out>
//                                         multi_scalar_mult (PLONK/utils/function.cu:396-412)
//                                         on 2^lgN affine points (96-byte x, y in
//                                         Montgomery form) and plain 32-byte
//                                         scalars; writes its Jacobian result
//                                         (3 x 48 bytes); reps > 0 adds wall-clock
//                                         times (its collection step runs on the host)
//   ref_* refmain <args...>               the reference driver's own main
// Every timing command prints one line "REFJSON {...}".
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#if defined(REF_UNIT_LDE)
// Called by the one line the staging recipe adds to the copy of lde.cu, just
// before our_lde returns; `p` is our_lde's result (`current`), `n` elements.
static void ref_lde_capture(const void* p, unsigned long long n);
#endif

#define main reference_unit_main
#if defined(REF_UNIT_NTT)
#include "ntt.cu"
#elif defined(REF_UNIT_LDE)
#include "lde.cu"
#elif defined(REF_UNIT_OPS)
#include "miss_ops.cu"
#else
#error "define one of REF_UNIT_NTT, REF_UNIT_LDE, REF_UNIT_OPS"
#endif
#undef main

namespace refdrv {

[[noreturn]] void die(const std::string& msg) {
  std::fprintf(stderr, "ref_gpu_driver: %s\n", msg.c_str());
  std::exit(2);
}

void check_cuda(const char* what) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) die(std::string(what) + ": " + cudaGetErrorString(e));
}

void read_exact(const char* path, void* dst, size_t bytes) {
  FILE* f = std::fopen(path, "rb");
  if (!f) die(std::string("cannot open ") + path);
  size_t got = std::fread(dst, 1, bytes, f);
  std::fclose(f);
  if (got != bytes) die(std::string("short file ") + path);
}

void write_all(const char* path, const void* src, size_t bytes) {
  FILE* f = std::fopen(path, "wb");
  if (!f) die(std::string("cannot create ") + path);
  size_t put = std::fwrite(src, 1, bytes, f);
  std::fclose(f);
  if (put != bytes) die(std::string("short write ") + path);
}

int lg_arg(const char* s) {
  int v = std::atoi(s);
  if (v < 1 || v > 28) die("lgN out of range");
  return v;
}

SyncedMemory host_vector(const char* path, uint64_t n) {
  SyncedMemory m(n * 32);
  read_exact(path, m.mutable_cpu_data(), n * 32);
  return m;
}

template <class F>
float event_ms(F&& f) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, 0);
  f();
  cudaEventRecord(b, 0);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

template <class F>
double wall_ms(F&& f) {
  auto t0 = std::chrono::steady_clock::now();
  f();
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

std::string stats_json(const std::vector<double>& v) {
  double mn = v.empty() ? 0 : v[0], sum = 0;
  for (double x : v) { mn = x < mn ? x : mn; sum += x; }
  char buf[160];
  std::snprintf(buf, sizeof buf, "{\"min_ms\": %.6f, \"mean_ms\": %.6f, \"reps\": %zu}", mn,
                v.empty() ? 0.0 : sum / v.size(), v.size());
  return buf;
}

}  // namespace refdrv

using namespace refdrv;

#if defined(REF_UNIT_NTT)
// The reference's CTkernel advances its stage counter by the kernel radix (at
// least 6) rather than by the kernel's iteration count
// (zksnark_ntt/ntt_kernel/ct_mixed_radix_wide.cuh:205,314), so Ntt::forward
// stays inside its buffer only when every one of CT_NTT's three kernels gets
// 6 or more iterations (algorithm.cuh:20-56): lgN >= 18.  Smaller sizes read
// and write past the buffer (2^13 raised an illegal address), so they are refused.
static int ntt_lg_arg(const char* s) {
  const int lg = lg_arg(s);
  if (lg < 18) die("the reference's Ntt::forward indexes past its buffer below lgN = 18");
  return lg;
}

static int unit_main(int argc, char** argv) {
  std::string cmd = argv[1];
  if ((cmd == "fwd" || cmd == "inv") && argc == 5) {
    const int lg = ntt_lg_arg(argv[2]);
    const uint64_t n = uint64_t{1} << lg;
    SyncedMemory in = host_vector(argv[3], n);
    SyncedMemory out;
    if (cmd == "fwd") {
      Ntt ntt(32);
      out = ntt.forward(in);
    } else {
      Intt intt(32);
      out = intt.forward(in);
    }
    check_cuda(cmd.c_str());
    write_all(argv[4], out.mutable_cpu_data(), n * 32);
    return 0;
  }
  if ((cmd == "split" || cmd == "std4") && argc == 5) {
    // the call sequences of run_check / run_standard4_check (ntt.cu:1276-1351)
    const int lg = lg_arg(argv[2]);
    const NttScaleConfig cfg = ntt_scale_config(lg);
    const uint64_t n = uint64_t{1} << lg;
    const int lg_i = cfg.lg_i, lg_j = lg - cfg.lg_i, lg_k = cfg.ours_lg_k;
    SyncedMemory in = host_vector(argv[3], n);
    Ntt ntt(32);
    if (cmd == "split") {
      const int step1_thread = step1_threads_default();
      const int step2_thread = step2_threads_for_lg_k(lg_k, lg);
      StageIndexMap map;
      StageIndexMap* map_ptr = nullptr;
      if (should_build_stage_map(cfg.map_policy, lg - lg_i)) {
        const uint64_t chunk_elems = (uint64_t{1} << lg_i) * (uint64_t{1} << lg_k);
        map = build_stage_index_map(chunk_elems, n / chunk_elems, lg_i, lg - lg_i, step2_thread);
        map_ptr = &map;
      }
      our_ntt(in, lg, lg_i, lg_j, lg_k, step1_thread, step2_thread, ntt, map_ptr);
    } else {
      standard4_ntt(in, lg, lg_i, lg_j, lg_k, step1_threads_default(), ntt);
    }
    check_cuda(cmd.c_str());
    write_all(argv[4], in.mutable_cpu_data(), n * 32);
    return 0;
  }
  if (cmd == "time" && argc == 5) {
    const int lg = ntt_lg_arg(argv[2]);
    const int reps = std::atoi(argv[3]);
    const uint64_t n = uint64_t{1} << lg;
    SyncedMemory in = host_vector(argv[4], n);
    in.mutable_gpu_data();
    Ntt ntt(32);
    Intt intt(32);
    SyncedMemory out(n * 32);
    out.mutable_gpu_data();
    check_cuda("setup");
    std::vector<double> f_alloc, f_pre, i_alloc, i_pre;
    SyncedMemory held;  // keeps each call's result alive past its stop event
    for (int r = -1; r < reps; ++r) {  // r = -1 is the warm-up
      double a = event_ms([&] { held = ntt.forward(in); });
      double b = event_ms([&] { ntt.forward_(in, out); });
      double c = event_ms([&] { held = intt.forward(in); });
      double d = event_ms([&] { intt.forward_(in, out); });
      check_cuda("time");
      if (r >= 0) {
        f_alloc.push_back(a); f_pre.push_back(b); i_alloc.push_back(c); i_pre.push_back(d);
      }
    }
    std::printf("REFJSON {\"op\": \"ntt_in_hbm\", \"lgN\": %d, \"forward\": %s, \"forward_prealloc\": %s, "
                "\"inverse\": %s, \"inverse_prealloc\": %s}\n",
                lg, stats_json(f_alloc).c_str(), stats_json(f_pre).c_str(),
                stats_json(i_alloc).c_str(), stats_json(i_pre).c_str());
    return 0;
  }
  return -1;
}
#endif

#if defined(REF_UNIT_LDE)
static std::vector<unsigned char>* g_capture = nullptr;
static void ref_lde_capture(const void* p, unsigned long long n) {
  if (g_capture) {
    g_capture->resize(n * 32);
    std::memcpy(g_capture->data(), p, n * 32);
  }
}

static int unit_main(int argc, char** argv) {
  std::string cmd = argv[1];
  if (cmd == "lde" && argc == 6) {
    // the call sequence of run_benchmark (lde.cu:1653-1700) for one repetition
    const int lg = lg_arg(argv[2]);
    const int lambda = std::atoi(argv[3]);
    const LdeScaleConfig cfg = lde_scale_config(lg, lambda);
    const uint64_t n = uint64_t{1} << lg;
    std::vector<unsigned char> input(n * 32), result;
    read_exact(argv[4], input.data(), n * 32);
    Ntt ntt(32);
    g_capture = &result;
    our_lde(reinterpret_cast<cpu::BLS12_381_Fr_G1*>(input.data()), lg, lambda, cfg.ours_lg_k,
            step1_threads_default(), our_lde_step2_threads_for_lg_k(lg, lambda, cfg.ours_lg_k), ntt);
    g_capture = nullptr;
    check_cuda("our_lde");
    if (result.size() != (n << lambda) * 32) die("our_lde result was not captured");
    write_all(argv[5], result.data(), result.size());
    return 0;
  }
  return -1;
}
#endif

#if defined(REF_UNIT_OPS)
static int unit_main(int argc, char** argv) {
  std::string cmd = argv[1];
  if (cmd == "gp" && argc == 5) {
    const uint64_t n = uint64_t{1} << lg_arg(argv[2]);
    SyncedMemory in = host_vector(argv[3], n);
    in.mutable_gpu_data();
    SyncedMemory out = accumulate_mul_poly(in);
    check_cuda("accumulate_mul_poly");
    write_all(argv[4], out.mutable_cpu_data(), n * 32);
    return 0;
  }
  if (cmd == "eval" && argc == 6) {
    const uint64_t n = uint64_t{1} << lg_arg(argv[2]);
    SyncedMemory in = host_vector(argv[3], n);
    SyncedMemory x = host_vector(argv[4], 1);
    in.mutable_gpu_data();
    x.mutable_gpu_data();
    SyncedMemory y = evaluate(in, x);
    check_cuda("evaluate");
    write_all(argv[5], y.mutable_cpu_data(), 32);
    return 0;
  }
  if (cmd == "div" && argc == 6) {
    const uint64_t n = uint64_t{1} << lg_arg(argv[2]);
    SyncedMemory in = host_vector(argv[3], n);
    SyncedMemory c = host_vector(argv[4], 1);
    in.mutable_gpu_data();
    c.mutable_gpu_data();
    SyncedMemory out = poly_div_poly(in, c);
    check_cuda("poly_div_poly");
    write_all(argv[5], out.mutable_cpu_data(), n * 32);
    return 0;
  }
  if (cmd == "msm" && argc == 7) {
    const int lg = lg_arg(argv[2]);
    const int reps = std::atoi(argv[3]);
    const uint64_t n = uint64_t{1} << lg;
    SyncedMemory pts(n * 96), sc(n * 32);
    read_exact(argv[4], pts.mutable_cpu_data(), n * 96);
    read_exact(argv[5], sc.mutable_cpu_data(), n * 32);
    pts.mutable_gpu_data();
    sc.mutable_gpu_data();
    check_cuda("upload");
    std::vector<double> t;
    SyncedMemory res;
    for (int r = -1; r < reps; ++r) {  // r = -1 is the warm-up (and the result kept)
      const double ms = wall_ms([&] {
        res = multi_scalar_mult(pts, sc);
        cudaDeviceSynchronize();
      });
      if (r >= 0) t.push_back(ms);
    }
    check_cuda("multi_scalar_mult");
    write_all(argv[6], res.mutable_cpu_data(), 3 * 48);
    if (reps > 0)
      std::printf("REFJSON {\"op\": \"msm\", \"lgN\": %d, \"multi_scalar_mult\": %s}\n", lg,
                  stats_json(t).c_str());
    return 0;
  }
  if (cmd == "time" && argc == 7) {
    // as miss_ops.cu:88-194 times them: inputs already on the device for the
    // GPU calls (their scratch allocation inside the timed call), the blst
    // functions on one host thread.
    const int lg = lg_arg(argv[2]);
    const int reps = std::atoi(argv[3]);
    const uint64_t n = uint64_t{1} << lg;
    std::vector<unsigned char> base(n * 32);
    read_exact(argv[4], base.data(), n * 32);
    SyncedMemory x = host_vector(argv[5], 1);
    SyncedMemory c = host_vector(argv[6], 1);
    x.mutable_gpu_data();
    std::vector<double> gp, ev, dv, ngp, ndv;
    SyncedMemory in(n * 32);
    SyncedMemory held;  // keeps each call's result alive past its stop event
    for (int r = -1; r < reps; ++r) {
      std::memcpy(in.mutable_cpu_data(), base.data(), n * 32);
      in.mutable_gpu_data();
      check_cuda("upload");
      double a = event_ms([&] { held = accumulate_mul_poly(in); });
      std::memcpy(in.mutable_cpu_data(), base.data(), n * 32);
      in.mutable_gpu_data();
      double b = event_ms([&] { held = evaluate(in, x); });
      std::memcpy(in.mutable_cpu_data(), base.data(), n * 32);
      in.mutable_gpu_data();
      SyncedMemory cc(32);
      std::memcpy(cc.mutable_cpu_data(), c.mutable_cpu_data(), 32);
      cc.mutable_gpu_data();
      check_cuda("upload");
      double d = event_ms([&] { held = poly_div_poly(in, cc); });
      check_cuda("time");
      if (r >= 0) { gp.push_back(a); ev.push_back(b); dv.push_back(d); }
    }
    // blst CPU baselines: naive_div divides by [c, 1] = X + c (miss_ops.cu:49-87)
    SyncedMemory divisor(64);
    std::memcpy(divisor.mutable_cpu_data(), c.mutable_cpu_data(), 32);
    std::memcpy(static_cast<char*>(divisor.mutable_cpu_data()) + 32, one().mutable_cpu_data(), 32);
    const int cpu_reps = reps < 3 ? reps : 3;
    for (int r = 0; r < cpu_reps; ++r) {
      std::memcpy(in.mutable_cpu_data(), base.data(), n * 32);
      ngp.push_back(wall_ms([&] { SyncedMemory o = naive_gp(lg, in); }));
      std::memcpy(in.mutable_cpu_data(), base.data(), n * 32);
      ndv.push_back(wall_ms([&] { SyncedMemory o = naive_div(lg, in, divisor); }));
    }
    std::printf("REFJSON {\"op\": \"miss_ops\", \"lgN\": %d, \"accumulate_mul_poly\": %s, "
                "\"evaluate\": %s, \"poly_div_poly\": %s, \"naive_gp_cpu_1thread\": %s, "
                "\"naive_div_cpu_1thread\": %s}\n",
                lg, stats_json(gp).c_str(), stats_json(ev).c_str(), stats_json(dv).c_str(),
                stats_json(ngp).c_str(), stats_json(ndv).c_str());
    return 0;
  }
  return -1;
}
#endif

int main(int argc, char** argv) {
  if (argc < 2) die("usage: see the header of ref_gpu_driver.cu");
  if (std::string(argv[1]) == "refmain") {
#if defined(REF_UNIT_OPS)
    return reference_unit_main();  // miss_ops.cu's main takes no arguments
#else
    argv[1] = argv[0];
    return reference_unit_main(argc - 1, argv + 1);
#endif
  }
  int rc = unit_main(argc, argv);
  if (rc < 0) die(std::string("unknown command or wrong arguments: ") + argv[1]);
  return rc;
}
