// batch.cu -- many polynomials of uneven power-of-two sizes per launch.
//
// A batch plan turns a list of jobs (NTT, INTT, the three LDE forms, grand
// products) into a short, fixed sequence of launches:
//  * every transform is split into its passes (the same radix plans and
//    tables as single calls); pass p of a job runs at "level" start + p, an
//    LDE from evaluations chains its INTT and its forward transform;
//  * one launch per level (per 128 job passes at that level) covers their
//    tiles (k_ntt_batch_level, one block per tile of a prefix-summed tile
//    list, the jobs' arguments passed as kernel parameters);
//  * the grand products run as two launches over the blocks of all of them.
// A plan owns its descriptors and workspaces (allocated once at creation), so
// running it allocates nothing and the whole sequence can be captured into a
// CUDA graph (pp_batch_capture) and replayed per prover round.
// The single-call entry points instead issue 2-3 launches per polynomial.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ntt.cuh"
#include "scan.cuh"

namespace pp {

struct BatchPlan {
  int dev = 0;
  // one level = one launch per chunk of at most kLevelJobs job passes, the
  // jobs' arguments passed as kernel parameters
  struct Level {
    std::vector<LevelParams> chunks;
  };
  std::vector<Level> levels;
  GpBatchJob *d_gp = nullptr;
  uint32_t *d_gp_start = nullptr;
  uint32_t gp_count = 0, gp_blocks = 0;
  void *d_mem = nullptr;   // workspaces of all jobs
  void *d_desc = nullptr;  // per-level descriptors and grand-product job table
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t launches = 0;
  uint64_t tiles = 0;
};

namespace {

struct SubTransform {
  const fr *in;
  fr *out;  // resolved later for chains that write into the job output
  uint32_t lg;
  bool inverse;
  NttInputDesc desc;
  uint32_t start_level;
  uint32_t passes;
};

int run_plan(BatchPlan *p, cudaStream_t s) {
  for (auto &lv : p->levels)
    for (auto &c : lv.chunks) {
      int st = ntt_launch_level(c, s);
      if (st) return st;
    }
  return gp_batch_launch(p->d_gp, p->d_gp_start, p->gp_count, p->gp_blocks, s);
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace
}  // namespace pp

using pp::fr;

extern "C" int pp_batch_create(const pp_job *jobs, uint32_t count, void **plan_out) {
  if (!plan_out || (count && !jobs)) {
    pp::set_error("pp_batch_create: null argument");
    return PP_E_INVAL;
  }
  *plan_out = nullptr;
  auto *p = new pp::BatchPlan();
  cudaGetDevice(&p->dev);
  // ---- expand jobs into sub-transforms and grand products
  std::vector<pp::SubTransform> subs;
  struct Gp {
    const fr *in;
    fr *out;
    uint64_t n;
  };
  std::vector<Gp> gps;
  for (uint32_t i = 0; i < count; ++i) {
    const pp_job &j = jobs[i];
    const bool al = (reinterpret_cast<uintptr_t>(j.d_in) & 15) == 0 &&
                    (reinterpret_cast<uintptr_t>(j.d_out) & 15) == 0;
    if (!j.d_in || !j.d_out || !al) {
      pp::set_error("pp_batch_create: job %u: buffers must be 16-byte aligned device pointers", i);
      delete p;
      return PP_E_INVAL;
    }
    const fr *in = static_cast<const fr *>(j.d_in);
    fr *out = static_cast<fr *>(j.d_out);
    const uint32_t L = j.lg_n + j.lambda;
    if (j.kind == PP_JOB_GP) {
      gps.push_back({in, out, 1ull << j.lg_n});
      continue;
    }
    if (j.kind > PP_JOB_GP || j.lambda > 8 || L > 28 || L < 3 ||
        ((j.kind == PP_JOB_NTT || j.kind == PP_JOB_INTT) && j.lambda)) {
      pp::set_error("pp_batch_create: job %u: kind %u, 2^%u (+%u) not supported in a batch", i, j.kind,
                    j.lg_n, j.lambda);
      delete p;
      return PP_E_UNSUPPORTED;
    }
    pp::SubTransform t{in, out, L, false, pp::NttInputDesc(), 0, 0};
    int st = PP_OK;
    switch (j.kind) {
      case PP_JOB_NTT:
        subs.push_back(t);
        break;
      case PP_JOB_INTT:
        t.inverse = true;
        subs.push_back(t);
        break;
      case PP_JOB_LDE_COEFFS: {
        const fr h = pp::host_pow(pp::host_mont_small(7), 1ull << j.lambda);
        t.desc.kind = pp::NTT_IN_DIAG;
        t.desc.diag = pp::pow_table(h, j.lg_n, &st);
        t.desc.n_valid = 1ull << j.lg_n;
        subs.push_back(t);
        break;
      }
      case PP_JOB_LDE_EVALS: {
        if (j.lg_n < 3) {
          pp::set_error("pp_batch_create: job %u: LDE from evaluations needs 2^3 or more points", i);
          delete p;
          return PP_E_UNSUPPORTED;
        }
        pp::SubTransform a{in, out, j.lg_n, true, pp::NttInputDesc(), 0, 0};
        subs.push_back(a);
        t.in = out;
        t.desc.kind = pp::NTT_IN_DIAG;
        t.desc.diag = pp::pow_table(pp::host_mont_small(7), j.lg_n, &st);
        t.desc.n_valid = 1ull << j.lg_n;
        t.start_level = 0xffffffffu;  // chained: starts after the INTT above
        subs.push_back(t);
        break;
      }
      case PP_JOB_LDE_SPREAD:
        t.desc.kind = pp::NTT_IN_SPREAD;
        t.desc.spread = j.lambda;
        subs.push_back(t);
        break;
    }
    if (st) {
      delete p;
      return st;
    }
  }
  // ---- workspace layout: one region per sub-transform (2^lg elements),
  //      then the grand-product scratch, then descriptors
  size_t ws_elems = 0;
  std::vector<size_t> ws_off(subs.size());
  for (size_t i = 0; i < subs.size(); ++i) {
    ws_off[i] = ws_elems;
    ws_elems += 1ull << subs[i].lg;
  }
  std::vector<pp::ScanGeom> gg(gps.size());
  std::vector<size_t> gp_off(gps.size());
  for (size_t i = 0; i < gps.size(); ++i) {
    gg[i] = pp::scan_geom(gps[i].n);
    gp_off[i] = ws_elems;
    ws_elems += gg[i].threads + gg[i].blocks;
  }
  size_t ws_bytes = pp::align_up(ws_elems * sizeof(fr), 256);
  PP_COUNT_ALLOC(ws_bytes ? ws_bytes : 256);
  cudaError_t e = cudaMalloc(&p->d_mem, ws_bytes ? ws_bytes : 256);
  if (e != cudaSuccess) {
    pp::set_error("pp_batch_create: %zu bytes of workspace: %s", ws_bytes, cudaGetErrorString(e));
    delete p;
    return PP_E_NOMEM;
  }
  fr *ws = static_cast<fr *>(p->d_mem);
  std::vector<std::vector<pp::PassArgs>> pass_args(subs.size());
  std::vector<std::vector<uint64_t>> pass_tiles(subs.size());
  uint32_t nlevels = 0;
  for (size_t i = 0; i < subs.size(); ++i) {
    auto &t = subs[i];
    const int st = pp::ntt_describe(t.in, t.out, ws + ws_off[i], t.lg, t.inverse, t.desc, pass_args[i],
                                    pass_tiles[i]);
    if (st) {
      cudaFree(p->d_mem);
      delete p;
      return st;
    }
    t.passes = (uint32_t)pass_args[i].size();
    t.start_level = t.start_level == 0xffffffffu ? subs[i - 1].start_level + subs[i - 1].passes : 0;
    nlevels = std::max(nlevels, t.start_level + t.passes);
  }
  // ---- per-level descriptor arrays
  std::vector<std::vector<pp::PassArgs>> lv_args(nlevels);
  std::vector<std::vector<uint64_t>> lv_start(nlevels);
  for (size_t i = 0; i < subs.size(); ++i)
    for (uint32_t q = 0; q < subs[i].passes; ++q) {
      const uint32_t L = subs[i].start_level + q;
      if (lv_start[L].empty()) lv_start[L].push_back(0);
      lv_args[L].push_back(pass_args[i][q]);
      lv_start[L].push_back(lv_start[L].back() + pass_tiles[i][q]);
    }
  std::vector<pp::GpBatchJob> gj(gps.size());
  std::vector<uint32_t> gstart(1, 0);
  for (size_t i = 0; i < gps.size(); ++i) {
    gj[i] = {gps[i].in, gps[i].out, gg[i], ws + gp_off[i], ws + gp_off[i] + gg[i].threads};
    gstart.push_back(gstart.back() + gg[i].blocks);
  }
  size_t desc_bytes = 0;
  desc_bytes += pp::align_up(gj.size() * sizeof(pp::GpBatchJob), 256) +
                pp::align_up(gstart.size() * sizeof(uint32_t), 256);
  char *d_desc = nullptr;
  PP_COUNT_ALLOC(desc_bytes ? desc_bytes : 256);
  e = cudaMalloc(reinterpret_cast<void **>(&d_desc), desc_bytes ? desc_bytes : 256);
  if (e != cudaSuccess) {
    cudaFree(p->d_mem);
    pp::set_error("pp_batch_create: descriptors: %s", cudaGetErrorString(e));
    delete p;
    return PP_E_NOMEM;
  }
  p->d_desc = d_desc;
  size_t off = 0;
  auto put = [&](const void *src, size_t bytes) -> void * {
    void *dst = d_desc + off;
    if (bytes) cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    off += pp::align_up(bytes, 256);
    return dst;
  };
  for (uint32_t L = 0; L < nlevels; ++L) {
    pp::BatchPlan::Level lv;
    const size_t count = lv_args[L].size();
    for (size_t j0 = 0; j0 < count; j0 += pp::kLevelJobs) {
      const size_t j1 = std::min(count, j0 + (size_t)pp::kLevelJobs);
      pp::LevelParams c;
      std::memset(&c, 0, sizeof(c));
      c.count = (uint32_t)(j1 - j0);
      for (size_t j = j0; j < j1; ++j) {
        c.args[j - j0] = lv_args[L][j];
        c.tile_start[j - j0] = lv_start[L][j] - lv_start[L][j0];
      }
      c.total_tiles = lv_start[L][j1] - lv_start[L][j0];
      lv.chunks.push_back(c);
      ++p->launches;
    }
    p->tiles += lv_start[L].back();
    p->levels.push_back(std::move(lv));
  }
  p->gp_count = (uint32_t)gj.size();
  p->gp_blocks = gstart.back();
  p->d_gp = static_cast<pp::GpBatchJob *>(put(gj.data(), gj.size() * sizeof(pp::GpBatchJob)));
  p->d_gp_start = static_cast<uint32_t *>(put(gstart.data(), gstart.size() * sizeof(uint32_t)));
  if (p->gp_count) p->launches += 2;
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    pp::set_error("pp_batch_create: %s", cudaGetErrorString(e));
    cudaFree(d_desc);
    cudaFree(p->d_mem);
    delete p;
    return PP_E_CUDA;
  }
  *plan_out = p;
  return PP_OK;
}

namespace {
pp::BatchPlan *unwrap(void *plan) { return static_cast<pp::BatchPlan *>(plan); }
}  // namespace

extern "C" int pp_batch_run(void *plan, void *stream) {
  pp::BatchPlan *p = unwrap(plan);
  if (!p) {
    pp::set_error("pp_batch_run: null plan");
    return PP_E_INVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (p->exec) {
    PP_CUDA_TRY(cudaGraphLaunch(p->exec, s));
    return PP_OK;
  }
  return pp::run_plan(p, s);
}

extern "C" int pp_batch_capture(void *plan) {
  pp::BatchPlan *p = unwrap(plan);
  if (!p) {
    pp::set_error("pp_batch_capture: null plan");
    return PP_E_INVAL;
  }
  if (p->exec) return PP_OK;
  cudaStream_t s;
  PP_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  int st = PP_OK;
  if (e == cudaSuccess) st = pp::run_plan(p, s);
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(s, &g);
  cudaStreamDestroy(s);
  if (e != cudaSuccess || e2 != cudaSuccess || st) {
    if (g) cudaGraphDestroy(g);
    if (st) return st;
    pp::set_error("pp_batch_capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    return PP_E_CUDA;
  }
  e = cudaGraphInstantiate(&p->exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    p->exec = nullptr;
    pp::set_error("pp_batch_capture: instantiate: %s", cudaGetErrorString(e));
    return PP_E_CUDA;
  }
  p->graph = g;
  return PP_OK;
}

extern "C" int pp_batch_info(void *plan, uint32_t *launches, uint64_t *tiles, uint32_t *levels) {
  pp::BatchPlan *p = unwrap(plan);
  if (!p) return PP_E_INVAL;
  if (launches) *launches = p->launches;
  if (tiles) *tiles = p->tiles;
  if (levels) *levels = (uint32_t)p->levels.size();
  return PP_OK;
}

extern "C" int pp_batch_destroy(void *plan) {
  if (!plan) return PP_OK;
  pp::BatchPlan *p = unwrap(plan);
  cudaDeviceSynchronize();
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  cudaFree(p->d_desc);
  cudaFree(p->d_mem);
  delete p;
  return PP_OK;
}
