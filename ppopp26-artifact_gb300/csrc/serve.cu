// serve.cu -- continuous-batching request loop for prover-round bundles.
//
// A bundle is the operator work of one PLONK prover round on polynomials of
// 2^lg_n coefficients:
//   3 coset LDEs of the wire polynomials (coefficients in, 2^lambda blowup),
//   the copy-constraint grand product z over the wires and sigmas,
//   one division by (X + c) (the quotient of an opening),
//   6 evaluations (the 3 wires and 3 sigmas at 6 points).
// A scheduler thread owns `slots` CUDA streams.  Submitted bundles wait in a
// FIFO queue; whenever a slot is free, the bundle's device memory fits in the
// HBM budget and (with max_inflight_mm) the estimated work of the running
// bundles leaves room for it, the bundle is admitted: its buffers come from a stream-
// ordered memory pool, its inputs are generated on the device from its seed
// or copied from pinned host memory, and its kernels are queued on the
// slot's stream, so bundles admitted while others run overlap on the GPU.
// Twiddle / coset tables and per-stream workspaces are built once at start
// and stay resident.  A bundle's results stay on the device until the client
// releases them; the memory returns to the budget then.  Every wait is
// bounded (PP_E_TIMEOUT), nothing spins on the GPU.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "ntt.cuh"
#include "scan.cuh"

namespace pp {
namespace {

using Clock = std::chrono::steady_clock;

double now_ms() {
  return std::chrono::duration<double, std::milli>(Clock::now().time_since_epoch()).count();
}

struct Bundle {
  uint64_t ticket = 0;
  pp_bundle req{};
  int status = PP_OK;
  enum State { QUEUED, RUNNING, DONE, CANCELLED } state = QUEUED;
  double t_submit = 0, t_start = 0, t_done = 0;
  int slot = -1;
  size_t bytes = 0;
  uint64_t work = 0;    // pp_bundle_work
  void *mem = nullptr;  // one allocation: inputs, params, results
  cudaEvent_t done_ev = nullptr;
  // views into mem
  fr *w[3] = {nullptr, nullptr, nullptr}, *sigma[3] = {nullptr, nullptr, nullptr};
  fr *divp = nullptr, *params = nullptr, *lde[3] = {nullptr, nullptr, nullptr}, *z = nullptr,
     *evals = nullptr;
};

size_t bundle_bytes(uint32_t lg, uint32_t lambda) {
  const size_t n = size_t{1} << lg;
  // w[3], sigma[3], div poly, params (16 slots), lde[3] (n << lambda), z, evals (6 -> 8)
  return (7 * n + 16 + 3 * (n << lambda) + n + 8) * sizeof(fr);
}

}  // namespace

struct Server {
  pp_server_config cfg{};
  int dev = 0;
  std::vector<cudaStream_t> streams;
  std::vector<uint64_t> slot_owner;  // ticket running on the slot, 0 = free
  cudaMemPool_t pool = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::map<uint64_t, Bundle> bundles;
  uint64_t next_ticket = 1;
  size_t budget_used = 0, budget_peak = 0;
  uint64_t inflight_work = 0;  // estimated multiplies of the running bundles
  std::atomic<bool> stop{false};
  std::thread worker;
  std::vector<double> latencies;
  double first_submit = 0, last_done = 0;
  uint64_t completed = 0, admitted_while_busy = 0, max_concurrent = 0;
  int fatal = PP_OK;
};

namespace {

// queue the bundle's work on its slot stream; called with the lock held
int launch_bundle(Server *S, Bundle &b) {
  cudaStream_t s = S->streams[b.slot];
  const uint32_t lg = b.req.lg_n, lam = b.req.lambda;
  const size_t n = size_t{1} << lg;
  PP_COUNT_ALLOC(b.bytes);
  cudaError_t e = cudaMallocFromPoolAsync(&b.mem, b.bytes, S->pool, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("bundle %llu: %zu bytes from the pool: %s", (unsigned long long)b.ticket, b.bytes,
              cudaGetErrorString(e));
    return PP_E_NOMEM;
  }
  fr *p = static_cast<fr *>(b.mem);
  for (int j = 0; j < 3; ++j) b.w[j] = p + j * n;
  for (int j = 0; j < 3; ++j) b.sigma[j] = p + (3 + j) * n;
  b.divp = p + 6 * n;
  b.params = p + 7 * n;  // beta, gamma, k1, k2, k3, c, z1..z6 (12 used)
  fr *q = b.params + 16;
  for (int j = 0; j < 3; ++j) b.lde[j] = q + j * (n << lam);
  b.z = q + 3 * (n << lam);
  b.evals = b.z + n;
  int st = PP_OK;
  if (b.req.h_inputs) {
    e = cudaMemcpyAsync(p, b.req.h_inputs, 7 * n * sizeof(fr), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return PP_E_CUDA;
  } else {
    st = pp_random_fr(p, 7 * n, b.req.seed, 0, s);
    if (st) return st;
  }
  if (b.req.h_params) {
    e = cudaMemcpyAsync(b.params, b.req.h_params, 12 * sizeof(fr), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return PP_E_CUDA;
  } else {
    st = pp_random_fr(b.params, 12, b.req.seed ^ 0x9a7a9a7aull, 0, s);
    if (st) return st;
  }
  for (int j = 0; j < 3 && !st; ++j) st = pp_lde(b.w[j], b.lde[j], lg, lam, PP_LDE_COEFFS, s);
  const void *wp[3] = {b.w[0], b.w[1], b.w[2]};
  const void *sp[3] = {b.sigma[0], b.sigma[1], b.sigma[2]};
  if (!st) st = pp_gp_perm(wp, sp, b.params, b.z, lg, s);
  if (!st) st = pp_div_xplusc(b.divp, n, b.params + 5, s);
  for (int k = 0; k < 6 && !st; ++k) {
    const fr *poly = k < 3 ? b.w[k] : b.sigma[k - 3];
    st = pp_eval(poly, n, b.params + 6 + k, b.evals + k, s);
  }
  if (st) return st;
  e = cudaEventRecord(b.done_ev, s);
  return e == cudaSuccess ? PP_OK : PP_E_CUDA;
}

void worker_loop(Server *S) {
  cudaSetDevice(S->dev);
  std::unique_lock<std::mutex> lk(S->mu);
  while (!S->stop.load()) {
    // 1. completions
    for (size_t sl = 0; sl < S->slot_owner.size(); ++sl) {
      const uint64_t t = S->slot_owner[sl];
      if (!t) continue;
      Bundle &b = S->bundles[t];
      const cudaError_t q = cudaEventQuery(b.done_ev);
      if (q == cudaErrorNotReady) continue;
      b.t_done = now_ms();
      b.status = q == cudaSuccess ? PP_OK : PP_E_CUDA;
      if (q != cudaSuccess) {
        cudaGetLastError();
        S->fatal = PP_E_CUDA;
      }
      b.state = Bundle::DONE;
      S->slot_owner[sl] = 0;
      S->inflight_work -= b.work;
      S->latencies.push_back(b.t_done - b.t_submit);
      S->last_done = b.t_done;
      ++S->completed;
      S->cv_done.notify_all();
    }
    // 2. admissions (FIFO: the head waits for memory rather than being overtaken)
    while (!S->queue.empty()) {
      int free_slot = -1;
      for (size_t sl = 0; sl < S->slot_owner.size(); ++sl)
        if (!S->slot_owner[sl]) {
          free_slot = (int)sl;
          break;
        }
      if (free_slot < 0) break;
      Bundle &b = S->bundles[S->queue.front()];
      if (b.state == Bundle::CANCELLED) {
        S->queue.pop_front();
        continue;
      }
      if (S->budget_used + b.bytes > S->cfg.budget_bytes) break;
      size_t busy = 0;
      for (auto o : S->slot_owner) busy += o != 0;
      // the work cap holds the head back while others run (never when idle)
      if (busy && S->cfg.max_inflight_mm && S->inflight_work + b.work > S->cfg.max_inflight_mm) break;
      S->queue.pop_front();
      if (busy) ++S->admitted_while_busy;
      S->max_concurrent = std::max<uint64_t>(S->max_concurrent, busy + 1);
      b.slot = free_slot;
      b.t_start = now_ms();
      S->budget_used += b.bytes;
      S->inflight_work += b.work;
      S->budget_peak = std::max(S->budget_peak, S->budget_used);
      const int st = launch_bundle(S, b);
      if (st) {
        // the work may be partly queued: wait for the slot's stream before
        // giving the memory back, then report the failure on this bundle
        cudaStreamSynchronize(S->streams[b.slot]);
        if (b.mem) cudaFreeAsync(b.mem, S->streams[b.slot]);
        b.mem = nullptr;
        S->budget_used -= b.bytes;
        S->inflight_work -= b.work;
        b.status = st;
        b.state = Bundle::DONE;
        b.t_done = now_ms();
        S->cv_done.notify_all();
        continue;
      }
      b.state = Bundle::RUNNING;
      S->slot_owner[free_slot] = b.ticket;
    }
    S->cv_work.wait_for(lk, std::chrono::microseconds(50));
  }
}

}  // namespace
}  // namespace pp

using pp::Server;

extern "C" uint64_t pp_bundle_work(uint32_t lg_n, uint32_t lambda) {
  const uint64_t n = 1ull << lg_n, lg_m = lg_n + lambda;
  const uint64_t lde = ((n << lambda) / 2) * lg_m + n;  // coset transform + the diagonal
  return 3 * lde + 16 * n + n + 6 * n;
}

extern "C" int pp_server_create(const pp_server_config *cfg, void **srv) {
  if (!cfg || !srv || cfg->slots == 0 || cfg->slots > 64 || cfg->min_lg > cfg->max_lg ||
      cfg->max_lg + cfg->lambda > 28) {
    pp::set_error("pp_server_create: bad configuration");
    return PP_E_INVAL;
  }
  *srv = nullptr;
  auto *S = new Server();
  S->cfg = *cfg;
  PP_CUDA_TRY(cudaGetDevice(&S->dev));
  // resident tables for every size this server accepts
  for (uint32_t lg = cfg->min_lg; lg <= cfg->max_lg; ++lg) {
    int st = pp::ntt_prepare(lg + cfg->lambda, false);
    const pp::fr h = pp::host_pow(pp::host_mont_small(7), 1ull << cfg->lambda);
    if (!st) pp::pow_table(h, lg, &st);
    if (!st) pp::pow_table(pp::host_root_of_unity((int)lg, false), lg, &st);
    if (st) {
      delete S;
      return st;
    }
  }
  S->streams.resize(cfg->slots);
  S->slot_owner.assign(cfg->slots, 0);
  const size_t nmax = size_t{1} << (cfg->max_lg + cfg->lambda);
  // the grand product of the largest bundle needs the most scan workspace
  const size_t npoly = size_t{1} << cfg->max_lg;
  const pp::ScanGeom sg = pp::scan_geom(npoly);
  const size_t scan_elems = 2 * npoly + sg.threads + sg.blocks;
  for (uint32_t i = 0; i < cfg->slots; ++i) {
    PP_CUDA_TRY(cudaStreamCreateWithFlags(&S->streams[i], cudaStreamNonBlocking));
    int st = PP_OK;
    pp::workspace_get(nmax * sizeof(pp::fr), S->streams[i], 0, &st);
    if (!st) pp::workspace_get(scan_elems * sizeof(pp::fr), S->streams[i], 1, &st);
    if (st) {
      delete S;
      return st;
    }
  }
  PP_CUDA_TRY(cudaDeviceGetDefaultMemPool(&S->pool, S->dev));
  uint64_t keep = cfg->budget_bytes;
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  PP_CUDA_TRY(cudaDeviceSynchronize());
  S->worker = std::thread(pp::worker_loop, S);
  *srv = S;
  return PP_OK;
}

extern "C" int pp_server_submit(void *srv, const pp_bundle *req, uint64_t *ticket) {
  Server *S = static_cast<Server *>(srv);
  if (!S || !req || !ticket) return PP_E_INVAL;
  if (req->lg_n < S->cfg.min_lg || req->lg_n > S->cfg.max_lg || req->lambda != S->cfg.lambda) {
    pp::set_error("pp_server_submit: bundle of 2^%u (lambda %u) outside this server's range", req->lg_n,
                  req->lambda);
    return PP_E_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->fatal) return S->fatal;
  const size_t bytes = pp::bundle_bytes(req->lg_n, req->lambda);
  if (bytes > S->cfg.budget_bytes) {
    pp::set_error("pp_server_submit: a bundle of 2^%u needs %zu bytes, over the whole budget", req->lg_n,
                  bytes);
    return PP_E_NOMEM;
  }
  if (S->queue.size() >= S->cfg.max_queue && S->cfg.max_queue) {
    pp::set_error("pp_server_submit: queue full");
    return PP_E_BUSY;
  }
  pp::Bundle b;
  b.ticket = S->next_ticket++;
  b.req = *req;
  b.bytes = bytes;
  b.work = pp_bundle_work(req->lg_n, req->lambda);
  b.t_submit = pp::now_ms();
  if (S->first_submit == 0) S->first_submit = b.t_submit;
  cudaError_t e = cudaEventCreateWithFlags(&b.done_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return PP_E_CUDA;
  *ticket = b.ticket;
  S->bundles[b.ticket] = b;
  S->queue.push_back(b.ticket);
  S->cv_work.notify_one();
  return PP_OK;
}

extern "C" int pp_server_wait(void *srv, uint64_t ticket, int timeout_ms, pp_bundle_result *out) {
  Server *S = static_cast<Server *>(srv);
  if (!S) return PP_E_INVAL;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->bundles.find(ticket);
  if (it == S->bundles.end()) return PP_E_INVAL;
  const bool ok = S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
    const auto st = S->bundles[ticket].state;
    return st == pp::Bundle::DONE || st == pp::Bundle::CANCELLED;
  });
  pp::Bundle &b = S->bundles[ticket];
  if (!ok) {
    pp::set_error("pp_server_wait: bundle %llu not done after %d ms", (unsigned long long)ticket,
                  timeout_ms);
    return PP_E_TIMEOUT;
  }
  if (b.state == pp::Bundle::CANCELLED) return PP_E_CANCELLED;
  if (out) {
    out->ticket = b.ticket;
    out->status = b.status;
    out->latency_ms = b.t_done - b.t_submit;
    out->queue_ms = b.t_start - b.t_submit;
    for (int j = 0; j < 3; ++j) out->d_lde[j] = b.lde[j];
    out->d_z = b.z;
    out->d_quotient = b.divp;
    out->d_evals = b.evals;
    for (int j = 0; j < 3; ++j) {
      out->d_w[j] = b.w[j];
      out->d_sigma[j] = b.sigma[j];
    }
    out->d_params = b.params;
  }
  return b.status;
}

extern "C" int pp_server_release(void *srv, uint64_t ticket) {
  Server *S = static_cast<Server *>(srv);
  if (!S) return PP_E_INVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->bundles.find(ticket);
  if (it == S->bundles.end()) return PP_E_INVAL;
  pp::Bundle &b = it->second;
  if (b.state == pp::Bundle::QUEUED || b.state == pp::Bundle::RUNNING) {
    pp::set_error("pp_server_release: bundle %llu is not finished", (unsigned long long)ticket);
    return PP_E_BUSY;
  }
  if (b.mem) {
    cudaFreeAsync(b.mem, S->streams[b.slot]);
    S->budget_used -= b.bytes;
  }
  if (b.done_ev) cudaEventDestroy(b.done_ev);
  S->bundles.erase(it);
  S->cv_work.notify_one();
  return PP_OK;
}

extern "C" int pp_server_cancel(void *srv, uint64_t ticket) {
  Server *S = static_cast<Server *>(srv);
  if (!S) return PP_E_INVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->bundles.find(ticket);
  if (it == S->bundles.end()) return PP_E_INVAL;
  if (it->second.state != pp::Bundle::QUEUED) return PP_E_BUSY;
  it->second.state = pp::Bundle::CANCELLED;
  S->cv_done.notify_all();
  return PP_OK;
}

extern "C" int pp_server_get_stats(void *srv, pp_server_stats *out) {
  Server *S = static_cast<Server *>(srv);
  if (!S || !out) return PP_E_INVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(out, 0, sizeof(*out));
  out->completed = S->completed;
  out->queued = S->queue.size();
  out->budget_used = S->budget_used;
  out->budget_peak = S->budget_peak;
  out->admitted_while_busy = S->admitted_while_busy;
  out->max_concurrent = S->max_concurrent;
  if (!S->latencies.empty()) {
    std::vector<double> l = S->latencies;
    std::sort(l.begin(), l.end());
    out->p50_ms = l[(l.size() - 1) / 2];
    out->p99_ms = l[(size_t)((l.size() - 1) * 0.99)];
    const double span = S->last_done - S->first_submit;
    out->bundles_per_s = span > 0 ? 1e3 * (double)S->completed / span : 0;
  }
  return PP_OK;
}

extern "C" int pp_server_reset_stats(void *srv) {
  Server *S = static_cast<Server *>(srv);
  if (!S) return PP_E_INVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  S->latencies.clear();
  S->completed = 0;
  S->first_submit = 0;
  S->last_done = 0;
  S->admitted_while_busy = 0;
  S->max_concurrent = 0;
  S->budget_peak = S->budget_used;
  return PP_OK;
}

extern "C" int pp_server_destroy(void *srv) {
  Server *S = static_cast<Server *>(srv);
  if (!S) return PP_OK;
  S->stop.store(true);
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  cudaDeviceSynchronize();
  for (auto &kv : S->bundles) {
    if (kv.second.mem) cudaFree(kv.second.mem);
    if (kv.second.done_ev) cudaEventDestroy(kv.second.done_ev);
  }
  for (auto s : S->streams) {
    pp::workspace_release_stream(s);
    cudaStreamDestroy(s);
  }
  delete S;
  return PP_OK;
}
