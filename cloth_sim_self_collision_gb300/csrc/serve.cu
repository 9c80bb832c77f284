// serve.cu -- continuous batching of cloth scenes on one GPU (the cs_server_*
// entry points of include/clothgpu.h).
//
// One worker thread owns a context whose arena holds every admitted scene and
// advances all unfinished ones together, one frame (StepTime,
// self_contact_sparse/main.cpp:213-263) per loop.  Scenes that arrive while
// frames run are packed, together with the unfinished resident ones, into a
// new arena by a builder thread on its own stream (host packing and upload
// overlap the frames); at the next frame boundary the worker copies the
// resident scenes' positions and velocities into the new arena on the device
// and swaps it in.  Finished scenes stay in the arena, masked out of the
// kernels, until the next swap drops them.  Admission is first come, first
// served by estimated device bytes: the arena being stepped plus the one being
// built stay within the budget.  A scene's frames compute exactly what they
// compute alone: every reduction, sort and schedule is per cloth.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include "ctx.h"

using namespace cs;
using namespace cs::host;

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

struct Request {
  int id = 0;
  std::unique_ptr<Cloth> cloth;  // until it is handed to the context
  int cloth_id = -1;             // its id inside the context once packed
  size_t bytes = 0;
  int np = 0, nsteps = 0, steps_done = 0;
  int status = CS_OK;
  bool in_arena = false, done = false;
  double t_submit = 0, t_admit = -1, t_first = -1, t_done = -1;
  std::vector<float> step_ms;
  std::vector<double> x, v;  // final state
};

// an arena being packed by the builder thread
struct Build {
  std::thread th;
  std::atomic<bool> ready{false};
  ArenaSet set;
  std::vector<int> members;  // request ids in slot order
  size_t bytes = 0;
  int status = CS_OK;
  std::string err;
  double ms = 0;
};

double percentile(std::vector<float> v, double q) {
  if (v.empty()) return 0.0;
  const size_t k = std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5));
  std::nth_element(v.begin(), v.begin() + k, v.end());
  return v[k];
}

}  // namespace

struct cs_server {
  cs_server_config cfg{};
  cs_ctx* ctx = nullptr;
  cudaStream_t build_stream = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int> queue;  // submitted, not yet packed
  std::map<int, std::unique_ptr<Request>> reqs;
  int next_req = 0;
  std::vector<int> slots;  // arena slot -> request id
  std::unique_ptr<Build> build;
  size_t arena_bytes = 0, peak_bytes = 0;
  std::thread worker;
  bool stop = false;
  int fatal = CS_OK;
  std::string err;
  Clock::time_point t0;
  long long frames = 0, vsteps = 0;
  int rebuilds = 0, submitted = 0, finished = 0, diverged = 0;
  double busy_s = 0, build_ms = 0, install_ms = 0;
  std::vector<float> samples, admit_ms;
};

namespace {

// Starts packing the next arena when scenes wait (or when finished scenes fill
// most of the arena).  Worker thread, no build running.
void maybe_start_build(cs_server* S) {
  std::vector<int> keep, add;
  size_t total = 0;
  bool release_now = false, do_build = false;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    long long live_np = 0, dead_np = 0;
    for (int rid : S->slots) {
      const Request& r = *S->reqs[rid];
      if (r.done) {
        dead_np += r.np;
      } else {
        live_np += r.np;
        keep.push_back(rid);
        total += r.bytes;
      }
    }
    const bool compact = dead_np > 0 && dead_np >= live_np;
    if (S->queue.empty() && !compact) return;
    // the arena being stepped stays resident while the next one is packed,
    // unless nothing in it is still running
    release_now = keep.empty() && !S->slots.empty();
    const double budget = S->cfg.hbm_budget_bytes;
    const double held = keep.empty() ? 0.0 : (double)S->arena_bytes;
    while (!S->queue.empty()) {
      Request& r = *S->reqs[S->queue.front()];
      if (held + (double)(total + r.bytes) > budget) break;
      if (S->cfg.max_cloths > 0 && (int)(keep.size() + add.size()) >= S->cfg.max_cloths) break;
      add.push_back(r.id);
      total += r.bytes;
      S->queue.pop_front();
    }
    do_build = !add.empty() || (compact && !keep.empty());
    if (!do_build && !release_now) return;
  }
  if (release_now) {
    ArenaSet empty;
    install(S->ctx, empty);  // `empty` now owns the old buffers and frees them
    std::lock_guard<std::mutex> lk(S->mu);
    for (int rid : S->slots) {
      Request& r = *S->reqs[rid];
      S->ctx->cloths.erase(r.cloth_id);
      r.in_arena = false;
    }
    S->slots.clear();
    S->arena_bytes = 0;
  }
  if (!do_build) return;
  std::unique_ptr<Build> b(new Build());
  std::vector<const Cloth*> members;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (int rid : add) {
      Request& r = *S->reqs[rid];
      r.cloth->id = S->ctx->next_id++;
      r.cloth_id = r.cloth->id;
      S->ctx->cloths[r.cloth_id] = std::move(r.cloth);
    }
    for (int rid : keep) b->members.push_back(rid);
    for (int rid : add) b->members.push_back(rid);
    for (int rid : b->members) members.push_back(S->ctx->cloths[S->reqs[rid]->cloth_id].get());
    b->bytes = total;
    S->peak_bytes = std::max(S->peak_bytes, S->arena_bytes + total);
  }
  Build* bp = b.get();
  const int device = S->cfg.device;
  cudaStream_t bs = S->build_stream;
  b->th = std::thread([S, bp, members, device, bs] {
    const Clock::time_point t = Clock::now();
    try {
      CK(cudaSetDevice(device));
      build_arena(bp->set, members, bs);
      CK(cudaStreamSynchronize(bs));
    } catch (const std::exception& e) {
      bp->status = status_of(e, &bp->err);
    }
    bp->ms = 1e3 * seconds_since(t);
    bp->ready = true;
    S->cv_work.notify_all();
  });
  S->build = std::move(b);
}

// Swaps a finished build in at a frame boundary.  Worker thread.
void install_build(cs_server* S) {
  Build& b = *S->build;
  b.th.join();
  if (b.status != CS_OK) {
    // the scenes that were to join fail; the resident ones keep running
    std::lock_guard<std::mutex> lk(S->mu);
    for (int rid : b.members) {
      Request& r = *S->reqs[rid];
      if (r.in_arena) continue;
      S->ctx->cloths.erase(r.cloth_id);
      r.status = b.status;
      r.done = true;
      r.t_done = seconds_since(S->t0);
      S->finished++;
    }
    S->err = b.err;
    S->build.reset();
    S->cv_done.notify_all();
    return;
  }
  const Clock::time_point t = Clock::now();
  cs_ctx* c = S->ctx;
  std::map<int, int> old_slot;
  for (size_t i = 0; i < S->slots.size(); i++) old_slot[S->slots[i]] = (int)i;
  for (size_t j = 0; j < b.members.size(); j++) {
    auto it = old_slot.find(b.members[j]);
    if (it == old_slot.end()) continue;
    const int i = it->second;
    const size_t n = 3 * (size_t)(c->voff[i + 1] - c->voff[i]);
    CK(cudaMemcpyAsync(b.set.A.x + 3 * (size_t)b.set.voff[j], c->A.x + 3 * (size_t)c->voff[i],
                       sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(b.set.A.v + 3 * (size_t)b.set.voff[j], c->A.v + 3 * (size_t)c->voff[i],
                       sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  install(c, b.set);
  b.set.mem.release();
  b.set.cmem.release();
  std::lock_guard<std::mutex> lk(S->mu);
  const double now = seconds_since(S->t0);
  std::map<int, int> in_new;
  for (int rid : b.members) in_new[rid] = 1;
  for (int rid : S->slots)
    if (!in_new.count(rid)) {
      Request& r = *S->reqs[rid];
      c->cloths.erase(r.cloth_id);
      r.in_arena = false;
    }
  for (int rid : b.members) {
    Request& r = *S->reqs[rid];
    r.in_arena = true;
    if (r.t_admit < 0) r.t_admit = now;
  }
  S->slots = b.members;
  S->arena_bytes = b.bytes;
  S->rebuilds++;
  S->build_ms += b.ms;
  S->install_ms += 1e3 * seconds_since(t);
  S->build.reset();
}

void fail_all(cs_server* S, int status, const std::string& msg) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->fatal = status;
  S->err = msg;
  for (auto& kv : S->reqs) {
    Request& r = *kv.second;
    if (r.done) continue;
    r.status = status;
    r.done = true;
    r.t_done = seconds_since(S->t0);
    S->finished++;
  }
  S->queue.clear();
  S->cv_done.notify_all();
}

void worker_main(cs_server* S) {
  try {
    CK(cudaSetDevice(S->cfg.device));
    for (;;) {
      if (S->build && S->build->ready) install_build(S);
      if (!S->build) maybe_start_build(S);
      std::vector<int> act(S->slots.size(), 0);
      bool any = false;
      {
        std::unique_lock<std::mutex> lk(S->mu);
        if (S->stop) break;
        for (size_t i = 0; i < S->slots.size(); i++) {
          act[i] = !S->reqs[S->slots[i]]->done;
          any |= act[i] != 0;
        }
        if (!any) {
          S->cv_work.wait_for(lk, std::chrono::milliseconds(2));
          continue;
        }
      }
      const Clock::time_point t = Clock::now();
      const double t_start = seconds_since(S->t0);
      frame(S->ctx, act);
      CK(cudaStreamSynchronize(S->ctx->stream));
      const float ms = (float)(1e3 * seconds_since(t));
      // final states of the scenes that finished with this frame (a scene that
      // blew up ends here with CS_ERR_DIVERGED)
      std::vector<int> fin;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        for (size_t i = 0; i < act.size(); i++)
          if (act[i] && !S->ctx->dead[i] && S->reqs[S->slots[i]]->steps_done + 1 == S->reqs[S->slots[i]]->nsteps)
            fin.push_back((int)i);
      }
      std::map<int, std::pair<std::vector<double>, std::vector<double>>> states;
      for (int i : fin) {
        const size_t n = 3 * (size_t)(S->ctx->voff[i + 1] - S->ctx->voff[i]);
        auto& st = states[i];
        st.first.resize(n);
        st.second.resize(n);
        CK(cudaMemcpyAsync(st.first.data(), S->ctx->A.x + 3 * (size_t)S->ctx->voff[i], sizeof(double) * n,
                           cudaMemcpyDeviceToHost, S->ctx->stream));
        CK(cudaMemcpyAsync(st.second.data(), S->ctx->A.v + 3 * (size_t)S->ctx->voff[i], sizeof(double) * n,
                           cudaMemcpyDeviceToHost, S->ctx->stream));
      }
      if (!fin.empty()) CK(cudaStreamSynchronize(S->ctx->stream));
      std::lock_guard<std::mutex> lk(S->mu);
      const double now = seconds_since(S->t0);
      S->frames++;
      S->busy_s += ms * 1e-3;
      for (size_t i = 0; i < act.size(); i++) {
        if (!act[i]) continue;
        Request& r = *S->reqs[S->slots[i]];
        if (r.t_first < 0) {
          r.t_first = t_start;
          S->admit_ms.push_back((float)(1e3 * (t_start - r.t_submit)));
        }
        if (S->ctx->dead[i]) {
          r.status = CS_ERR_DIVERGED;
          r.done = true;
          r.t_done = now;
          S->finished++;
          S->diverged++;
          fin.push_back((int)i);
          continue;
        }
        r.steps_done++;
        r.step_ms.push_back(ms);
        S->samples.push_back(ms);
        S->vsteps += r.np;
        auto it = states.find((int)i);
        if (it != states.end()) {
          r.x = std::move(it->second.first);
          r.v = std::move(it->second.second);
          r.done = true;
          r.t_done = now;
          S->finished++;
        }
      }
      if (!fin.empty()) S->cv_done.notify_all();
    }
  } catch (const std::exception& e) {
    std::string msg;
    const int st = status_of(e, &msg);
    fail_all(S, st, msg);
  }
}

int set_err(cs_server* S, int status, const std::string& msg) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->err = msg;
  return status;
}

}  // namespace

extern "C" {

int cs_server_create(const cs_server_config* cfg, cs_server** out) {
  if (!cfg || !out) return CS_ERR_ARG;
  *out = nullptr;
  if (cfg->hbm_budget_bytes <= 0 || cfg->max_cloths < 0) return CS_ERR_ARG;
  cs_ctx* ctx = nullptr;
  const int st = cs_create(cfg->device, cfg->precision, &ctx);
  if (st != CS_OK) return st;
  // The serving arena changes at every admission and retirement, and a frame
  // graph is captured again after each change: measured at 2 scenes/s, graph
  // frames tripled the admission latency (the capture and instantiation on the
  // worker thread, the builder's packing slowed beside them) and lowered the
  // throughput.  So the worker steps host-driven frames unless
  // CLOTHGPU_FRAME_MODE=graph asks otherwise.
  {
    const char* e = std::getenv("CLOTHGPU_FRAME_MODE");
    if (!e || std::strcmp(e, "graph") != 0) cs_set_frame_mode(ctx, CS_FRAME_HOST);
  }
  cs_server* S = new cs_server();
  S->cfg = *cfg;
  S->ctx = ctx;
  if (cudaStreamCreateWithFlags(&S->build_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cs_destroy(ctx);
    delete S;
    return CS_ERR_CUDA;
  }
  S->t0 = Clock::now();
  S->worker = std::thread(worker_main, S);
  *out = S;
  return CS_OK;
}

int cs_server_submit(cs_server* S, int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                     const int* quad, const double* x, const double* v, const cs_params* prm, int nsteps,
                     int* req) {
  if (!S) return CS_ERR_ARG;
  if (nsteps <= 0) return set_err(S, CS_ERR_ARG, "cs_server_submit: nsteps must be positive");
  std::unique_ptr<Request> r(new Request());
  try {
    r->cloth = make_cloth(np, X0, bc, nt, tri, nq, quad, prm);
  } catch (const std::exception& e) {
    std::string msg;
    const int st = status_of(e, &msg);
    return set_err(S, st, "cs_server_submit: " + msg);
  }
  if (x) r->cloth->x.assign(x, x + 3 * (size_t)np);
  if (v) r->cloth->v.assign(v, v + 3 * (size_t)np);
  r->bytes = cloth_device_bytes(r->cloth->topo);
  r->np = np;
  r->nsteps = nsteps;
  if ((double)r->bytes > S->cfg.hbm_budget_bytes)
    return set_err(S, CS_ERR_CAPACITY, "cs_server_submit: the scene needs " + std::to_string(r->bytes) +
                                           " device bytes, more than the budget");
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->fatal != CS_OK) return S->fatal;
    r->id = S->next_req++;
    r->t_submit = seconds_since(S->t0);
    if (req) *req = r->id;
    S->queue.push_back(r->id);
    S->reqs[r->id] = std::move(r);
    S->submitted++;
  }
  S->cv_work.notify_all();
  return CS_OK;
}

int cs_server_wait(cs_server* S, int req, double timeout_s, double* x, double* v, cs_request_info* info) {
  if (!S) return CS_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(req);
  if (it == S->reqs.end()) {
    S->err = "cs_server_wait: unknown request " + std::to_string(req);
    return CS_ERR_ARG;
  }
  Request& r = *it->second;
  const auto pred = [&] { return r.done; };
  if (timeout_s < 0)
    S->cv_done.wait(lk, pred);
  else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
    return CS_ERR_TIMEOUT;
  if (r.status == CS_OK) {
    if (x) std::copy(r.x.begin(), r.x.end(), x);
    if (v) std::copy(r.v.begin(), r.v.end(), v);
  }
  if (info) {
    info->np = r.np;
    info->nsteps = r.nsteps;
    info->steps_done = r.steps_done;
    info->status = r.status;
    info->t_submit = r.t_submit;
    info->t_admit = r.t_admit;
    info->t_first_frame = r.t_first;
    info->t_done = r.t_done;
    info->step_ms_p50 = percentile(r.step_ms, 0.50);
    info->step_ms_p99 = percentile(r.step_ms, 0.99);
  }
  return r.status;
}

int cs_server_release(cs_server* S, int req) {
  if (!S) return CS_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(req);
  if (it == S->reqs.end() || !it->second->done) {
    S->err = "cs_server_release: unknown or unfinished request " + std::to_string(req);
    return CS_ERR_ARG;
  }
  std::vector<double>().swap(it->second->x);
  std::vector<double>().swap(it->second->v);
  return CS_OK;
}

int cs_server_drain(cs_server* S, double timeout_s) {
  if (!S) return CS_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  const auto pred = [&] { return S->finished == S->submitted; };
  if (timeout_s < 0)
    S->cv_done.wait(lk, pred);
  else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
    return CS_ERR_TIMEOUT;
  return S->fatal;
}

int cs_server_get_stats(cs_server* S, cs_server_stats* st) {
  if (!S || !st) return CS_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(st, 0, sizeof(*st));
  st->frames = S->frames;
  st->vertex_steps = S->vsteps;
  st->submitted = S->submitted;
  st->finished = S->finished;
  st->queued = (int)S->queue.size();
  for (int rid : S->slots) st->resident += S->reqs[rid]->done ? 0 : 1;
  st->rebuilds = S->rebuilds;
  st->diverged = S->diverged;
  st->elapsed_s = seconds_since(S->t0);
  st->busy_s = S->busy_s;
  st->step_ms_p50 = percentile(S->samples, 0.50);
  st->step_ms_p99 = percentile(S->samples, 0.99);
  st->step_ms_max = S->samples.empty() ? 0.0 : *std::max_element(S->samples.begin(), S->samples.end());
  st->admit_ms_p50 = percentile(S->admit_ms, 0.50);
  st->admit_ms_p99 = percentile(S->admit_ms, 0.99);
  st->build_ms_total = S->build_ms;
  st->install_ms_total = S->install_ms;
  st->arena_bytes = (double)S->arena_bytes;
  st->peak_bytes = (double)S->peak_bytes;
  return S->fatal;
}

const char* cs_server_last_error(cs_server* S) { return S ? S->err.c_str() : "null server"; }

void cs_server_destroy(cs_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  if (S->build && S->build->th.joinable()) S->build->th.join();
  S->build.reset();
  cudaSetDevice(S->cfg.device);
  cs_destroy(S->ctx);
  cudaStreamDestroy(S->build_stream);
  delete S;
}

size_t cs_scene_device_bytes(int np, const double* X0, int nt, const int* tri, int nq, const int* quad,
                             const cs_params* prm) {
  try {
    return cloth_device_bytes(make_cloth(np, X0, nullptr, nt, tri, nq, quad, prm)->topo);
  } catch (const std::exception&) {
    return 0;
  }
}

}  // extern "C"
