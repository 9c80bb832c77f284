// frame_graph.cu -- one frame (StepTime, self_contact_sparse/main.cpp:213-263)
// captured as a CUDA graph, its control flow decided on the device.
//
// The host-driven frame (api.cu: frame, resolve, detect, run_mixed, run_cg)
// reads device counters after every detection and solver cycle to decide what
// runs next.  Here those decisions are kernels: per-cloth flags in InstState
// (want, phase, applied) replace the host's vectors, FrameCtl counts the passes,
// and the loops of the reference become conditional graph nodes:
//   * the refinement cycles of the mixed solve (at most 12) or the CG
//     iterations of the FP64 solve: WHILE nodes;
//   * up to 5 CCD impulse passes (self_collision_cloth.cpp:398-420): a WHILE node;
//   * the rigid-impact-zone passes (at most 100, :421-455): a WHILE node inside an
//     IF node that runs only when some cloth is still in contact.
// Every kernel is the one the host-driven frame launches, in the same order,
// so a graph frame equals a host-driven frame bit for bit.  Launch sizes are
// fixed at capture: counts are read on the device, and the candidate and zone
// sorts run at padded sizes chosen from the counts the host-driven frames saw.
// A count beyond a fixed size sets FrameCtl::overflow; the host then restores
// the frame's start state and re-runs it host-driven, which grows the buffers,
// and captures a new graph for the next frame.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ctx.h"

namespace cs {
namespace host {
void set_active(cs_ctx* c, const std::vector<int>& act);
void pull_states(cs_ctx* c);
void note_divergence(cs_ctx* c);
}  // namespace host

namespace {

constexpr int kCtlThreads = 256;
constexpr int kMaxCycles = 12;  // refinement cycles of the mixed solve (run_mixed)

enum ActiveFrom { kFromWant = 0, kFromPhase = 1, kFromApplied = 2, kFromWantCg = 3 };

// A.active from one of the per-cloth flags (never a cloth that blew up)
__global__ void k_ctl_active(Arena A, int from) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ni) return;
  const InstState& S = A.st[i];
  int a = from == kFromPhase ? S.phase : from == kFromApplied ? S.applied : S.want;
  if (from == kFromWantCg) a = a && A.prm[i].solver_kind == CS_SOLVER_CG;
  A.active[i] = a && !S.diverged;
}

// frame start: the host's mask becomes `want`; counters reset
__global__ void k_ctl_begin(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    FrameCtl* c = A.ctl;
    c->ccd_pass = c->riz_pass = c->cycle = 0;
    c->overflow = 0;
  }
  if (i >= A.ni) return;
  InstState& S = A.st[i];
  S.want = A.active[i];
  S.phase = S.applied = 0;
}

// start of GetIntermidiateVelocityContactResolved: every live cloth in phase,
// the frame's contact counters cleared
__global__ void k_ctl_resolve_begin(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ni) return;
  InstState& S = A.st[i];
  S.phase = S.want && !S.diverged;
  S.applied = 0;
  S.st_prx = S.st_ccd_passes = S.st_riz_passes = S.st_riz_last = S.st_riz_total = S.st_riz_nodes = 0;
  for (int k = 0; k < 5; k++) S.st_ccd[k] = 0;
}

// after the proximity detection (self_collision_cloth.cpp:386-392)
__global__ void k_ctl_after_prx(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ni) return;
  InstState& S = A.st[i];
  if (!S.want) return;
  S.st_prx = S.n_contacts;
  if (S.diverged)
    S.phase = S.applied = 0;
  else
    S.applied = S.n_contacts > 0;
}

// after a CCD detection (:398-420): counts, and cloths without contacts leave
__global__ void k_ctl_after_ccd(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ni) return;
  InstState& S = A.st[i];
  if (S.diverged) S.phase = S.applied = 0;
  if (!S.phase) return;
  const int pass = A.ctl->ccd_pass;
  S.st_ccd[pass] = S.n_contacts;
  S.st_ccd_passes = pass + 1;
  if (S.n_contacts == 0)
    S.phase = 0;
  else
    S.applied = 1;
}

// after an impact-zone detection (:421-455)
__global__ void k_ctl_after_riz(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ni) return;
  InstState& S = A.st[i];
  if (S.diverged) S.phase = S.applied = 0;
  if (!S.phase) return;
  const int n = S.n_contacts;
  S.st_riz_passes++;
  S.st_riz_last = n;
  S.st_riz_total += n;
  S.st_riz_nodes = S.riz_nodes;
  if (n == 0) S.phase = 0;
}

// one block: whether any cloth is still in phase (what 0) or active and unsolved (1)
__device__ bool any_cloth(const Arena& A, int what) {
  __shared__ int s_any;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  int mine = 0;
  for (int i = threadIdx.x; i < A.ni; i += blockDim.x) {
    const InstState& S = A.st[i];
    mine |= what == 0 ? (S.phase && !S.diverged) : (A.active[i] && !S.done);
  }
  if (mine) s_any = 1;
  __syncthreads();
  return s_any != 0;
}

__global__ void k_ctl_ccd_cond(Arena A, cudaGraphConditionalHandle h) {
  const bool any = any_cloth(A, 0);
  if (threadIdx.x == 0) {
    const int pass = ++A.ctl->ccd_pass;
    cudaGraphSetConditional(h, pass < 5 && any ? 1u : 0u);
  }
}

__global__ void k_ctl_any_phase(Arena A, cudaGraphConditionalHandle h) {
  const bool any = any_cloth(A, 0);
  if (threadIdx.x == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
}

__global__ void k_ctl_riz_cond(Arena A, cudaGraphConditionalHandle h) {
  const bool any = any_cloth(A, 0);
  if (threadIdx.x == 0) {
    const int pass = ++A.ctl->riz_pass;
    cudaGraphSetConditional(h, pass < 100 && any ? 1u : 0u);
  }
}

// mixed solve: another refinement cycle while a cloth is unsolved (run_mixed);
// a grid barrier that gave up ends the frame as an overflow (the host re-runs it)
__global__ void k_ctl_mx_cond(Arena A, cudaGraphConditionalHandle h) {
  const bool any = any_cloth(A, 1);
  if (threadIdx.x == 0) {
    FrameCtl* c = A.ctl;
    const int cyc = ++c->cycle;
    const bool gave_up = ((volatile unsigned*)A.grid_bar)[2] != 0u;
    if (gave_up) c->overflow |= kOverflowSolver;
    cudaGraphSetConditional(h, cyc < kMaxCycles && any && !gave_up ? 1u : 0u);
  }
}

__global__ void k_ctl_set_cycle(Arena A, int v) { A.ctl->cycle = v; }

// FP64 CG: the next iteration while a cloth is unsolved and below the cap (run_cg)
__global__ void k_ctl_cg_cond(Arena A, cudaGraphConditionalHandle h, int cap) {
  const bool any = any_cloth(A, 1);
  if (threadIdx.x == 0) {
    const int it = ++A.ctl->cycle;
    cudaGraphSetConditional(h, it < cap && any ? 1u : 0u);
  }
}

__global__ void k_ctl_finish(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ni) return;
  A.st[i].impulse_applied = A.st[i].applied;
}

// ---- capture helpers --------------------------------------------------------------
void ck(cudaError_t e, const char* what) { launch_check(e, what); }

cudaGraph_t capturing_graph(cudaStream_t s, const cudaGraphNode_t** deps, const cudaGraphEdgeData** edges,
                            size_t* nd) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  ck(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, deps, edges, nd), "cudaStreamGetCaptureInfo");
  if (st != cudaStreamCaptureStatusActive) throw CudaError("frame graph: stream is not capturing");
  return g;
}

// a conditional handle of the graph being captured on s
cudaGraphConditionalHandle new_handle(cudaStream_t s, unsigned defval) {
  const cudaGraphNode_t* deps;
  const cudaGraphEdgeData* edges;
  size_t nd;
  cudaGraph_t g = capturing_graph(s, &deps, &edges, &nd);
  cudaGraphConditionalHandle h;
  ck(cudaGraphConditionalHandleCreate(&h, g, defval, cudaGraphCondAssignDefault),
     "cudaGraphConditionalHandleCreate");
  return h;
}

// Appends a conditional node (WHILE or IF) with handle h to the capture on s
// and captures its body on the stream bs.
template <typename F>
void conditional(cudaStream_t s, cudaStream_t bs, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                 F&& body) {
  const cudaGraphNode_t* deps;
  const cudaGraphEdgeData* edges;
  size_t nd;
  cudaGraph_t g = capturing_graph(s, &deps, &edges, &nd);
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  ck(cudaGraphAddNode(&node, g, deps, edges, nd, &p), "cudaGraphAddNode(conditional)");
  ck(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
     "cudaStreamUpdateCaptureDependencies");
  cudaGraph_t bg = p.conditional.phGraph_out[0];
  ck(cudaStreamBeginCaptureToGraph(bs, bg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
     "cudaStreamBeginCaptureToGraph(body)");
  try {
    body(bs);
  } catch (...) {
    cudaStreamEndCapture(bs, &bg);  // leave the body stream usable
    throw;
  }
  ck(cudaStreamEndCapture(bs, &bg), "cudaStreamEndCapture(body)");
}

inline int nb(int n) { return (n + kCtlThreads - 1) / kCtlThreads; }

int pow2_at_least(long long n) {
  long long p = 1;
  while (p < n) p <<= 1;
  return (int)std::min<long long>(p, 0x40000000LL);
}

}  // namespace

namespace host {

// launches of one frame, captured on stream s (bodies on c->gstream[0..1])
void emit_frame(cs_ctx* c, cudaStream_t s) {
  Arena& A = c->A;
  ContactBufs& C = c->C;
  const int ni = A.ni;
  cudaStream_t b1 = c->gstream[0], b2 = c->gstream[1];
  auto active = [&](cudaStream_t st, int from) { k_ctl_active<<<nb(ni), kCtlThreads, 0, st>>>(A, from); };

  k_ctl_begin<<<nb(ni), kCtlThreads, 0, s>>>(A);
  ck(cudaMemcpyAsync(A.x1, A.x, sizeof(double) * 3 * (size_t)A.nv, cudaMemcpyDeviceToDevice, s), "copy x1");
  // ---- implicit step (StepTime_InternalDynamics[ILU], solve_internal_sparse.h:185-326)
  launch_elements(A, true, true, s);
  launch_slot_reduce(A, s);
  launch_rhs(A, s);
  if (c->precision == CS_PREC_MIXED) {
    launch_mx_outer_init(A, s);
    launch_mx_warm_start(A, s);
    const cudaGraphConditionalHandle h = new_handle(s, 1);
    conditional(s, b1, h, cudaGraphCondTypeWhile, [&](cudaStream_t bs) {
      launch_mx_inner_persistent(A, c->mx_eta, c->mx_cap, c->mx_blocks_per_sm, c->mx_threads, c->mx_tail_slices, bs);
      launch_mx_refine(A, -1.0, kMaxCycles, bs);
      k_ctl_mx_cond<<<1, kCtlThreads, 0, bs>>>(A, h);
    });
  } else {
    if (!c->g_ilu.empty()) {
      launch_ilu_factor(A, c->g_ilu_list, (int)c->g_ilu.size(), s, true);
      launch_pcg(A, c->g_ilu_list, (int)c->g_ilu.size(), -1.0, -1, s, true);
    }
    if (c->g_cg_cap > 1) {
      active(s, kFromWantCg);
      launch_cg_init(A, -1.0, -1, s);
      k_ctl_set_cycle<<<1, 1, 0, s>>>(A, 1);
      const cudaGraphConditionalHandle h = new_handle(s, 1);
      conditional(s, b1, h, cudaGraphCondTypeWhile, [&](cudaStream_t bs) {
        launch_cg_iteration(A, -1, -1.0, -1, c->g_cg_serial, bs);
        k_ctl_cg_cond<<<1, kCtlThreads, 0, bs>>>(A, h, c->g_cg_cap);
      });
      active(s, kFromWant);
    }
  }
  launch_finish_implicit(A, s);
  // ---- GetIntermidiateVelocityContactResolved (self_collision_cloth.cpp:355-456)
  k_ctl_resolve_begin<<<nb(ni), kCtlThreads, 0, s>>>(A);
  active(s, kFromPhase);
  detect_dev(A, C, 0, kGateAlways, -1, c->g_scand, A.x1, nullptr, s);
  k_ctl_after_prx<<<nb(ni), kCtlThreads, 0, s>>>(A);
  launch_impulses(A, C, 0, A.x1, A.v, s);
  {
    const cudaGraphConditionalHandle h = new_handle(s, 1);
    conditional(s, b1, h, cudaGraphCondTypeWhile, [&](cudaStream_t bs) {
      active(bs, kFromPhase);
      mark_dirty_dev(A, C, kGateCcdLater, -1, bs);
      detect_dev(A, C, 1, kGateCcdFirst, kGateCcdLater, c->g_scand, A.x1, A.v, bs);
      k_ctl_after_ccd<<<nb(ni), kCtlThreads, 0, bs>>>(A);
      active(bs, kFromPhase);
      launch_impulses(A, C, 1, A.x1, A.v, bs);
      k_ctl_ccd_cond<<<1, kCtlThreads, 0, bs>>>(A, h);
    });
  }
  {
    const cudaGraphConditionalHandle hif = new_handle(s, 0);
    k_ctl_any_phase<<<1, kCtlThreads, 0, s>>>(A, hif);
    conditional(s, b1, hif, cudaGraphCondTypeIf, [&](cudaStream_t bs) {
      active(bs, kFromPhase);
      ck(cudaMemcpyAsync(A.v0, A.v, sizeof(double) * 3 * (size_t)A.nv, cudaMemcpyDeviceToDevice, bs), "copy v0");
      launch_riz_reset(A, bs);
      const cudaGraphConditionalHandle h = new_handle(bs, 1);
      conditional(bs, b2, h, cudaGraphCondTypeWhile, [&](cudaStream_t ws) {
        active(ws, kFromPhase);
        mark_dirty_dev(A, C, kGateRizFirst, kGateRizLater, ws);
        detect_dev(A, C, 1, -1, kGateAlways, c->g_scand, A.x1, A.v, ws);
        launch_riz_count(A, ws);
        k_ctl_after_riz<<<nb(ni), kCtlThreads, 0, ws>>>(A);
        active(ws, kFromPhase);
        riz_add_dev(A, C, ws);
        riz_apply_dev(A, C, c->g_szone, A.x1, A.v, A.v0, ws);
        k_ctl_riz_cond<<<1, kCtlThreads, 0, ws>>>(A, h);
      });
    });
  }
  // ---- re-integration and velocity update of the cloths that got impulses
  // (self_contact_sparse/main.cpp:246-261)
  active(s, kFromApplied);
  launch_reintegrate(A, s);
  launch_elements(A, false, true, s);
  launch_update_velocity(A, s);
  k_ctl_finish<<<nb(ni), kCtlThreads, 0, s>>>(A);
  active(s, kFromWant);
}

void graph_release(cs_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  if (c->g_ilu_list) cudaFree(c->g_ilu_list);
  c->g_ilu_list = nullptr;
}

// Captures the frame graph for the current arena and contact buffers.
void graph_capture(cs_ctx* c) {
  graph_release(c);
  Arena& A = c->A;
  for (int k = 0; k < 2; k++)
    if (!c->gstream[k]) CK(cudaStreamCreateWithFlags(&c->gstream[k], cudaStreamNonBlocking));
  // padded sort sizes: four times the largest counts the frames so far saw
  // (contacts grow as cloths settle into contact, and a frame that outgrows
  // the graph costs a graph frame, a host-driven frame and a capture, far more
  // than sorting padded keys), at least CLOTHGPU_GRAPH_SORT_MIN candidates and
  // CLOTHGPU_GRAPH_ZONE_MIN zone members (tests lower them to make graph
  // frames outgrow their sizes)
  const char* es = std::getenv("CLOTHGPU_GRAPH_SORT_MIN");
  const char* ez = std::getenv("CLOTHGPU_GRAPH_ZONE_MIN");
  const long long smin = es ? std::max(1LL, std::atoll(es)) : 65536, zmin = ez ? std::max(1LL, std::atoll(ez)) : 16384;
  const long long smul = es ? 2 : 4, zmul = ez ? 2 : 4;
  c->g_scand = std::min(c->C.cand_cap, pow2_at_least(std::max<long long>(smul * c->max_ncand, smin)));
  c->g_szone = std::min(A.nv, pow2_at_least(std::max<long long>(zmul * c->max_zone, zmin)));
  {
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    A.dev_grid = std::max(1, sms * c->graph_grid_per_sm);
  }
  // the static solver lists of the FP64 path
  c->g_ilu.clear();
  c->g_cg_cap = 0;
  c->g_cg_serial = false;
  for (int i = 0; i < A.ni; i++) {
    const cs_params& p = c->cloths[c->order[i]]->prm;
    if (c->solver[i] == CS_SOLVER_CG) {
      c->g_cg_cap = std::max(c->g_cg_cap, p.maxit);
      c->g_cg_serial |= (p.flags & CS_FLAG_EXACT_DOTS) != 0;
    } else {
      c->g_ilu.push_back(i);
    }
  }
  if (!c->g_ilu.empty()) {
    CK(cudaMalloc(&c->g_ilu_list, sizeof(int) * c->g_ilu.size()));
    CK(cudaMemcpy(c->g_ilu_list, c->g_ilu.data(), sizeof(int) * c->g_ilu.size(), cudaMemcpyHostToDevice));
  }
  CK(cudaStreamSynchronize(c->stream));
  const long long launches = g_launches;
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    CK(e);
  }
  try {
    emit_frame(c, c->stream);
  } catch (...) {
    cudaGraph_t dummy = nullptr;
    cudaStreamEndCapture(c->stream, &dummy);
    cudaGraphDestroy(g);
    cudaGetLastError();
    g_launches = launches;
    throw;
  }
  e = cudaStreamEndCapture(c->stream, &g);
  g_launches = launches;  // captured, not launched
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c->gexec = nullptr;
    cudaGetLastError();
    CK(e);
  }
  c->g_captures++;
}

// One frame through the graph; false when the frame overflowed a fixed size and
// was restored to its start (the caller then runs it host-driven).
bool graph_frame(cs_ctx* c, const std::vector<int>& act) {
  Arena& A = c->A;
  const size_t n3 = 3 * (size_t)A.nv;
  if (c->gsave_n != n3) {
    if (c->gsave) cudaFree(c->gsave);
    c->gsave = nullptr;
    c->gsave_n = 0;
    CK(cudaMalloc(&c->gsave, sizeof(double) * 2 * std::max<size_t>(n3, 1)));
    c->gsave_n = n3;
  }
  if (!c->gexec) {
    try {
      graph_capture(c);
    } catch (const CudaError& e) {
      // a graph this context cannot capture: frames stay host-driven
      c->graph_mode = false;
      std::fprintf(stderr, "clothgpu: frame graph off, frames run host-driven: %s\n", e.what());
      return false;
    }
  }
  CK(cudaMemcpyAsync(c->gsave, A.x, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->gsave + n3, A.v, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
  set_active(c, act);
  CK(cudaGraphLaunch(c->gexec, c->stream));
  g_launches += 1;
  FrameCtl ctl;
  CK(cudaMemcpyAsync(&ctl, A.ctl, sizeof(FrameCtl), cudaMemcpyDeviceToHost, c->stream));
  pull_states(c);  // synchronises
  if (ctl.overflow) {
    CK(cudaMemcpyAsync(A.x, c->gsave, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(A.v, c->gsave + n3, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    graph_release(c);
    c->g_overflows++;
    for (int k = 0; k < 4; k++)
      if (ctl.overflow & (1 << k)) c->g_over_reason[k]++;
    return false;
  }
  note_divergence(c);
  for (int i = 0; i < A.ni; i++) {
    if (!act[i]) continue;
    const InstState& h = c->hst[i];
    cs_stats& st = c->cloths[c->order[i]]->stats;
    const int diverged = st.diverged;
    std::memset(&st, 0, sizeof(st));
    st.diverged = diverged;
    st.solver_iterations = h.solver_iterations;
    st.solver_conv = h.solver_conv;
    st.ilu_singular = c->solver[i] == CS_SOLVER_ILU_PCG ? h.ilu_singular : 0;
    st.n_prx = h.st_prx;
    for (int k = 0; k < 5; k++) st.n_ccd[k] = h.st_ccd[k];
    st.n_ccd_passes = h.st_ccd_passes;
    st.n_riz_passes = h.st_riz_passes;
    st.n_riz_last = h.st_riz_last;
    st.n_riz_total = h.st_riz_total;
    st.riz_nodes = h.st_riz_nodes;
    st.impulse_applied = h.impulse_applied;
  }
  c->g_frames++;
  return true;
}

}  // namespace host
}  // namespace cs
