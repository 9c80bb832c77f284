// ctx.h -- host-side internals of a context (include/clothgpu.h's cs_ctx):
// the cloths it holds, the device arena they are packed into, and the frame
// orchestration that the C ABI (api.cu) and the serving loop (serve.cu) share.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/clothgpu.h"
#include "kernels.h"
#include "topology.h"

namespace cs {
namespace host {

struct ArgError : std::runtime_error {
  explicit ArgError(const std::string& s) : std::runtime_error(s) {}
};
struct CapacityError : std::runtime_error {
  explicit CapacityError(const std::string& s) : std::runtime_error(s) {}
};

#define CK(expr)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (expr);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      throw CudaError(std::string(#expr) + ": " + cudaGetErrorString(e_) + " (" __FILE__ ":" +   \
                      std::to_string(__LINE__) + ")");                                            \
  } while (0)

struct Cloth {
  int id = 0;
  ClothTopo topo;
  cs_params prm{};
  std::vector<double> x, v;  // host copy, authoritative only while the arena is rebuilt
  cs_stats stats{};
};

// device allocation with ownership in the context
struct DevMem {
  std::vector<void*> ptrs;
  template <typename T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&p, n * sizeof(T));
    if (e != cudaSuccess) throw CudaError(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    ptrs.push_back(p);
    return (T*)p;
  }
  template <typename T>
  T* upload(const std::vector<T>& h, cudaStream_t s) {
    T* d = alloc<T>(h.size());
    if (!h.empty()) CK(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

// one packing of cloths into a device arena, with its host mirrors
struct ArenaSet {
  Arena A;
  ContactBufs C;
  DevMem mem, cmem;
  std::vector<int> order;  // arena slot -> cloth id
  std::vector<int> voff, toff, qoff, boff, noff, solver;
  int* d_list = nullptr;
  std::vector<InstState> hst;
  ~ArenaSet() {
    mem.release();
    cmem.release();
  }
};

}  // namespace host
}  // namespace cs

struct cs_ctx {
  int device = 0;
  int precision = CS_PREC_FP64;
  cudaStream_t stream = nullptr;
  std::string err;
  std::map<int, std::unique_ptr<cs::host::Cloth>> cloths;
  std::vector<int> order;  // arena slot -> cloth id
  int next_id = 0;
  bool dirty = true;
  cs::Arena A;
  cs::ContactBufs C;
  cs::host::DevMem mem, cmem;  // arena / contact buffers
  // host mirrors of arena offsets
  std::vector<int> voff, toff, boff, noff, qoff;
  std::vector<int> solver;  // per slot
  int* d_list = nullptr;    // scratch list of cloth slots
  int last_ncand = 0;  // candidates of the last detection (kept in C.cand)
  int last_nce = 0;    // contacts of the last detection (in C.ce)
  std::vector<cs::InstState> hst;
  long long launches0 = 0;
  // mixed precision: whole inner solves as one cooperative launch (else one
  // launch per kernel and iteration), and its blocks per SM (0: occupancy limit)
  bool mx_persistent = true;
  int mx_blocks_per_sm = 0;
  int mx_threads = 256;  // threads per block of the persistent solve
  // slices still iterating below which the persistent solve continues in a
  // smaller launch (cheaper grid barriers for the last cloths); 0: one launch
  int mx_tail_slices = 1216;
  // blocks per SM of the grid-stride narrow-phase kernels of a graph frame
  int graph_grid_per_sm = 8;
  // register variant of the FP64 narrow-phase kernels (0 free, 128 capped)
  int narrow_regs = 0;
  // pause between polls of the persistent solver's grid barrier (ns), its
  // time-out, and the test hook that keeps block 0 from arriving
  int bar_sleep_ns = 256;
  int impulse_cluster = 1;  // blocks per cloth of the impulse sweep (a cluster when > 1)
  long long bar_timeout_ns = 2000000000;
  int bar_hold = 0;
  // inner FP32 solve of a refinement cycle: relative residual target and cap
  float mx_eta = 1.0e-3f;
  float mx_eta_big = 1.0e-4f;  // inner tolerance of cloths over 16384 vertices
  int mx_cap = 300;
  // per slot: the cloth blew up (CS_ERR_DIVERGED) and is no longer stepped
  std::vector<int> dead;
  // slots of the last set_active (cloths that the next launches touch)
  std::vector<int> cur_act;
  // contact log (cs_contact_log): per cloth id, one entry per detection of its last resolve
  struct LogEntry {
    int kind, count;
    unsigned long long digest;
  };
  bool log_on = false;
  std::map<int, std::vector<LogEntry>> clog;
  // largest candidate and zone-member counts of the host-driven detections
  // (the padded sort sizes of a frame graph are chosen from them)
  long long max_ncand = 0, max_zone = 0;
  // frame graph (frame_graph.cu): on by default; its executable, capture
  // streams, fixed sizes, static solver lists, start-state snapshot, counters
  bool graph_mode = true;
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t gstream[2] = {nullptr, nullptr};
  int g_scand = 0, g_szone = 0, g_cg_cap = 0;
  bool g_cg_serial = false;
  std::vector<int> g_ilu;
  int* g_ilu_list = nullptr;
  double* gsave = nullptr;
  size_t gsave_n = 0;
  long long g_frames = 0, g_captures = 0, g_overflows = 0, host_frames = 0;
  long long g_over_reason[4] = {0, 0, 0, 0};  // overflows by reason: sort, zone, buffers, solver
};

namespace cs {
namespace host {

// Validates the arguments and builds the cloth's host topology (adjacency,
// BVH, matrix pattern, ILU schedule): the expensive host part of admitting a
// cloth.  Touches no context, so any thread may call it.
std::unique_ptr<Cloth> make_cloth(int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                                  const int* quad, const cs_params* prm);
// device bytes a cloth adds to an arena (buffers sized by its vertices,
// triangles, stencils, blocks and BVH nodes), used for admission by memory
size_t cloth_device_bytes(const ClothTopo& t);
// Packs cloths into a fresh arena on stream s; reads only the cloths.
void build_arena(ArenaSet& o, const std::vector<const Cloth*>& cl, cudaStream_t s);
// Makes o the context's arena; o receives the previous arena's buffers.
void install(cs_ctx* c, ArenaSet& o);
// one frame (StepTime) for the arena slots with act[slot] != 0
void frame(cs_ctx* c, const std::vector<int>& act);
// maps an exception from the host layer to a CS_* status and records its message
int status_of(const std::exception& e, std::string* msg);
// frame graph (frame_graph.cu): capture for the current arena, release, and one
// frame through it (false: a fixed size overflowed and the start state was
// restored, so the caller runs the frame host-driven)
void graph_capture(cs_ctx* c);
void graph_release(cs_ctx* c);
bool graph_frame(cs_ctx* c, const std::vector<int>& act);

}  // namespace host
}  // namespace cs
