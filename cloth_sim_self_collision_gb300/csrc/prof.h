// prof.h -- optional per-kernel device timing: CUDA events recorded on the
// launching stream around each launch of a kernel class, resolved on demand.
#pragma once
#include <cuda_runtime.h>

namespace cs {

enum ProfKernel {
  PK_TRI_ELEMENTS = 0,
  PK_SLOT_REDUCE,
  PK_RHS,
  PK_ILU_FACTOR,
  PK_PCG,
  PK_CG_SPMV,
  PK_CG_UPDATE,
  PK_CG_DIRECTION,
  PK_REFIT,
  PK_TRAVERSE,
  PK_NARROW,
  PK_IMPULSE,
  PK_MX_SPMV,
  PK_MX_UPDATE,
  PK_MX_DIRECTION,
  PK_MX_RESIDUAL,
  PK_MX_PERSIST,
  PK_NARROW_FILTER,
  PK_NARROW_FV,
  PK_NARROW_EE,
  PK_SORT,
  PK_NARROW_CCD64,
  PK_COUNT
};

extern const char* const kProfNames[PK_COUNT];

// begin / end a timed launch on stream s (no-ops while profiling is off)
void prof_begin(ProfKernel k, cudaStream_t s);
void prof_end(ProfKernel k, cudaStream_t s);
void prof_enable(bool on);
bool prof_enabled();
// resolves recorded events (synchronises them) and accumulates totals
void prof_collect();
void prof_reset();
bool prof_read(const char* name, double* total_ms, long long* launches);
// host-side counters read through prof_read: "pairs", "candidates", "contacts", "detections"
void prof_count(const char* name, long long n);

}  // namespace cs
