// The ensemble's persistent stage launch (passes_ens.cu): one kernel per RK3
// stage advances every eligible member through all five passes.
//
// The host records each member's stage as segments, a segment being one
// pass (or vel_max's wave-space sums or its completion) of one member with
// its argument block and its number of tiles; the segments are ordered by
// pass level (z inverse and the wave-space sums, y inverse, x pass, then
// vel_max's completion and y forward, then z forward), so that every segment
// a segment depends on has all of its tickets before it.  Persistent CTAs
// draw tickets from an atomic counter and run the ticket's tile; before
// starting, a CTA waits (bounded) until each segment its segment depends on
// has counted all of its tiles done.  Because a CTA only waits for lower
// tickets, already drawn by running CTAs that wait only for lower ones
// still, the launch always makes progress.  A wait that exceeds its bound
// sets the error flag, skips the tile and still counts it, so that the
// launch ends and the host reports the failure.
#pragma once
#include <vector>

#include "passes.cuh"

namespace samgpu {

enum EnsKind : int { kEnsZInv = 0, kEnsYInv, kEnsX, kEnsYFwd, kEnsZFwd, kEnsParseval, kEnsFinish };

// arguments of the wave-space sums (parseval_body) and of the completion
struct EnsParsevalArgs {
  const float2* u;
  Grid g;
  double* pv;
};
struct EnsFinishArgs {
  const double* partials;
  int nblk;
  Grid g;
  DevState* st;
  int i_cfl;
  double cfl0, adv_cfl_limit;
  const double* pv;
  int npv;
  int* vmax;
};

// virtual blocks of the wave-space sums per work item
constexpr int kEnsParsevalChunk = 32;

// tiles of a transform segment per work item
constexpr int kEnsChunk = 8;

struct EnsSeg {
  int kind, path;     // EnsKind; FFT path (the transform length)
  int first, ntiles;  // work items (tickets) first .. first + ntiles - 1
  int tiles, chunk;   // the segment's tiles, tiles per work item
  int dep[2];         // segments that must be complete first (-1: none)
  int args_off;       // byte offset of the argument block in the launch's blob
  int pad;
  const FftPlan* plan;
};

// One member's stage as recorded: segments with member-local dependencies.
struct EnsRecSeg {
  int kind, path, ntiles, level;
  int dep[2];
  size_t smem;
  std::vector<unsigned char> args;
  const FftPlan* plan;
};
struct EnsRecorder {
  std::vector<EnsRecSeg> segs;
};

// Recording of the FP32 passes (the eligible members' precision).
void ens_record_z_inv(EnsRecorder& r, const ZInvArgs<float>& a, const FftPlan* pl, size_t smem);
void ens_record_y_inv(EnsRecorder& r, const YInvArgs<float>& a, const FftPlan* pl, size_t smem);
void ens_record_x_pass(EnsRecorder& r, const XPassArgs<float>& a, const FftPlan* pl, size_t smem, bool stats,
                       const EnsParsevalArgs* pa, const EnsFinishArgs* fa);
void ens_record_y_fwd(EnsRecorder& r, const YFwdArgs<float>& a, const FftPlan* pl, size_t smem);
void ens_record_z_fwd(EnsRecorder& r, const ZFwdArgs<float>& a, const FftPlan* pl, size_t smem);
// whether the persistent kernel has a code path for this transform length
bool ens_length_ok(int n);

// A stage's launch: the members' records merged in pass-level order (larger
// members first within a level), device copies of the segments and the
// argument blob, and the counters (one per segment, then the ticket).
struct EnsStageLaunch {
  EnsSeg* seg = nullptr;
  unsigned char* blob = nullptr;
  unsigned* counters = nullptr;
  int nseg = 0, total = 0;
  size_t smem = 0;
};
// 0 ok, -1 device allocation failed, -2 a segment the kernel cannot run (a
// length without a path, or tiles too large beside its static shared memory)
int ens_build_stage(const std::vector<EnsRecorder*>& members, EnsStageLaunch& out);
void ens_free_stage(EnsStageLaunch& s);
// the counters' reset and the persistent launch (grid: the CTAs that can be
// resident, at most ctas_per_sm per SM)
void ens_launch_stage(const EnsStageLaunch& s, int ctas_per_sm, int* err, cudaStream_t st);

}  // namespace samgpu
