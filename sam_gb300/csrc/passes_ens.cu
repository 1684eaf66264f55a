// The ensemble's persistent stage kernel and its recorder (ens.cuh): the
// FP32 pass bodies of passes_impl.cuh, instantiated with L2-coherent loads
// for the transform lengths that have a compile-time FFT path (32, 64, 96,
// 128), run as work items drawn from one ticket counter.
#include <algorithm>
#include <cstring>

#include "ens.cuh"
#include "passes_impl.cuh"

namespace samgpu {

constexpr int kEnsArgsMax = 512;  // bytes of the largest argument block
static_assert(sizeof(XPassArgs<float>) <= kEnsArgsMax && sizeof(ZFwdArgs<float>) <= kEnsArgsMax &&
                  sizeof(ZInvArgs<float>) <= kEnsArgsMax && sizeof(YInvArgs<float>) <= kEnsArgsMax &&
                  sizeof(YFwdArgs<float>) <= kEnsArgsMax && sizeof(EnsFinishArgs) <= kEnsArgsMax,
              "argument block larger than the kernel's staging area");
constexpr unsigned kEnsWaitLimit = 1u << 22;  // polls of a dependency (about a second with the back-off)

bool ens_length_ok(int n) { return n == 32 || n == 64 || n == 96 || n == 128; }

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Each (pass, length) body is its own function, not inlined into the
// scheduler: its registers are then allocated for it alone, as in the pass's
// own kernel, instead of for the union of twenty bodies.  A call runs the
// tiles t0 .. t1 - 1 of its segment, so that the saving and restoring of
// registers around the call is paid once per group of tiles.
#define SAMGPU_ENS_BODY(NAME, BODY, ARGS)                                                                   \
  template <int PATH>                                                                                       \
  __device__ __noinline__ void NAME(const unsigned char* args, const FftPlan* plan, int t0, int t1) {         \
    for (int tile = t0; tile < t1; ++tile) {                                                                \
      BODY<float, PATH, true>(*reinterpret_cast<const ARGS<float>*>(args), plan, tile);                      \
      __syncthreads();                                                                                      \
    }                                                                                                       \
  }
SAMGPU_ENS_BODY(ens_z_inv, z_inv_body, ZInvArgs)
SAMGPU_ENS_BODY(ens_y_inv, y_inv_body, YInvArgs)
SAMGPU_ENS_BODY(ens_x, x_pass_body, XPassArgs)
SAMGPU_ENS_BODY(ens_y_fwd, y_fwd_body, YFwdArgs)
SAMGPU_ENS_BODY(ens_z_fwd, z_fwd_body, ZFwdArgs)
#undef SAMGPU_ENS_BODY
__device__ __noinline__ void ens_parseval(const unsigned char* args, int tile) {
  const EnsParsevalArgs& pa = *reinterpret_cast<const EnsParsevalArgs*>(args);
  const int b0 = tile * kEnsParsevalChunk;
  for (int b = b0; b < b0 + kEnsParsevalChunk && b < kParsevalBlocks; ++b) {
    parseval_body<float>(pa.u, pa.g, pa.pv, b, kParsevalBlocks);
    __syncthreads();
  }
}
__device__ __noinline__ void ens_finish(const unsigned char* args) {
  const EnsFinishArgs& fa = *reinterpret_cast<const EnsFinishArgs*>(args);
  vel_max_finish_body<true>(fa.partials, fa.nblk, fa.g, fa.st, fa.i_cfl, fa.cfl0, fa.adv_cfl_limit, fa.pv, fa.npv,
                            fa.vmax, 0);
}

template <int PATH>
__device__ __forceinline__ void ens_pass(int kind, const unsigned char* args, const FftPlan* plan, int t0, int t1) {
  switch (kind) {
    case kEnsZInv: ens_z_inv<PATH>(args, plan, t0, t1); break;
    case kEnsYInv: ens_y_inv<PATH>(args, plan, t0, t1); break;
    case kEnsX: ens_x<PATH>(args, plan, t0, t1); break;
    case kEnsYFwd: ens_y_fwd<PATH>(args, plan, t0, t1); break;
    default: ens_z_fwd<PATH>(args, plan, t0, t1); break;
  }
}

__global__ void __launch_bounds__(kThreads, 3)
    k_ens_stage(const EnsSeg* __restrict__ seg, int nseg, int total, const unsigned char* __restrict__ blob,
                unsigned* counters, int* err) {
  __shared__ int s_tk, s_seg, s_ok;
  __shared__ __align__(16) unsigned char s_args[kEnsArgsMax];
  for (;;) {
    if (threadIdx.x == 0) {
      const int tk = (int)atomicAdd(counters + nseg, 1u);
      int si = -1, ok = 1;
      if (tk < total) {
        // the segment holding ticket tk (segments in ticket order)
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (seg[mid].first <= tk) lo = mid;
          else hi = mid - 1;
        }
        si = lo;
        // after a timeout anywhere in the launch, tiles are only counted
        if (ld_acquire(reinterpret_cast<const unsigned*>(err))) ok = 0;
        for (int d = 0; d < 2 && ok; ++d) {
          const int ds = seg[si].dep[d];
          if (ds < 0) continue;
          const unsigned need = (unsigned)seg[ds].ntiles;
          unsigned it = 0;
          while (ld_acquire(counters + ds) < need) {
            if (++it > kEnsWaitLimit || ld_acquire(reinterpret_cast<const unsigned*>(err))) {
              ok = 0;
              atomicExch(err, 1);
              break;
            }
            __nanosleep(256);
          }
        }
      }
      s_tk = tk;
      s_seg = si;
      s_ok = ok;
    }
    __syncthreads();
    const int tk = s_tk, si = s_seg;
    if (tk >= total) break;
    const EnsSeg sg = seg[si];
    {
      const int4* src = reinterpret_cast<const int4*>(blob + sg.args_off);
      for (int w = threadIdx.x; w < kEnsArgsMax / 16; w += blockDim.x) reinterpret_cast<int4*>(s_args)[w] = src[w];
    }
    __syncthreads();
    if (s_ok) {
      const int item = tk - sg.first;
      if (sg.kind == kEnsParseval) {
        ens_parseval(s_args, item);
      } else if (sg.kind == kEnsFinish) {
        ens_finish(s_args);
      } else {
        const int t0 = item * sg.chunk, t1 = min(t0 + sg.chunk, sg.tiles);
        switch (sg.path) {  // (ens_build_stage admits these four only)
          case 32: ens_pass<32>(sg.kind, s_args, sg.plan, t0, t1); break;
          case 64: ens_pass<64>(sg.kind, s_args, sg.plan, t0, t1); break;
          case 96: ens_pass<96>(sg.kind, s_args, sg.plan, t0, t1); break;
          case 128: ens_pass<128>(sg.kind, s_args, sg.plan, t0, t1); break;
          default: break;
        }
      }
    }
    // every thread's writes of this tile are visible device-wide before
    // the tile is counted
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(counters + si, 1u);
  }
}

// ---------------------------------------------------------------- recording
template <typename A>
static void push(EnsRecorder& r, int kind, int path, int ntiles, int level, int d0, int d1, size_t smem, const A& a,
                 const FftPlan* pl) {
  EnsRecSeg s;
  s.kind = kind;
  s.path = path;
  s.ntiles = ntiles;
  s.level = level;
  s.dep[0] = d0;
  s.dep[1] = d1;
  s.smem = smem;
  s.args.resize(sizeof(A));
  std::memcpy(s.args.data(), &a, sizeof(A));
  s.plan = pl;
  r.segs.push_back(std::move(s));
}
static int last_of(const EnsRecorder& r, int kind) {
  for (int i = (int)r.segs.size() - 1; i >= 0; --i)
    if (r.segs[(size_t)i].kind == kind) return i;
  return -1;
}

void ens_record_z_inv(EnsRecorder& r, const ZInvArgs<float>& a, const FftPlan* pl, size_t smem) {
  const int nty = (a.g.my + a.ty - 1) / a.ty;
  push(r, kEnsZInv, a.g.nz, a.nvar * a.g.mx * nty, 0, -1, -1, smem, a, pl);
}
void ens_record_y_inv(EnsRecorder& r, const YInvArgs<float>& a, const FftPlan* pl, size_t smem) {
  const int ntx = (a.g.mx + a.tx - 1) / a.tx;
  push(r, kEnsYInv, a.g.ny, a.nvar * a.g.nz * ntx, 1, last_of(r, kEnsZInv), -1, smem, a, pl);
}
void ens_record_x_pass(EnsRecorder& r, const XPassArgs<float>& a0, const FftPlan* pl, size_t smem, bool stats,
                       const EnsParsevalArgs* pa, const EnsFinishArgs* fa) {
  const XPassArgs<float> a = prep_x_pass(a0);
  push(r, kEnsX, a.g.nx, x_pass_blocks(a), 2, last_of(r, kEnsYInv), -1, smem, a, pl);
  if (stats) {
    const int ix = (int)r.segs.size() - 1;
    push(r, kEnsParseval, 0, (kParsevalBlocks + kEnsParsevalChunk - 1) / kEnsParsevalChunk, 0, -1, -1, 0, *pa,
         nullptr);
    const int ip = (int)r.segs.size() - 1;
    push(r, kEnsFinish, 0, 1, 3, ix, ip, 0, *fa, nullptr);
  }
}
void ens_record_y_fwd(EnsRecorder& r, const YFwdArgs<float>& a, const FftPlan* pl, size_t smem) {
  const int ntz = (a.g.nz + a.tz - 1) / a.tz;
  push(r, kEnsYFwd, a.g.ny, a.nvar * a.g.mx * ntz, 3, last_of(r, kEnsX), -1, smem, a, pl);
}
void ens_record_z_fwd(EnsRecorder& r, const ZFwdArgs<float>& a0, const FftPlan* pl, size_t smem) {
  const ZFwdArgs<float> a = prep_z_fwd(a0);
  const int nty = (a.g.my + a.ty - 1) / a.ty;
  push(r, kEnsZFwd, a.g.nz, a.g.mx * nty, 4, last_of(r, kEnsYFwd), last_of(r, kEnsFinish), smem, a, pl);
}

// ----------------------------------------------------------------- launches
int ens_build_stage(const std::vector<EnsRecorder*>& members, EnsStageLaunch& out) {
  struct Ref {
    int level, member, local;
  };
  std::vector<Ref> order;
  for (int m = 0; m < (int)members.size(); ++m)
    for (int i = 0; i < (int)members[(size_t)m]->segs.size(); ++i)
      order.push_back({members[(size_t)m]->segs[(size_t)i].level, m, i});
  std::stable_sort(order.begin(), order.end(), [](const Ref& x, const Ref& y) { return x.level < y.level; });
  std::vector<std::vector<int>> gidx(members.size());
  for (size_t m = 0; m < members.size(); ++m) gidx[m].assign(members[m]->segs.size(), -1);
  for (int k = 0; k < (int)order.size(); ++k) gidx[(size_t)order[(size_t)k].member][(size_t)order[(size_t)k].local] = k;
  std::vector<EnsSeg> segs(order.size());
  std::vector<unsigned char> blob;
  int ticket = 0;
  size_t smem = 0;
  for (size_t k = 0; k < order.size(); ++k) {
    const EnsRecSeg& r = members[(size_t)order[k].member]->segs[(size_t)order[k].local];
    EnsSeg& s = segs[k];
    s.kind = r.kind;
    s.path = r.path;
    // transform segments: kEnsChunk tiles per work item (per ticket)
    const bool xform = r.kind != kEnsParseval && r.kind != kEnsFinish;
    s.tiles = r.ntiles;
    s.chunk = xform ? kEnsChunk : 1;
    s.first = ticket;
    s.ntiles = xform ? (r.ntiles + kEnsChunk - 1) / kEnsChunk : r.ntiles;
    for (int d = 0; d < 2; ++d) s.dep[d] = r.dep[d] < 0 ? -1 : gidx[(size_t)order[k].member][(size_t)r.dep[d]];
    s.args_off = (int)blob.size();
    s.pad = 0;
    s.plan = r.plan;
    blob.insert(blob.end(), r.args.begin(), r.args.end());
    blob.resize(blob.size() + kEnsArgsMax);  // room for the kernel's full-size copy; keeps 16-byte alignment
    blob.resize((blob.size() + 15) & ~(size_t)15);
    ticket += s.ntiles;
    smem = std::max(smem, r.smem);
  }
  // every transform segment on a length the kernel has a path for, and the
  // largest tile's shared memory beside the kernel's static shared memory
  for (const EnsSeg& s : segs)
    if (s.kind != kEnsParseval && s.kind != kEnsFinish && !ens_length_ok(s.path)) return -2;
  {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes at;
    if (cudaFuncGetAttributes(&at, k_ens_stage) != cudaSuccess || smem + at.sharedSizeBytes > (size_t)optin)
      return -2;
  }
  ens_free_stage(out);
  out.nseg = (int)segs.size();
  out.total = ticket;
  out.smem = smem;
  if (cudaMalloc(&out.seg, sizeof(EnsSeg) * segs.size()) != cudaSuccess ||
      cudaMalloc(&out.blob, blob.size()) != cudaSuccess ||
      cudaMalloc(&out.counters, sizeof(unsigned) * (segs.size() + 1)) != cudaSuccess)
    return -1;
  if (cudaMemcpy(out.seg, segs.data(), sizeof(EnsSeg) * segs.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(out.blob, blob.data(), blob.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return -1;
  return 0;
}

void ens_free_stage(EnsStageLaunch& s) {
  cudaFree(s.seg);
  cudaFree(s.blob);
  cudaFree(s.counters);
  s.seg = nullptr;
  s.blob = nullptr;
  s.counters = nullptr;
  s.nseg = s.total = 0;
}

void ens_launch_stage(const EnsStageLaunch& s, int ctas_per_sm, int* err, cudaStream_t st) {
  if (s.total == 0) return;
  static size_t attr_smem = 0;
  if (s.smem > attr_smem) {
    cudaFuncAttributes at;
    cudaFuncGetAttributes(&at, k_ens_stage);
    cudaFuncSetAttribute(k_ens_stage, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    attr_smem = s.smem;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ens_stage, kThreads, s.smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  int grid = per_sm * sm_count();
  if (grid > s.total) grid = s.total;
  cudaMemsetAsync(s.counters, 0, sizeof(unsigned) * ((size_t)s.nseg + 1), st);
  k_ens_stage<<<grid, kThreads, s.smem, st>>>(s.seg, s.nseg, s.total, s.blob, s.counters, err);
}

}  // namespace samgpu
