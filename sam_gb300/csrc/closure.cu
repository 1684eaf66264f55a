// Learned subgrid closure: the 12 -> 64 -> 64 -> 2 MLP on sm_103a.
//
// Inference: a warpgroup (128 threads) per tile of 128 points, four
// warpgroups per CTA, each with its own tiles.  The inputs and the weights
// sit in shared memory in the canonical K-major no-swizzle layout of the
// tensor cores (8 x 16-byte core matrices: element (r, k) at (r/8)*SBO +
// (k/8)*LBO + (r%8)*16 + (k%8)*2 with LBO = 128 B and SBO = (K/8)*128 B).
// One thread per warpgroup issues tcgen05.mma (kind::f16, BF16 x BF16 ->
// FP32 in TMEM, M = 128), tcgen05.commit arrives on an mbarrier, the
// warpgroup's four warps read their 32 TMEM lanes back with tcgen05.ld; the
// ReLU epilogue writes the next layer's BF16 operand into shared memory (the
// biases are in the MMAs, against constant-1 input columns).  Three MMA
// groups per tile (K = 16, then 5 x K = 16 twice).  Every wait is bounded:
// on timeout the kernel sets *err, waits (bounded again) for its TMA load and
// its MMA group still in flight, frees its TMEM and returns; the outputs of a
// launch that timed out are undefined.
//
// Training: the backward pass of the loss mean (C - y)^2 and Adam run on the
// CUDA cores in FP32 (the network is small; the weight gradients are
// per-CTA partial sums reduced in a fixed order, so runs are reproducible).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "closure.cuh"
#include "common.cuh"
#include "tc05.cuh"

namespace samgpu {

// ------------------------------------------------------------- MMA selftest
// D(128 x 64) = A(128 x 16) B(64 x 16)^T: the smallest use of the path the
// forward kernel takes, checked against a host product in the tests.
__global__ void __launch_bounds__(128) k_mma_selftest(const __nv_bfloat16* __restrict__ a,
                                                      const __nv_bfloat16* __restrict__ b, float* __restrict__ d,
                                                      int* err) {
  __shared__ __align__(1024) uint8_t sa[128 * 16 * 2];
  __shared__ __align__(1024) uint8_t sb[64 * 16 * 2];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  if (threadIdx.x < 32) tmem_alloc(&tbase, 64);
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  stage_matrix(sa, a, 128, 16);
  stage_matrix(sb, b, 64, 16);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = tbase;
  if (threadIdx.x == 0) {
    mma_bf16(tm, sdesc(smem_u32(sa), 128, 256), sdesc(smem_u32(sb), 128, 256), idesc_bf16(128, 64), 0);
    mma_commit(&bar);
  }
  int bad = mbar_wait(&bar, 0);
  tc_fence_after();
  bad = __syncthreads_or(bad);
  if (!bad) {
    const int w = threadIdx.x >> 5;
    for (int c = 0; c < 64; c += 16) {
      float v[16];
      tmem_ld16(tm + ((uint32_t)(32 * w) << 16) + (uint32_t)c, v);
      for (int i = 0; i < 16; ++i) d[threadIdx.x * 64 + c + i] = v[i];
    }
  } else if (threadIdx.x == 0) {
    atomicExch(err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    tmem_dealloc(tm, 64);
  }
}

void mlp_mma_selftest(const __nv_bfloat16* a, const __nv_bfloat16* b, float* d, int* err, cudaStream_t s) {
  k_mma_selftest<<<1, 128, 0, s>>>(a, b, d, err);
}

// ------------------------------------------------------------ forward pass
// One hidden layer's epilogue for this thread's row: TMEM (the bias is
// already in the accumulator) -> ReLU -> BF16 K-major operand tile columns
// 0..63 (and, when hg is given, the activations), 16 columns at a time; the
// ReLU is the conversion's (cvt.relu).
__device__ __forceinline__ void epilogue(uint32_t tl, uint8_t* tile, int r, __nv_bfloat16* __restrict__ hg,
                                         long long row, bool live) {
#pragma unroll
  for (int c0 = 0; c0 < kMlpH; c0 += 16) {
    float h[16];
    tmem_ld16(tl + (uint32_t)c0, h);
    uint32_t q[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) q[k] = pack_relu_bf16(h[2 * k], h[2 * k + 1]);
#pragma unroll
    for (int j = 0; j < 2; ++j)
      *reinterpret_cast<uint4*>(tile + kmaj(r, c0 + 8 * j, kMlpK2)) =
          make_uint4(q[4 * j], q[4 * j + 1], q[4 * j + 2], q[4 * j + 3]);
    if (hg && live) {
      uint4* dst = reinterpret_cast<uint4*>(hg + row * kMlpH + c0);
#pragma unroll
      for (int j = 0; j < 2; ++j) dst[j] = make_uint4(q[4 * j], q[4 * j + 1], q[4 * j + 2], q[4 * j + 3]);
    }
  }
}

// Shared memory of the forward kernel: the BF16 weights in the K-major
// layout (shared by the CTA's warpgroups), then per warpgroup its input tile
// and its 128 x 80 hidden operand tile (columns 64..66 hold 1.0, the bias
// inputs of layers 2 and 3; 67..79 zero), and the barriers.  Every operand
// starts on a 128-byte boundary.
constexpr int kMlpWG = 4;  // warpgroups per CTA, each with its own tiles
struct MlpWgTiles {
  uint8_t a1[kMlpTile * kMlpK1 * 2];
  uint8_t a2[kMlpTile * kMlpK2 * 2];
};
struct MlpFwdSmem {
  uint8_t w1[kMlpH * kMlpK1 * 2];
  uint8_t w2[kMlpH * kMlpK2 * 2];
  uint8_t w3[kMlpN3 * kMlpK2 * 2];
  MlpWgTiles wg[kMlpWG];
  uint64_t mbar[kMlpWG], tbar[kMlpWG];
  uint32_t tbase;
};
constexpr size_t kMlpFwdSmemBytes = sizeof(MlpFwdSmem) + 1024;  // + room to align the base to 1024 bytes
constexpr int kMlpFwdCtas = 2;  // per SM: 112 KB of shared memory and 256 TMEM columns each

// Persistent CTAs of four warpgroups; each warpgroup runs its own tiles of
// 128 points (thread r of the warpgroup owns row r: its TMEM lane) through
// the three layers with its own TMEM columns (64 per warpgroup), barriers
// and named-barrier synchronisation, so a CTA keeps four independent MMA
// chains in flight and an SM eight.  Optionally stores the activations for
// the backward pass.  The input tiles arrive by TMA: a 2-D tensor map over
// x16 ([n][16] BF16, 32-byte rows) with a box of 8 x 128 (16 bytes x 128
// rows), loaded at x = 0 and x = 8, writes the two K halves of a 128 x 16
// tile one after the other: element (r, k) at (k/8)*2048 + r*16 + (k%8)*2,
// the canonical no-swizzle K-major layout with LBO = 2048 B and SBO = 128 B.
// A warpgroup's next input is loaded as soon as its layer-1 MMA has read the
// current one.
__global__ void __launch_bounds__(128 * kMlpWG, kMlpFwdCtas)
    k_mlp_fwd(const __grid_constant__ CUtensorMap xmap, long long n, const MlpDev* __restrict__ P,
              float2* __restrict__ coef, __nv_bfloat16* __restrict__ h1g, __nv_bfloat16* __restrict__ h2g,
              float* __restrict__ og, int* err) {
  extern __shared__ __align__(1024) uint8_t mlp_smem[];
  MlpFwdSmem& S = *reinterpret_cast<MlpFwdSmem*>(mlp_smem + ((1024u - (smem_u32(mlp_smem) & 1023u)) & 1023u));
  const int tid = threadIdx.x, g = tid >> 7, r = tid & 127;
  const int bid = 1 + g;  // this warpgroup's named barrier (0 is __syncthreads)
  const long long ntiles = (n + kMlpTile - 1) / kMlpTile;
  const long long nslots = (long long)gridDim.x * kMlpWG;
  const long long first = (long long)blockIdx.x * kMlpWG + g;
  constexpr uint32_t kTileBytes = kMlpTile * kMlpK1 * 2;
  uint8_t* a1 = S.wg[g].a1;
  uint8_t* a2 = S.wg[g].a2;
  auto load_tile = [&](long long t) {
    mbar_expect_tx(&S.tbar[g], kTileBytes);
    tma_load_2d(a1, &xmap, 0, (int)(t * kMlpTile), &S.tbar[g]);
    tma_load_2d(a1 + kTileBytes / 2, &xmap, 8, (int)(t * kMlpTile), &S.tbar[g]);
  };
  if (tid < 32) tmem_alloc(&S.tbase, 64 * kMlpWG);
  if (r == 0) {
    mbar_init(&S.mbar[g], 1);
    mbar_init(&S.tbar[g], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (first < ntiles) load_tile(first);
  }
  stage_matrix(S.w1, P->w1, kMlpH, kMlpK1);
  stage_matrix(S.w2, P->w2, kMlpH, kMlpK2);
  stage_matrix(S.w3, P->w3, kMlpN3, kMlpK2);
  {
    // the constant columns of this thread's row of its hidden operand tile
    const uint32_t one = 0x3F80u;  // 1.0 in BF16
    *reinterpret_cast<uint4*>(a2 + kmaj(r, kMlpH, kMlpK2)) = make_uint4(one | (one << 16), one, 0u, 0u);
    *reinterpret_cast<uint4*>(a2 + kmaj(r, kMlpH + 8, kMlpK2)) = make_uint4(0u, 0u, 0u, 0u);
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = S.tbase + 64u * (uint32_t)g;                    // this warpgroup's columns
  const uint32_t tl = tm + ((uint32_t)(32 * ((tid >> 5) & 3)) << 16);  // this warp's lanes
  const uint32_t sa1 = smem_u32(a1), sa2 = smem_u32(a2);
  const uint32_t w1 = smem_u32(S.w1), w2 = smem_u32(S.w2), w3 = smem_u32(S.w3);
  const uint32_t id64 = idesc_bf16(kMlpTile, kMlpH), id16 = idesc_bf16(kMlpTile, kMlpN3);
  uint32_t mph = 0, tph = 0;
  int bad = 0;
  bool pend = first < ntiles;  // a TMA load not yet waited for (the same in every thread of the warpgroup)
  bool mpend = false;          // an MMA group committed and not yet waited for
  // one thread polls each barrier; the warpgroup's named barrier releases
  // the others and makes bad the same in all of them
  auto wait_mma = [&]() {
    int b = r == 0 ? mbar_wait(&S.mbar[g], mph) : 0;
    b = bar_named_or(bid, 128, b);
    if (!b) {
      mph ^= 1u;
      mpend = false;
    }
    tc_fence_after();
    return b;
  };
  auto to_mma = [&]() {  // operand tile written: visible to the tensor cores
    fence_async_smem();
    tc_fence_before();
    bar_named(bid, 128);
    tc_fence_after();
  };
  for (long long t = first; t < ntiles; t += nslots) {
    const long long row = t * kMlpTile + r;
    const bool live = row < n;
    bad = r == 0 ? mbar_wait(&S.tbar[g], tph) : 0;
    bad = bar_named_or(bid, 128, bad);
    if (bad) break;
    tph ^= 1u;
    pend = false;
    // layer 1: D = X W1^T (K = 16; the bias through input columns 12..14)
    if (r == 0) {
      tc_fence_after();
      mma_bf16(tm, sdesc(sa1, 2048, 128), sdesc(w1, 128, 256), id64, 0);
      mma_commit(&S.mbar[g]);
    }
    mpend = true;
    if ((bad = wait_mma())) break;
    // the input tile has been read: the next one loads during this tile's chain
    const long long tn = t + nslots;
    pend = tn < ntiles;
    if (r == 0 && pend) load_tile(tn);
    epilogue(tl, a2, r, h1g, row, live);
    to_mma();
    // layer 2: D = H1 W2^T (K = 80 as five K = 16 steps, the last with the
    // bias columns)
    if (r == 0) {
#pragma unroll
      for (int kk = 0; kk < kMlpK2 / 16; ++kk)
        mma_bf16(tm, sdesc(sa2 + 256 * kk, 128, kMlpK2 * 16), sdesc(w2 + 256 * kk, 128, kMlpK2 * 16), id64, kk > 0);
      mma_commit(&S.mbar[g]);
    }
    mpend = true;
    if ((bad = wait_mma())) break;
    epilogue(tl, a2, r, h2g, row, live);
    to_mma();
    // layer 3: D = H2 W3^T (N = 16, two rows used; K = 80 as for layer 2)
    if (r == 0) {
#pragma unroll
      for (int kk = 0; kk < kMlpK2 / 16; ++kk)
        mma_bf16(tm, sdesc(sa2 + 256 * kk, 128, kMlpK2 * 16), sdesc(w3 + 256 * kk, 128, kMlpK2 * 16), id16, kk > 0);
      mma_commit(&S.mbar[g]);
    }
    mpend = true;
    if ((bad = wait_mma())) break;
    float o[2];
    tmem_ld2(tl, o);
    if (live) {
      coef[row] = make_float2(kMlpScale * softplus(o[0]), kMlpScale * softplus(o[1]));
      if (og) {
        og[2 * row] = o[0];
        og[2 * row + 1] = o[1];
      }
    }
    // the accumulator is read before the next tile's layer 1 writes it
    tc_fence_before();
    bar_named(bid, 128);
    tc_fence_after();
  }
  if (bad && r == 0) atomicExch(err, 1);
  // a load or an MMA group still in flight (the loop left early) completes
  // before the shared memory and the TMEM it uses are released
  if (pend && r == 0) mbar_wait(&S.tbar[g], tph);
  if (mpend && r == 0) mbar_wait(&S.mbar[g], mph);
  tc_fence_before();
  __syncthreads();
  if (tid < 32) {
    tc_fence_after();
    tmem_dealloc(S.tbase, 64 * kMlpWG);
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda); the map of x16 as [n][16] BF16 with 8 x 128 boxes
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static bool x16_map(const __nv_bfloat16* x16, long long n, CUtensorMap* m) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(x16) & 15)) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)kMlpK1, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)kMlpK1 * 2};
  const cuuint32_t box[2] = {8, (cuuint32_t)kMlpTile};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(x16), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int mlp_forward(const __nv_bfloat16* x16, long long n, const MlpDev* dev, float2* coef, const MlpBatch* batch,
                int* err, cudaStream_t s) {
  const long long ntiles = (n + kMlpTile - 1) / kMlpTile;
  long long grid = (long long)sm_count() * kMlpFwdCtas;  // persistent: one wave
  if (grid > (ntiles + kMlpWG - 1) / kMlpWG) grid = (ntiles + kMlpWG - 1) / kMlpWG;
  if (grid < 1) return 0;
  CUtensorMap m;
  if (!x16_map(x16, n, &m)) return -1;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMlpFwdSmemBytes) !=
        cudaSuccess)
      return -1;
    attr = true;
  }
  k_mlp_fwd<<<(int)grid, 128 * kMlpWG, kMlpFwdSmemBytes, s>>>(m, n, dev, coef, batch ? batch->h1 : nullptr,
                                                              batch ? batch->h2 : nullptr, batch ? batch->o : nullptr,
                                                              err);
  return (int)grid;
}

// -------------------------------------------------------------- parameters
// part j (0, 1, 2) of the exact split of b into three BF16 values:
// b = hi + mid + lo, each part the nearest BF16 of what the previous left
__device__ __forceinline__ __nv_bfloat16 bias_part(float b, int j) {
  __nv_bfloat16 h = __float2bfloat16_rn(b);
  for (int i = 0; i < j; ++i) {
    b -= __bfloat162float(h);
    h = __float2bfloat16_rn(b);
  }
  return h;
}

__global__ void k_mlp_pack(const float* __restrict__ p, MlpDev* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const __nv_bfloat16 z = __float2bfloat16_rn(0.f);
  if (i < kMlpH * kMlpK1) {
    const int r = i / kMlpK1, k = i - r * kMlpK1;
    d->w1[i] = k < kMlpIn ? __float2bfloat16_rn(p[kMlpOffW1 + r * kMlpIn + k])
                          : (k < kMlpOne + 3 ? bias_part(p[kMlpOffB1 + r], k - kMlpOne) : z);
  }
  if (i < kMlpH * kMlpK2) {
    const int r = i / kMlpK2, k = i - r * kMlpK2;
    d->w2[i] = k < kMlpH ? __float2bfloat16_rn(p[kMlpOffW2 + r * kMlpH + k])
                         : (k < kMlpH + 3 ? bias_part(p[kMlpOffB2 + r], k - kMlpH) : z);
  }
  if (i < kMlpN3 * kMlpK2) {
    const int r = i / kMlpK2, k = i - r * kMlpK2;
    d->w3[i] = r >= kMlpOut ? z
                            : (k < kMlpH ? __float2bfloat16_rn(p[kMlpOffW3 + r * kMlpH + k])
                                         : (k < kMlpH + 3 ? bias_part(p[kMlpOffB3 + r], k - kMlpH) : z));
  }
}

void mlp_pack(const float* params, MlpDev* dev, cudaStream_t s) {
  k_mlp_pack<<<(kMlpH * kMlpK2 + 255) / 256, 256, 0, s>>>(params, dev);
}

__global__ void k_features_bf16(const float* __restrict__ f, __nv_bfloat16* __restrict__ x, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n * kMlpK1;
       e += (long long)gridDim.x * blockDim.x) {
    const long long r = e / kMlpK1;
    const int k = (int)(e - r * kMlpK1);
    x[e] = __float2bfloat16_rn(k < kMlpIn ? f[r * kMlpIn + k] : (k < kMlpOne + 3 ? 1.f : 0.f));
  }
}

void mlp_features_bf16(const float* f, __nv_bfloat16* x16, long long n, cudaStream_t s) {
  long long g = (n * kMlpK1 + 255) / 256;
  if (g > sm_count() * 32) g = sm_count() * 32;
  if (g < 1) g = 1;
  k_features_bf16<<<(int)g, 256, 0, s>>>(f, x16, n);
}

// ----------------------------------------------------------- backward pass
// One CTA per tile of 128 points, thread t owns point t: it forms the
// output, hidden-2 and hidden-1 deltas of L = (1/(2n)) sum (C - y)^2 in FP32
// with the BF16 weights the forward pass used, stages them in shared memory,
// and the CTA writes its partial weight gradients (and loss sum) to
// part[blockIdx.x][kMlpParams + 1].
constexpr int kBwdLd = kMlpH + 1;  // padded row of the shared delta tiles
constexpr size_t kBwdSmem = sizeof(float) * ((size_t)kMlpTile * kBwdLd * 4 + (size_t)kMlpTile * (kMlpIn + 2) +
                                             (size_t)kMlpH * kBwdLd + (size_t)kMlpOut * kMlpH);

__global__ void __launch_bounds__(128) k_mlp_bwd(const __nv_bfloat16* __restrict__ x16, const float2* __restrict__ y,
                                                 long long n, const MlpDev* __restrict__ P,
                                                 const __nv_bfloat16* __restrict__ h1g,
                                                 const __nv_bfloat16* __restrict__ h2g, const float* __restrict__ og,
                                                 float* __restrict__ part) {
  extern __shared__ __align__(16) float sm[];
  float* d2 = sm;                         // [128][65] hidden-2 deltas
  float* d1 = d2 + kMlpTile * kBwdLd;     // [128][65] hidden-1 deltas
  float* h1 = d1 + kMlpTile * kBwdLd;     // [128][65]
  float* h2 = h1 + kMlpTile * kBwdLd;     // [128][65]
  float* xo = h2 + kMlpTile * kBwdLd;     // [128][14]: 12 inputs, 2 output deltas
  float* w2 = xo + kMlpTile * (kMlpIn + 2);  // [64][65] W2[n][k]
  float* w3 = w2 + kMlpH * kBwdLd;        // [2][64]
  __shared__ float s_loss[4];
  const int tid = threadIdx.x;
  for (int e = tid; e < kMlpH * kMlpH; e += blockDim.x)
    w2[(e / kMlpH) * kBwdLd + e % kMlpH] = __bfloat162float(P->w2[(e / kMlpH) * kMlpK2 + e % kMlpH]);
  for (int e = tid; e < kMlpOut * kMlpH; e += blockDim.x) w3[e] = __bfloat162float(P->w3[(e / kMlpH) * kMlpK2 + e % kMlpH]);
  __syncthreads();
  const long long row = (long long)blockIdx.x * kMlpTile + tid;
  const bool live = row < n;
  const float inv_n = 1.0f / (float)n;
  float loss = 0.f;
  float dout[kMlpOut] = {0.f, 0.f};
  float a1[kMlpH], a2[kMlpH];
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) {
    a1[k] = live ? __bfloat162float(h1g[row * kMlpH + k]) : 0.f;
    a2[k] = live ? __bfloat162float(h2g[row * kMlpH + k]) : 0.f;
  }
  if (live) {
    const float2 yy = y[row];
    const float tgt[2] = {yy.x, yy.y};
#pragma unroll
    for (int j = 0; j < kMlpOut; ++j) {
      const float o = og[2 * row + j];
      const float sig = 1.f / (1.f + expf(-o));
      const float c = kMlpScale * softplus(o);
      const float r = c - tgt[j];
      loss += r * r;
      dout[j] = r * inv_n * kMlpScale * sig;
    }
  }
  // hidden 2
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) {
    const float g = dout[0] * w3[k] + dout[1] * w3[kMlpH + k];
    d2[tid * kBwdLd + k] = a2[k] > 0.f ? g : 0.f;
    h1[tid * kBwdLd + k] = a1[k];
    h2[tid * kBwdLd + k] = a2[k];
  }
  // hidden 1: (d2 W2)_k = sum_n d2_n W2[n][k]
  for (int k = 0; k < kMlpH; ++k) {
    float g = 0.f;
#pragma unroll 8
    for (int m = 0; m < kMlpH; ++m) g += d2[tid * kBwdLd + m] * w2[m * kBwdLd + k];
    d1[tid * kBwdLd + k] = a1[k] > 0.f ? g : 0.f;
  }
#pragma unroll
  for (int i = 0; i < kMlpIn; ++i) xo[tid * (kMlpIn + 2) + i] = live ? __bfloat162float(x16[row * kMlpK1 + i]) : 0.f;
  xo[tid * (kMlpIn + 2) + kMlpIn] = dout[0];
  xo[tid * (kMlpIn + 2) + kMlpIn + 1] = dout[1];
  // loss sum of the tile (fixed order)
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if ((tid & 31) == 0) s_loss[tid >> 5] = loss;
  __syncthreads();
  float* out = part + (long long)blockIdx.x * (kMlpParams + 1);
  // weight gradients as sums over the tile's points
  for (int e = tid; e < kMlpH * kMlpIn; e += blockDim.x) {
    const int r = e / kMlpIn, i = e - r * kMlpIn;
    float g = 0.f;
    for (int p = 0; p < kMlpTile; ++p) g += d1[p * kBwdLd + r] * xo[p * (kMlpIn + 2) + i];
    out[kMlpOffW1 + e] = g;
  }
  for (int e = tid; e < kMlpH * kMlpH; e += blockDim.x) {
    const int r = e / kMlpH, k = e - r * kMlpH;
    float g = 0.f;
    for (int p = 0; p < kMlpTile; ++p) g += d2[p * kBwdLd + r] * h1[p * kBwdLd + k];
    out[kMlpOffW2 + e] = g;
  }
  for (int e = tid; e < kMlpOut * kMlpH; e += blockDim.x) {
    const int j = e / kMlpH, k = e - j * kMlpH;
    float g = 0.f;
    for (int p = 0; p < kMlpTile; ++p) g += xo[p * (kMlpIn + 2) + kMlpIn + j] * h2[p * kBwdLd + k];
    out[kMlpOffW3 + e] = g;
  }
  if (tid < kMlpH) {
    float g1 = 0.f, g2 = 0.f;
    for (int p = 0; p < kMlpTile; ++p) {
      g1 += d1[p * kBwdLd + tid];
      g2 += d2[p * kBwdLd + tid];
    }
    out[kMlpOffB1 + tid] = g1;
    out[kMlpOffB2 + tid] = g2;
  }
  if (tid < kMlpOut) {
    float g = 0.f;
    for (int p = 0; p < kMlpTile; ++p) g += xo[p * (kMlpIn + 2) + kMlpIn + tid];
    out[kMlpOffB3 + tid] = g;
  }
  if (tid == 0) out[kMlpParams] = (s_loss[0] + s_loss[1]) + (s_loss[2] + s_loss[3]);
}

// -------------------------------------------- backward pass on tensor cores
// The three contractions of the backward pass as tcgen05 MMAs, per tile of
// 128 points (thread t owns point t, TMEM lane t):
//   (1) hidden-1 pre-deltas   G1  = D2 W2          M = 128 points, N = 64, K = 64
//   (2) layer 1 and 2 weights [D2^T; D1^T] [H1 | 1 | X | 1]^T
//                                                  M = 128, N = 96, K = 128 points
//       rows 0..63 x columns 0..79 give dW2 and db2 (H1's constant-1
//       columns), rows 64..127 x columns 80..95 give dW1 and db1 (the input
//       tile's constant-1 column); the two off-diagonal blocks are unused
//   (3) layer 3 weights       [H2^T; 1] [DO_hi | DO_lo]^T
//                                                  M = 128 (65 used), N = 16 (4 used), K = 128
// The deltas are FP32; each enters the BF16 MMAs as an exact two-part split
// hi + lo (hi = bf16(d), lo = bf16(d - hi): 16 significand bits), so the
// products with the BF16 activations and weights lose nothing beyond 2^-17
// of the delta.  The weight gradients accumulate in TMEM over the CTA's tiles
// (persistent CTAs, fixed tile order); the CTA then writes its partial sums,
// reduced over CTAs in a fixed order by k_mlp_reduce as before.
constexpr int kBk = 128;  // K of the weight-gradient MMAs: the points of a tile
struct MlpBwdSmem {
  uint8_t w2t[kMlpH * kMlpH * 2];         // W2^T as [k][n] (N = 64, K = 64)
  uint8_t ad2[2][kMlpTile * kMlpH * 2];   // D2 [point][n], hi and lo (M = 128, K = 64)
  uint8_t ast[2][128 * kBk * 2];          // [D2^T; D1^T], hi and lo (M = 128, K = 128)
  uint8_t bst[96 * kBk * 2];              // [H1^T; 1; X^T] (N = 96, K = 128)
  uint8_t a3[128 * kBk * 2];              // [H2^T; 1; 0] (M = 128, K = 128)
  uint8_t b3[16 * kBk * 2];               // [DO_hi; DO_lo; 0] (N = 16, K = 128)
  float w3[kMlpOut * kMlpH];
  float red[4][kMlpOut];
  uint64_t mbar;
  uint32_t tbase;
};
constexpr size_t kMlpBwdSmemBytes = sizeof(MlpBwdSmem) + 1024;

__device__ __forceinline__ void st_bf16(uint8_t* tile, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + off) = __float2bfloat16_rn(v);
}
// the two-part split of v into the hi and lo tiles
__device__ __forceinline__ void st_split(uint8_t* hi, uint8_t* lo, uint32_t off, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  *reinterpret_cast<__nv_bfloat16*>(hi + off) = h;
  *reinterpret_cast<__nv_bfloat16*>(lo + off) = __float2bfloat16_rn(v - __bfloat162float(h));
}

__global__ void __launch_bounds__(128, 1)
    k_mlp_bwd_tc(const __nv_bfloat16* __restrict__ x16, const float2* __restrict__ y, long long n,
                 const MlpDev* __restrict__ P, const __nv_bfloat16* __restrict__ h1g,
                 const __nv_bfloat16* __restrict__ h2g, const float* __restrict__ og, float* __restrict__ part,
                 int* err) {
  extern __shared__ __align__(1024) uint8_t bwd_smem[];
  MlpBwdSmem& S = *reinterpret_cast<MlpBwdSmem*>(bwd_smem + ((1024u - (smem_u32(bwd_smem) & 1023u)) & 1023u));
  const int t = threadIdx.x;
  const long long ntiles = (n + kMlpTile - 1) / kMlpTile;
  if (t < 32) tmem_alloc(&S.tbase, 256);
  if (t == 0) {
    mbar_init(&S.mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // W2^T (element (k, n) = W2[n][k]) and the FP32 copy of W3
  for (int e = t; e < kMlpH * kMlpH; e += blockDim.x) {
    const int nn = e / kMlpH, k = e - nn * kMlpH;
    *reinterpret_cast<__nv_bfloat16*>(S.w2t + kmaj(k, nn, kMlpH)) = P->w2[nn * kMlpK2 + k];
  }
  for (int e = t; e < kMlpOut * kMlpH; e += blockDim.x)
    S.w3[e] = __bfloat162float(P->w3[(e / kMlpH) * kMlpK2 + e % kMlpH]);
  // the constant rows of this thread's column (point t) of the operand tiles
  for (int r = 64; r < 80; ++r) st_bf16(S.bst, kmaj(r, t, kBk), r < 67 ? 1.f : 0.f);
  for (int r = 64; r < 128; ++r) st_bf16(S.a3, kmaj(r, t, kBk), r == 64 ? 1.f : 0.f);
  for (int r = 4; r < 16; ++r) st_bf16(S.b3, kmaj(r, t, kBk), 0.f);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = S.tbase;
  const uint32_t tl = tm + ((uint32_t)(32 * (t >> 5)) << 16);  // this warp's lanes
  const uint32_t c_g1 = 0, c_st = 64, c_3 = 160;                // TMEM columns of the three results
  const float inv_n = 1.0f / (float)n;
  float loss = 0.f;
  uint32_t ph = 0;
  int bad = 0;
  bool mpend = false;
  auto wait_mma = [&]() {
    int b = t == 0 ? mbar_wait(&S.mbar, ph) : 0;
    b = __syncthreads_or(b);
    if (!b) {
      ph ^= 1u;
      mpend = false;
    }
    tc_fence_after();
    return b;
  };
  bool first = true;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long row = tile * kMlpTile + t;
    const bool live = row < n;
    // ---- this point's deltas (FP32)
    float dout[kMlpOut] = {0.f, 0.f};
    if (live) {
      const float2 yy = y[row];
      const float tg[2] = {yy.x, yy.y};
#pragma unroll
      for (int j = 0; j < kMlpOut; ++j) {
        const float o = og[2 * row + j];
        const float sig = 1.f / (1.f + expf(-o));
        const float r = kMlpScale * softplus(o) - tg[j];
        loss += r * r;
        dout[j] = r * inv_n * kMlpScale * sig;
      }
    }
    for (int k0 = 0; k0 < kMlpH; k0 += 8) {
      uint4 q1 = make_uint4(0u, 0u, 0u, 0u), q2 = q1;
      if (live) {
        q1 = *reinterpret_cast<const uint4*>(h1g + row * kMlpH + k0);
        q2 = *reinterpret_cast<const uint4*>(h2g + row * kMlpH + k0);
      }
      const __nv_bfloat16* a1 = reinterpret_cast<const __nv_bfloat16*>(&q1);
      const __nv_bfloat16* a2 = reinterpret_cast<const __nv_bfloat16*>(&q2);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int k = k0 + i;
        const float h2v = __bfloat162float(a2[i]);
        const float g = dout[0] * S.w3[k] + dout[1] * S.w3[kMlpH + k];
        const float d2 = h2v > 0.f ? g : 0.f;
        st_split(S.ad2[0], S.ad2[1], kmaj(t, k, kMlpH), d2);
        st_split(S.ast[0], S.ast[1], kmaj(k, t, kBk), d2);
        *reinterpret_cast<__nv_bfloat16*>(S.bst + kmaj(k, t, kBk)) = a1[i];
        *reinterpret_cast<__nv_bfloat16*>(S.a3 + kmaj(k, t, kBk)) = a2[i];
      }
    }
    {
      uint4 qx[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
      if (live) {
        qx[0] = *reinterpret_cast<const uint4*>(x16 + row * kMlpK1);
        qx[1] = *reinterpret_cast<const uint4*>(x16 + row * kMlpK1 + 8);
      }
      const __nv_bfloat16* xv = reinterpret_cast<const __nv_bfloat16*>(qx);
#pragma unroll
      for (int c = 0; c < kMlpK1; ++c) *reinterpret_cast<__nv_bfloat16*>(S.bst + kmaj(80 + c, t, kBk)) = xv[c];
      // rows j and 2 + j of [DO_hi; DO_lo]
#pragma unroll
      for (int j = 0; j < kMlpOut; ++j) st_split(S.b3 + kmaj(j, 0, kBk), S.b3 + kmaj(2 + j, 0, kBk), kmaj(0, t, kBk),
                                                 dout[j]);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- (1) G1 = D2 W2 (hi and lo parts) and (3) the layer-3 gradients
    if (t == 0) {
      const uint32_t id64 = idesc_bf16(128, 64), id16 = idesc_bf16(128, 16);
      const uint32_t w2 = smem_u32(S.w2t);
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int kk = 0; kk < kMlpH / 16; ++kk)
          mma_bf16(tm + c_g1, sdesc(smem_u32(S.ad2[h]) + 256 * kk, 128, kMlpH * 16), sdesc(w2 + 256 * kk, 128, kMlpH * 16),
                   id64, (h | kk) != 0);
#pragma unroll
      for (int kk = 0; kk < kBk / 16; ++kk)
        mma_bf16(tm + c_3, sdesc(smem_u32(S.a3) + 256 * kk, 128, kBk * 16), sdesc(smem_u32(S.b3) + 256 * kk, 128, kBk * 16),
                 id16, !(first && kk == 0));
      mma_commit(&S.mbar);
    }
    mpend = true;
    if ((bad = wait_mma())) break;
    // ---- hidden-1 deltas from G1 (this thread's lane), into rows 64..127 of [D2^T; D1^T]
    {
      uint4 q1[8];
      if (live)
#pragma unroll
        for (int j = 0; j < 8; ++j) q1[j] = *reinterpret_cast<const uint4*>(h1g + row * kMlpH + 8 * j);
      else
#pragma unroll
        for (int j = 0; j < 8; ++j) q1[j] = make_uint4(0u, 0u, 0u, 0u);
      const __nv_bfloat16* a1 = reinterpret_cast<const __nv_bfloat16*>(q1);
#pragma unroll
      for (int c0 = 0; c0 < kMlpH; c0 += 16) {
        float g[16];
        tmem_ld16(tl + c_g1 + (uint32_t)c0, g);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int k = c0 + i;
          const float d1 = __bfloat162float(a1[k]) > 0.f ? g[i] : 0.f;
          st_split(S.ast[0], S.ast[1], kmaj(64 + k, t, kBk), d1);
        }
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- (2) the layer-1 and layer-2 weight gradients, accumulated over tiles
    if (t == 0) {
      const uint32_t id96 = idesc_bf16(128, 96);
      const uint32_t bst = smem_u32(S.bst);
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int kk = 0; kk < kBk / 16; ++kk)
          mma_bf16(tm + c_st, sdesc(smem_u32(S.ast[h]) + 256 * kk, 128, kBk * 16), sdesc(bst + 256 * kk, 128, kBk * 16),
                   id96, !(first && h == 0 && kk == 0));
      mma_commit(&S.mbar);
    }
    mpend = true;
    if ((bad = wait_mma())) break;
    first = false;
  }
  if (bad && t == 0) atomicExch(err, 1);
  // an MMA group still in flight (the loop left early) completes before the
  // shared memory and TMEM it uses are released
  if (mpend && t == 0) mbar_wait(&S.mbar, ph);
  // ---- this CTA's partial sums (a CTA without tiles writes zeros)
  float* out = part + (long long)blockIdx.x * (kMlpParams + 1);
  if (!bad) {
    float v[16];
    if (t < kMlpH) {
      // row t: dW2[t][0..63] and db2[t] (column 64)
      for (int c0 = 0; c0 < 80; c0 += 16) {
        if (!first) tmem_ld16(tl + c_st + (uint32_t)c0, v);
        else for (int i = 0; i < 16; ++i) v[i] = 0.f;
        for (int i = 0; i < 16; ++i) {
          const int k = c0 + i;
          if (k < kMlpH) out[kMlpOffW2 + t * kMlpH + k] = v[i];
          else if (k == kMlpH) out[kMlpOffB2 + t] = v[i];
        }
      }
    } else {
      // row 64 + r: dW1[r][0..11] and db1[r] (columns 80..92)
      const int r = t - kMlpH;
      if (!first) tmem_ld16(tl + c_st + 80u, v);
      else for (int i = 0; i < 16; ++i) v[i] = 0.f;
      for (int c = 0; c < kMlpIn; ++c) out[kMlpOffW1 + r * kMlpIn + c] = v[c];
      out[kMlpOffB1 + r] = v[kMlpOne];
    }
    // layer 3: row k < 64 -> dW3[j][k] = hi + lo columns, row 64 -> db3[j]
    if (!first) tmem_ld16(tl + c_3, v);
    else for (int i = 0; i < 16; ++i) v[i] = 0.f;
    if (t < kMlpH) {
      for (int j = 0; j < kMlpOut; ++j) out[kMlpOffW3 + j * kMlpH + t] = v[j] + v[2 + j];
    } else if (t == kMlpH) {
      for (int j = 0; j < kMlpOut; ++j) out[kMlpOffB3 + j] = v[j] + v[2 + j];
    }
  }
  // the loss sum of the CTA's points (fixed order)
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if ((t & 31) == 0) S.red[t >> 5][0] = loss;
  tc_fence_before();
  __syncthreads();
  if (t == 0) out[kMlpParams] = (S.red[0][0] + S.red[1][0]) + (S.red[2][0] + S.red[3][0]);
  if (t < 32) {
    tc_fence_after();
    tmem_dealloc(tm, 256);
  }
}

// grad[p] = sum over CTAs of part[b][p] in CTA order; loss[0] likewise
__global__ void k_mlp_reduce(const float* __restrict__ part, int nblk, float* __restrict__ grad,
                             float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kMlpParams) return;
  float g = 0.f;
  for (int b = 0; b < nblk; ++b) g += part[(long long)b * (kMlpParams + 1) + p];
  if (p < kMlpParams) grad[p] = g;
  else loss[0] = g;
}

long long mlp_partials(long long n) { return ((n + kMlpTile - 1) / kMlpTile) * (kMlpParams + 1); }

void mlp_backward(const __nv_bfloat16* x16, const float2* y, long long n, const MlpDev* dev, const MlpBatch& batch,
                  float* part, float* grad, float* loss, int* err, bool tensor_cores, cudaStream_t s) {
  const long long ntiles = (n + kMlpTile - 1) / kMlpTile;
  int nblk;
  if (tensor_cores) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_mlp_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMlpBwdSmemBytes);
      attr = true;
    }
    // persistent: one CTA per SM (the operand tiles take 165 KB of shared memory)
    nblk = (int)(ntiles < sm_count() ? ntiles : sm_count());
    k_mlp_bwd_tc<<<nblk, kMlpTile, kMlpBwdSmemBytes, s>>>(x16, y, n, dev, batch.h1, batch.h2, batch.o, part, err);
  } else {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
      attr = true;
    }
    nblk = (int)ntiles;
    k_mlp_bwd<<<nblk, kMlpTile, kBwdSmem, s>>>(x16, y, n, dev, batch.h1, batch.h2, batch.o, part);
  }
  k_mlp_reduce<<<(kMlpParams + 1 + 255) / 256, 256, 0, s>>>(part, nblk, grad, loss);
}

// Adam (Kingma & Ba 2015): beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected
__global__ void k_mlp_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ g, float lr_t, float b1, float b2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr_t * mi / (sqrtf(vi) + 1e-8f);
}

void mlp_adam(float* params, float* m, float* v, const float* grad, int step, float lr, MlpDev* dev,
              cudaStream_t s) {
  const double b1 = 0.9, b2 = 0.999;
  const double lr_t = lr * sqrt(1.0 - pow(b2, step)) / (1.0 - pow(b1, step));
  k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(params, m, v, grad, (float)lr_t, (float)b1, (float)b2);
  mlp_pack(params, dev, s);
}

}  // namespace samgpu
