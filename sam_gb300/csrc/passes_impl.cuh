// Kernel templates of the five HBM passes (included by the translation
// units that instantiate them, one per working precision: passes.cu
// (FP64, plus the precision-independent kernels), passes_f32.cu and
// passes_dd.cu).
// The five HBM passes of one RK3 stage and the reference-layout variants of
// each transform.  Every pass moves a tile of pencils from HBM into shared
// memory, transforms it there (fft_engine.cuh) and writes it back transposed
// for the next pass, so the reference's MPI slab transposes (x2z_decomp.f,
// z2x_decomp.f) become the store patterns of these kernels.
//
//   z_inv  : z_trans_b.f:30-52     wave (kx,ky,kz)  -> (z, kx, ky)
//   y_inv  : xy_trans_b.f:14-38      (z, kx, ky)      -> (z, y, kx)
//   x_pass : xy_trans_b.f:39-60 + rhs.f:26-61 + xy_trans_f.f:26-37
//            (z, y, kx) -> physical line -> vel_max partials, products ->
//            (m, z, kx, y)
//   y_fwd  : xy_trans_f.f:39-54      (m, z, kx, y)    -> (m, kx, ky, z)
//   z_fwd  : z_trans_f.f:21-31 + rhs.f:108-142 + sam.f:210-221,293-314
//            (m, kx, ky, z) -> projected rhs, RK3 update of u
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "common.cuh"
#include "passes.cuh"

namespace samgpu {

template <typename T>
__device__ __forceinline__ void load_twiddles(cx_t<T>* s_tw, const cx_t<T>* __restrict__ g_tw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) s_tw[i] = g_tw[i];
}

// Element-wise tile copy with kBatch independent loads in flight per thread:
// v = get(e) for a batch of e, then put(e, v) for the same batch.
constexpr int kBatch = 8;

// Resident CTAs per SM each kernel's register budget is sized for (measured
// at 256^3): in FP32 the transpose passes of the 16 x 16 register path fit
// 64 registers (four CTAs; the y inverse 48 with five, 5 % faster; the y
// forward at six measured 12 % slower) and the x pass 72 (three CTAs of 288
// threads) without spills; the compile-time Stockham transposes (lengths 32-512)
// spilled 40-110 bytes at 64 and keep three CTAs (80 registers; 128^3 y
// forward 10 % faster); the FP32 z_fwd epilogue spills below 128 and keeps
// two (three measured slower); FP64 CTAs are bound by the FP64 pipe.
// The run-time-radix path (kFftGeneric, lengths without a compile-time
// path) needs more registers: one x pass CTA per SM, two of the others.
enum PassKind { kPassZInv, kPassYInv, kPassX, kPassYFwd, kPassZFwd };
template <typename T, int K, int PATH = kFft256> struct MinBlocks {
  static constexpr int value =
      PATH == kFftGeneric ? (K == kPassX ? 1 : 2) : (K == kPassZFwd ? 2 : (K == kPassX ? 3 : (PATH == kFft256 ? (K == kPassYInv ? 5 : 4) : 3)));
};
template <int K, int PATH> struct MinBlocks<double, K, PATH> {
  static constexpr int value = PATH == kFftGeneric ? 1 : 2;
};
// double-float pairs: the 16 x 16 register path holds 16 complex pairs (64
// registers) per thread, as in FP64
// (the z-forward epilogue keeps one CTA: its tiles fill the shared memory of
// an SM anyway, and two modes' inputs in flight need the registers)
template <int K, int PATH> struct MinBlocks<dd, K, PATH> {
  static constexpr int value = PATH == kFftGeneric || K == kPassZFwd ? 1 : 2;
};
template <typename V, typename Get, typename Put>
__device__ __forceinline__ void batched(int count, Get get, Put put) {
  for (int base = threadIdx.x; base < count; base += kBatch * blockDim.x) {
    V v[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int e = base + u * blockDim.x;
      if (e < count) v[u] = get(e);
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int e = base + u * blockDim.x;
      if (e < count) put(e, v[u]);
    }
  }
}

// v * s for a constant s of the launch: in the double-float form, when s is
// a power of two (1/Nz, 1/(2 Nx Ny) on power-of-two grids), two exact FP32
// products instead of a pair product
template <typename W> __device__ __forceinline__ W scale_by(W v, W s, bool pow2) { return v * s; }
template <> __device__ __forceinline__ dd scale_by<dd>(dd v, dd s, bool pow2) {
  return pow2 ? dd(__fmul_rn(v.hi, s.hi), __fmul_rn(v.lo, s.hi)) : v * s;
}
__host__ __device__ inline bool is_pow2_inv(int n) { return n > 0 && (n & (n - 1)) == 0; }

// First-stage loader reading element idx of a row in global memory.
// Store phase of the transposes: line t (t < nl) of a tile of `tile` lines
// in shared memory goes to dst[r * ostride + t] for output rows r < nr,
// taking its element at line position pos(r).  A thread keeps one line and
// walks r with a running pointer (consecutive threads: consecutive t of one
// row, so the stores coalesce); no division per element.
template <typename C, typename Pos>
__device__ __forceinline__ void store_tile_rows(C* __restrict__ dst, long long ostride, const C* s_ln, int ld, int tile,
                                                int nl, int nr, Pos pos) {
  const int span = min(tile, (int)blockDim.x);  // lines per sweep
  const int rs = (int)blockDim.x / span, r0 = (int)threadIdx.x / span;
  if (r0 >= rs) return;
  const long long step = (long long)rs * ostride;
  for (int t = (int)threadIdx.x - r0 * span; t < nl; t += span) {
    const C* src = s_ln + t * ld;
    C* o = dst + (long long)r0 * ostride + t;
#pragma unroll 4
    for (int r = r0; r < nr; r += rs, o += step) *o = src[sidx(pos(r))];
  }
}

// Loads of data that another CTA of the same launch wrote (the persistent
// ensemble stage kernel, COH = true) go to L2 (ld.global.cg), never to a
// possibly stale L1 line; the per-pass kernels (COH = false) load as usual.
template <bool COH, typename V> __device__ __forceinline__ V ldc(const V* p) {
  if constexpr (COH) return __ldcg(p);
  else return *p;
}

template <typename C, bool COH = false> struct RowLoad {
  const C* __restrict__ row;
  __device__ __forceinline__ C operator()(int idx) const { return ldc<COH>(row + idx); }
};

// First-stage loader of a row of stored modes 0..k, then -k..-1, padded to
// the transform length: idx <= lo from row[idx], idx >= hi from
// row[idx - gap], the band between as zero.
template <typename C, bool COH = false> struct BandRowLoad {
  const C* __restrict__ row;
  int lo, hi, gap;
  __device__ __forceinline__ C operator()(int idx) const {
    if (idx <= lo) return ldc<COH>(row + idx);
    if (idx >= hi) return ldc<COH>(row + idx - gap);
    return mk<C>((decltype(C::x))0, (decltype(C::x))0);
  }
};

// First-stage loader of a subgrid gradient field in k_z_inv: element p of
// the z line is i (alpha u_a + beta u_b) at the stored mode of p (zero in
// the truncated band), alpha = a0 + a1 kz and beta = b0 + b1 kz with kz the
// wave number of p; rb is null when beta = 0.
template <typename C> struct DeriveLoad {
  const C* __restrict__ ra;
  const C* __restrict__ rb;
  decltype(C::x) a0, a1, b0, b1;
  int km, nz, gap;
  __device__ __forceinline__ C operator()(int p) const {
    using T = decltype(C::x);
    if (p > km && p < nz - km) return mk<C>((T)0, (T)0);
    const bool lo = p <= km;
    const int q = lo ? p : p - gap;
    const T kz = (T)(lo ? p : p - nz);
    const C ua = ra[q];
    const T al = a0 + a1 * kz;
    T zr = al * ua.x, zi = al * ua.y;
    if (rb) {
      const C ub = rb[q];
      const T be = b0 + b1 * kz;
      zr += be * ub.x;
      zi += be * ub.y;
    }
    return mk<C>(-zi, zr);
  }
};

// --------------------------------------------------------------- z inverse
// Tile: field n, kx index i, ky rows j0 .. j0+TY-1.  Input rows hold Nz_min
// modes; output A(n, z, kx, ky) with ky fastest.
template <typename T, int PATH, bool COH = false>
__device__ __forceinline__ void z_inv_body(const ZInvArgs<T>& a, const FftPlan* __restrict__ gpl, int bid) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  load_plan(&pl, gpl);
  __syncthreads();
  C* s_tw = reinterpret_cast<C*>(smem_raw);
  C* s_ln = s_tw + tw_load<PATH>(pl);
  const int nz = a.g.nz, mz = a.g.mz, km = a.g.kz, my = a.g.my;
  const int ld = a.ld;
  const int nty = (my + a.ty - 1) / a.ty;
  int b = bid;
  const int jt = b % nty; b /= nty;
  const int i = b % a.g.mx; b /= a.g.mx;
  const int n = b;
  const int j0 = jt * a.ty;
  const int nl = min(a.ty, my - j0);
  load_twiddles<T>(s_tw, a.tw, tw_load<PATH>(pl));
  const C* src = a.in + (long long)n * a.in_n + (long long)i * a.in_kx + (long long)j0 * a.in_ky;
  __syncthreads();
  if (!a.derive || n < a.g.lu) {
    // the first stage reads the stored modes straight from the row, the
    // truncated band as zero (no shared-memory staging)
    fft_lines_from<+1, PATH>(s_ln, ld, nl, s_tw, pl, [&](int L) {
      return BandRowLoad<C, COH>{src + (long long)L * a.in_ky, km, nz - km, nz - mz};
    });
  } else {
    // gradient field m of the subgrid stress: S_ab = (i/2)(k_b u_a + k_a u_b)
    // (i k_a u_a when a = b) for the six velocity products in rhs.f's order,
    // i k_a T for the three buoyancy products
    // (fields m >= Lr: the vorticity w_a = i (k_b u_c - k_c u_b), (a, b, c)
    // cyclic, which only the learned closure's invariants use); formed from
    // the rows of u_a and u_b while the first stage loads them
    const int m = n - a.g.lu;
    const bool vort = m >= a.g.lr;
    int fa, fb;
    if (vort) {
      fa = (m - a.g.lr + 2) % 3;  // u_c, multiplied by k_b
      fb = (m - a.g.lr + 1) % 3;  // u_b, multiplied by k_c
    } else if (m < 6) {
      fb = m < 1 ? 0 : (m < 3 ? 1 : 2);
      fa = m - (fb * (fb + 1)) / 2;
    } else {
      fa = m - 6;
      fb = 3;
    }
    const long long off = (long long)i * a.in_kx + (long long)j0 * a.in_ky;
    const C* srca = a.in + (long long)(vort || m < 6 ? fa : 3) * a.in_n + off;
    const C* srcb = a.in + (long long)(vort || m < 6 ? fb : 3) * a.in_n + off;
    // alpha multiplies u_a, beta u_b: wave-number component and scale of each
    int da, db;
    T sa, sb;
    if (vort) {
      da = fb; sa = (T)1; db = fa; sb = (T)-1;
    } else if (m >= 6 || fa == fb) {
      da = fa; sa = (T)1; db = -1; sb = (T)0;
    } else {
      da = fb; sa = (T)0.5; db = fa; sb = (T)0.5;
    }
    const T kxv = (T)a.g.wave_x * (T)i, wz = (T)a.g.wave_z;
    fft_lines_from<+1, PATH>(s_ln, ld, nl, s_tw, pl, [&](int L) {
      const T kyv = (T)a.g.wave_y * (T)kwave(j0 + L, a.g.ky, my);
      const T kfix = da == 0 ? kxv : kyv, kfixb = db == 0 ? kxv : kyv;
      DeriveLoad<C> d;
      d.ra = srca + (long long)L * a.in_ky;
      d.rb = db >= 0 ? srcb + (long long)L * a.in_ky : nullptr;
      d.a0 = da < 2 ? sa * kfix : (T)0;
      d.a1 = da < 2 ? (T)0 : sa * wz;
      d.b0 = db >= 0 && db < 2 ? sb * kfixb : (T)0;
      d.b1 = db == 2 ? sb * wz : (T)0;
      d.km = km;
      d.nz = nz;
      d.gap = nz - mz;
      return d;
    });
  }
  __syncthreads();
  // store: a thread keeps row t of the tile and walks z with a running
  // pointer; consecutive threads write consecutive ky of one z
  C* dst = a.out + (long long)n * a.out_n + (long long)i * a.out_kx + j0;
  store_tile_rows(dst, a.out_z, s_ln, ld, a.ty, nl, nz, [](int z) { return z; });
}
template <typename T, int PATH>
__global__ void __launch_bounds__(kThreads, MinBlocks<T, kPassZInv, PATH>::value)
    k_z_inv(const __grid_constant__ ZInvArgs<T> a, const FftPlan* __restrict__ gpl) {
  z_inv_body<T, PATH>(a, gpl, blockIdx.x);
}

// --------------------------------------------------------------- y inverse
// Tile: field n, plane z, kx columns i0 .. i0+TX-1.  Input rows (one per kx)
// hold either Ny_min compact modes (zero band inserted here, as
// x2z_decomp.f:111-124 does) or Ny values with the band already present.
template <typename T, int PATH, bool COH = false>
__device__ __forceinline__ void y_inv_body(const YInvArgs<T>& a, const FftPlan* __restrict__ gpl, int bid) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  load_plan(&pl, gpl);
  __syncthreads();
  C* s_tw = reinterpret_cast<C*>(smem_raw);
  C* s_ln = s_tw + tw_load<PATH>(pl);
  const int ny = a.g.ny, my = a.g.my, km = a.g.ky, mx = a.g.mx;
  const int ld = a.ld;
  const int ntx = (mx + a.tx - 1) / a.tx;
  int b = bid;
  const int it = b % ntx; b /= ntx;
  const int z = b % a.g.nz; b /= a.g.nz;
  const int n = b;
  const int i0 = it * a.tx;
  const int nl = min(a.tx, mx - i0);
  load_twiddles<T>(s_tw, a.tw, tw_load<PATH>(pl));
  const C* src = a.in + (long long)n * a.in_n + (long long)z * a.in_z + (long long)i0 * a.in_kx;
  __syncthreads();
  // the first stage reads the rows straight from memory: all Ny values
  // (in_full) or the stored modes with the truncated band as zero
  if (a.in_full)
    fft_lines_from<+1, PATH>(s_ln, ld, nl, s_tw, pl,
                             [&](int L) { return RowLoad<C, COH>{src + (long long)L * a.in_kx}; });
  else
    fft_lines_from<+1, PATH>(s_ln, ld, nl, s_tw, pl,
                             [&](int L) { return BandRowLoad<C, COH>{src + (long long)L * a.in_kx, km, ny - km, ny - my}; });
  __syncthreads();
  C* dst = a.out + (long long)n * a.out_n + (long long)z * a.out_z + i0;
  store_tile_rows(dst, a.out_y, s_ln, ld, a.tx, nl, ny, [](int y) { return y; });
}
template <typename T, int PATH>
__global__ void __launch_bounds__(kThreads, MinBlocks<T, kPassYInv, PATH>::value)
    k_y_inv(const __grid_constant__ YInvArgs<T> a, const FftPlan* __restrict__ gpl) {
  y_inv_body<T, PATH>(a, gpl, blockIdx.x);
}

// Two adjacent complex values in one store (one 16-byte store in FP32, two in
// FP64); o must be aligned to twice the element size.
__device__ __forceinline__ void store_pair(float2* o, float2 a, float2 b) {
  *reinterpret_cast<float4*>(o) = make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void store_pair(double2* o, double2 a, double2 b) {
  o[0] = a;
  o[1] = b;
}
__device__ __forceinline__ void store_pair(ddc* o, ddc a, ddc b) {
  o[0] = a;
  o[1] = b;
}

// First-stage loader of the backward x transform: the stored half spectrum
// with the truncated band lo < idx < hi read as zero.
template <typename C> struct BandLoad {
  const C* line;
  int lo, hi;
  __device__ __forceinline__ C operator()(int idx) const {
    if (idx > lo && idx < hi) return mk<C>((decltype(C::x))0, (decltype(C::x))0);
    return line[sidx(idx)];
  }
};

// Error-free FP32 accumulation (Knuth's TwoSum, Dekker/FMA TwoProduct): a
// running sum kept as an unevaluated pair hi + lo carries about 48 bits,
// enough for the FP64-accurate vel_max sums of the FP32 form without FP64
// arithmetic (which runs at 1/64 of the FP32 rate on this GPU).
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b - bb);
  const float lo = a.lo + err;
  const float h = s + lo;
  return DF{h, lo - (h - s)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  DF r = df_add(a, b.hi);
  return df_add(r, b.lo);
}
__device__ __forceinline__ DF df_add_sq(DF a, float v) {
  const float p = v * v;
  const float e = fmaf(v, v, -p);  // p + e = v^2 exactly
  return df_add(df_add(a, p), e);
}

// The products of rhs.f:46-60, rounded once each.  In FP32 the rounding is
// spelled out (__fmul_rn is never fused into a neighbouring sum), so the
// general kernel and the fused FP32 x pass compute the same bits.  (A packed
// mul.rn.f32x2 would not do: where its result feeds an add/sub.rn.f32x2 the
// compiler fuses the pair into one FMA despite the .rn modifiers; measured
// on 2^20 random operand pairs, every differing result equalled fmaf.)
__device__ __forceinline__ float pmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double pmul(double a, double b) { return a * b; }
__device__ __forceinline__ dd pmul(dd a, dd b) { return a * b; }

// First-stage loader of the forward x transform: element idx of line a, or,
// when b is given, of line a times line b component by component (the two
// real rows of a pair multiply separately), i.e. a product line of rhs.f.
template <typename C> struct ProductLoad {
  const C* a;
  const C* b;
  const C* g;  // subgrid term added to the product (may be null)
  __device__ __forceinline__ C operator()(int idx) const {
    const C va = a[sidx(idx)];
    if (!b) return va;
    const C vb = b[sidx(idx)];
    if (!g) return mk<C>(pmul(va.x, vb.x), pmul(va.y, vb.y));
    const C vg = g[sidx(idx)];
    return mk<C>(pmul(va.x, vb.x) + vg.x, pmul(va.y, vb.y) + vg.y);
  }
};

// Subgrid stress on one physical point: s[0..5] the strain in product order
// (S11 S12 S22 S13 S23 S33), s[6..8] dT/dx_a; on return s holds the terms
// the products receive, -2 nu_t S and -kappa_t dT/dx with
// nu_t = cds |S|, |S| = sqrt(2 sum ifact S^2), kappa_t = nu_t prt_inv.
template <typename T>
__device__ __forceinline__ void sgs_point(T* s, int nf, T cds, T prt_inv) {
  T sum = (T)0;
#pragma unroll
  for (int m = 0; m < 6; ++m) sum += (m == 1 || m == 3 || m == 4 ? (T)2 : (T)1) * s[m] * s[m];
  const T nu = cds * sqrt((T)2 * sum);
  const T nu2 = (T)2 * nu, kap = nu * prt_inv;
#pragma unroll
  for (int m = 0; m < 6; ++m) s[m] = -nu2 * s[m];
#pragma unroll
  for (int m = 6; m < 9; ++m)
    if (m < nf) s[m] = -kap * s[m];
}

// As sgs_point with per-point coefficients: nu_t = cnu |S|, kappa_t = ckap |S|.
template <typename T>
__device__ __forceinline__ void sgs_point_c(T* s, int nf, T cnu, T ckap) {
  T sum = (T)0;
#pragma unroll
  for (int m = 0; m < 6; ++m) sum += (m == 1 || m == 3 || m == 4 ? (T)2 : (T)1) * s[m] * s[m];
  const T sm = sqrt((T)2 * sum);
  const T nu = cnu * sm, kap = ckap * sm;
  const T nu2 = (T)2 * nu;
#pragma unroll
  for (int m = 0; m < 6; ++m) s[m] = -nu2 * s[m];
#pragma unroll
  for (int m = 6; m < 9; ++m)
    if (m < nf) s[m] = -kap * s[m];
}

// The learned closure's 12 inputs at one point from the strain S (product
// order S11 S12 S22 S13 S23 S33), the temperature gradient g and the
// vorticity w; |S| = sqrt(2 S:S), eps = 1e-30:
//   f0 log(1 + |w|^2/|S|^2)           f6  S33 / |S|
//   f1 tr(S^3) / |S|^3                f7  w_z / (|S| + |w|)
//   f2 w.S.w / (|S| |w|^2)            f8  g.S.g / (|S| |g|^2)
//   f3 log(1 + |N^2| / |S|^2)         f9  w.g / (|w| |g|)
//   f4 asinh(b g_z / |S|^2)           f10 log(1 + |S| delta^2 / nu)
//   f5 log(1 + |b| |g_h| / |S|^2)     f11 4 (S13^2 + S23^2) / |S|^2
// (b = buoy_fac_z, g_h the horizontal part of g).
// Division in the invariants: exact in FP64; in FP32 the 2-ulp fast
// division (the invariants are rounded to BF16, 2^-8 relative, afterwards)
__device__ __forceinline__ double fdv(double a, double b) { return a / b; }
__device__ __forceinline__ float fdv(float a, float b) { return __fdividef(a, b); }

template <typename T>
__device__ __forceinline__ void closure_invariants(const T* S, const T* g, const T* w, T bz, T n2, T dsq, T nu,
                                                   float* f) {
  const T eps = (T)1e-30;
  const T M[3][3] = {{S[0], S[1], S[3]}, {S[1], S[2], S[4]}, {S[3], S[4], S[5]}};
  T s2 = (T)0, tr3 = (T)0, wSw = (T)0, gSg = (T)0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      s2 += M[i][j] * M[i][j];
      T sq = (T)0;
#pragma unroll
      for (int k = 0; k < 3; ++k) sq += M[i][k] * M[k][j];
      tr3 += sq * M[j][i];
      wSw += w[i] * M[i][j] * w[j];
      gSg += g[i] * M[i][j] * g[j];
    }
  s2 = (T)2 * s2;
  const T sn = sqrt(s2);
  const T w2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], wn = sqrt(w2);
  const T g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2], gn = sqrt(g2);
  const T inv_s2 = fdv((T)1, s2 + eps);
  f[0] = (float)log1p(w2 * inv_s2);
  f[1] = (float)fdv(tr3, s2 * sn + eps);
  f[2] = (float)fdv(wSw, sn * w2 + eps);
  f[3] = (float)log1p(fabs(n2) * inv_s2);
  f[4] = (float)asinh(bz * g[2] * inv_s2);
  f[5] = (float)log1p(fabs(bz) * sqrt(g[0] * g[0] + g[1] * g[1]) * inv_s2);
  f[6] = (float)fdv(M[2][2], sn + eps);
  f[7] = (float)fdv(w[2], sn + wn + eps);
  f[8] = (float)fdv(gSg, sn * g2 + eps);
  f[9] = (float)fdv(w[0] * g[0] + w[1] * g[1] + w[2] * g[2], wn * gn + eps);
  f[10] = (float)log1p(fdv(sn * dsq, nu));
  f[11] = (float)((T)4 * (S[3] * S[3] + S[4] * S[4]) * inv_s2);
}

__device__ __forceinline__ void store_features(void* feat, long long pt, const float* f) {
  uint32_t q[8];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    q[i] = *reinterpret_cast<const uint32_t*>(&h);
  }
  q[6] = 0x3F803F80u;  // columns 12, 13: 1.0 (the network's bias inputs)
  q[7] = 0x00003F80u;  // column 14: 1.0, column 15: 0
  uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(feat) + pt * 16);
  dst[0] = make_uint4(q[0], q[1], q[2], q[3]);
  dst[1] = make_uint4(q[4], q[5], q[6], q[7]);
}

// ------------------------------------------------------------------ x pass
// Tile: plane z, rows y0 .. y0+Y-1 (Y even).  Two real x-lines (rows y0+2c
// and y0+2c+1 of the same field) share one complex line: x + i y.
__device__ __forceinline__ void product_pair(int m, int& a, int& b) {
  // rhs.f:49-57 column order of the upper triangle: uu uv vv uw vw ww ut vt wt
  // (m = 0..5 is the triangle of the velocity, 6..8 pair u,v,w with T)
  if (m < 6) {
    b = m < 1 ? 0 : (m < 3 ? 1 : 2);
    a = m - (b * (b + 1)) / 2;
  } else {
    b = 3;
    a = m - 6;
  }
}

template <typename T, int PATH, bool COH = false>
__device__ __forceinline__ void x_pass_body(const XPassArgs<T>& a, const FftPlan* __restrict__ gpl, int bid) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  load_plan(&pl, gpl);
  __syncthreads();
  C* s_tw = reinterpret_cast<C*>(smem_raw);
  C* s_in = s_tw + tw_load<PATH>(pl);                  // nin * yp lines
  const int nx = a.g.nx, ny = a.g.ny, kmx = a.g.kx, mx = a.g.mx;
  const int Y = a.yt, yp = Y / 2, ld = a.ld;
  const int nin = a.nin;
  C* s_pr = s_in + nin * yp * ld;                // group product lines
  // vel_max's reduction scratch shares the product lines' space (it is done
  // before the first product is formed)
  double* s_red = reinterpret_cast<double*>(s_pr);
  const int nyt = (ny + Y - 1) / Y;
  const int yt = bid % nyt;
  const int z = bid / nyt;
  const int y0 = yt * Y;
  const int yv = min(Y, ny - y0);  // valid rows in the tile
  load_twiddles<T>(s_tw, a.tw, tw_load<PATH>(pl));

  // ---- build the input lines
  if (a.in_mode == 0) {
    // spectral rows of B(n, z, y, kx): Hermitian half spectra with kx <= kx_max
    // (the truncated band kx_max < p < Nx - kx_max is never stored: the
    // transform's first stage reads it as zero)
    // FP32: a thread keeps one kx (consecutive threads: consecutive kx of a
    // row) and takes the lines L = lane + u * lanes, u < kBatch: all loads of
    // the batch (two rows per line) are issued before the first store.  (In
    // FP64, 256 threads over Mx = 86 leave a third idle: measured slower
    // there, so FP64 keeps the element-wise batches.)
    if constexpr (sizeof(T) == 4) {
      const int nl = nin * yp;
      const int kspan = min(mx, (int)blockDim.x);
      const int lanes = (int)blockDim.x / kspan;
      const int lane = (int)threadIdx.x / kspan;
      if (lane < lanes)
        for (int kx = (int)threadIdx.x - lane * kspan; kx < mx; kx += kspan) {
          const C* src0 = a.in + (long long)z * a.in_z + kx;
          const int sa = sidx(kx), sb = sidx(kx == 0 ? 0 : nx - kx);
          for (int L0 = lane; L0 < nl; L0 += kBatch * lanes) {
            C X[kBatch], Yv[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
              const int L = L0 + u * lanes;
              X[u] = mk<C>((T)0, (T)0);
              Yv[u] = mk<C>((T)0, (T)0);
              if (L < nl) {
                const int f = (int)fdiv(L, a.fd_yp), c = L - f * yp;
                const int ya = y0 + 2 * c;
                const C* src = src0 + (long long)f * a.in_n + (long long)ya * a.in_y;
                if (ya < ny) X[u] = ldc<COH>(src);
                if (ya + 1 < ny) Yv[u] = ldc<COH>(src + a.in_y);
              }
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
              const int L = L0 + u * lanes;
              if (L < nl) {
                if (kx == 0) {  // xy_trans_b.f:28-31 keeps only the real part of kx = 0
                  X[u].y = (T)0;
                  Yv[u].y = (T)0;
                }
                s_in[L * ld + sa] = mk<C>(X[u].x - Yv[u].y, X[u].y + Yv[u].x);
                if (kx > 0) s_in[L * ld + sb] = mk<C>(X[u].x + Yv[u].y, Yv[u].x - X[u].y);
              }
            }
          }
        }
    } else {
      // element e -> line L = (f, c) and kx; loads the two rows of the pair
      struct Pair { C x, y; };
      batched<Pair>(
          nin * yp * mx,
          [&](int e) {
            const int L = (int)fdiv(e, a.fd_mx), kx = e - L * mx;
            const int f = (int)fdiv(L, a.fd_yp), c = L - f * yp;
            const int ya = y0 + 2 * c, yb = ya + 1;
            const C* src = a.in + (long long)f * a.in_n + (long long)z * a.in_z;
            Pair q;
            q.x = ya < ny ? ldc<COH>(src + (long long)ya * a.in_y + kx) : mk<C>((T)0, (T)0);
            q.y = yb < ny ? ldc<COH>(src + (long long)yb * a.in_y + kx) : mk<C>((T)0, (T)0);
            return q;
          },
          [&](int e, Pair q) {
            const int L = (int)fdiv(e, a.fd_mx), kx = e - L * mx;
            C X = q.x, Yv = q.y;
            if (kx == 0) {  // xy_trans_b.f:28-31 keeps only the real part of kx = 0
              X.y = (T)0;
              Yv.y = (T)0;
            }
            s_in[L * ld + sidx(kx)] = mk<C>(X.x - Yv.y, X.y + Yv.x);
            if (kx > 0) s_in[L * ld + sidx(nx - kx)] = mk<C>(X.x + Yv.y, Yv.x - X.y);
          });
    }
    __syncthreads();
    fft_lines_from<+1, PATH>(s_in, ld, nin * yp, s_tw, pl,
                       [&](int L) { return BandLoad<C>{s_in + L * ld, kmx, nx - kmx}; });
  } else {
    // physical rows of P(n, z, y, x)
    struct Pair { T x, y; };
    batched<Pair>(
        nin * yp * nx,
        [&](int e) {
          const int L = (int)fdiv(e, a.fd_nx), x = e - L * nx;
          const int f = (int)fdiv(L, a.fd_yp), c = L - f * yp;
          const int ya = y0 + 2 * c, yb = ya + 1;
          const T* src = a.in_phys + (long long)f * a.in_n + (long long)z * a.in_z;
          Pair q;
          q.x = ya < ny ? src[(long long)ya * a.in_y + x] : (T)0;
          q.y = yb < ny ? src[(long long)yb * a.in_y + x] : (T)0;
          return q;
        },
        [&](int e, Pair q) {
          const int L = (int)fdiv(e, a.fd_nx), x = e - L * nx;
          s_in[L * ld + sidx(x)] = mk<C>(q.x, q.y);
        });
  }
  __syncthreads();

  // ---- vel_max partial sums (vel_max.f:11-21), FP64-accurate,
  // deterministic order (FP64 arithmetic in the FP64 form; error-free FP32
  // pairs in the FP32 form, turned into FP64 per warp)
  if constexpr (kIsDD<T>) {
    if (a.partials) {
      // the double-float form: max |u| as order-preserving 64-bit keys of
      // the pairs (FP32 and integer work only), the non-finite flag; the
      // sums come from wave space (k_parseval, FP64)
      unsigned long long km[4] = {0ull, 0ull, 0ull, 0ull};
      int bad = 0;
      for (int e = threadIdx.x; e < yp * nx; e += blockDim.x) {
        const int c = (int)fdiv(e, a.fd_nx), x = e - c * nx;
        const bool ra = y0 + 2 * c < ny, rb = y0 + 2 * c + 1 < ny;
#pragma unroll
        for (int f = 0; f < 4; ++f)
          if (f < a.g.lu) {
            const C v = s_in[(f * yp + c) * ld + sidx(x)];
            if (ra) {
              km[f] = max(km[f], dd_abs_key(v.x));
              bad |= !dd_isfinite(v.x);
            }
            if (rb) {
              km[f] = max(km[f], dd_abs_key(v.y));
              bad |= !dd_isfinite(v.y);
            }
          }
      }
      for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int f = 0; f < 4; ++f) km[f] = max(km[f], __shfl_xor_sync(0xffffffffu, km[f], o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
      }
      const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
      unsigned long long* s_km = reinterpret_cast<unsigned long long*>(s_red);
      int* s_bad = reinterpret_cast<int*>(s_km + 4 * nw);
      if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int f = 0; f < 4; ++f) s_km[w * 4 + f] = km[f];
        s_bad[w] = bad;
      }
      __syncthreads();
      if (threadIdx.x < a.g.lu) {
        const int f = threadIdx.x;
        unsigned long long tm = 0ull;
        int tb = 0;
        for (int k = 0; k < nw; ++k) {
          tm = max(tm, s_km[k * 4 + f]);
          tb |= s_bad[k];
        }
        atomicMax(reinterpret_cast<unsigned long long*>(a.vmax) + f, tm);
        if (f == 0 && tb) atomicOr(a.vmax + 8, 1);
      }
      __syncthreads();
    }
  } else if (a.partials && a.max_only) {
    // the FP32 form: max |u| and the non-finite flag here, the sums from
    // wave space (k_parseval); all four fields in one reduction
    T mx4[4] = {(T)0, (T)0, (T)0, (T)0};
    int bad = 0;
    for (int e = threadIdx.x; e < yp * nx; e += blockDim.x) {
      const int c = (int)fdiv(e, a.fd_nx), x = e - c * nx;
      const bool ra = y0 + 2 * c < ny, rb = y0 + 2 * c + 1 < ny;
#pragma unroll
      for (int f = 0; f < 4; ++f)
        if (f < a.g.lu) {
          const C v = s_in[(f * yp + c) * ld + sidx(x)];
          if (ra) {
            mx4[f] = fmax(mx4[f], fabs(v.x));
            bad |= !isfinite(v.x);
          }
          if (rb) {
            mx4[f] = fmax(mx4[f], fabs(v.y));
            bad |= !isfinite(v.y);
          }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int f = 0; f < 4; ++f) mx4[f] = fmax(mx4[f], __shfl_xor_sync(0xffffffffu, mx4[f], o));
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // (FP32 and integer only: an FP64 conversion here is issued by every warp)
    float* s_mx = reinterpret_cast<float*>(s_red);
    int* s_bad = reinterpret_cast<int*>(s_mx + 4 * nw);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int f = 0; f < 4; ++f) s_mx[w * 4 + f] = (float)mx4[f];
      s_bad[w] = bad;
    }
    __syncthreads();
    // one atomic per field and CTA: the max of non-negative floats is the max
    // of their bit patterns (order-independent, so deterministic)
    if (threadIdx.x < a.g.lu) {
      const int f = threadIdx.x;
      float tm = 0.f;
      int tb = 0;
      for (int k = 0; k < nw; ++k) {
        tm = fmaxf(tm, s_mx[k * 4 + f]);
        tb |= s_bad[k];
      }
      atomicMax(a.vmax + f, __float_as_int(tm));
      if (f == 0 && tb) atomicOr(a.vmax + 8, 1);
    }
    __syncthreads();
  } else if (a.partials) {
    for (int f = 0; f < a.g.lu; ++f) {
      double s1 = 0.0, s2 = 0.0;
      DF d1{0.f, 0.f}, d2{0.f, 0.f};
      T mxv = (T)0;
      int bad = 0;
      for (int e = threadIdx.x; e < yp * nx; e += blockDim.x) {
        const int c = (int)fdiv(e, a.fd_nx), x = e - c * nx;
        const C v = s_in[(f * yp + c) * ld + sidx(x)];
        if (y0 + 2 * c < ny) {
          if (sizeof(T) == 8) {
            const double d = (double)v.x;
            s1 += d; s2 += d * d;
          } else {
            d1 = df_add(d1, (float)v.x);
            d2 = df_add_sq(d2, (float)v.x);
          }
          mxv = fmax(mxv, fabs(v.x));
          bad |= !isfinite(v.x);
        }
        if (y0 + 2 * c + 1 < ny) {
          if (sizeof(T) == 8) {
            const double d = (double)v.y;
            s1 += d; s2 += d * d;
          } else {
            d1 = df_add(d1, (float)v.y);
            d2 = df_add_sq(d2, (float)v.y);
          }
          mxv = fmax(mxv, fabs(v.y));
          bad |= !isfinite(v.y);
        }
      }
      if (sizeof(T) == 4) {
        for (int o = 16; o > 0; o >>= 1) {
          d1 = df_add(d1, DF{__shfl_xor_sync(0xffffffffu, d1.hi, o), __shfl_xor_sync(0xffffffffu, d1.lo, o)});
          d2 = df_add(d2, DF{__shfl_xor_sync(0xffffffffu, d2.hi, o), __shfl_xor_sync(0xffffffffu, d2.lo, o)});
        }
        s1 = (double)d1.hi + (double)d1.lo;
        s2 = (double)d2.hi + (double)d2.lo;
      }
      // warp reduce then CTA reduce
      for (int o = 16; o > 0; o >>= 1) {
        if (sizeof(T) == 8) {
          s1 += __shfl_xor_sync(0xffffffffu, s1, o);
          s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        mxv = fmax(mxv, __shfl_xor_sync(0xffffffffu, mxv, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
      }
      const double mxd = (double)mxv;
      const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
      if ((threadIdx.x & 31) == 0) {
        s_red[w * 4 + 0] = s1; s_red[w * 4 + 1] = s2; s_red[w * 4 + 2] = mxd; s_red[w * 4 + 3] = (double)bad;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double t1 = 0, t2 = 0, tm = 0, tb = 0;
        for (int k = 0; k < nw; ++k) {
          t1 += s_red[k * 4 + 0]; t2 += s_red[k * 4 + 1];
          tm = fmax(tm, s_red[k * 4 + 2]); tb += s_red[k * 4 + 3];
        }
        double* dst = a.partials + ((long long)bid * a.g.lu + f) * 4;
        dst[0] = t1; dst[1] = t2; dst[2] = tm; dst[3] = tb;
      }
      __syncthreads();
    }
  }

  // ---- the closure's invariants (out_mode 4): inputs are S (6), dT/dx (3
  // when Lr = 9) and w (3)
  if (a.out_mode == 4) {
    if constexpr (!kIsDD<T>) {  // (the double-float form has no closure)
    const int lr = a.g.lr;
    const T bz = (T)a.f_bz, n2 = (T)a.f_n2, dsq = (T)a.f_dsq, nu = (T)a.f_nu;
    for (int e = threadIdx.x; e < yp * nx; e += blockDim.x) {
      const int c = (int)fdiv(e, a.fd_nx), x = e - c * nx;
      T sx[6], sy[6], gx[3] = {(T)0, (T)0, (T)0}, gy[3] = {(T)0, (T)0, (T)0}, wx[3], wy[3];
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const C v = s_in[(m * yp + c) * ld + sidx(x)];
        sx[m] = v.x;
        sy[m] = v.y;
      }
      if (lr == 9)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const C v = s_in[((6 + m) * yp + c) * ld + sidx(x)];
          gx[m] = v.x;
          gy[m] = v.y;
        }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const C v = s_in[((lr + m) * yp + c) * ld + sidx(x)];
        wx[m] = v.x;
        wy[m] = v.y;
      }
      float f[12];
      const int ya = y0 + 2 * c;
      if (ya < ny) {
        closure_invariants<T>(sx, gx, wx, bz, n2, dsq, nu, f);
        store_features(a.feat, ((long long)z * ny + ya) * nx + x, f);
      }
      if (ya + 1 < ny) {
        closure_invariants<T>(sy, gy, wy, bz, n2, dsq, nu, f);
        store_features(a.feat, ((long long)z * ny + ya + 1) * nx + x, f);
      }
    }
    }
    return;
  }

  // ---- subgrid stress: the gradient lines become -2 nu_t S and -kappa_t dT
  if (a.les) {
    if constexpr (!kIsDD<T>) {  // (the double-float form has no closure)
    const int lu = a.g.lu, lr = a.g.lr;
    const T cds = a.les == 1 ? (T)a.les_cds[0] : (T)0, prt = (T)a.les_prt_inv;
    for (int e = threadIdx.x; e < yp * nx; e += blockDim.x) {
      const int c = (int)fdiv(e, a.fd_nx), x = e - c * nx;
      C v[9];
      T sx[9], sy[9];
#pragma unroll
      for (int m = 0; m < 9; ++m)
        if (m < lr) {
          v[m] = s_in[((lu + m) * yp + c) * ld + sidx(x)];
          sx[m] = v[m].x;
          sy[m] = v[m].y;
        }
      if (a.les == 2) {
        // learned closure: per-point coefficients (rows past Ny are padding)
        const int ya = min(y0 + 2 * c, ny - 1), yb = min(y0 + 2 * c + 1, ny - 1);
        const float2 ca = a.les_coef[((long long)z * ny + ya) * nx + x];
        const float2 cb = a.les_coef[((long long)z * ny + yb) * nx + x];
        // C delta^2 in the working precision (no FP64 per point in FP32)
        const T dsq = (T)a.les_dsq;
        sgs_point_c<T>(sx, lr, (T)ca.x * dsq, (T)ca.y * dsq);
        sgs_point_c<T>(sy, lr, (T)cb.x * dsq, (T)cb.y * dsq);
      } else {
        sgs_point<T>(sx, lr, cds, prt);
        sgs_point<T>(sy, lr, cds, prt);
      }
#pragma unroll
      for (int m = 0; m < 9; ++m)
        if (m < lr) s_in[((lu + m) * yp + c) * ld + sidx(x)] = mk<C>(sx[m], sy[m]);
    }
    }
    __syncthreads();
  }

  // ---- outputs
  if (a.out_mode == 3) return;  // statistics only (vel_max.f)
  if (a.out_mode == 0) {
    // physical rows (xy_trans_b.f:57-59)
    for (int e = threadIdx.x; e < nin * Y * nx; e += blockDim.x) {
      const int r = (int)fdiv(e, a.fd_nx), x = e - r * nx;
      const int f = (int)fdiv(r, a.fd_y), yy = r - f * Y;
      if (yy < yv) {
        const C v = s_in[(f * yp + (yy >> 1)) * ld + sidx(x)];
        a.out_phys[(long long)f * a.out_pn + (long long)z * a.out_pz + (long long)(y0 + yy) * a.out_py + x] =
            (yy & 1) ? v.y : v.x;
      }
    }
    return;
  }
  const T fn = a.fn;  // 1/(Nx Ny) (xy_trans_f.f:20) and the 1/2 of the split
  const bool fn_pow2 = is_pow2_inv(nx) && is_pow2_inv(ny);
  // output line q = m * Y/2 + c: pair c of output field m.  out_mode 1
  // transforms the input lines in place, all at once; out_mode 2 forms the
  // products `group` lines at a time (group >= 1 by construction)
  const int nlo = (a.out_mode == 1 ? nin : a.g.lr) * yp;
  const int gstep = a.out_mode == 1 ? nlo : max(a.group, 1);
  for (int l0 = 0; l0 < nlo; l0 += gstep) {
    const int gl = min(gstep, nlo - l0);
    // out_mode 2 (rhs.f:46-60): the products of the physical lines, formed
    // while the first FFT stage loads them, straight into the product lines
    C* lines = a.out_mode == 1 ? s_in : s_pr;
    fft_lines_from<-1, PATH>(lines, ld, gl, s_tw, pl, [&](int L) {
      if (a.out_mode == 1) return ProductLoad<C>{lines + L * ld, nullptr, nullptr};
      const int q = l0 + L;
      const int m = (int)fdiv(q, a.fd_yp), c = q - m * yp;
      int fa, fb;
      product_pair(m, fa, fb);
      const C* gl_ = a.les ? s_in + ((a.g.lu + m) * yp + c) * ld : nullptr;
      return ProductLoad<C>{s_in + (fa * yp + c) * ld, s_in + (fb * yp + c) * ld, gl_};
    });
    __syncthreads();
    // split the two real transforms, keep kx <= kx_max, scale, store
    // C(m, z, kx, y): a thread keeps one line (the rows y0+2c, y0+2c+1 of
    // field m) and steps through kx with running pointers; consecutive
    // threads take consecutive lines (rows, then fields) of one kx
    {
      const int span = min(gstep, (int)blockDim.x);
      const int lanes = (int)blockDim.x / span;
      const int lane = (int)threadIdx.x / span;
      const long long ostep = (long long)lanes * a.out_kx;
      if (lane < lanes)
        for (int L = (int)threadIdx.x - lane * span; L < gl; L += span) {
          const int q = l0 + L;
          const int m = (int)fdiv(q, a.fd_yp), c = q - m * yp;
          const C* ln = lines + L * ld;
          C* o = a.out + (long long)z * a.out_z + y0 + (long long)m * a.out_n + (long long)lane * a.out_kx + 2 * c;
          const bool two = 2 * c + 1 < yv, one = 2 * c < yv;
          for (int kx = lane; kx < mx; kx += lanes, o += ostep) {
            const C z1 = ln[sidx(kx)];
            const C z2 = ln[sidx(kx == 0 ? 0 : nx - kx)];
            const C ve = mk<C>(scale_by(z1.x + z2.x, fn, fn_pow2), scale_by(z1.y - z2.y, fn, fn_pow2));
            const C vo = mk<C>(scale_by(z1.y + z2.y, fn, fn_pow2), scale_by(z2.x - z1.x, fn, fn_pow2));
            if (two) {
              if ((reinterpret_cast<uintptr_t>(o) & (2 * sizeof(C) - 1)) == 0) {
                store_pair(o, ve, vo);
              } else {  // odd Ny: the pair straddles a vector boundary
                o[0] = ve;
                o[1] = vo;
              }
            } else if (one) {
              o[0] = ve;
            }
          }
        }
    }
    __syncthreads();
  }
}
template <typename T, int PATH>
__global__ void __launch_bounds__(x_threads(sizeof(T), PATH == kFft256), MinBlocks<T, kPassX, PATH>::value)
    k_x_pass(const __grid_constant__ XPassArgs<T> a, const FftPlan* __restrict__ gpl) {
  x_pass_body<T, PATH>(a, gpl, blockIdx.x);
}

// ------------------------------------------------ x pass, FP32 at Nx = 256
// The x pass of the plain FP32 step with 256-point x lines (spectral input
// rows, products out, no subgrid terms; at stage 1 vel_max's max |u| and
// non-finite flag) as one kernel without run-time generality.  Its
// arithmetic is x_pass_body's 16 x 16 register path operation for operation,
// so the results are bit-identical; the bookkeeping around it differs:
//  - the truncated band kx_max < p < Nx - kx_max of each staged line is
//    written as zeros once, so the first transform stage reads plain shared
//    memory (no per-element band test);
//  - a team of 16 threads owns one scratch line and takes a product line
//    from its first transform stage to HBM by itself: it forms the product
//    while loading, transforms it, pairs Z(kx) with Z(Nx - kx) by shuffles
//    within the team (thread k holds Z(k + 16 j) after the second stage, and
//    Z(256 - k - 16 j) sits in thread (16 - k) mod 16 at j' = 15 - j, or at
//    (16 - j) mod 16 for k = 0) and stores the split pair.  Teams synchronise
//    only among their own 16 threads: the product phase has no CTA barrier
//    and no separate output loop.
// Shared memory: the 16 x 16 twiddles w_256^{k q} at [16 q + k], the Nin *
// Y/2 input lines, one scratch line per team (vel_max's reduction scratch
// before the products).
constexpr int kXf256Threads = 288;                  // 18 teams of 16 (two rounds of 9 x 4 product lines)
constexpr int kXf256Teams = kXf256Threads / 16;
constexpr int kXf256Ld = 271;                       // line_stride(256)
static_assert(kXf256Ld == ((256 + (255 >> 4)) | 1), "line stride of a 256-point line");
__host__ __device__ constexpr size_t x_f256_smem(int lines) {
  return sizeof(float2) * (256 + (size_t)(lines + kXf256Teams) * kXf256Ld);
}

// the second stage of the 16 x 16 path on a line already in shared memory:
// thread k reads row 16 k + q, applies w_256^{k q} and transforms it, leaving
// Z(k + 16 j) in v[j]
template <int SIGN>
__device__ __forceinline__ void f256_rows(float2* v, const float2* line, const float2* w, int k) {
  v[0] = line[17 * k];
#pragma unroll
  for (int q = 1; q < 16; ++q) v[q] = ctw<SIGN>(line[17 * k + q], w[16 * q]);
  dft16<SIGN>(v);
}

// (a template only so that the translation units including this header
// share one instantiation)
template <int V = 0>
__global__ void __launch_bounds__(kXf256Threads, 3) k_x_pass_f256(const __grid_constant__ XPassArgs<float> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int nx = 256, LD = kXf256Ld;
  float2* s_tw = reinterpret_cast<float2*>(smem_raw);
  float2* s_in = s_tw + 256;
  const int ny = a.g.ny, kmx = a.g.kx, mx = a.g.mx;
  const int Y = a.yt, yp = Y / 2, nl = a.nin * yp;
  float2* s_pr = s_in + nl * LD;
  const int nyt = (ny + Y - 1) / Y;
  const int z = blockIdx.x / nyt;
  const int y0 = (blockIdx.x - z * nyt) * Y;
  const int yv = min(Y, ny - y0);
  const int tid = threadIdx.x;
  if (tid < 256) s_tw[tid] = a.tw[tid];
  {
    // zeros in the truncated band (sidx of its ends: one contiguous run)
    const int b0 = sidx(kmx + 1), nb = sidx(nx - kmx - 1) - b0 + 1;
    for (int L = tid / 18; L < nl; L += kXf256Threads / 18)
      for (int j = tid % 18; j < nb; j += 18) s_in[L * LD + b0 + j] = make_float2(0.f, 0.f);
  }
  {
    // the stored half spectra, two rows per line (x + i y): a thread keeps
    // one kx and issues the loads of a batch of lines before its stores
    const int kspan = min(mx, kXf256Threads);
    const int lanes = kXf256Threads / kspan;
    const int lane = tid / kspan;
    if (lane < lanes)
      for (int kx = tid - lane * kspan; kx < mx; kx += kspan) {
        const float2* src0 = a.in + (long long)z * a.in_z + kx;
        const int sa = sidx(kx), sb = sidx(kx == 0 ? 0 : nx - kx);
        for (int L0 = lane; L0 < nl; L0 += kBatch * lanes) {
          float2 X[kBatch], Yv[kBatch];
#pragma unroll
          for (int u = 0; u < kBatch; ++u) {
            const int L = L0 + u * lanes;
            X[u] = make_float2(0.f, 0.f);
            Yv[u] = make_float2(0.f, 0.f);
            if (L < nl) {
              const int f = (int)fdiv(L, a.fd_yp), c = L - f * yp;
              const int ya = y0 + 2 * c;
              const float2* src = src0 + (long long)f * a.in_n + (long long)ya * a.in_y;
              if (ya < ny) X[u] = src[0];
              if (ya + 1 < ny) Yv[u] = src[a.in_y];
            }
          }
#pragma unroll
          for (int u = 0; u < kBatch; ++u) {
            const int L = L0 + u * lanes;
            if (L < nl) {
              if (kx == 0) {  // xy_trans_b.f:28-31 keeps only the real part of kx = 0
                X[u].y = 0.f;
                Yv[u].y = 0.f;
              }
              s_in[L * LD + sa] = make_float2(X[u].x - Yv[u].y, X[u].y + Yv[u].x);
              if (kx > 0) s_in[L * LD + sb] = make_float2(X[u].x + Yv[u].y, Yv[u].x - X[u].y);
            }
          }
        }
      }
  }
  __syncthreads();

  // ---- the backward transforms (xy_trans_b.f:39-60), in place
  const int team = tid >> 4, k = tid & 15;
  const unsigned tmask = 0xFFFFu << (tid & 16);
  const float2* w = s_tw + k;
  for (int L = team; L < nl; L += kXf256Teams) {
    float2* line = s_in + L * LD;
    float2 v[16];
    // the first stage reads and writes the thread's own column (k + 17 q)
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = line[k + 17 * q];
    dft16<+1>(v);
#pragma unroll
    for (int s = 0; s < 16; ++s) line[17 * s + k] = v[s];
    __syncwarp(tmask);
    f256_rows<+1>(v, line, w, k);
    __syncwarp(tmask);
#pragma unroll
    for (int s = 0; s < 16; ++s) line[k + 17 * s] = v[s];
  }
  __syncthreads();

  // ---- vel_max (vel_max.f:11-21): max |u| of each field and the
  // non-finite flag; the sums come from wave space (k_parseval)
  if (a.partials) {
    float mx4[4] = {0.f, 0.f, 0.f, 0.f};
    int bad = 0;
    for (int e = tid; e < yp * nx; e += kXf256Threads) {
      const int c = e >> 8, x = e & 255;
      const bool ra = y0 + 2 * c < ny, rb = y0 + 2 * c + 1 < ny;
#pragma unroll
      for (int f = 0; f < 4; ++f)
        if (f < a.g.lu) {
          const float2 v = s_in[(f * yp + c) * LD + sidx(x)];
          if (ra) {
            mx4[f] = fmaxf(mx4[f], fabsf(v.x));
            bad |= !isfinite(v.x);
          }
          if (rb) {
            mx4[f] = fmaxf(mx4[f], fabsf(v.y));
            bad |= !isfinite(v.y);
          }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int f = 0; f < 4; ++f) mx4[f] = fmaxf(mx4[f], __shfl_xor_sync(0xffffffffu, mx4[f], o));
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    constexpr int nw = kXf256Threads / 32;
    float* s_mx = reinterpret_cast<float*>(s_pr);
    int* s_bad = reinterpret_cast<int*>(s_mx + 4 * nw);
    if ((tid & 31) == 0) {
#pragma unroll
      for (int f = 0; f < 4; ++f) s_mx[(tid >> 5) * 4 + f] = mx4[f];
      s_bad[tid >> 5] = bad;
    }
    __syncthreads();
    // one atomic per field and CTA: the max of non-negative floats is the
    // max of their bit patterns (order-independent, so deterministic)
    if (tid < a.g.lu) {
      float tm = 0.f;
      int tb = 0;
      for (int q = 0; q < nw; ++q) {
        tm = fmaxf(tm, s_mx[q * 4 + tid]);
        tb |= s_bad[q];
      }
      atomicMax(a.vmax + tid, __float_as_int(tm));
      if (tid == 0 && tb) atomicOr(a.vmax + 8, 1);
    }
    __syncthreads();
  }

  // ---- products (rhs.f:46-60), forward transforms, split, scale, store
  // C(m, z, kx, y) (xy_trans_f.f:20-37)
  const float fn = a.fn;
  float2* tline = s_pr + team * LD;
  const int partner = (tid & 16) | ((16 - k) & 15);
  const int nq = a.g.lr * yp;
  for (int q = team; q < nq; q += kXf256Teams) {
    const int m = (int)fdiv(q, a.fd_yp), c = q - m * yp;
    int fa, fb;
    product_pair(m, fa, fb);
    const float2* pa = s_in + (fa * yp + c) * LD + k;
    const float2* pb = s_in + (fb * yp + c) * LD + k;
    float2 v[16];
    // (scalar products: a packed mul.rn.f32x2 feeding the first stage's
    // packed sums is fused by the compiler into an FMA despite the .rn)
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float2 ea = pa[17 * j], eb = pb[17 * j];
      v[j] = make_float2(pmul(ea.x, eb.x), pmul(ea.y, eb.y));
    }
    dft16<-1>(v);
    __syncwarp(tmask);  // the team's reads of its previous line are done
#pragma unroll
    for (int s = 0; s < 16; ++s) tline[17 * s + k] = v[s];
    __syncwarp(tmask);
    f256_rows<-1>(v, tline, w, k);
    float2* o = a.out + (long long)z * a.out_z + (long long)m * a.out_n + (long long)k * a.out_kx + y0 + 2 * c;
    const bool two = 2 * c + 1 < yv, one = 2 * c < yv;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (16 * j > kmx) break;
      // Z(Nx - kx) for kx = k + 16 j, from the partner thread
      const float2 snd = k == 0 ? v[(16 - j) & 15] : v[15 - j];
      float2 z2;
      z2.x = __shfl_sync(tmask, snd.x, partner);
      z2.y = __shfl_sync(tmask, snd.y, partner);
      const float2 z1 = v[j];
      if (k + 16 * j <= kmx) {
        const float2 ve = make_float2((z1.x + z2.x) * fn, (z1.y - z2.y) * fn);
        const float2 vo = make_float2((z1.y + z2.y) * fn, (z2.x - z1.x) * fn);
        float2* oj = o + (long long)(16 * j) * a.out_kx;
        if (two) {
          if ((reinterpret_cast<uintptr_t>(oj) & 15) == 0) {
            store_pair(oj, ve, vo);
          } else {  // odd Ny: the pair straddles a vector boundary
            oj[0] = ve;
            oj[1] = vo;
          }
        } else if (one) {
          oj[0] = ve;
        }
      }
    }
  }
}

// whether k_x_pass_f256 runs this launch (else the general kernel)
__host__ __device__ inline bool x_f256_applies(const XPassArgs<float>& a) {
  return a.g.nx == 256 && a.sched == 0 && a.in_mode == 0 && a.out_mode == 2 && a.les == 0 && a.nin == a.g.lu &&
         a.nin <= 4 && (a.g.lr == 6 || a.g.lr == 9) && (!a.partials || a.max_only) && a.yt >= 2 && a.yt % 2 == 0;
}

// --------------------------------------------------------------- y forward
// Tile: field m, kx column i, planes z0 .. z0+TZ-1.  Output D(m, kx, ky, z)
// keeps |ky| <= ky_max (xy_trans_f.f:45-52).
template <typename T, int PATH, bool COH = false>
__device__ __forceinline__ void y_fwd_body(const YFwdArgs<T>& a, const FftPlan* __restrict__ gpl, int bid) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  load_plan(&pl, gpl);
  __syncthreads();
  C* s_tw = reinterpret_cast<C*>(smem_raw);
  C* s_ln = s_tw + tw_load<PATH>(pl);
  const int ny = a.g.ny, my = a.g.my, km = a.g.ky, nz = a.g.nz;
  const int ld = a.ld;
  const int ntz = (nz + a.tz - 1) / a.tz;
  int b = bid;
  const int zt = b % ntz; b /= ntz;
  const int i = b % a.g.mx; b /= a.g.mx;
  const int m = b;
  const int z0 = zt * a.tz;
  const int nl = min(a.tz, nz - z0);
  load_twiddles<T>(s_tw, a.tw, tw_load<PATH>(pl));
  const C* src = a.in + (long long)m * a.in_n + (long long)i * a.in_kx + (long long)z0 * a.in_z;
  __syncthreads();
  // the first stage reads its inputs straight from the rows of C (no
  // shared-memory staging); the rows are contiguous in y
  fft_lines_from<-1, PATH>(s_ln, ld, nl, s_tw, pl,
                           [&](int L) { return RowLoad<C, COH>{src + (long long)L * a.in_z}; });
  __syncthreads();
  C* dst = a.out + (long long)m * a.out_n + (long long)i * a.out_kx + z0;
  store_tile_rows(dst, a.out_ky, s_ln, ld, a.tz, nl, my, [&](int j) { return kpos(j, km, my, ny); });
}
template <typename T, int PATH>
__global__ void __launch_bounds__(kThreads, MinBlocks<T, kPassYFwd, PATH>::value)
    k_y_fwd(const __grid_constant__ YFwdArgs<T> a, const FftPlan* __restrict__ gpl) {
  y_fwd_body<T, PATH>(a, gpl, blockIdx.x);
}

__device__ __forceinline__ double wexp(double x) { return exp(x); }
__device__ __forceinline__ float wexp(float x) { return expf(x); }

// Per-launch constants of the epilogue in working type W, formed once per
// thread: the FP32 form then touches no FP64 arithmetic per mode.
template <typename W> struct EpiConst {
  W wave_x, wave_y, wave_z, nz_inv, dt_fac1, dt_fac2, mvis_f, mvis_t, bx, bz, lapse, cth, sth;
  bool same_t, nz_pow2;
};

template <typename W, typename T>
__device__ __forceinline__ EpiConst<W> epi_const(const ZFwdArgs<T>& a, double dt) {
  const StageConsts& sc = a.sc;
  EpiConst<W> e;
  e.wave_x = (W)a.g.wave_x; e.wave_y = (W)a.g.wave_y; e.wave_z = (W)a.g.wave_z;
  e.nz_inv = (W)a.nz_inv;
  e.nz_pow2 = is_pow2_inv(a.g.nz);
  e.dt_fac1 = (W)(sc.gamma * dt);
  e.dt_fac2 = (W)(sc.zeta * dt);
  const double vis_f = sc.vis * (sc.gamma * dt + sc.zeta * dt);  // sam.f:293-295
  e.mvis_f = (W)(-vis_f);
  e.mvis_t = (W)(-(vis_f * sc.pr_inv));                           // sam.f:297
  e.same_t = sc.pr_inv == 1.0;
  e.bx = (W)sc.buoy_fac_x; e.bz = (W)sc.buoy_fac_z; e.lapse = (W)sc.lapse;
  e.cth = (W)sc.cos_theta; e.sth = (W)sc.sin_theta;
  return e;
}

// u and r_old of one mode (mode 2) or u_sav (mode 1), loaded ahead of use.
template <typename W> struct EpiIn {
  W ur[4], ui[4], rr[4], ri[4];
};

template <typename W, typename T>
__device__ __forceinline__ void epi_load(const ZFwdArgs<T>& a, int i, int j, int k, EpiIn<W>& in) {
  using C = cx_t<T>;
  const Grid& g = a.g;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    in.ur[f] = in.ui[f] = in.rr[f] = in.ri[f] = (W)0;
  }
  if (a.mode == 2) {
    const long long uidx = (long long)i * a.u_kx + (long long)j * a.u_ky + k;
#pragma unroll
    for (int f = 0; f < 4; ++f)
      if (f < g.lu) {
        const C v = a.u[(long long)f * a.u_n + uidx];
        in.ur[f] = (W)v.x; in.ui[f] = (W)v.y;
        if (a.sc.nrk > 1) {
          const C ro = a.r[(long long)f * a.u_n + uidx];
          in.rr[f] = (W)ro.x; in.ri[f] = (W)ro.y;
        }
      }
  } else if (a.sc.i_strat) {  // mode 1: (w, T) of u_sav in slots 2, 3
    const long long s = (long long)i * a.sav_kx + (long long)j * a.sav_ky + k;
    const C w = a.usav[s];
    const C th = a.usav[a.sav_n + s];
    in.ur[2] = (W)w.x; in.ui[2] = (W)w.y; in.ur[3] = (W)th.x; in.ui[3] = (W)th.y;
  }
}

// rhs.f:108-142 for one mode (kx i, ky j, kz k) in working type W, then
// (mode 2) sam.f:210-221 and 293-314.  ln points at field 0 of this mode in
// shared memory; field f is at ln[f * fstride].
template <typename W, typename T>
__device__ __forceinline__ void epi_mode(const ZFwdArgs<T>& a, const cx_t<T>* ln, int fstride, int i, int j, int k,
                                         const EpiConst<W>& c, const EpiIn<W>& in) {
  using C = cx_t<T>;
  const Grid& g = a.g;
  const StageConsts& sc = a.sc;
  const int nf = a.nf;
  const W rkx = c.wave_x * (W)i;
  const W rky = c.wave_y * (W)kwave(j, g.ky, g.my);
  const W rkz = c.wave_z * (W)kwave(k, g.kz, g.mz);
  const W rk_sq_raw = rkx * rkx + rky * rky + rkz * rkz;
  const W rk_sq = rk_sq_raw > (W)1.0e-10 ? rk_sq_raw : (W)1.0e-10;
  W tr[9], ti[9];
#pragma unroll
  for (int f = 0; f < 9; ++f) {
    if (f < nf) {
      const C v = ln[f * fstride];
      tr[f] = scale_by((W)v.x, c.nz_inv, c.nz_pow2);
      ti[f] = scale_by((W)v.y, c.nz_inv, c.nz_pow2);
    } else {
      tr[f] = (W)0; ti[f] = (W)0;
    }
  }
  // -i (a + i b) = b - i a
  const W s1r = rkx * tr[0] + rky * tr[1] + rkz * tr[3], s1i = rkx * ti[0] + rky * ti[1] + rkz * ti[3];
  const W s2r = rkx * tr[1] + rky * tr[2] + rkz * tr[4], s2i = rkx * ti[1] + rky * ti[2] + rkz * ti[4];
  const W s3r = rkx * tr[3] + rky * tr[4] + rkz * tr[5], s3i = rkx * ti[3] + rky * ti[4] + rkz * ti[5];
  W r1r = s1i, r1i = -s1r, r2r = s2i, r2i = -s2r, r3r = s3i, r3i = -s3r, r4r = (W)0, r4i = (W)0;
  if (sc.i_strat) {
    W wr = in.ur[2], wi = in.ui[2];
    if (a.mode == 2 && sc.rot_sav) {  // sam.f:180-181
      wr = c.cth * in.ur[2] - c.sth * in.ur[0];
      wi = c.cth * in.ui[2] - c.sth * in.ui[0];
    }
    const W thr = in.ur[3], thi = in.ui[3];
    r1r += c.bx * thr; r1i += c.bx * thi;
    r3r += c.bz * thr; r3i += c.bz * thi;
    const W s4r = rkx * tr[6] + rky * tr[7] + rkz * tr[8];
    const W s4i = rkx * ti[6] + rky * ti[7] + rkz * ti[8];
    r4r = s4i - c.lapse * wr;
    r4i = -s4r - c.lapse * wi;
  }
  // p = -i (k . R) / k^2 ;  R -= i k p   (rhs.f:134-139)
  const W qr = rkx * r1r + rky * r2r + rkz * r3r, qi = rkx * r1i + rky * r2i + rkz * r3i;
  const W pr = qi / rk_sq, pim = -qr / rk_sq;
  // -i rk p = rk * (p.i, -p.r)
  r1r += rkx * pim; r1i -= rkx * pr;
  r2r += rky * pim; r2i -= rky * pr;
  r3r += rkz * pim; r3i -= rkz * pr;
  const W rr[4] = {r1r, r2r, r3r, r4r}, ri[4] = {r1i, r2i, r3i, r4i};
  if (a.mode == 1) {
    const long long ridx = (long long)i * a.r_kx + (long long)j * a.r_ky + k;
#pragma unroll
    for (int f = 0; f < 4; ++f)
      if (f < g.lu) a.r[(long long)f * a.r_n + ridx] = mk<C>((T)rr[f], (T)ri[f]);
    a.r[(long long)g.lu * a.r_n + ridx] = mk<C>((T)pr, (T)pim);
    return;
  }
  const long long uidx = (long long)i * a.u_kx + (long long)j * a.u_ky + k;
  W ef, et;
  if constexpr (kIsDD<W>) {
    // exp(-nu_f k^2) = e(kx) e(ky) e(kz), tabulated for this stage in FP64
    // and rounded to pairs (launch_if_tables)
    const dd* tb = a.ift;
    const int oy = g.mx, oz = g.mx + g.my, tw = g.mx + g.my + g.mz;
    ef = tb[i] * tb[oy + j] * tb[oz + k];
    et = c.same_t ? ef : tb[tw + i] * tb[tw + oy + j] * tb[tw + oz + k];
  } else {
    ef = wexp(c.mvis_f * rk_sq_raw);
    et = c.same_t ? ef : wexp(c.mvis_t * rk_sq_raw);
  }
#pragma unroll
  for (int f = 0; f < 4; ++f)
    if (f < g.lu) {
      W ur = in.ur[f], ui = in.ui[f];
      if (sc.nrk > 1) {  // sam.f:211-221
        ur = ur + c.dt_fac2 * in.rr[f];
        ui = ui + c.dt_fac2 * in.ri[f];
      }
      const W vf = f == 3 ? et : ef;  // sam.f:297
      ur = (ur + c.dt_fac1 * rr[f]) * vf;
      ui = (ui + c.dt_fac1 * ri[f]) * vf;
      a.u[(long long)f * a.u_n + uidx] = mk<C>((T)ur, (T)ui);
      a.r[(long long)f * a.u_n + uidx] = mk<C>((T)rr[f], (T)ri[f]);
    }
  if (sc.write_p) a.p[uidx] = mk<C>((T)pr, (T)pim);
}

// --------------------------------------------------------------- z forward
// Tile: kx column i, ky rows j0 .. j0+TY-1, all nf fields.  Forward z
// transform, truncation to Nz_min and 1/Nz (z_trans_f.f:25-30), then one of
//   mode 0: write the truncated modes back in place (z_trans_f),
//   mode 1: rhs epilogue (rhs.f:108-142) into r with u_sav from memory,
//   mode 2: full stage epilogue: rhs, then sam.f:210-221 and 293-314.
template <typename T, int PATH, bool COH = false>
__device__ __forceinline__ void z_fwd_body(const ZFwdArgs<T>& a, const FftPlan* __restrict__ gpl, int bid) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  load_plan(&pl, gpl);
  __syncthreads();
  C* s_tw = reinterpret_cast<C*>(smem_raw);
  C* s_ln = s_tw + tw_load<PATH>(pl);
  const Grid& g = a.g;
  const int nz = g.nz, mz = g.mz, km = g.kz, my = g.my;
  const int ld = a.ld, nf = a.nf;
  const int nty = (my + a.ty - 1) / a.ty;
  const int jt = bid % nty;
  const int i = bid / nty;
  const int j0 = jt * a.ty;
  const int nl = min(a.ty, my - j0);
  load_twiddles<T>(s_tw, a.tw, tw_load<PATH>(pl));
  // lines of all nf fields for the nl rows of this tile, packed as f * nl + t;
  // the first stage reads the z-contiguous rows of D straight from memory
  __syncthreads();
  fft_lines_from<-1, PATH>(s_ln, ld, nf * nl, s_tw, pl, [&](int L) {
    const int f = L / nl, t = L - f * nl;
    return RowLoad<C, COH>{a.in + (long long)f * a.in_n + (long long)i * a.in_kx + (long long)(j0 + t) * a.in_ky};
  });
  __syncthreads();
  const T nz_inv = a.nz_inv;
  if (a.mode == 0) {
    for (int e = threadIdx.x; e < nf * a.ty * mz; e += blockDim.x) {
      const int r = (int)fdiv(e, a.fd_m), k = e - r * mz;
      const int f = (int)fdiv(r, a.fd_t), t = r - f * a.ty;
      if (t >= nl) continue;
      C v = s_ln[(f * nl + t) * ld + sidx(kpos(k, km, mz, nz))];
      v.x *= nz_inv;
      v.y *= nz_inv;
      a.in[(long long)f * a.in_n + (long long)i * a.in_kx + (long long)(j0 + t) * a.in_ky + k] = v;
    }
    return;
  }
  double dt = 0.0;
  if (a.mode == 2) dt = ldc<COH>(&a.state->dt);
  // the epilogue constants once per CTA (FP64 arithmetic on one thread)
  __shared__ EpiConst<T> s_cw;
  if (threadIdx.x == 0) s_cw = epi_const<T>(a, dt);
  __syncthreads();
  const EpiConst<T> cw = s_cw;
  // two modes per iteration: their global loads are issued together
  for (int e0 = threadIdx.x; e0 < nl * mz; e0 += 2 * blockDim.x) {
    const int e1 = e0 + blockDim.x;
    const bool has1 = e1 < nl * mz;
    const int t0 = (int)fdiv(e0, a.fd_m), k0 = e0 - t0 * mz;
    const int t1 = has1 ? (int)fdiv(e1, a.fd_m) : t0, k1 = has1 ? e1 - t1 * mz : k0;
    EpiIn<T> in0, in1;
    epi_load<T>(a, i, j0 + t0, k0, in0);
    if (has1) epi_load<T>(a, i, j0 + t1, k1, in1);
    for (int h = 0; h < 2; ++h) {
      if (h == 1 && !has1) break;
      const int t = h ? t1 : t0, k = h ? k1 : k0, j = j0 + t;
      const C* ln = s_ln + t * ld + sidx(kpos(k, km, mz, nz));
      // (the FP32 form treats the mean mode in FP64 below)
      if (sizeof(T) == 8 || i != 0 || j != 0 || k != 0) epi_mode<T, T>(a, ln, nl * ld, i, j, k, cw, h ? in1 : in0);
    }
  }
  if (sizeof(T) == 4 && i == 0 && j0 == 0 && threadIdx.x == 0) {
    // the FP32 form keeps the mean (k = 0) mode in FP64; one thread, outside
    // the per-mode loop so that no FP64 instruction is issued per mode
    EpiIn<double> ind;
    epi_load<double>(a, 0, 0, 0, ind);
    epi_mode<double, T>(a, s_ln + sidx(kpos(0, km, mz, nz)), nl * ld, 0, 0, 0, epi_const<double>(a, dt), ind);
  }
  if (a.mode == 2 && a.sc.last && bid == 0 && threadIdx.x == 0) {
    // sam.f:318 time = time + dt, once per step (no CTA of this launch reads
    // time, and none writes dt)
    a.state->time = a.state->time + dt;
  }
}
template <typename T, int PATH>
__global__ void __launch_bounds__(kThreads, MinBlocks<T, kPassZFwd, PATH>::value)
    k_z_fwd(const __grid_constant__ ZFwdArgs<T> a, const FftPlan* __restrict__ gpl) {
  z_fwd_body<T, PATH>(a, gpl, blockIdx.x);
}

// ----------------------------------------------------- vel_max completion
// vel_max.f:28-49 on the per-CTA partials written by k_x_pass.
// Parseval sums of vel_max (see launch_parseval): sums of the stored modes'
// squares, FP64-accurate, per-thread strided order, block tree, fixed launch
// shape.  The FP32 form (the only user) accumulates the exact squares of its
// FP32 values in error-free FP32 pairs (about 48 bits: FP64 arithmetic, one
// instruction per value pair of the 1/64-rate FP64 pipe plus a conversion,
// made this kernel FP64-bound); the FP64 form would use FP64.
__device__ __forceinline__ DF df_add_wsq(DF a, float v, float w) {
  // a + w v^2 with w a power of two (exact scaling of the exact square p + e)
  const float p = v * v;
  const float e = fmaf(v, v, -p);
  return df_add(df_add(a, p * w), e * w);
}

template <typename T>
__device__ __forceinline__ void parseval_body(const cx_t<T>* __restrict__ u, const Grid& g, double* __restrict__ pv,
                                              int bid, int nblk) {
  __shared__ double red[4][kThreads];
  const long long nm = (long long)g.mx * g.my * g.mz;
  const int plane = g.my * g.mz;
  if constexpr (sizeof(T) == 4) {
    // kx = 0 modes count once, kx > 0 twice (their conjugates): sum w |u|^2
    // with w = 1/2 for kx = 0 and 1 otherwise, then double
    DF acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (long long m = bid * (long long)blockDim.x + threadIdx.x; m < nm;
         m += (long long)nblk * blockDim.x) {
      const float w = m < plane ? 0.5f : 1.0f;
#pragma unroll
      for (int f = 0; f < 4; ++f)
        if (f < g.lu) {
          const cx_t<T> v = u[f * nm + m];
          acc[f] = df_add_wsq(df_add_wsq(acc[f], v.y, w), v.x, w);
        }
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) red[f][threadIdx.x] = 2.0 * ((double)acc[f].hi + (double)acc[f].lo);
  } else {
    // kx = 0 modes count once, kx > 0 twice (their conjugates): separate sums
    double acc0[4] = {0.0, 0.0, 0.0, 0.0}, acc1[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long m = bid * (long long)blockDim.x + threadIdx.x; m < nm;
         m += (long long)nblk * blockDim.x) {
      const bool kx0 = m < plane;
#pragma unroll
      for (int f = 0; f < 4; ++f)
        if (f < g.lu) {
          const cx_t<T> v = u[f * nm + m];
          const double re = (double)v.x, im = (double)v.y;
          if (kx0) acc0[f] = fma(re, re, fma(im, im, acc0[f]));
          else acc1[f] = fma(re, re, fma(im, im, acc1[f]));
        }
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) red[f][threadIdx.x] = acc0[f] + 2.0 * acc1[f];
  }
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int f = 0; f < 4; ++f) red[f][threadIdx.x] += red[f][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < g.lu) pv[(long long)bid * g.lu + threadIdx.x] = red[threadIdx.x][0];
  if (bid == 0 && threadIdx.x < g.lu) pv[(long long)nblk * g.lu + threadIdx.x] = (double)u[threadIdx.x * nm].x;
}
template <typename T>
__global__ void __launch_bounds__(kThreads) k_parseval(const cx_t<T>* __restrict__ u, Grid g, double* __restrict__ pv) {
  parseval_body<T>(u, g, pv, blockIdx.x, gridDim.x);
}

template <typename T>
void launch_parseval(const cx_t<T>* u, const Grid& g, double* pv, cudaStream_t s) {
  k_parseval<T><<<kParsevalBlocks, kThreads, 0, s>>>(u, g, pv);
}
// vel_max.f:28-49 on the per-CTA partials written by the x pass (or, in the
// FP32 and double-float forms, on the wave-space sums and the max keys).
template <bool COH = false>
__device__ __forceinline__ void vel_max_finish_body(const double* __restrict__ partials, int nblk, const Grid& g,
                                                    DevState* st, int i_cfl, double cfl0, double adv_cfl_limit,
                                                    const double* __restrict__ pv, int npv, int* __restrict__ vmax,
                                                    int vkind) {
  __shared__ double red[kThreads];
  __shared__ double fin[4][4];
  if (!pv) {
    // a thread reads whole per-CTA records (lu x 4 doubles, contiguous) of
    // the CTAs b = t, t + 256, ... into 16 accumulators, then one fixed-order
    // tree per quantity: deterministic for a given number of CTAs
    __shared__ double redq[16][kThreads / 2];
    double v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = 0.0;
    const int nq = 4 * g.lu;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
      const double2* rec = reinterpret_cast<const double2*>(partials + (long long)b * nq);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (2 * i < nq) {
          const double2 x = ldc<COH>(rec + i);
          v[2 * i] = ((2 * i) % 4 == 2) ? fmax(v[2 * i], x.x) : v[2 * i] + x.x;
          v[2 * i + 1] = ((2 * i + 1) % 4 == 2) ? fmax(v[2 * i + 1], x.y) : v[2 * i + 1] + x.y;
        }
    }
    // first tree level straight from the registers (threads t and t + 128)
    const int h = blockDim.x / 2;
    if (threadIdx.x >= h)
#pragma unroll
      for (int i = 0; i < 16; ++i) redq[i][threadIdx.x - h] = v[i];
    __syncthreads();
    if (threadIdx.x < h)
#pragma unroll
      for (int i = 0; i < 16; ++i)
        redq[i][threadIdx.x] = (i % 4 == 2) ? fmax(v[i], redq[i][threadIdx.x]) : v[i] + redq[i][threadIdx.x];
    __syncthreads();
    for (int st = h / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          redq[i][threadIdx.x] = (i % 4 == 2) ? fmax(redq[i][threadIdx.x], redq[i][threadIdx.x + st])
                                              : redq[i][threadIdx.x] + redq[i][threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x < nq) fin[threadIdx.x / 4][threadIdx.x % 4] = redq[threadIdx.x][0];
    __syncthreads();
  }
  if (pv) {
    // sums from wave space: sum u = N u(0,0,0), sum u^2 = N sum w |u|^2
    for (int f = 0; f < g.lu; ++f) {
      double v = 0.0;
      for (int b = threadIdx.x; b < npv; b += blockDim.x) v += ldc<COH>(pv + (long long)b * g.lu + f);
      red[threadIdx.x] = v;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        const double n = (double)g.nx * (double)g.ny * (double)g.nz;
        fin[f][0] = ldc<COH>(pv + (long long)npv * g.lu + f) * n;
        fin[f][1] = red[0] * n;
        fin[f][2] = vkind ? dd_key_value(ldc<COH>(reinterpret_cast<const unsigned long long*>(vmax) + f))
                          : (double)__int_as_float(ldc<COH>(vmax + f));
        fin[f][3] = (double)ldc<COH>(vmax + 8);
      }
      __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x < kVmaxInts) vmax[threadIdx.x] = 0;  // ready for the next step's maxima
  }
  if (threadIdx.x == 0) {
    const double inv = 1.0 / ((double)g.nx * (double)g.ny * (double)g.nz);
    int bad = 0;
    for (int f = 0; f < g.lu; ++f) {
      st->u_avg[f] = fin[f][0] * inv;
      st->u_var[f] = fin[f][1] * inv - st->u_avg[f] * st->u_avg[f];
      st->u_max[f] = fin[f][2];
      bad |= fin[f][3] != 0.0;
    }
    st->energy = 0.5 * (st->u_var[0] + st->u_var[1] + st->u_var[2]);
    const double cx = st->u_max[0] * g.kx * g.wave_x;
    const double cy = st->u_max[1] * g.ky * g.wave_y;
    const double cz = st->u_max[2] * g.kz * g.wave_z;
    if (i_cfl == 1) {
      const double cb = fmax(cx, fmax(cy, cz));
      if (cb > 0.0 && !bad) st->dt = cfl0 * adv_cfl_limit / cb;
    }
    st->cfl_x = cx * st->dt;
    st->cfl_y = cy * st->dt;
    st->cfl_z = cz * st->dt;
    if (bad) st->nonfinite = 1;
  }
}

// ------------------------------------------------------------------ launchers
template <typename T>
void launch_z_inv(const ZInvArgs<T>& a0, const FftPlan* pl, size_t smem, cudaStream_t s) {
  ZInvArgs<T> a = a0;
  const int nty = (a.g.my + a.ty - 1) / a.ty;
  const int grid = a.nvar * a.g.mx * nty;
  switch (a.g.nz) {
    case 256:
      if (a.sched) k_z_inv<T, 256><<<grid, kThreads, smem, s>>>(a, pl);
      else k_z_inv<T, kFft256><<<grid, kThreads, smem, s>>>(a, pl);
      break;
    case 32: k_z_inv<T, 32><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 64: k_z_inv<T, 64><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 128: k_z_inv<T, 128><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 512: k_z_inv<T, 512><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 96: k_z_inv<T, 96><<<grid, kThreads, smem, s>>>(a, pl); break;
    default: k_z_inv<T, kFftGeneric><<<grid, kThreads, smem, s>>>(a, pl);
  }
}
template <typename T>
void launch_y_inv(const YInvArgs<T>& a0, const FftPlan* pl, size_t smem, cudaStream_t s) {
  YInvArgs<T> a = a0;
  const int ntx = (a.g.mx + a.tx - 1) / a.tx;
  const int grid = a.nvar * a.g.nz * ntx;
  switch (a.g.ny) {
    case 256:
      if (a.sched) k_y_inv<T, 256><<<grid, kThreads, smem, s>>>(a, pl);
      else k_y_inv<T, kFft256><<<grid, kThreads, smem, s>>>(a, pl);
      break;
    case 32: k_y_inv<T, 32><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 64: k_y_inv<T, 64><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 128: k_y_inv<T, 128><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 512: k_y_inv<T, 512><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 96: k_y_inv<T, 96><<<grid, kThreads, smem, s>>>(a, pl); break;
    default: k_y_inv<T, kFftGeneric><<<grid, kThreads, smem, s>>>(a, pl);
  }
}
template <typename T>
int x_pass_blocks(const XPassArgs<T>& a) {
  return a.g.nz * ((a.g.ny + a.yt - 1) / a.yt);
}
// the launch-time fields of the x pass's and the z-forward pass's argument
// blocks (fast divisors, scales), shared by the launchers and the ensemble
// stage recorder
template <typename T>
XPassArgs<T> prep_x_pass(const XPassArgs<T>& a0) {
  XPassArgs<T> a = a0;
  a.fd_mx = make_fastdiv(a.g.mx);
  a.fd_yp = make_fastdiv(a.yt / 2);
  a.fd_nx = make_fastdiv(a.g.nx);
  a.fd_y = make_fastdiv(a.yt);
  a.fn = (T)(0.5 / ((double)a.g.nx * (double)a.g.ny));
  return a;
}
template <typename T>
ZFwdArgs<T> prep_z_fwd(const ZFwdArgs<T>& a0) {
  ZFwdArgs<T> a = a0;
  a.fd_t = make_fastdiv(a.ty);
  a.fd_m = make_fastdiv(a.g.mz);
  a.nz_inv = (T)(1.0 / (double)a.g.nz);
  return a;
}

template <typename T>
void launch_x_pass(const XPassArgs<T>& a0, const FftPlan* pl, size_t smem, cudaStream_t s) {
  const XPassArgs<T> a = prep_x_pass(a0);
  switch (a.g.nx) {
    case 256:
      if (a.sched == 1) {
        k_x_pass<T, 256><<<x_pass_blocks(a), x_threads(sizeof(T), false), smem, s>>>(a, pl);
        break;
      }
      if constexpr (std::is_same<T, float>::value) {
        const size_t fsm = x_f256_smem(a.nin * (a.yt / 2));
        if (x_f256_applies(a) && fsm <= (size_t)smem_optin()) {
          k_x_pass_f256<><<<x_pass_blocks(a), kXf256Threads, fsm, s>>>(a);
          break;
        }
      }
      k_x_pass<T, kFft256><<<x_pass_blocks(a), x_threads(sizeof(T), true), smem, s>>>(a, pl);
      break;
    case 32: k_x_pass<T, 32><<<x_pass_blocks(a), kThreads, smem, s>>>(a, pl); break;
    case 64: k_x_pass<T, 64><<<x_pass_blocks(a), kThreads, smem, s>>>(a, pl); break;
    case 128: k_x_pass<T, 128><<<x_pass_blocks(a), kThreads, smem, s>>>(a, pl); break;
    case 512: k_x_pass<T, 512><<<x_pass_blocks(a), kThreads, smem, s>>>(a, pl); break;
    case 96: k_x_pass<T, 96><<<x_pass_blocks(a), kThreads, smem, s>>>(a, pl); break;
    default: k_x_pass<T, kFftGeneric><<<x_pass_blocks(a), kThreads, smem, s>>>(a, pl);
  }
}
template <typename T>
void launch_y_fwd(const YFwdArgs<T>& a0, const FftPlan* pl, size_t smem, cudaStream_t s) {
  YFwdArgs<T> a = a0;
  const int ntz = (a.g.nz + a.tz - 1) / a.tz;
  const int grid = a.nvar * a.g.mx * ntz;
  switch (a.g.ny) {
    case 256:
      if (a.sched) k_y_fwd<T, 256><<<grid, kThreads, smem, s>>>(a, pl);
      else k_y_fwd<T, kFft256><<<grid, kThreads, smem, s>>>(a, pl);
      break;
    case 32: k_y_fwd<T, 32><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 64: k_y_fwd<T, 64><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 128: k_y_fwd<T, 128><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 512: k_y_fwd<T, 512><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 96: k_y_fwd<T, 96><<<grid, kThreads, smem, s>>>(a, pl); break;
    default: k_y_fwd<T, kFftGeneric><<<grid, kThreads, smem, s>>>(a, pl);
  }
}
template <typename T>
void launch_z_fwd(const ZFwdArgs<T>& a0, const FftPlan* pl, size_t smem, cudaStream_t s) {
  const ZFwdArgs<T> a = prep_z_fwd(a0);
  const int nty = (a.g.my + a.ty - 1) / a.ty;
  const int grid = a.g.mx * nty;
  switch (a.g.nz) {
    case 256:
      if (a.sched) k_z_fwd<T, 256><<<grid, kThreads, smem, s>>>(a, pl);
      else k_z_fwd<T, kFft256><<<grid, kThreads, smem, s>>>(a, pl);
      break;
    case 32: k_z_fwd<T, 32><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 64: k_z_fwd<T, 64><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 128: k_z_fwd<T, 128><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 512: k_z_fwd<T, 512><<<grid, kThreads, smem, s>>>(a, pl); break;
    case 96: k_z_fwd<T, 96><<<grid, kThreads, smem, s>>>(a, pl); break;
    default: k_z_fwd<T, kFftGeneric><<<grid, kThreads, smem, s>>>(a, pl);
  }
}
static inline void allow_dynamic_smem(const void* fn, int optin) {
  cudaFuncAttributes at;
  if (cudaFuncGetAttributes(&at, fn) != cudaSuccess) return;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)at.sharedSizeBytes);
}

// Opt every pass into the largest dynamic shared memory the device allows
// (the per-block opt-in limit less the kernel's static shared memory), per
// group of passes (each group is instantiated in its own translation unit).
template <typename T>
void smem_limits_zinv(int optin) {
  allow_dynamic_smem((const void*)k_z_inv<T, kFft256>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, kFftGeneric>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, 32>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, 64>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, 128>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, 512>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, 96>, optin);
  allow_dynamic_smem((const void*)k_z_inv<T, 256>, optin);
}
template <typename T>
void smem_limits_yinv(int optin) {
  allow_dynamic_smem((const void*)k_y_inv<T, kFft256>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, kFftGeneric>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, 32>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, 64>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, 128>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, 512>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, 96>, optin);
  allow_dynamic_smem((const void*)k_y_inv<T, 256>, optin);
}
template <typename T>
void smem_limits_x(int optin) {
  if constexpr (std::is_same<T, float>::value) allow_dynamic_smem((const void*)k_x_pass_f256<>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, kFft256>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, kFftGeneric>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, 32>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, 64>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, 128>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, 512>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, 96>, optin);
  allow_dynamic_smem((const void*)k_x_pass<T, 256>, optin);
}
template <typename T>
void smem_limits_yfwd(int optin) {
  allow_dynamic_smem((const void*)k_y_fwd<T, kFft256>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, kFftGeneric>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, 32>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, 64>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, 128>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, 512>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, 96>, optin);
  allow_dynamic_smem((const void*)k_y_fwd<T, 256>, optin);
}
template <typename T>
void smem_limits_zfwd(int optin) {
  allow_dynamic_smem((const void*)k_z_fwd<T, kFft256>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, kFftGeneric>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, 32>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, 64>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, 128>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, 512>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, 96>, optin);
  allow_dynamic_smem((const void*)k_z_fwd<T, 256>, optin);
}

#define SAMGPU_INST_ZINV(T)                                                                   \
  template void launch_z_inv<T>(const ZInvArgs<T>&, const FftPlan*, size_t, cudaStream_t);     \
  template void smem_limits_zinv<T>(int);
#define SAMGPU_INST_YINV(T)                                                                   \
  template void launch_y_inv<T>(const YInvArgs<T>&, const FftPlan*, size_t, cudaStream_t);     \
  template void smem_limits_yinv<T>(int);
#define SAMGPU_INST_X(T)                                                                      \
  template void launch_x_pass<T>(const XPassArgs<T>&, const FftPlan*, size_t, cudaStream_t);   \
  template int x_pass_blocks<T>(const XPassArgs<T>&);                                          \
  template void smem_limits_x<T>(int);
#define SAMGPU_INST_YFWD(T)                                                                   \
  template void launch_y_fwd<T>(const YFwdArgs<T>&, const FftPlan*, size_t, cudaStream_t);     \
  template void smem_limits_yfwd<T>(int);
#define SAMGPU_INST_ZFWD(T)                                                                   \
  template void launch_z_fwd<T>(const ZFwdArgs<T>&, const FftPlan*, size_t, cudaStream_t);     \
  template void smem_limits_zfwd<T>(int);
#define SAMGPU_INST(T) \
  SAMGPU_INST_ZINV(T) SAMGPU_INST_YINV(T) SAMGPU_INST_X(T) SAMGPU_INST_YFWD(T) SAMGPU_INST_ZFWD(T)

}  // namespace samgpu
