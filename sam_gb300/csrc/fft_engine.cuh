// Batched mixed-radix FFT engine for sm_103a: lines of length n <= 1024 held
// in shared memory, each line transformed by a team of TW threads (TW a power
// of two, TW >= n/8; teams wider than a warp synchronise on a named barrier).
// A stage of radix p (2, 3, 4, 5, 8) is a self-sorting Stockham step done in
// place: every thread first loads all of its butterfly inputs (at most 8
// complex values) into registers, the team synchronises, then the thread
// computes and writes its outputs.  The plan is read from shared memory.
//
// Conventions are FFTPACK's (the reference's fft.f): unnormalised transforms,
// SIGN = -1 is cfftf (exp(-i ...)), SIGN = +1 is cfftb (exp(+i ...)).
// Twiddles w_{l p}^{f q} are tabulated per stage (forward sign) by the host in
// extended precision and rounded once; the backward transform conjugates them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ddfloat.cuh"

namespace samgpu {

template <typename T> struct Cx;
template <> struct Cx<double> { using type = double2; };
template <> struct Cx<float> { using type = float2; };
template <> struct Cx<dd> { using type = ddc; };
template <typename T> using cx_t = typename Cx<T>::type;

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) a, decltype(C::x) b) { C r; r.x = a; r.y = b; return r; }

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
// FP32 complex sums as one packed instruction (add/sub.rn.f32x2: two IEEE
// round-to-nearest operations, the same results as the scalar pair)
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
// Double-float complex sums with the real and imaginary parts in one packed
// pair per instruction: the high parts' TwoSum, the low parts' sum and the
// renormalisation of ddfloat.cuh's operator+, each step on (re, im) at once
// (the same IEEE operations and results as two scalar pair sums).
__device__ __forceinline__ unsigned long long f2p(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2u(unsigned long long r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ unsigned long long f2add(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2sub(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// s + e = H +- K exactly (TwoSum; for the difference with -K folded in), then
// the low parts' sum L added and the pair renormalised
template <bool SUB>
__device__ __forceinline__ ddc dd_cplx_sum(unsigned long long H, unsigned long long K, unsigned long long L) {
  const unsigned long long s = SUB ? f2sub(H, K) : f2add(H, K);
  const unsigned long long bb = f2sub(s, H);
  const unsigned long long t = f2sub(H, f2sub(s, bb));
  unsigned long long e = SUB ? f2sub(t, f2add(K, bb)) : f2add(t, f2sub(K, bb));
  e = f2add(e, L);
  const unsigned long long h = f2add(s, e);
  const unsigned long long l = f2sub(e, f2sub(h, s));
  ddc r;
  f2u(h, r.x.hi, r.y.hi);
  f2u(l, r.x.lo, r.y.lo);
  return r;
}
__device__ __forceinline__ ddc cadd(ddc a, ddc b) {
  return dd_cplx_sum<false>(f2p(a.x.hi, a.y.hi), f2p(b.x.hi, b.y.hi),
                            f2add(f2p(a.x.lo, a.y.lo), f2p(b.x.lo, b.y.lo)));
}
__device__ __forceinline__ ddc csub(ddc a, ddc b) {
  return dd_cplx_sum<true>(f2p(a.x.hi, a.y.hi), f2p(b.x.hi, b.y.hi),
                           f2sub(f2p(a.x.lo, a.y.lo), f2p(b.x.lo, b.y.lo)));
}
// a * w (SIGN=-1) or a * conj(w) (SIGN=+1)
template <int SIGN, typename C> __device__ __forceinline__ C ctw(C a, C w) {
  if (SIGN < 0) return mk<C>(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
  return mk<C>(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
__device__ __forceinline__ unsigned long long f2mul(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
// Complex double-float product a * (u + i v)-style: the real and imaginary
// parts as one packed pair each step, lane k = x (0) or y (1):
//   R_k = ax * U_k + ay * V_k
// with U = (c1, c3), V = (c2, c4) the caller's coefficient pairs, given as
// their high and low parts.  The two exact products (FMA TwoProduct, the
// error terms formed negated from -ax, -ay so no packed negation is needed),
// a TwoSum of them, the four cross terms and one renormalisation: the
// operations of dd_mul_sub on both parts at once.
__device__ __forceinline__ ddc dd_cplx_dot(ddc a, unsigned long long Uh, unsigned long long Ul,
                                           unsigned long long Vh, unsigned long long Vl) {
  const unsigned long long Xh = f2p(a.x.hi, a.x.hi), Xl = f2p(a.x.lo, a.x.lo), nXh = f2p(-a.x.hi, -a.x.hi);
  const unsigned long long Yh = f2p(a.y.hi, a.y.hi), Yl = f2p(a.y.lo, a.y.lo), nYh = f2p(-a.y.hi, -a.y.hi);
  const unsigned long long P = f2mul(Xh, Uh), Q = f2mul(Yh, Vh);
  const unsigned long long nEP = f2fma(nXh, Uh, P), nEQ = f2fma(nYh, Vh, Q);  // -(exact error of P, Q)
  const unsigned long long s = f2add(P, Q);
  const unsigned long long bb = f2sub(s, P);
  unsigned long long e = f2add(f2sub(P, f2sub(s, bb)), f2sub(Q, bb));
  e = f2sub(e, f2add(nEP, nEQ));
  e = f2fma(Xh, Ul, e);
  e = f2fma(Xl, Uh, e);
  e = f2fma(Yh, Vl, e);
  e = f2fma(Yl, Vh, e);
  const unsigned long long h = f2add(s, e);
  const unsigned long long l = f2sub(e, f2sub(h, s));
  ddc r;
  f2u(h, r.x.hi, r.y.hi);
  f2u(l, r.x.lo, r.y.lo);
  return r;
}
// double-float pairs: a * w as a packed pair (SIGN = -1: U = (wx, wy),
// V = (-wy, wx); SIGN = +1, a * conj(w): U = (wx, -wy), V = (wy, wx))
template <int SIGN> __device__ __forceinline__ ddc ctw(ddc a, ddc w) {
  if (SIGN < 0)
    return dd_cplx_dot(a, f2p(w.x.hi, w.y.hi), f2p(w.x.lo, w.y.lo), f2p(-w.y.hi, w.x.hi), f2p(-w.y.lo, w.x.lo));
  return dd_cplx_dot(a, f2p(w.x.hi, -w.y.hi), f2p(w.x.lo, -w.y.lo), f2p(w.y.hi, w.x.hi), f2p(w.y.lo, w.x.lo));
}
// FP32: the same products with their rounding spelled out (the second
// product rounded, the first fused with the sum), so every kernel computes
// the same bits whatever the compiler would contract at each call site
template <int SIGN> __device__ __forceinline__ float2 ctw(float2 a, float2 w) {
  if (SIGN < 0) return make_float2(__fmaf_rn(a.x, w.x, -__fmul_rn(a.y, w.y)), __fmaf_rn(a.x, w.y, __fmul_rn(a.y, w.x)));
  return make_float2(__fmaf_rn(a.x, w.x, __fmul_rn(a.y, w.y)), __fmaf_rn(a.y, w.x, -__fmul_rn(a.x, w.y)));
}
// multiply by SIGN * i  (exp(SIGN i pi/2))
template <int SIGN, typename C> __device__ __forceinline__ C cmul_si(C a) {
  if (SIGN < 0) return mk<C>(a.y, -a.x);
  return mk<C>(-a.y, a.x);
}

struct FftStage {
  int p;       // radix
  int l;       // length of the sub-transforms already combined
  int m;       // n / (l p)
  int tw_off;  // offset of this stage's l*(p-1) twiddles
  uint32_t mmul;  // exact b / m == (b * mmul) >> 21 for b < 2^11
};

struct FftPlan {
  int n;
  int nst;
  int tw_total;
  int team;     // threads per line in FP64 (at most 8 values per thread)
  int team_sp;  // threads per line in FP32 (at most 8 values per thread)
  int tw16_off; // n == 256: offset of the 16 x 16 table w_256^{f q} (else -1)
  int tw_pass;  // twiddles the pass kernels load: the 16 x 16 table (at 0) for n = 256, else all
  FftStage st[10];
};

// Values a thread holds per stage (8 complex: 16 in FP32 spills registers
// with five radices compiled into each stage loop).
template <typename C> struct Emax { static constexpr int value = 8; };
template <typename C> __device__ __forceinline__ int team_of(const FftPlan& pl) {
  return sizeof(C) <= 8 ? pl.team_sp : pl.team;
}

__device__ __forceinline__ int div_m(int b, const FftStage& s) { return (int)(((uint32_t)b * s.mmul) >> 21); }

// Shared-memory position of element p of a line: one pad slot after every 16
// elements, so the stride-16 row reads of the 16 x 16 path (and the strided
// reads of late Stockham stages) fall in distinct banks.
__host__ __device__ __forceinline__ int sidx(int p) { return p + (p >> 4); }
// Stride between consecutive lines: room for sidx(n - 1), rounded up to odd
// so lines start in rotating banks.
__host__ __device__ __forceinline__ int line_stride(int n) {
  const int s = n + ((n - 1) >> 4);
  return s | 1;
}

// Exact unsigned division by a runtime divisor d >= 1 for n < 2^31
// (round-up multiplier method): q = (umulhi(n, mul) + n) >> shift.
struct FastDiv {
  uint32_t d, mul, shift;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  uint32_t s = 0;
  while ((1ull << s) < d) ++s;
  f.shift = s;
  f.mul = (uint32_t)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  return (uint32_t)(((uint64_t)__umulhi(n, f.mul) + n) >> f.shift);
}

// ---- radix-p DFT kernels on registers (in place on a[0..P-1])
template <int SIGN, typename C> __device__ __forceinline__ void dft2(C* a) {
  C t = a[1];
  a[1] = csub(a[0], t);
  a[0] = cadd(a[0], t);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft4(C* a) {
  C t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]);
  C t2 = cadd(a[1], a[3]), t3 = cmul_si<SIGN>(csub(a[1], a[3]));
  a[0] = cadd(t0, t2);
  a[2] = csub(t0, t2);
  a[1] = cadd(t1, t3);
  a[3] = csub(t1, t3);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft8(C* a) {
  using T = decltype(C::x);
  const T h = (T)0.70710678118654752440084436210484903928;  // sqrt(2)/2
  // first level: pairs (q, q+4)
  C b0 = cadd(a[0], a[4]), b4 = csub(a[0], a[4]);
  C b1 = cadd(a[1], a[5]), b5 = csub(a[1], a[5]);
  C b2 = cadd(a[2], a[6]), b6 = csub(a[2], a[6]);
  C b3 = cadd(a[3], a[7]), b7 = csub(a[3], a[7]);
  // twiddles w8^{q} on the odd half: q=1 -> (1 + SIGN i) h, q=2 -> SIGN i, q=3 -> (-1 + SIGN i) h
  b6 = cmul_si<SIGN>(b6);
  {
    C t = b5;  // (t.x - SIGN? ) : multiply by h (1 + SIGN i)
    if (SIGN < 0) b5 = mk<C>((t.x + t.y) * h, (t.y - t.x) * h);
    else b5 = mk<C>((t.x - t.y) * h, (t.y + t.x) * h);
    t = b7;  // multiply by h (-1 + SIGN i)
    if (SIGN < 0) b7 = mk<C>((-t.x + t.y) * h, (-t.y - t.x) * h);
    else b7 = mk<C>((-t.x - t.y) * h, (-t.y + t.x) * h);
  }
  // two length-4 DFTs on (b0,b1,b2,b3) and (b4,b5,b6,b7)
  C e[4] = {b0, b1, b2, b3};
  C o[4] = {b4, b5, b6, b7};
  dft4<SIGN>(e);
  dft4<SIGN>(o);
  // outputs: even-indexed from e, odd-indexed from o
  a[0] = e[0]; a[2] = e[1]; a[4] = e[2]; a[6] = e[3];
  a[1] = o[0]; a[3] = o[1]; a[5] = o[2]; a[7] = o[3];
}

template <int SIGN, typename C> __device__ __forceinline__ void dft3(C* a) {
  using T = decltype(C::x);
  const T c1 = (T)-0.5;
  const T s1 = (T)SIGN * (T)0.86602540378443864676372317075293618347;  // SIGN*sin(2pi/3)
  C t = cadd(a[1], a[2]);
  C d = csub(a[1], a[2]);
  C y0 = cadd(a[0], t);
  C m = mk<C>(a[0].x + c1 * t.x, a[0].y + c1 * t.y);
  // SIGN i s * d
  C r = mk<C>(-s1 * d.y, s1 * d.x);
  a[0] = y0;
  a[1] = cadd(m, r);
  a[2] = csub(m, r);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft5(C* a) {
  using T = decltype(C::x);
  const T c1 = (T)0.30901699437494742410229341718281905886;   // cos(2pi/5)
  const T c2 = (T)-0.80901699437494742410229341718281905886;  // cos(4pi/5)
  const T s1 = (T)SIGN * (T)0.95105651629515357211643933337938214340;  // sin(2pi/5)
  const T s2 = (T)SIGN * (T)0.58778525229247312916870595463907276860;  // sin(4pi/5)
  C t1 = cadd(a[1], a[4]), d1 = csub(a[1], a[4]);
  C t2 = cadd(a[2], a[3]), d2 = csub(a[2], a[3]);
  C y0 = cadd(a[0], cadd(t1, t2));
  C m1 = mk<C>(a[0].x + c1 * t1.x + c2 * t2.x, a[0].y + c1 * t1.y + c2 * t2.y);
  C m2 = mk<C>(a[0].x + c2 * t1.x + c1 * t2.x, a[0].y + c2 * t1.y + c1 * t2.y);
  // i*(s1 d1 + s2 d2) and i*(s2 d1 - s1 d2)
  C n1 = mk<C>(-(s1 * d1.y + s2 * d2.y), s1 * d1.x + s2 * d2.x);
  C n2 = mk<C>(-(s2 * d1.y - s1 * d2.y), s2 * d1.x - s1 * d2.x);
  a[0] = y0;
  a[1] = cadd(m1, n1);
  a[4] = csub(m1, n1);
  a[2] = cadd(m2, n2);
  a[3] = csub(m2, n2);
}

// v * (cr + i si) for real constants cr, si
template <typename C, typename T> __device__ __forceinline__ C crot(C v, T cr, T si) {
  return mk<C>(v.x * cr - v.y * si, v.x * si + v.y * cr);
}
__device__ __forceinline__ float2 crot(float2 v, float cr, float si) {
  return make_float2(__fmaf_rn(v.x, cr, -__fmul_rn(v.y, si)), __fmaf_rn(v.x, si, __fmul_rn(v.y, cr)));
}
__device__ __forceinline__ ddc crot(ddc v, dd cr, dd si) {
  return dd_cplx_dot(v, f2p(cr.hi, si.hi), f2p(cr.lo, si.lo), f2p(-si.hi, cr.hi), f2p(-si.lo, cr.lo));
}

// 16-point DFT in registers as 4 x 4: DFT4 over n1 of x[4 n1 + n2], the
// twiddles w16^{n2 k1}, DFT4 over n2; output k1 + 4 k2 in place.
template <int SIGN, typename C> __device__ __forceinline__ void dft16(C* a) {
  using T = decltype(C::x);
  const T c1 = (T)0.92387953251128675612818318939678828682;  // cos(pi/8)
  const T s1 = (T)0.38268343236508977172845998403039886676;  // sin(pi/8)
  const T h = (T)0.70710678118654752440084436210484903928;   // sqrt(2)/2
  C b[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    C t[4] = {a[n2], a[4 + n2], a[8 + n2], a[12 + n2]};
    dft4<SIGN>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) b[n2][k1] = t[k1];
  }
  // w16^j = (cos(2 pi j/16), SIGN sin(2 pi j/16)) for j = n2 k1
  auto rot = [&](C v, T cr, T si) { return crot(v, cr, si); };
  const T sg = (T)SIGN;
  b[1][1] = rot(b[1][1], c1, sg * s1);   // j = 1
  b[1][2] = rot(b[1][2], h, sg * h);     // j = 2
  b[1][3] = rot(b[1][3], s1, sg * c1);   // j = 3
  b[2][1] = rot(b[2][1], h, sg * h);     // j = 2
  b[2][2] = cmul_si<SIGN>(b[2][2]);      // j = 4
  b[2][3] = rot(b[2][3], -h, sg * h);    // j = 6
  b[3][1] = rot(b[3][1], s1, sg * c1);   // j = 3
  b[3][2] = rot(b[3][2], -h, sg * h);    // j = 6
  b[3][3] = rot(b[3][3], -c1, -sg * s1); // j = 9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    C t[4] = {b[0][k1], b[1][k1], b[2][k1], b[3][k1]};
    dft4<SIGN>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) a[k1 + 4 * k2] = t[k2];
  }
}

template <int P, int SIGN, typename C> __device__ __forceinline__ void dftp(C* a) {
  if (P == 2) dft2<SIGN>(a);
  else if (P == 3) dft3<SIGN>(a);
  else if (P == 4) dft4<SIGN>(a);
  else if (P == 5) dft5<SIGN>(a);
  else dft8<SIGN>(a);
}

// One Stockham stage of radix P on one line held in shared memory.
// tl: lane index within the team, TW: team width.
__device__ __forceinline__ void team_sync(int TW) {
  if (TW <= 32) {
    __syncwarp();
  } else {
    const int id = 1 + (int)(threadIdx.x / TW);
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(TW) : "memory");
  }
}

// Reads element idx of the line being transformed (the stage's input).
template <typename C> struct LineLoad {
  const C* line;
  __device__ __forceinline__ C operator()(int idx) const { return line[sidx(idx)]; }
};

template <int P, int SIGN, typename C, typename Ld>
__device__ __forceinline__ void fft_stage(C* line, const C* __restrict__ tw, const FftStage& s, int n, int tl,
                                          int TW, Ld load) {
  constexpr int MAXB = Emax<C>::value / P;
  const int nb = n / P;
  C a[MAXB][P];
  int fo[MAXB], ko[MAXB];
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = tl + i * TW;
    fo[i] = 0; ko[i] = 0;
    if (b < nb) {
      const int f = div_m(b, s);
      const int k = b - f * s.m;
      fo[i] = f; ko[i] = k;
      const int src = f * s.m * P + k;
      a[i][0] = load(src);
      if (s.l == 1) {
#pragma unroll
        for (int q = 1; q < P; ++q) a[i][q] = load(src + s.m * q);
      } else {
        const C* w = tw + s.tw_off + f * (P - 1);
#pragma unroll
        for (int q = 1; q < P; ++q) a[i][q] = ctw<SIGN>(load(src + s.m * q), w[q - 1]);
      }
    }
  }
  team_sync(TW);
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = tl + i * TW;
    if (b < nb) {
      dftp<P, SIGN>(a[i]);
      const int dst = fo[i] * s.m + ko[i];
      const int os = s.l * s.m;
#pragma unroll
      for (int q = 0; q < P; ++q) line[sidx(dst + q * os)] = a[i][q];
    }
  }
  team_sync(TW);
}

// Full transform of one line (all threads of the team call this together;
// a team with no line passes active=false and still synchronises).
template <int SIGN, typename C, typename Ld>
__device__ __forceinline__ void fft_stage_p(C* line, const C* __restrict__ tw, const FftStage& st, int n, int tl,
                                            int TW, Ld load) {
  switch (st.p) {
    case 8: fft_stage<8, SIGN>(line, tw, st, n, tl, TW, load); break;
    case 4: fft_stage<4, SIGN>(line, tw, st, n, tl, TW, load); break;
    case 2: fft_stage<2, SIGN>(line, tw, st, n, tl, TW, load); break;
    case 3: fft_stage<3, SIGN>(line, tw, st, n, tl, TW, load); break;
    default: fft_stage<5, SIGN>(line, tw, st, n, tl, TW, load); break;
  }
}

// Full transform of one line (all threads of the team call this together;
// a team with no line passes active=false and still synchronises).
template <int SIGN, typename C>
__device__ __forceinline__ void fft_line(C* line, const C* __restrict__ tw, const FftPlan& pl, int tl, bool active) {
  const int n = pl.n;
  const int TW = team_of<C>(pl);
  const int tla = active ? tl : (1 << 20);  // inactive lanes own no butterfly
  for (int s = 0; s < pl.nst; ++s) fft_stage_p<SIGN>(line, tw, pl.st[s], n, tla, TW, LineLoad<C>{line});
}

// As fft_line, but the first stage reads its inputs through first(idx), so a
// caller can form the line on the fly (e.g. the product of two other lines).
template <int SIGN, typename C, typename First>
__device__ __forceinline__ void fft_line_from(C* line, const C* __restrict__ tw, const FftPlan& pl, int tl,
                                              bool active, First first) {
  const int n = pl.n;
  const int TW = team_of<C>(pl);
  const int tla = active ? tl : (1 << 20);
  fft_stage_p<SIGN>(line, tw, pl.st[0], n, tla, TW, first);
  for (int s = 1; s < pl.nst; ++s) fft_stage_p<SIGN>(line, tw, pl.st[s], n, tla, TW, LineLoad<C>{line});
}

// n = 256 as 16 x 16 in registers: a team of 16 threads per line, two lines
// per warp.  Thread k first transforms the column x[k + 16 q] (the l = 1
// Stockham stage of radix 16) and writes it back; thread f then reads row
// 16 f + q, applies w_256^{f q} and transforms it (the l = 16 stage).  One
// shared-memory exchange and four warp barriers per line.
template <int SIGN, typename C, typename First>
__device__ __forceinline__ void fft256_lines(C* base, int ld, int nlines, const C* __restrict__ tw,
                                             const FftPlan& pl, First first) {
  const int team = threadIdx.x >> 4;
  const int k = threadIdx.x & 15;
  const int nteams = blockDim.x >> 4;
  const int rounds = (nlines + nteams - 1) / nteams;
  const C* w = tw + pl.tw16_off + k;  // w[16 q] = w_256^{k q}
  for (int r = 0; r < rounds; ++r) {
    const int L = r * nteams + team;
    const bool active = L < nlines;
    C* line = base + (active ? L : 0) * ld;
    C a[16];
    if (active) {
      const auto ld0 = first(L);
#pragma unroll
      for (int q = 0; q < 16; ++q) a[q] = ld0(k + 16 * q);
      dft16<SIGN>(a);
    }
    __syncwarp();
    if (active) {
#pragma unroll
      for (int s = 0; s < 16; ++s) line[sidx(16 * s + k)] = a[s];
    }
    __syncwarp();
    if (active) {
      a[0] = line[sidx(16 * k)];
#pragma unroll
      for (int q = 1; q < 16; ++q) a[q] = ctw<SIGN>(line[sidx(16 * k + q)], w[16 * q]);
      dft16<SIGN>(a);
    }
    __syncwarp();
    if (active) {
#pragma unroll
      for (int s = 0; s < 16; ++s) line[sidx(k + 16 * s)] = a[s];
    }
    __syncwarp();
  }
}

// Code paths of the line transforms: kFftAny picks at run time (the plan's
// length); kFft256 compiles only the 16 x 16 register path (n = 256) and
// kFftGeneric only the Stockham stages with the radix chosen at run time;
// PATH = n (32, 64, 96, 128, 256, 512) compiles the Stockham stages of that length
// with their radices fixed at compile time.  A kernel built for one length
// thus carries no registers for another path.
constexpr int kFftAny = 0, kFft256 = 1, kFftGeneric = 2;

// The s-th radix of the plan for length n (build_plan's order: 8s, then 4,
// 2, 3, 5) and the number of stages, at compile time.
__host__ __device__ constexpr int ct_radix(int n, int s) {
  int r = n, k = 0;
  while (r % 8 == 0) { if (k == s) return 8; r /= 8; ++k; }
  while (r % 4 == 0) { if (k == s) return 4; r /= 4; ++k; }
  while (r % 2 == 0) { if (k == s) return 2; r /= 2; ++k; }
  while (r % 3 == 0) { if (k == s) return 3; r /= 3; ++k; }
  while (r % 5 == 0) { if (k == s) return 5; r /= 5; ++k; }
  return 0;
}
__host__ __device__ constexpr int ct_nst(int n) {
  int s = 0;
  while (ct_radix(n, s) != 0) ++s;
  return s;
}
// lengths with a compile-time path
__host__ __device__ constexpr bool ct_length(int n) {
  return n == 32 || n == 64 || n == 96 || n == 128 || n == 256 || n == 512;
}
// Twiddles a kernel compiled for PATH loads: the 16 x 16 table alone (at the
// start of the table) for the register path, all of them otherwise.
template <int PATH> __device__ __forceinline__ int tw_load(const FftPlan& pl) {
  return PATH == kFft256 ? pl.tw_pass : pl.tw_total;
}

// Stages S.. of a compile-time length N on one line; stage 0 reads through first.
template <int SIGN, int N, int S, typename C, typename First>
__device__ __forceinline__ void fft_ct_stages(C* line, const C* __restrict__ tw, const FftPlan& pl, int tl, int TW,
                                              First first) {
  if constexpr (S < ct_nst(N)) {
    if constexpr (S == 0) fft_stage<ct_radix(N, 0), SIGN>(line, tw, pl.st[0], N, tl, TW, first);
    else fft_stage<ct_radix(N, S), SIGN>(line, tw, pl.st[S], N, tl, TW, LineLoad<C>{line});
    fft_ct_stages<SIGN, N, S + 1>(line, tw, pl, tl, TW, first);
  }
}

// Transform `nlines` lines of a CTA's shared-memory tile.  Line L starts at
// base + L*ld.  Every thread of the CTA must call this with the same plan.
template <int SIGN, int PATH = kFftAny, typename C>
__device__ __forceinline__ void fft_lines(C* base, int ld, int nlines, const C* __restrict__ tw, const FftPlan& pl) {
  if (pl.n == 1) return;
  if (PATH == kFft256 || (PATH == kFftAny && pl.tw16_off >= 0)) {
    fft256_lines<SIGN>(base, ld, nlines, tw, pl, [&](int L) { return LineLoad<C>{base + L * ld}; });
    return;
  }
  if (PATH == kFft256) return;
  const int TW = team_of<C>(pl);
  const int nteams = blockDim.x / TW;
  const int team = threadIdx.x / TW;
  const int tl = threadIdx.x - team * TW;
  const int rounds = (nlines + nteams - 1) / nteams;
  for (int r = 0; r < rounds; ++r) {
    const int L = r * nteams + team;
    const bool active = L < nlines;
    if constexpr (ct_length(PATH)) {
      C* line = base + (active ? L : 0) * ld;
      fft_ct_stages<SIGN, PATH, 0>(line, tw, pl, active ? tl : (1 << 20), TW, LineLoad<C>{line});
    } else {
      fft_line<SIGN>(base + (active ? L : 0) * ld, tw, pl, tl, active);
    }
  }
}

// As fft_lines, with the first stage of line L reading through the loader
// first(L) returns (a functor idx -> value).  A length-1 transform is the
// identity: the inputs are only copied into place.
template <int SIGN, int PATH = kFftAny, typename C, typename First>
__device__ __forceinline__ void fft_lines_from(C* base, int ld, int nlines, const C* __restrict__ tw,
                                               const FftPlan& pl, First first) {
  if (pl.n == 1 || pl.nst == 0) {
    for (int L = threadIdx.x; L < nlines; L += blockDim.x) base[L * ld] = first(L)(0);
    return;
  }
  if (PATH == kFft256 || (PATH == kFftAny && pl.tw16_off >= 0)) {
    fft256_lines<SIGN>(base, ld, nlines, tw, pl, first);
    return;
  }
  if (PATH == kFft256) return;
  const int TW = team_of<C>(pl);
  const int nteams = blockDim.x / TW;
  const int team = threadIdx.x / TW;
  const int tl = threadIdx.x - team * TW;
  const int rounds = (nlines + nteams - 1) / nteams;
  for (int r = 0; r < rounds; ++r) {
    const int L = r * nteams + team;
    const bool active = L < nlines;
    const int Lc = active ? L : 0;
    if constexpr (ct_length(PATH)) {
      fft_ct_stages<SIGN, PATH, 0>(base + Lc * ld, tw, pl, active ? tl : (1 << 20), TW, first(Lc));
    } else {
      fft_line_from<SIGN>(base + Lc * ld, tw, pl, tl, active, first(Lc));
    }
  }
}

// Copy a plan from global memory into shared memory (call before a barrier).
__device__ __forceinline__ void load_plan(FftPlan* s_plan, const FftPlan* __restrict__ g_plan) {
  const int nw = (int)(sizeof(FftPlan) / sizeof(int));
  const int* src = reinterpret_cast<const int*>(g_plan);
  int* dst = reinterpret_cast<int*>(s_plan);
  for (int i = threadIdx.x; i < nw; i += blockDim.x) dst[i] = src[i];
}

}  // namespace samgpu
