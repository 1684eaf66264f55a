/*
 * CPU oracle -- test infrastructure, never part of the shipped product.
 *
 * Mixed-radix FFTs with FFTPACK v4 conventions (fft.f, vendored in the
 * reference):
 *   cfftf  (fft.f:189-268):  c(j) = sum_k c(k) exp(-i (j-1)(k-1) 2 pi / n)
 *   cfftb  (fft.f:24-60):    c(j) = sum_k c(k) exp(+i (j-1)(k-1) 2 pi / n)
 *   rfftf  (fft.f:2350-2403): r(1)=sum r, r(2k-2)=Re X(k-1), r(2k-1)=Im X(k-1),
 *                             r(n)=Nyquist (n even); X uses exp(-i ...)
 *   rfftb: the inverse synthesis of that packing (unnormalised).
 * All transforms are unnormalised, exactly as FFTPACK's.
 *
 * The algorithm here is a self-sorting (Stockham) decimation-in-time
 * factorisation written for this oracle; it is not FFTPACK's code.  A stage of
 * radix p combines p sub-transforms of length l into one of length l*p:
 *   Y'[(f + l s) m + k] = sum_q w_p^{s q} ( w_{lp}^{f q} Y[f m p + k + m q] )
 * with m = n/(l p).  Twiddles are evaluated in long double and rounded.
 */
#include "so_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const long double SO_TWO_PI_L = 6.283185307179586476925286766559005768L;

static int factorize(int n, int *fac) {
  int nf = 0;
  /* radix 4 first, then 2, 3, 5, then any remaining odd prime */
  while (n % 4 == 0) { fac[nf++] = 4; n /= 4; }
  while (n % 2 == 0) { fac[nf++] = 2; n /= 2; }
  for (int p = 3; n > 1; p += 2) {
    while (n % p == 0) { fac[nf++] = p; n /= p; }
  }
  return nf;
}

static so_cplx cexp_sign(int sign, long double num, long double den) {
  long double a = SO_TWO_PI_L * num / den;
  return (double)cosl(a) + (double)(sign * sinl(a)) * I;
}

int so_cplan_init(so_cplan *p, int n) {
  memset(p, 0, sizeof(*p));
  if (n < 1) return -1;
  p->n = n;
  p->nf = factorize(n, p->fac);
  /* twiddle tables for both signs: per stage, l*(radix-1) entries */
  int total = 0, l = 1;
  for (int s = 0; s < p->nf; ++s) { total += l * (p->fac[s] - 1); l *= p->fac[s]; }
  p->ntw = total;
  p->twf = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(total + 1));
  p->twb = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(total + 1));
  /* per-stage roots of unity exp(-+ 2 pi i e / r), e = 0..r-1, for odd radices */
  for (int s = 0; s < p->nf; ++s)
    if (p->fac[s] > 64) return -2; /* radices above 64 are not supported */
  int nroot = 0;
  for (int s = 0; s < p->nf; ++s) nroot += p->fac[s];
  p->rootf = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)nroot);
  p->rootb = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)nroot);
  for (int s = 0, o = 0; s < p->nf; o += p->fac[s], ++s)
    for (int e = 0; e < p->fac[s]; ++e) {
      p->rootf[o + e] = cexp_sign(-1, (long double)e, (long double)p->fac[s]);
      p->rootb[o + e] = cexp_sign(+1, (long double)e, (long double)p->fac[s]);
    }
  int off = 0;
  l = 1;
  for (int s = 0; s < p->nf; ++s) {
    int r = p->fac[s];
    long double L = (long double)l * r;
    for (int f = 0; f < l; ++f)
      for (int q = 1; q < r; ++q) {
        p->twf[off + f * (r - 1) + (q - 1)] = cexp_sign(-1, (long double)f * q, L);
        p->twb[off + f * (r - 1) + (q - 1)] = cexp_sign(+1, (long double)f * q, L);
      }
    off += l * (r - 1);
    l *= r;
  }
  return 0;
}

void so_cplan_free(so_cplan *p) {
  free(p->twf); free(p->twb); free(p->rootf); free(p->rootb);
  memset(p, 0, sizeof(*p));
}

/* one transform of length n; work must hold n complex values */
static void cfft_run(const so_cplan *p, so_cplx *c, so_cplx *work, int sign) {
  const int n = p->n;
  if (n == 1) return;
  so_cplx *x = c, *y = work;
  const so_cplx *tw = sign < 0 ? p->twf : p->twb;
  int l = 1, off = 0, roff = 0;
  for (int s = 0; s < p->nf; ++s) {
    const int r = p->fac[s];
    const int m = n / (l * r);
    const so_cplx *root = (sign < 0 ? p->rootf : p->rootb) + roff;
    for (int f = 0; f < l; ++f) {
      const so_cplx *w = tw + off + f * (r - 1);
      for (int k = 0; k < m; ++k) {
        so_cplx a[64];
        const so_cplx *src = x + (size_t)f * m * r + k;
        a[0] = src[0];
        for (int q = 1; q < r; ++q) a[q] = src[(size_t)m * q] * w[q - 1];
        so_cplx *dst = y + (size_t)f * m + k;
        const size_t os = (size_t)l * m;
        if (r == 2) {
          dst[0] = a[0] + a[1];
          dst[os] = a[0] - a[1];
        } else if (r == 4) {
          so_cplx t0 = a[0] + a[2], t1 = a[0] - a[2];
          so_cplx t2 = a[1] + a[3], t3 = a[1] - a[3];
          /* multiply t3 by sign*i: exp(sign*i*pi/2) */
          so_cplx t3r = sign < 0 ? (cimag(t3) - creal(t3) * I) : (-cimag(t3) + creal(t3) * I);
          dst[0] = t0 + t2;
          dst[os] = t1 + t3r;
          dst[2 * os] = t0 - t2;
          dst[3 * os] = t1 - t3r;
        } else {
          /* generic radix: direct DFT over q, roots of unity of order r */
          for (int s2 = 0; s2 < r; ++s2) {
            so_cplx acc = a[0];
            for (int q = 1; q < r; ++q) acc += a[q] * root[(s2 * q) % r];
            dst[(size_t)s2 * os] = acc;
          }
        }
      }
    }
    off += l * (r - 1);
    roff += r;
    l *= r;
    so_cplx *t = x; x = y; y = t;
  }
  if (x != c) memcpy(c, x, sizeof(so_cplx) * (size_t)n);
}

void so_cfftf(const so_cplan *p, so_cplx *c, so_cplx *work) { cfft_run(p, c, work, -1); }
void so_cfftb(const so_cplan *p, so_cplx *c, so_cplx *work) { cfft_run(p, c, work, +1); }

int so_rplan_init(so_rplan *p, int n) {
  memset(p, 0, sizeof(*p));
  if (n < 1) return -1;
  p->n = n;
  if (n % 2 == 0) {
    so_cplan_init(&p->half, n / 2);
    p->wr = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(n / 2 + 1));
    for (int k = 0; k <= n / 2; ++k) p->wr[k] = cexp_sign(-1, (long double)k, (long double)n);
  } else {
    so_cplan_init(&p->full, n);
  }
  return 0;
}

void so_rplan_free(so_rplan *p) {
  if (p->n % 2 == 0) so_cplan_free(&p->half); else so_cplan_free(&p->full);
  free(p->wr);
  memset(p, 0, sizeof(*p));
}

/* work must hold n+2 complex values */
void so_rfftf(const so_rplan *p, double *r, so_cplx *work) {
  const int n = p->n;
  if (n == 1) return;
  if (n % 2) {
    so_cplx *z = work, *w2 = work + n;
    for (int i = 0; i < n; ++i) z[i] = r[i];
    so_cfftf(&p->full, z, w2);
    r[0] = creal(z[0]);
    for (int k = 1; k <= (n - 1) / 2; ++k) { r[2 * k - 1] = creal(z[k]); r[2 * k] = cimag(z[k]); }
    return;
  }
  const int h = n / 2;
  so_cplx *z = work, *w2 = work + h + 1;
  for (int j = 0; j < h; ++j) z[j] = r[2 * j] + r[2 * j + 1] * I;
  so_cfftf(&p->half, z, w2);
  /* X_k = E_k + w^k O_k with E_k = (Z_k + conj Z_{h-k})/2, O_k = (Z_k - conj Z_{h-k})/(2i) */
  so_cplx X0 = creal(z[0]) + cimag(z[0]);
  so_cplx Xh = creal(z[0]) - cimag(z[0]);
  r[0] = creal(X0);
  for (int k = 1; k < h; ++k) {
    so_cplx zk = z[k], zc = conj(z[h - k]);
    so_cplx E = 0.5 * (zk + zc);
    so_cplx O = -0.5 * I * (zk - zc);
    so_cplx X = E + p->wr[k] * O;
    r[2 * k - 1] = creal(X);
    r[2 * k] = cimag(X);
  }
  r[n - 1] = creal(Xh);
}

void so_rfftb(const so_rplan *p, double *r, so_cplx *work) {
  const int n = p->n;
  if (n == 1) return;
  if (n % 2) {
    so_cplx *z = work, *w2 = work + n;
    z[0] = r[0];
    for (int k = 1; k <= (n - 1) / 2; ++k) {
      so_cplx v = r[2 * k - 1] + r[2 * k] * I;
      z[k] = v;
      z[n - k] = conj(v);
    }
    so_cfftb(&p->full, z, w2);
    for (int i = 0; i < n; ++i) r[i] = creal(z[i]);
    return;
  }
  const int h = n / 2;
  so_cplx *z = work, *w2 = work + h + 1;
  /* rebuild X_0..X_h, then Z_k = E_k + i O_k with E_k=(X_k+conj X_{h-k}), O_k = conj(w^k)(X_k - conj X_{h-k}) */
  double x0 = r[0], xh = r[n - 1];
  z[0] = (x0 + xh) + (x0 - xh) * I;
  for (int k = 1; k < h; ++k) {
    so_cplx Xk = r[2 * k - 1] + r[2 * k] * I;
    int kk = h - k;
    so_cplx Xc = conj(r[2 * kk - 1] + r[2 * kk] * I);
    so_cplx E = Xk + Xc;
    so_cplx O = (Xk - Xc) * conj(p->wr[k]);
    z[k] = E + I * O;
  }
  so_cfftb(&p->half, z, w2);
  for (int j = 0; j < h; ++j) { r[2 * j] = creal(z[j]); r[2 * j + 1] = cimag(z[j]); }
}
