/*
 * CPU oracle -- test infrastructure, never part of the shipped product.
 * FFTPACK-convention transforms (fft.f of the reference), restated.
 */
#ifndef SO_FFT_H
#define SO_FFT_H
#include <complex.h>

typedef double _Complex so_cplx;

typedef struct {
  int n, nf, fac[40], ntw;
  so_cplx *twf, *twb;     /* stage twiddles, forward / backward sign */
  so_cplx *rootf, *rootb; /* per-stage roots of unity for odd radices */
} so_cplan;

typedef struct {
  int n;
  so_cplan half; /* even n: complex transform of length n/2 */
  so_cplan full; /* odd n: complex transform of length n */
  so_cplx *wr;   /* exp(-2 pi i k / n), k = 0..n/2 */
} so_rplan;

int so_cplan_init(so_cplan *p, int n);
void so_cplan_free(so_cplan *p);
/* work: n complex */
void so_cfftf(const so_cplan *p, so_cplx *c, so_cplx *work);
void so_cfftb(const so_cplan *p, so_cplx *c, so_cplx *work);

int so_rplan_init(so_rplan *p, int n);
void so_rplan_free(so_rplan *p);
/* work: 2n+2 complex */
void so_rfftf(const so_rplan *p, double *r, so_cplx *work);
void so_rfftb(const so_rplan *p, double *r, so_cplx *work);
#endif
