/* C restatement of the reference optimizer on C^-1 (test infrastructure only).
 * See pngf_port.h. Loop structure follows pngf-opt/pngfopt.hpp so that the
 * CPU baseline costs what the reference costs: O(k^2 N) per evaluation
 * (pngfopt.hpp:435-455) and O(k N^2) per accept (pngfopt.hpp:294-307, 350-358).
 */
#include "pngf_port.h"

#include <complex.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zc;

typedef void (*zgetrf_t)(int *, int *, zc *, int *, int *, int *);
typedef void (*zgetri_t)(int *, zc *, int *, int *, zc *, int *, int *);
typedef void (*zgetrs_t)(char *, int *, int *, zc *, int *, int *, zc *, int *, int *);
typedef void (*zgemm_t)(char *, char *, int *, int *, int *, zc *, zc *, int *, zc *, int *, zc *, zc *, int *);

static zgetrf_t p_zgetrf;
static zgetri_t p_zgetri;
static zgetrs_t p_zgetrs;
static zgemm_t p_zgemm;

void port_set_lapack(void *a, void *b, void *c, void *d) {
  p_zgetrf = (zgetrf_t)a;
  p_zgetri = (zgetri_t)b;
  p_zgetrs = (zgetrs_t)c;
  p_zgemm = (zgemm_t)d;
}

int port_threads(void) { return omp_get_max_threads(); }

struct port_state {
  long n;
  int E, kmax;
  zc *G, *Cinv, *Gobj, *R, *Einc, *PEinc, *S, *Snew, *Eobj, *newEobj;
  signed char *P;
  /* last evaluation */
  int k;
  int *s, *d, *ipiv;
  zc *V, *K, *VS, *RU, *CinvU, *VCinv, *work;
};

static void *xmalloc(size_t b) { return b ? malloc(b) : NULL; }

/* compute_R_matrix: R = Gobj C^-1, S = C^-1 PEinc (pngfopt.hpp:237-250). */
static void compute_R(port_state *s, int compute_eobj) {
  int n = (int)s->n, E = s->E, one = 1;
  zc alpha = 1.0, beta = 0.0;
  char N = 'N';
  p_zgemm(&N, &N, &E, &n, &n, &alpha, s->Gobj, &E, s->Cinv, &n, &beta, s->R, &E);
  p_zgemm(&N, &N, &n, &one, &n, &alpha, s->Cinv, &n, s->PEinc, &n, &beta, s->S, &n);
  if (compute_eobj) {
    p_zgemm(&N, &N, &E, &one, &n, &alpha, s->R, &E, s->PEinc, &n, &beta, s->Eobj, &E);
    memcpy(s->newEobj, s->Eobj, sizeof(zc) * E);
  } else {
    memcpy(s->Eobj, s->newEobj, sizeof(zc) * E);
  }
}

static void compute_PEinc(port_state *s) {
#pragma omp parallel for
  for (long i = 0; i < s->n; ++i) s->PEinc[i] = s->P[i] ? -s->Einc[i] : 0.0;
}

port_state *port_create(long n, int E, int kmax, const double *G, const double *Gobj, const double *Einc,
                        const signed char *P) {
  if (!p_zgetrf || !p_zgetri || !p_zgetrs || !p_zgemm) return NULL;
  port_state *s = (port_state *)calloc(1, sizeof(port_state));
  s->n = n;
  s->E = E;
  s->kmax = kmax;
  const size_t nn = (size_t)n * n;
  s->G = xmalloc(sizeof(zc) * nn);
  s->Cinv = xmalloc(sizeof(zc) * nn);
  s->Gobj = xmalloc(sizeof(zc) * E * n);
  s->R = xmalloc(sizeof(zc) * E * n);
  s->Einc = xmalloc(sizeof(zc) * n);
  s->PEinc = xmalloc(sizeof(zc) * n);
  s->S = xmalloc(sizeof(zc) * n);
  s->Snew = xmalloc(sizeof(zc) * n);
  s->Eobj = xmalloc(sizeof(zc) * E);
  s->newEobj = xmalloc(sizeof(zc) * E);
  s->P = xmalloc(n);
  s->s = xmalloc(sizeof(int) * kmax);
  s->d = xmalloc(sizeof(int) * kmax);
  s->ipiv = xmalloc(sizeof(int) * (n > kmax ? n : kmax));
  s->V = xmalloc(sizeof(zc) * kmax * n);
  s->K = xmalloc(sizeof(zc) * kmax * kmax);
  s->VS = xmalloc(sizeof(zc) * kmax);
  s->RU = xmalloc(sizeof(zc) * kmax * E);
  s->CinvU = xmalloc(sizeof(zc) * kmax * n);
  s->VCinv = xmalloc(sizeof(zc) * kmax * n);
  s->work = xmalloc(sizeof(zc) * 100 * (size_t)(kmax > 1 ? kmax : 1));
  if (!s->G || !s->Cinv || !s->V || !s->VCinv || !s->CinvU) {
    port_destroy(s);
    return NULL;
  }
  memcpy(s->G, G, sizeof(zc) * nn);
  memcpy(s->Gobj, Gobj, sizeof(zc) * E * n);
  memcpy(s->Einc, Einc, sizeof(zc) * n);
  memcpy(s->P, P, n);
  /* compute_C_matrix, column-major branch (pngfopt.hpp:215-231) */
#pragma omp parallel for
  for (long ii = 0; ii < n; ++ii) {
    zc *col = s->Cinv + (size_t)ii * n;
    const zc *g = s->G + (size_t)ii * n;
    for (long jj = 0; jj < n; ++jj) col[jj] = s->P[jj] ? g[jj] : (ii == jj ? 1.0 : 0.0);
  }
  /* LinAlg::invertMatrix (linalg.hpp:34-85) */
  int nn_ = (int)n, info = 0, lwork = -1;
  zc wq;
  p_zgetrf(&nn_, &nn_, s->Cinv, &nn_, s->ipiv, &info);
  if (info != 0) {
    port_destroy(s);
    return NULL;
  }
  p_zgetri(&nn_, s->Cinv, &nn_, s->ipiv, &wq, &lwork, &info);
  lwork = (int)creal(wq);
  zc *work = xmalloc(sizeof(zc) * (lwork > 1 ? lwork : 1));
  p_zgetri(&nn_, s->Cinv, &nn_, s->ipiv, work, &lwork, &info);
  free(work);
  if (info != 0) {
    port_destroy(s);
    return NULL;
  }
  compute_PEinc(s);
  compute_R(s, 1);
  return s;
}

void port_destroy(port_state *s) {
  if (!s) return;
  free(s->G); free(s->Cinv); free(s->Gobj); free(s->R); free(s->Einc); free(s->PEinc); free(s->S);
  free(s->Snew); free(s->Eobj); free(s->newEobj); free(s->P); free(s->s); free(s->d); free(s->ipiv);
  free(s->V); free(s->K); free(s->VS); free(s->RU); free(s->CinvU); free(s->VCinv); free(s->work);
  free(s);
}

int port_eval(port_state *st, const int *edges, const int *signs, int k, double *new_eobj) {
  if (k < 0 || k > st->kmax) return 1;
  const long n = st->n;
  const int E = st->E;
  st->k = k;
  memcpy(st->s, edges, sizeof(int) * k);
  memcpy(st->d, signs, sizeof(int) * k);
  const int *s = st->s, *d = st->d;
  /* RU = +-R[:, s] (pngfopt.hpp:398-418) */
  for (int q = 0; q < k; ++q)
    for (int e = 0; e < E; ++e) st->RU[q * E + e] = d[q] > 0 ? st->R[(size_t)s[q] * E + e] : -st->R[(size_t)s[q] * E + e];
  /* V = (G - I)[s, :], stored as V^T column-major (pngfopt.hpp:422-432) */
#pragma omp parallel for
  for (int jj = 0; jj < k; ++jj) {
    zc *v = st->V + (size_t)jj * n;
    for (long ii = 0; ii < n; ++ii) v[ii] = st->G[s[jj] + (size_t)ii * n];
    v[s[jj]] -= 1.0;
  }
  /* K = I + V C^-1[:, s] D (pngfopt.hpp:435-455) */
#pragma omp parallel for
  for (int ii = 0; ii < k * k; ++ii) {
    const int col = ii / k, row = ii - col * k;
    const zc *v = st->V + (size_t)row * n;
    const zc *c = st->Cinv + (size_t)s[col] * n;
    zc acc = 0.0;
    for (long i = 0; i < n; ++i) acc += v[i] * c[i];
    if (d[col] < 0) acc = -acc;
    if (row == col) acc += 1.0;
    st->K[ii] = acc;
  }
  /* Snew = S - C^-1[:, s] D Einc_s (pngfopt.hpp:458-465) */
#pragma omp parallel for
  for (long ii = 0; ii < n; ++ii) {
    zc acc = 0.0;
    for (int jj = 0; jj < k; ++jj) acc += st->Cinv[ii + (size_t)s[jj] * n] * st->Einc[s[jj]] * (double)d[jj];
    st->Snew[ii] = st->S[ii] - acc;
  }
  /* VSnew = V Snew (pngfopt.hpp:467-480) */
#pragma omp parallel for
  for (int ii = 0; ii < k; ++ii) {
    const zc *v = st->V + (size_t)ii * n;
    zc acc = 0.0;
    for (long jj = 0; jj < n; ++jj) acc += v[jj] * st->Snew[jj];
    st->VS[ii] = acc;
  }
  /* zgetrf + zgetrs (pngfopt.hpp:493-510) */
  int kk = k, one = 1, info = 0;
  char N = 'N';
  if (k > 0) {
    p_zgetrf(&kk, &kk, st->K, &kk, st->ipiv, &info);
    p_zgetrs(&N, &kk, &one, st->K, &kk, st->ipiv, st->VS, &kk, &info);
  }
  /* newEobj = Gobj Snew - RU x (pngfopt.hpp:514-537) */
  for (int j = 0; j < E; ++j) {
    zc acc = 0.0;
    for (long i = 0; i < n; ++i) acc += st->Gobj[j + (size_t)i * E] * st->Snew[i];
    zc r = 0.0;
    for (int i = 0; i < k; ++i) r += st->RU[i * E + j] * st->VS[i];
    st->newEobj[j] = acc - r;
    new_eobj[2 * j] = creal(st->newEobj[j]);
    new_eobj[2 * j + 1] = cimag(st->newEobj[j]);
  }
  return info != 0 ? 2 : 0;
}

int port_accept(port_state *st) {
  const long n = st->n;
  const int k = st->k;
  const int *s = st->s, *d = st->d;
  if (k > 0) {
    /* CinvU = +-C^-1[:, s] (pngfopt.hpp:260-274) */
#pragma omp parallel for
    for (int ii = 0; ii < k; ++ii) {
      const zc *c = st->Cinv + (size_t)s[ii] * n;
      zc *o = st->CinvU + (size_t)ii * n;
      for (long jj = 0; jj < n; ++jj) o[jj] = d[ii] > 0 ? c[jj] : -c[jj];
    }
    /* K^-1 from the factors (pngfopt.hpp:284-291) */
    int kk = k, lwork = 100 * k, info = 0;
    p_zgetri(&kk, st->K, &kk, st->ipiv, st->work, &lwork, &info);
    /* VCinv = V C^-1, the naive loop of pngfopt.hpp:294-307 */
#pragma omp parallel for
    for (long ii = 0; ii < (long)k * n; ++ii) {
      const long col = ii / k, row = ii - col * k;
      const zc *v = st->V + (size_t)row * n;
      const zc *c = st->Cinv + (size_t)col * n;
      zc acc = 0.0;
      for (long i = 0; i < n; ++i) acc += v[i] * c[i];
      st->VCinv[ii] = acc;
    }
    /* V <- K^-1 VCinv; C^-1 <- C^-1 - CinvU V (pngfopt.hpp:324-358) */
    int nn = (int)n;
    zc alpha = 1.0, beta = 0.0;
    char N = 'N';
    p_zgemm(&N, &N, &kk, &nn, &kk, &alpha, st->K, &kk, st->VCinv, &kk, &beta, st->V, &kk);
    alpha = -1.0;
    beta = 1.0;
    p_zgemm(&N, &N, &nn, &nn, &kk, &alpha, st->CinvU, &nn, st->V, &kk, &beta, st->Cinv, &nn);
    for (int q = 0; q < k; ++q) st->P[s[q]] = (signed char)(st->P[s[q]] + d[q]);
  }
  compute_PEinc(st);
  compute_R(st, 0);
  return 0;
}

void port_eobj(const port_state *s, double *eobj) {
  for (int e = 0; e < s->E; ++e) {
    eobj[2 * e] = creal(s->Eobj[e]);
    eobj[2 * e + 1] = cimag(s->Eobj[e]);
  }
}
