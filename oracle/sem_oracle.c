/*
 * sem_oracle.c — CPU restatement (plain C + OpenMP) of SpectralElements.jl's
 * operator apply and PCG, used ONLY as test infrastructure: the parity checker
 * at sizes where the NumPy oracle is slow, and the optimised CPU baseline of
 * bench.py.  It is never linked into, loaded by, or called from the product.
 *
 * Layout: column-major (n*Ex) x (n*Ey) local fields (src/semmesh.jl:19).
 *   laplace : src/lapl.jl:70-81   (ur = Dr u, us = u Ds', wr/ws, Dr' wr + ws Ds)
 *   hlmz    : src/hlmz.jl:12-19   (nu .* lapl + k .* (B .* u))
 *   QQ'     : src/gatherScatter.jl:8-16 with src/semq.jl:6-25 (sum of copies:
 *             x pairs, then y pairs, in increasing index order)
 *   mask    : src/mask.jl:10-18 with src/mesh.jl:149-175
 *   pcg     : src/pcg.jl:16-60
 * Parity status: unpinned (see sem_oracle.py); this file is checked against
 * the NumPy restatement by the CPU test suite.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int n, Ex, Ey, perx, pery;
  int dxmin, dxmax, dymin, dymax; /* Dirichlet flags (ignored in a periodic direction) */
} so_grid;

static int keep(const so_grid* g, int64_t r, int64_t c) {
  const int64_t NX = (int64_t)g->n * g->Ex, NY = (int64_t)g->n * g->Ey;
  if (!g->perx && ((g->dxmin && r == 0) || (g->dxmax && r == NX - 1))) return 0;
  if (!g->pery && ((g->dymin && c == 0) || (g->dymax && c == NY - 1))) return 0;
  return 1;
}

static int64_t partner(int64_t r, int n, int E, int per) {
  const int64_t NX = (int64_t)n * E;
  const int64_t e = r / n;
  const int i = (int)(r - e * n);
  if (i == 0) {
    if (e > 0) return r - 1;
    if (per) return NX - 1;
  }
  if (i == n - 1) {
    if (e < E - 1) return r + 1;
    if (per) return 0;
  }
  return -1;
}

/* out = QQ' u (out != u) */
void so_gather_scatter(const so_grid* g, const double* u, double* out) {
  const int64_t NX = (int64_t)g->n * g->Ex, NY = (int64_t)g->n * g->Ey;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < NY; ++c) {
    const int64_t pc = partner(c, g->n, g->Ey, g->pery);
    for (int64_t r = 0; r < NX; ++r) {
      const int64_t pr = partner(r, g->n, g->Ex, g->perx);
      const int64_t r0 = (pr >= 0 && pr < r) ? pr : r, r1 = (pr >= 0 && pr < r) ? r : pr;
      double v;
      if (pc < 0) {
        v = u[r0 + c * NX];
        if (r1 >= 0) v += u[r1 + c * NX];
      } else {
        const int64_t c0 = pc < c ? pc : c, c1 = pc < c ? c : pc;
        double a = u[r0 + c0 * NX], b = u[r0 + c1 * NX];
        if (r1 >= 0) {
          a += u[r1 + c0 * NX];
          b += u[r1 + c1 * NX];
        }
        v = a + b;
      }
      out[r + c * NX] = v;
    }
  }
}

/* out = mask(QQ'(nu .* lapl(u) + k B u)) with the optional steps of flags:
 * 1 = QQ', 2 = mask; nu_f (nullable) multiplies the lapl output pointwise
 * (lapl(u,nu,msh)), nug (nullable) is folded into G (variable coefficient). */
void so_apply(const so_grid* g, const double* Dr, const double* Ds, const double* G11,
              const double* G12, const double* G22, const double* B, const double* nu_f,
              const double* nug, double nu, double k, int flags, const double* u, double* out,
              double* work) {
  const int n = g->n;
  const int64_t NX = (int64_t)n * g->Ex, NY = (int64_t)n * g->Ey;
  double* loc = (flags & 1) ? work : out;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ey = 0; ey < g->Ey; ++ey)
    for (int ex = 0; ex < g->Ex; ++ex) {
      double ur[32 * 32], us[32 * 32], wr[32 * 32], ws[32 * 32];
      const int64_t r0 = (int64_t)ex * n, c0 = (int64_t)ey * n;
#define AT(a, i, j) a[(r0 + (i)) + (c0 + (j)) * NX]
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double sr = 0.0, ss = 0.0;
          for (int q = 0; q < n; ++q) {
            sr += Dr[i + q * n] * AT(u, q, j);
            ss += AT(u, i, q) * Ds[j + q * n];
          }
          ur[i + j * n] = sr;
          us[i + j * n] = ss;
        }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const double a = ur[i + j * n], b = us[i + j * n];
          double w1 = AT(G11, i, j) * a + AT(G12, i, j) * b;
          double w2 = AT(G12, i, j) * a + AT(G22, i, j) * b;
          if (nug) {
            w1 *= AT(nug, i, j);
            w2 *= AT(nug, i, j);
          }
          wr[i + j * n] = w1;
          ws[i + j * n] = w2;
        }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double s1 = 0.0, s2 = 0.0;
          for (int q = 0; q < n; ++q) {
            s1 += Dr[q + i * n] * wr[q + j * n];
            s2 += ws[i + q * n] * Ds[q + j * n];
          }
          double v = s1 + s2;
          v = nu_f ? AT(nu_f, i, j) * v : nu * v;
          if (B && k != 0.0) v += k * (AT(B, i, j) * AT(u, i, j));
          AT(loc, i, j) = v;
        }
#undef AT
    }
  if (flags & 1) so_gather_scatter(g, work, out);
  if (flags & 2) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < NY; ++c)
      for (int64_t r = 0; r < NX; ++r)
        if (!keep(g, r, c)) out[r + c * NX] = 0.0 * out[r + c * NX];
  }
}

static double mult_at(const so_grid* g, int64_t r, int64_t c) {
  const int cx = partner(r, g->n, g->Ex, g->perx) >= 0 ? 2 : 1;
  const int cy = partner(c, g->n, g->Ey, g->pery) >= 0 ? 2 : 1;
  return 1.0 / (double)(cx * cy);
}

/* pcg of src/pcg.jl:16-60 with opA = mask(QQ'(hlmz(., nu, k))) and opM =
 * r ./ d (d = NULL: identity).  Returns the iteration count; *res = final
 * Inf-norm residual.  x must hold length(b) doubles. */
int so_pcg(const so_grid* g, const double* Dr, const double* Ds, const double* G11,
           const double* G12, const double* G22, const double* B, const double* nug, double nu,
           double k, const double* d, const double* b, double* x, double tol, int maxiter,
           double* res) {
  const int64_t NX = (int64_t)g->n * g->Ex, NY = (int64_t)g->n * g->Ey, L = NX * NY;
  double* r = (double*)malloc(sizeof(double) * L);
  double* h = (double*)malloc(sizeof(double) * L);
  double* p = (double*)malloc(sizeof(double) * L);
  double* Ap = (double*)malloc(sizeof(double) * L);
  double* work = (double*)malloc(sizeof(double) * L);
  double* mult = (double*)malloc(sizeof(double) * L);
  for (int64_t c = 0; c < NY; ++c)
    for (int64_t rr = 0; rr < NX; ++rr) mult[rr + c * NX] = mult_at(g, rr, c);
  memset(x, 0, sizeof(double) * L);
  memcpy(r, b, sizeof(double) * L);
  double tprev = 1.0;
  int it = 0;
  for (;;) {
    double rm = 0.0;
    for (int64_t i = 0; i < L; ++i) rm = fabs(r[i]) > rm || r[i] != r[i] ? fabs(r[i]) : rm;
    *res = rm;
    if (!(rm > tol)) break;
    if (it == maxiter) break;
    ++it;
    double t = 0.0;
    for (int64_t i = 0; i < L; ++i) {
      h[i] = d ? r[i] / d[i] : r[i];
      t += r[i] * h[i] * mult[i];
    }
    const double beta = it == 1 ? 0.0 : t / tprev;
    for (int64_t i = 0; i < L; ++i) p[i] = it == 1 ? h[i] : h[i] + beta * p[i];
    so_apply(g, Dr, Ds, G11, G12, G22, B, NULL, nug, nu, k, 3, p, Ap, work);
    double pap = 0.0;
    for (int64_t i = 0; i < L; ++i) pap += p[i] * Ap[i] * mult[i];
    const double alpha = t / pap;
    for (int64_t i = 0; i < L; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * Ap[i];
    }
    tprev = t;
  }
  free(r);
  free(h);
  free(p);
  free(Ap);
  free(work);
  free(mult);
  return it;
}
