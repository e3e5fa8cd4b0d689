/* CPU restatement of the reference recursive-skeletonization solver.
 * TEST INFRASTRUCTURE ONLY (the checker); see rs_oracle.h.
 *
 * Sources restated (paths within jpryan1/ie-solver):
 *   tree        ie_solver/quadtree/quadtree.cpp:39-432, 997-1074
 *   kernels     ie_solver/kernel/kernel.cpp:29-290, 293-591
 *   ID          ie_solver/ie_mat.cpp:548-588 with LAPACK dgeqp3/dlaqp2/dlarfg
 *               (published algorithm, Businger-Golub pivoting with the
 *               Drmac-Bujanovic norm-downdating safeguard) and dtrtrs
 *   LU          ie_solver/ie_mat.cpp:449-519 with LAPACK dgetrf/dgetrs
 *   factor      ie_solver/skel_factorization/skel_factorization.cpp:38-310, 323-381
 *   solve       ie_solver/skel_factorization/skel_factorization.cpp:388-426, 507-777
 *   border      ie_solver/linear_solve.cpp:20-112
 */
#include "rs_oracle.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define MIN_DOFS_TO_COMPRESS 16 /* skel_factorization.h:11 */
#define RADIUS_RATIO 1.5        /* kernel.h:12 */

/* ------------------------------------------------------------------ */
/* growable int vector                                                 */
/* ------------------------------------------------------------------ */
typedef struct {
  int* v;
  int n, cap;
} ivec;

static void iv_push(ivec* a, int x) {
  if (a->n == a->cap) {
    a->cap = a->cap ? 2 * a->cap : 8;
    a->v = (int*)realloc(a->v, sizeof(int) * (size_t)a->cap);
  }
  a->v[a->n++] = x;
}
static void iv_clear(ivec* a) { a->n = 0; }
static void iv_free(ivec* a) { free(a->v); a->v = NULL; a->n = a->cap = 0; }
static void iv_append(ivec* a, const ivec* b) { for (int i = 0; i < b->n; ++i) iv_push(a, b->v[i]); }
static void iv_copy(ivec* a, const ivec* b) { iv_clear(a); iv_append(a, b); }

/* ------------------------------------------------------------------ */
/* data structures (quadtree.h:16-139)                                 */
/* ------------------------------------------------------------------ */
typedef struct {
  int level, is_leaf, parent;
  int bl, tl, tr, br;
  int children[4]; /* {bl, tl, tr, br}, quadtree.cpp:356-359 */
  double corners[8], side;
  ivec nbr;
  ivec orig, active, skel, red, near, perm;
  int compressed;
  int k, r;
  double *T, *L, *U, *Xrr, *Xlu, *schur;
  int* piv;
} node_t;

struct orc_solver {
  int pde, sd, n, nholes, leaf, npp, nthreads;
  double tol;
  double *pts, *nrm, *w, *curv, *hc, *hr;
  node_t* nodes;
  int num_nodes, cap_nodes;
  ivec* levels;
  int num_levels, cap_levels;
  double tmin, tmax;
  int root;
  /* root and bordered blocks */
  int ns;          /* |allskel| */
  int* allskel;
  double* allskel_mat; /* ns x ns before LU */
  double* allskel_lu;
  int* allskel_piv;
  int nb;          /* bordered dimension (3h Stokes, h Laplace), 0 = none */
  double *U, *Psi; /* (n*sd x nb), (nb x n*sd) */
  double* S_lu;
  int* S_piv;
  double t_factor, t_solve;
  int tree_built, factored;
};

/* ------------------------------------------------------------------ */
/* small dense helpers (column major)                                  */
/* ------------------------------------------------------------------ */
static double* dalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* C (m x n) = alpha * op(A) * op(B) + beta * C; op = transpose when ta/tb. */
static void gemm(int ta, int tb, int m, int n, int k, double alpha, const double* A, int lda,
                 const double* B, int ldb, double beta, double* C, int ldc) {
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < m; ++i) C[i + (size_t)ldc * j] *= beta;
    for (int l = 0; l < k; ++l) {
      double b = tb ? B[j + (size_t)ldb * l] : B[l + (size_t)ldb * j];
      b *= alpha;
      if (b == 0.0) continue;
      if (!ta) {
        const double* a = A + (size_t)lda * l;
        double* c = C + (size_t)ldc * j;
        for (int i = 0; i < m; ++i) c[i] += a[i] * b;
      } else {
        double* c = C + (size_t)ldc * j;
        for (int i = 0; i < m; ++i) c[i] += A[l + (size_t)lda * i] * b;
      }
    }
  }
}

static double nrm2(int n, const double* x) {
  /* scaled two-norm (overflow/underflow safe) */
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n; ++i) {
    if (x[i] != 0.0) {
      double a = fabs(x[i]);
      if (scale < a) {
        ssq = 1.0 + ssq * (scale / a) * (scale / a);
        scale = a;
      } else {
        ssq += (a / scale) * (a / scale);
      }
    }
  }
  return scale * sqrt(ssq);
}

/* LAPACK dgetrf (right-looking, partial pivoting); piv is 0-based row index
 * swapped with row j at step j.  Returns 0, or j+1 if U(j,j) == 0. */
static int getrf(int n, double* A, int lda, int* piv) {
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int p = j;
    double mx = fabs(A[j + (size_t)lda * j]);
    for (int i = j + 1; i < n; ++i) {
      double v = fabs(A[i + (size_t)lda * j]);
      if (v > mx) { mx = v; p = i; }
    }
    piv[j] = p;
    if (A[p + (size_t)lda * j] != 0.0) {
      if (p != j)
        for (int c = 0; c < n; ++c) {
          double t = A[j + (size_t)lda * c];
          A[j + (size_t)lda * c] = A[p + (size_t)lda * c];
          A[p + (size_t)lda * c] = t;
        }
      double inv = 1.0 / A[j + (size_t)lda * j];
      for (int i = j + 1; i < n; ++i) A[i + (size_t)lda * j] *= inv;
    } else if (info == 0) {
      info = j + 1;
    }
    for (int c = j + 1; c < n; ++c) {
      double b = A[j + (size_t)lda * c];
      if (b == 0.0) continue;
      double* col = A + (size_t)lda * c;
      const double* lcol = A + (size_t)lda * j;
      for (int i = j + 1; i < n; ++i) col[i] -= lcol[i] * b;
    }
  }
  return info;
}

/* dgetrs 'N': B (n x nrhs) <- A^{-1} B. */
static void getrs_n(int n, const double* LU, int lda, const int* piv, double* B, int ldb,
                    int nrhs) {
  for (int c = 0; c < nrhs; ++c) {
    double* b = B + (size_t)ldb * c;
    for (int j = 0; j < n; ++j)
      if (piv[j] != j) { double t = b[j]; b[j] = b[piv[j]]; b[piv[j]] = t; }
    for (int j = 0; j < n; ++j) {
      double v = b[j];
      if (v != 0.0)
        for (int i = j + 1; i < n; ++i) b[i] -= v * LU[i + (size_t)lda * j];
    }
    for (int j = n - 1; j >= 0; --j) {
      if (b[j] != 0.0) {
        b[j] /= LU[j + (size_t)lda * j];
        double v = b[j];
        for (int i = 0; i < j; ++i) b[i] -= v * LU[i + (size_t)lda * j];
      }
    }
  }
}

/* dgetrs 'T': B <- A^{-T} B. */
static void getrs_t(int n, const double* LU, int lda, const int* piv, double* B, int ldb,
                    int nrhs) {
  for (int c = 0; c < nrhs; ++c) {
    double* b = B + (size_t)ldb * c;
    for (int j = 0; j < n; ++j) { /* U^T y = b */
      double v = b[j];
      for (int i = 0; i < j; ++i) v -= LU[i + (size_t)lda * j] * b[i];
      b[j] = v / LU[j + (size_t)lda * j];
    }
    for (int j = n - 1; j >= 0; --j) { /* L^T z = y */
      double v = b[j];
      for (int i = j + 1; i < n; ++i) v -= LU[i + (size_t)lda * j] * b[i];
      b[j] = v;
    }
    for (int j = n - 1; j >= 0; --j)
      if (piv[j] != j) { double t = b[j]; b[j] = b[piv[j]]; b[piv[j]] = t; }
  }
}

/* ------------------------------------------------------------------ */
/* interpolative decomposition: ie_mat.cpp:548-588                    */
/* ------------------------------------------------------------------ */

/* LAPACK dlarfg: on return alpha = beta, x = v(2:), returns tau. */
static double larfg(int n, double* alpha, double* x) {
  if (n <= 1) return 0.0;
  double xnorm = nrm2(n - 1, x);
  if (xnorm == 0.0) return 0.0;
  double beta = -copysign(hypot(*alpha, xnorm), *alpha);
  double tau = (beta - *alpha) / beta;
  double scal = 1.0 / (*alpha - beta);
  for (int i = 0; i < n - 1; ++i) x[i] *= scal;
  *alpha = beta;
  return tau;
}

int orc_id(const double* Ain, int m, int n, double tol, int* perm, double* Z, double* rdiag) {
  if (m <= 0 || n <= 0) return 0;
  double* A = dalloc((size_t)m * n);
  memcpy(A, Ain, sizeof(double) * (size_t)m * n);
  int* jp = (int*)malloc(sizeof(int) * (size_t)n);
  double* vn1 = dalloc(n);
  double* vn2 = dalloc(n);
  double* work = dalloc(n);
  const double tol3z = sqrt(DBL_EPSILON * 0.5);
  int mn = m < n ? m : n;
  for (int j = 0; j < n; ++j) {
    jp[j] = j;
    vn1[j] = nrm2(m, A + (size_t)m * j);
    vn2[j] = vn1[j];
  }
  /* dlaqp2: unblocked column-pivoted Householder QR */
  for (int i = 0; i < mn; ++i) {
    int pvt = i;
    double mx = fabs(vn1[i]);
    for (int j = i + 1; j < n; ++j)
      if (fabs(vn1[j]) > mx) { mx = fabs(vn1[j]); pvt = j; }
    if (pvt != i) {
      double* a = A + (size_t)m * pvt;
      double* b = A + (size_t)m * i;
      for (int r = 0; r < m; ++r) { double t = a[r]; a[r] = b[r]; b[r] = t; }
      int t = jp[pvt]; jp[pvt] = jp[i]; jp[i] = t;
      vn1[pvt] = vn1[i];
      vn2[pvt] = vn2[i];
    }
    double* col = A + (size_t)m * i;
    double tau = larfg(m - i, &col[i], &col[i + 1]);
    if (i < n - 1 && tau != 0.0) {
      double aii = col[i];
      col[i] = 1.0;
      for (int c = i + 1; c < n; ++c) {
        double* cc = A + (size_t)m * c;
        double s = 0.0;
        for (int r = i; r < m; ++r) s += col[r] * cc[r];
        s *= tau;
        for (int r = i; r < m; ++r) cc[r] -= s * col[r];
      }
      col[i] = aii;
    }
    for (int j = i + 1; j < n; ++j) {
      if (vn1[j] != 0.0) {
        double temp = fabs(A[i + (size_t)m * j]) / vn1[j];
        temp = 1.0 - temp * temp;
        if (temp < 0.0) temp = 0.0;
        double temp2 = temp * (vn1[j] / vn2[j]) * (vn1[j] / vn2[j]);
        if (temp2 <= tol3z) {
          if (i < m - 1) {
            vn1[j] = nrm2(m - i - 1, A + (size_t)m * j + i + 1);
            vn2[j] = vn1[j];
          } else {
            vn1[j] = 0.0;
            vn2[j] = 0.0;
          }
        } else {
          vn1[j] *= sqrt(temp);
        }
      }
    }
  }
  for (int i = 0; i < n; ++i) {
    if (rdiag) rdiag[i] = i < mn ? A[i + (size_t)m * i] : 0.0;
    if (perm) perm[i] = jp[i];
  }
  /* rank scan, ie_mat.cpp:559-568 */
  int skel = 0;
  double thresh = fabs(tol * A[0]);
  for (int i = 1; i < n; ++i) {
    double rii = i < mn ? A[i + (size_t)m * i] : 0.0;
    if (fabs(rii) < thresh) { skel = i; break; }
  }
  if (skel > 0 && Z) {
    /* Z = R11^{-1} R12 by back substitution (dtrtrs 'U','N','N') */
    int red = n - skel;
    for (int c = 0; c < red; ++c) {
      double* z = Z + (size_t)skel * c;
      for (int r = 0; r < skel; ++r) z[r] = A[r + (size_t)m * (skel + c)];
      for (int r = skel - 1; r >= 0; --r) {
        z[r] /= A[r + (size_t)m * r];
        double v = z[r];
        for (int q = 0; q < r; ++q) z[q] -= v * A[q + (size_t)m * r];
      }
    }
  }
  free(A); free(jp); free(vn1); free(vn2); free(work);
  return skel;
}

/* ------------------------------------------------------------------ */
/* kernels: kernel.cpp:105-290                                         */
/* ------------------------------------------------------------------ */
static double laplace_entry(const orc_solver* s, int t, int j) {
  const double scale = 1.0 / (2 * M_PI);
  double sp1 = s->pts[2 * j], sp2 = s->pts[2 * j + 1];
  double sn1 = s->nrm[2 * j], sn2 = s->nrm[2 * j + 1];
  double sw = s->w[j], sc = s->curv[j];
  double tp1 = s->pts[2 * t], tp2 = s->pts[2 * t + 1];
  if (tp1 == sp1 && sp2 == tp2) return 0 + 0.5 + 0.5 * sc * sw * scale;
  double r0 = tp1 - sp1, r1 = tp2 - sp2;
  return -sw * scale * (r0 * sn1 + r1 * sn2) / (r0 * r0 + r1 * r1);
}

static double laplace_neumann_entry(const orc_solver* s, int t, int j) {
  const double scale = 1.0 / (2 * M_PI);
  double sp1 = s->pts[2 * j], sp2 = s->pts[2 * j + 1];
  double sw = s->w[j], sc = s->curv[j];
  double tp1 = s->pts[2 * t], tp2 = s->pts[2 * t + 1];
  double tn1 = s->nrm[2 * t], tn2 = s->nrm[2 * t + 1];
  if (tp1 == sp1 && sp2 == tp2) return 0 + sw - 0.5 + 0.5 * sc * sw * scale;
  double r0 = tp1 - sp1, r1 = tp2 - sp2;
  return sw + sw * scale * (r0 * tn1 + r1 * tn2) / (r0 * r0 + r1 * r1);
}

static double stokes_entry(const orc_solver* s, int tgt, int src) {
  const double scale = 1.0 / M_PI;
  int jp = src / 2, ip = tgt / 2;
  double sp1 = s->pts[2 * jp], sp2 = s->pts[2 * jp + 1];
  double sn1 = s->nrm[2 * jp], sn2 = s->nrm[2 * jp + 1];
  double sw = s->w[jp], sc = s->curv[jp];
  double tp1 = s->pts[2 * ip], tp2 = s->pts[2 * ip + 1];
  double tn1 = s->nrm[2 * ip], tn2 = s->nrm[2 * ip + 1];
  if (tp1 == sp1 && sp2 == tp2) {
    double potential = -0.5 * sc * sw * scale;
    if (tgt % 2 == 0) {
      if (src % 2 == 0) return 0 - 0.5 + potential * sn2 * sn2 + sw * tn1 * sn1;
      return -potential * sn1 * sn2 + sw * tn2 * sn1;
    }
    if (src % 2 == 0) return -potential * sn1 * sn2 + sw * tn2 * sn1;
    return 0 - 0.5 + potential * sn1 * sn1 + sw * tn2 * sn2;
  }
  double r0 = tp1 - sp1, r1 = tp2 - sp2;
  double d = r0 * r0 + r1 * r1;
  double potential = sw * scale * (r0 * sn1 + r1 * sn2) / (d * d);
  if (tgt % 2 == 0) {
    if (src % 2 == 0) return potential * r0 * r0 + sw * tn1 * sn1;
    return potential * r0 * r1 + sw * tn1 * sn2;
  }
  if (src % 2 == 0) return potential * r1 * r0 + sw * tn2 * sn1;
  return potential * r1 * r1 + sw * tn2 * sn2;
}

static double kentry(const orc_solver* s, int i, int j) {
  if (s->pde == ORC_STOKES) return stokes_entry(s, i, j);
  if (s->pde == ORC_LAPLACE_NEUMANN) return laplace_neumann_entry(s, i, j);
  return laplace_entry(s, i, j);
}

void orc_kernel_block(const orc_solver* s, const int* I, int nI, const int* J, int nJ,
                      double* out) {
  for (int j = 0; j < nJ; ++j)
    for (int i = 0; i < nI; ++i) out[i + (size_t)nI * j] = kentry(s, I[i], J[j]);
}

/* Proxy rows [K(pxy <- box); K(box <- pxy)^T], kernel.cpp:426-591. */
static void proxy_block(const orc_solver* s, double cx, double cy, double r, const ivec* box,
                        double* out, int ldo) {
  int npp = s->npp;
  double pw = 2.0 * M_PI * r / npp;
  int n = box->n;
  for (int p = 0; p < npp; ++p) {
    double ang = 2 * M_PI * p * (1.0 / npp);
    double px = cx + (r + 0.0) * cos(ang), py = cy + (r + 0.0) * sin(ang);
    double pn1 = cos(ang), pn2 = sin(ang);
    if (s->pde == ORC_STOKES) {
      const double scale = 1.0 / M_PI;
      for (int j = 0; j < n; ++j) {
        int src = box->v[j], jp = src / 2;
        double sp1 = s->pts[2 * jp], sp2 = s->pts[2 * jp + 1];
        double sn1 = s->nrm[2 * jp], sn2 = s->nrm[2 * jp + 1], sw = s->w[jp];
        double r0 = px - sp1, r1 = py - sp2;
        double d = r0 * r0 + r1 * r1;
        double pot = sw * scale * (r0 * sn1 + r1 * sn2) / (d * d);
        double* c = out + (size_t)ldo * j;
        if (src % 2 == 0) {
          c[2 * p] = pot * r0 * r0 + sw * pn1 * sn1;
          c[2 * p + 1] = pot * r1 * r0 + sw * pn2 * sn1;
        } else {
          c[2 * p] = pot * r0 * r1 + sw * pn1 * sn2;
          c[2 * p + 1] = pot * r1 * r1 + sw * pn2 * sn2;
        }
      }
      for (int i = 0; i < n; ++i) {
        int tgt = box->v[i], ip = tgt / 2;
        double tp1 = s->pts[2 * ip], tp2 = s->pts[2 * ip + 1];
        double tn1 = s->nrm[2 * ip], tn2 = s->nrm[2 * ip + 1];
        double r0 = tp1 - px, r1 = tp2 - py;
        double d = r0 * r0 + r1 * r1;
        double pot = pw * scale * (r0 * pn1 + r1 * pn2) / (d * d);
        double* c = out + (size_t)ldo * i + 2 * npp;
        if (tgt % 2 == 0) {
          c[2 * p] = pot * r0 * r0 + pw * tn1 * pn1;
          c[2 * p + 1] = pot * r0 * r1 + pw * tn1 * pn2;
        } else {
          c[2 * p] = pot * r1 * r0 + pw * tn2 * pn1;
          c[2 * p + 1] = pot * r1 * r1 + pw * tn2 * pn2;
        }
      }
    } else if (s->pde == ORC_LAPLACE) {
      const double scale = 1.0 / (2 * M_PI);
      for (int j = 0; j < n; ++j) {
        int src = box->v[j];
        double r0 = px - s->pts[2 * src], r1 = py - s->pts[2 * src + 1];
        out[p + (size_t)ldo * j] = -s->w[src] * scale *
            (r0 * s->nrm[2 * src] + r1 * s->nrm[2 * src + 1]) / (r0 * r0 + r1 * r1);
      }
      for (int i = 0; i < n; ++i) {
        int tgt = box->v[i];
        double r0 = s->pts[2 * tgt] - px, r1 = s->pts[2 * tgt + 1] - py;
        out[npp + (size_t)ldo * i + p] = -pw * scale * (r0 * pn1 + r1 * pn2) /
                                         (r0 * r0 + r1 * r1);
      }
    } else { /* Laplace-Neumann, kernel.cpp:594-646 */
      const double scale = 1.0 / (2 * M_PI);
      for (int j = 0; j < n; ++j) {
        int src = box->v[j];
        double r0 = px - s->pts[2 * src], r1 = py - s->pts[2 * src + 1];
        double sw = s->w[src];
        out[p + (size_t)ldo * j] = sw + sw * scale * (r0 * pn1 + r1 * pn2) / (r0 * r0 + r1 * r1);
      }
      for (int i = 0; i < n; ++i) {
        int tgt = box->v[i];
        double r0 = s->pts[2 * tgt] - px, r1 = s->pts[2 * tgt + 1] - py;
        out[npp + (size_t)ldo * i + p] =
            pw + pw * scale * (r0 * s->nrm[2 * tgt] + r1 * s->nrm[2 * tgt + 1]) /
                     (r0 * r0 + r1 * r1);
      }
    }
  }
}

static int proxy_rows(const orc_solver* s) { return (s->pde == ORC_STOKES ? 4 : 2) * s->npp; }

/* ------------------------------------------------------------------ */
/* quadtree: quadtree.cpp:39-432                                       */
/* ------------------------------------------------------------------ */
static int new_node(orc_solver* s) {
  if (s->num_nodes == s->cap_nodes) {
    s->cap_nodes = s->cap_nodes ? 2 * s->cap_nodes : 64;
    s->nodes = (node_t*)realloc(s->nodes, sizeof(node_t) * (size_t)s->cap_nodes);
  }
  node_t* nd = &s->nodes[s->num_nodes];
  memset(nd, 0, sizeof(*nd));
  nd->is_leaf = 1;
  nd->parent = -1;
  nd->bl = nd->tl = nd->tr = nd->br = -1;
  for (int c = 0; c < 4; ++c) nd->children[c] = -1;
  return s->num_nodes++;
}

static void level_push(orc_solver* s, int level, int node) {
  while (s->num_levels <= level) {
    if (s->num_levels == s->cap_levels) {
      s->cap_levels = s->cap_levels ? 2 * s->cap_levels : 16;
      s->levels = (ivec*)realloc(s->levels, sizeof(ivec) * (size_t)s->cap_levels);
    }
    memset(&s->levels[s->num_levels], 0, sizeof(ivec));
    s->num_levels++;
  }
  iv_push(&s->levels[level], node);
}

static void node_subdivide(orc_solver* s, int ni);

/* quadtree.cpp:230-269 */
static void recursive_add(orc_solver* s, int ni, double x, double y, int point_ind) {
  for (int i = 0; i < s->sd; ++i) iv_push(&s->nodes[ni].orig, s->sd * point_ind + i);
  node_t* nd = &s->nodes[ni];
  double midx = ((nd->corners[6] - nd->corners[0]) / 2.0) + nd->corners[0];
  double midy = ((nd->corners[3] - nd->corners[1]) / 2.0) + nd->corners[1];
  int child;
  if (x < midx && y < midy) child = nd->bl;
  else if (x < midx && y >= midy) child = nd->tl;
  else if (x >= midx && y < midy) child = nd->br;
  else child = nd->tr;
  if (child >= 0) {
    recursive_add(s, child, x, y, point_ind);
  } else if (nd->is_leaf && nd->orig.n > s->leaf) {
    node_subdivide(s, ni);
  }
}

/* quadtree.cpp:275-432 */
static void node_subdivide(orc_solver* s, int ni) {
  s->nodes[ni].is_leaf = 0;
  double c[8];
  memcpy(c, s->nodes[ni].corners, sizeof(c));
  double midx = ((c[6] - c[0]) / 2.0) + c[0];
  double midy = ((c[3] - c[1]) / 2.0) + c[1];
  int bl = new_node(s), tl = new_node(s), tr = new_node(s), br = new_node(s);
  node_t* nd = &s->nodes[ni]; /* re-fetch after realloc */
  double* B = s->nodes[bl].corners;
  B[0] = c[0]; B[1] = c[1]; B[2] = c[2]; B[3] = midy; B[4] = midx; B[5] = midy; B[6] = midx; B[7] = c[7];
  double* TL = s->nodes[tl].corners;
  TL[0] = c[0]; TL[1] = midy; TL[2] = c[2]; TL[3] = c[3]; TL[4] = midx; TL[5] = c[5]; TL[6] = midx; TL[7] = midy;
  double* TR = s->nodes[tr].corners;
  TR[0] = midx; TR[1] = midy; TR[2] = midx; TR[3] = c[3]; TR[4] = c[4]; TR[5] = c[5]; TR[6] = c[6]; TR[7] = midy;
  double* BR = s->nodes[br].corners;
  BR[0] = midx; BR[1] = c[1]; BR[2] = midx; BR[3] = midy; BR[4] = c[4]; BR[5] = midy; BR[6] = c[6]; BR[7] = c[7];
  int kids[4] = {bl, tl, tr, br};
  for (int q = 0; q < 4; ++q) {
    node_t* k = &s->nodes[kids[q]];
    k->level = nd->level + 1;
    k->side = nd->side / 2.0;
    k->parent = ni;
  }
  /* level order bl, br, tr, tl (quadtree.cpp:338-350) */
  level_push(s, nd->level + 1, bl);
  level_push(s, nd->level + 1, br);
  level_push(s, nd->level + 1, tr);
  level_push(s, nd->level + 1, tl);
  nd = &s->nodes[ni];
  nd->bl = bl; nd->tl = tl; nd->tr = tr; nd->br = br;
  nd->children[0] = bl; nd->children[1] = tl; nd->children[2] = tr; nd->children[3] = br;
  for (int idx = 0; idx < nd->orig.n; idx += s->sd) {
    int mi = nd->orig.v[idx];
    int pv = (mi / s->sd) * 2;
    double x = s->pts[pv], y = s->pts[pv + 1];
    int dst;
    if (x < midx && y < midy) dst = bl;
    else if (x < midx && y >= midy) dst = tl;
    else if (x >= midx && y < midy) dst = br;
    else dst = tr;
    for (int i = 0; i < s->sd; ++i) iv_push(&s->nodes[dst].orig, mi + i);
  }
  if (s->nodes[bl].orig.n > s->leaf) node_subdivide(s, bl);
  if (s->nodes[tl].orig.n > s->leaf) node_subdivide(s, tl);
  if (s->nodes[tr].orig.n > s->leaf) node_subdivide(s, tr);
  if (s->nodes[br].orig.n > s->leaf) node_subdivide(s, br);
}

/* quadtree.cpp:185-227 */
static void get_descendent_neighbors(orc_solver* s, int big, int small) {
  double top = s->nodes[big].corners[3];
  double bottom = s->nodes[big].corners[1];
  double left = s->nodes[big].corners[0];
  double right = s->nodes[big].corners[4];
  for (int i = 0; i < 8; i += 2) {
    double x = s->nodes[small].corners[i];
    double y = s->nodes[small].corners[i + 1];
    int hit = 0;
    if (x > left && x < right) {
      if (fabs(y - top) < 1e-14) hit = 1;
      else if (fabs(y - bottom) < 1e-14) hit = 1;
    }
    if (!hit && y < top && y < bottom) { /* the reference's condition, kept */
      if (fabs(x - left) < 1e-14) hit = 1;
      else if (fabs(x - right) < 1e-14) hit = 1;
    }
    if (hit) {
      iv_push(&s->nodes[big].nbr, small);
      iv_push(&s->nodes[small].nbr, big);
      break;
    }
  }
  for (int c = 0; c < 4; ++c) {
    int ch = s->nodes[small].children[c];
    if (ch >= 0) get_descendent_neighbors(s, big, ch);
  }
}

int orc_build_tree(orc_solver* s) {
  if (s->n <= 0) return 1;
  double mn = s->pts[0], mx = s->pts[0];
  for (int i = 0; i < 2 * s->n; ++i) {
    if (s->pts[i] < mn) mn = s->pts[i];
    if (s->pts[i] > mx) mx = s->pts[i];
  }
  s->tmin = mn;
  s->tmax = mx;
  double lo = mn - 0.01, hi = mx + 0.01;
  int root = new_node(s);
  node_t* r = &s->nodes[root];
  r->level = 0;
  r->corners[0] = lo; r->corners[1] = lo; r->corners[2] = lo; r->corners[3] = hi;
  r->corners[4] = hi; r->corners[5] = hi; r->corners[6] = hi; r->corners[7] = lo;
  r->side = hi - lo;
  level_push(s, 0, root);
  s->root = root;
  for (int i = 0; i < s->n; ++i) recursive_add(s, root, s->pts[2 * i], s->pts[2 * i + 1], i);
  /* neighbor lists, quadtree.cpp:131-175 */
  for (int lv = 0; lv < s->num_levels; ++lv) {
    for (int k = 0; k < s->levels[lv].n; ++k) {
      int a = s->levels[lv].v[k];
      int par = s->nodes[a].parent;
      if (par >= 0) {
        for (int c = 0; c < 4; ++c) {
          int sib = s->nodes[par].children[c];
          if (sib != a) iv_push(&s->nodes[a].nbr, sib);
        }
        int np = s->nodes[par].nbr.n;
        for (int q = 0; q < np; ++q) {
          int pn = s->nodes[par].nbr.v[q];
          for (int c = 0; c < 4; ++c) {
            int cousin = s->nodes[pn].children[c];
            if (cousin < 0) continue;
            if (s->nodes[cousin].level != s->nodes[a].level) continue;
            double dist = sqrt(pow(s->nodes[a].corners[0] - s->nodes[cousin].corners[0], 2) +
                               pow(s->nodes[a].corners[1] - s->nodes[cousin].corners[1], 2));
            if (dist < s->nodes[a].side * sqrt(2) + 1e-5) iv_push(&s->nodes[a].nbr, cousin);
          }
        }
      }
      if (s->nodes[a].is_leaf) {
        for (int q = 0; q < s->nodes[a].nbr.n; ++q) {
          int nb = s->nodes[a].nbr.v[q];
          if (s->nodes[nb].level != s->nodes[a].level) continue;
          for (int c = 0; c < 4; ++c) {
            int ch = s->nodes[nb].children[c];
            if (ch >= 0) get_descendent_neighbors(s, a, ch);
          }
        }
      }
    }
  }
  s->tree_built = 1;
  return 0;
}

/* quadtree.cpp:1032-1074 */
static void remove_inactive_dofs_at_box(orc_solver* s, int ni) {
  node_t* nd = &s->nodes[ni];
  iv_clear(&nd->skel);
  iv_clear(&nd->red);
  iv_clear(&nd->active);
  if (!nd->is_leaf) {
    for (int c = 0; c < 4; ++c) {
      node_t* ch = &s->nodes[nd->children[c]];
      iv_append(&nd->active, ch->compressed ? &ch->skel : &ch->active);
    }
  } else {
    iv_copy(&nd->active, &nd->orig);
  }
}

/* quadtree.cpp:997-1025 */
static void remove_inactive_dofs_at_level(orc_solver* s, int level) {
  ivec* lv = &s->levels[level];
  for (int k = 0; k < lv->n; ++k)
    if (!s->nodes[lv->v[k]].compressed) remove_inactive_dofs_at_box(s, lv->v[k]);
  for (int k = 0; k < lv->n; ++k) {
    node_t* a = &s->nodes[lv->v[k]];
    iv_clear(&a->near);
    for (int q = 0; q < a->nbr.n; ++q) {
      node_t* nb = &s->nodes[a->nbr.v[q]];
      if (nb->level > a->level) continue;
      iv_append(&a->near, nb->is_leaf ? &nb->orig : &nb->active);
    }
  }
}

/* ------------------------------------------------------------------ */
/* ID matrix: kernel.cpp:293-423                                       */
/* ------------------------------------------------------------------ */
static void center_of(const node_t* nd, double* cx, double* cy) {
  *cx = nd->corners[0] + nd->side / 2.0;
  *cy = nd->corners[1] + nd->side / 2.0;
}

/* Gathers the row-source DOFs; *use_proxy tells whether proxy rows follow. */
static void id_rows(const orc_solver* s, int ni, ivec* rows, int* use_proxy) {
  const node_t* nd = &s->nodes[ni];
  iv_clear(rows);
  *use_proxy = 0;
  if (nd->level == 1 || nd->level == 2) {
    const ivec* lv = &s->levels[nd->level];
    for (int k = 0; k < lv->n; ++k)
      if (lv->v[k] != ni) iv_append(rows, &s->nodes[lv->v[k]].active);
    if (nd->level == 2) {
      const ivec* up = &s->levels[1];
      for (int k = 0; k < up->n; ++k)
        if (s->nodes[up->v[k]].is_leaf) iv_append(rows, &s->nodes[up->v[k]].orig);
    }
    return;
  }
  double cx, cy;
  center_of(nd, &cx, &cy);
  for (int q = 0; q < nd->near.n; ++q) {
    int mi = nd->near.v[q];
    int pv = (mi / s->sd) * 2;
    double x = s->pts[pv], y = s->pts[pv + 1];
    double dist = sqrt(pow(cx - x, 2) + pow(cy - y, 2));
    if (dist < RADIUS_RATIO * nd->side) iv_push(rows, mi);
  }
  *use_proxy = 1;
}

static double* build_id_matrix(const orc_solver* s, int ni, int* m_out) {
  const node_t* nd = &s->nodes[ni];
  ivec rows = {0};
  int use_proxy;
  id_rows(s, ni, &rows, &use_proxy);
  int n = nd->active.n, q = rows.n;
  int m = 2 * q + (use_proxy ? proxy_rows(s) : 0);
  double* A = dalloc((size_t)m * n);
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < q; ++i) {
      A[i + (size_t)m * j] = kentry(s, rows.v[i], nd->active.v[j]);
      A[q + i + (size_t)m * j] = kentry(s, nd->active.v[j], rows.v[i]);
    }
  }
  if (use_proxy) {
    double cx, cy;
    center_of(nd, &cx, &cy);
    proxy_block(s, cx, cy, nd->side * RADIUS_RATIO, &nd->active, A + 2 * q, m);
  }
  iv_free(&rows);
  *m_out = m;
  return A;
}

static int level_order_node(const orc_solver* s, int idx);

int orc_id_matrix(const orc_solver* s, int node, double* out, long cap, int* n_out) {
  int m;
  node = level_order_node(s, node);
  double* A = build_id_matrix(s, node, &m);
  int n = s->nodes[node].active.n;
  long cnt = (long)m * n;
  if (out) memcpy(out, A, sizeof(double) * (size_t)(cnt < cap ? cnt : cap));
  free(A);
  if (n_out) *n_out = n;
  return m;
}

/* ------------------------------------------------------------------ */
/* factorization: skel_factorization.cpp:38-381                        */
/* ------------------------------------------------------------------ */
/* get_update, skel_factorization.cpp:354-381 */
static void get_update(const orc_solver* s, double* upd, const ivec* BN, const node_t* d) {
  int nb = BN->n;
  int k = d->skel.n;
  int* bi = (int*)malloc(sizeof(int) * (size_t)(k ? k : 1));
  int* si = (int*)malloc(sizeof(int) * (size_t)(k ? k : 1));
  int cnt = 0;
  for (int a = 0; a < k; ++a)
    for (int b = 0; b < nb; ++b)
      if (BN->v[b] == d->skel.v[a]) { si[cnt] = a; bi[cnt] = b; ++cnt; }
  for (int i = 0; i < cnt; ++i)
    for (int j = 0; j < cnt; ++j)
      upd[bi[i] + (size_t)nb * bi[j]] += d->schur[si[i] + (size_t)k * si[j]];
  free(bi); free(si);
}

/* get_descendents_updates, skel_factorization.cpp:340-351 */
static void get_descendents_updates(const orc_solver* s, double* upd, const ivec* BN, int ni) {
  const node_t* nd = &s->nodes[ni];
  for (int c = 0; c < 4; ++c) {
    const node_t* ch = &s->nodes[nd->children[c]];
    if (ch->compressed) get_update(s, upd, BN, ch);
    if (!ch->is_leaf) get_descendents_updates(s, upd, BN, nd->children[c]);
  }
}

/* id_compress, skel_factorization.cpp:38-68 */
static int id_compress(orc_solver* s, int ni) {
  int m;
  double* A = build_id_matrix(s, ni, &m);
  node_t* nd = &s->nodes[ni];
  int n = nd->active.n;
  if (m == 0) { free(A); return 0; }
  int* p = (int*)malloc(sizeof(int) * (size_t)n);
  double* Z = dalloc((size_t)n * n);
  int k = orc_id(A, m, n, s->tol, p, Z, NULL);
  free(A);
  if (k == 0) { free(p); free(Z); return 0; }
  nd->k = k;
  nd->r = n - k;
  nd->T = dalloc((size_t)k * nd->r);
  memcpy(nd->T, Z, sizeof(double) * (size_t)k * nd->r);
  iv_clear(&nd->skel); iv_clear(&nd->red); iv_clear(&nd->perm);
  for (int i = 0; i < k; ++i) { iv_push(&nd->skel, nd->active.v[p[i]]); iv_push(&nd->perm, p[i]); }
  for (int i = k; i < n; ++i) { iv_push(&nd->red, nd->active.v[p[i]]); iv_push(&nd->perm, p[i]); }
  free(p); free(Z);
  return k;
}

/* decouple, skel_factorization.cpp:77-128 */
static void decouple(orc_solver* s, int ni) {
  node_t* nd = &s->nodes[ni];
  const ivec* BN = &nd->active;
  int nb = BN->n, k = nd->k, r = nd->r;
  double* KBN = dalloc((size_t)nb * nb);
  orc_kernel_block(s, BN->v, nb, BN->v, nb, KBN);
  double* upd = dalloc((size_t)nb * nb);
  if (!nd->is_leaf) get_descendents_updates(s, upd, BN, ni);
  for (size_t i = 0; i < (size_t)nb * nb; ++i) KBN[i] -= upd[i];
  free(upd);
  const int* sidx = nd->perm.v;
  const int* ridx = nd->perm.v + k;
  double* Kss = dalloc((size_t)k * k);
  double* Ksr = dalloc((size_t)k * r);
  double* Krs = dalloc((size_t)r * k);
  double* Krr = dalloc((size_t)r * r);
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i < k; ++i) Kss[i + (size_t)k * j] = KBN[sidx[i] + (size_t)nb * sidx[j]];
    for (int i = 0; i < r; ++i) Krs[i + (size_t)r * j] = KBN[ridx[i] + (size_t)nb * sidx[j]];
  }
  for (int j = 0; j < r; ++j) {
    for (int i = 0; i < k; ++i) Ksr[i + (size_t)k * j] = KBN[sidx[i] + (size_t)nb * ridx[j]];
    for (int i = 0; i < r; ++i) Krr[i + (size_t)r * j] = KBN[ridx[i] + (size_t)nb * ridx[j]];
  }
  free(KBN);
  const double* T = nd->T; /* k x r */
  /* K_BN_r_sn = Krs - T^T Kss  (r x k) */
  double* Krsn = dalloc((size_t)r * k);
  memcpy(Krsn, Krs, sizeof(double) * (size_t)r * k);
  {
    double* tmp = dalloc((size_t)r * k);
    gemm(1, 0, r, k, k, 1.0, T, k, Kss, k, 0.0, tmp, r);
    for (size_t i = 0; i < (size_t)r * k; ++i) Krsn[i] = Krs[i] - tmp[i];
    free(tmp);
  }
  /* X_rr = Krr - T^T Ksr - Krsn T */
  double* X = dalloc((size_t)r * r);
  {
    double* t1 = dalloc((size_t)r * r);
    double* t2 = dalloc((size_t)r * r);
    gemm(1, 0, r, r, k, 1.0, T, k, Ksr, k, 0.0, t1, r);
    gemm(0, 0, r, r, k, 1.0, Krsn, r, T, k, 0.0, t2, r);
    for (size_t i = 0; i < (size_t)r * r; ++i) X[i] = (Krr[i] - t1[i]) - t2[i];
    free(t1); free(t2);
  }
  /* K_BN_sn_r = Ksr - Kss T  (k x r) */
  double* Ksnr = dalloc((size_t)k * r);
  {
    double* tmp = dalloc((size_t)k * r);
    gemm(0, 0, k, r, k, 1.0, Kss, k, T, k, 0.0, tmp, k);
    for (size_t i = 0; i < (size_t)k * r; ++i) Ksnr[i] = Ksr[i] - tmp[i];
    free(tmp);
  }
  nd->Xrr = X;
  nd->Xlu = dalloc((size_t)r * r);
  memcpy(nd->Xlu, X, sizeof(double) * (size_t)r * r);
  nd->piv = (int*)malloc(sizeof(int) * (size_t)(r ? r : 1));
  getrf(r, nd->Xlu, r, nd->piv);
  /* L = Ksnr X^{-1}: (X^T)^{-1} Ksnr^T then transpose (ie_mat.cpp:506-519) */
  nd->L = dalloc((size_t)k * r);
  {
    double* kt = dalloc((size_t)r * k);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < r; ++j) kt[j + (size_t)r * i] = Ksnr[i + (size_t)k * j];
    getrs_t(r, nd->Xlu, r, nd->piv, kt, r, k);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < r; ++j) nd->L[i + (size_t)k * j] = kt[j + (size_t)r * i];
    free(kt);
  }
  /* U = X^{-1} Krsn */
  nd->U = dalloc((size_t)r * k);
  memcpy(nd->U, Krsn, sizeof(double) * (size_t)r * k);
  getrs_n(r, nd->Xlu, r, nd->piv, nd->U, r, k);
  /* schur_update = L Krsn (k x k) */
  nd->schur = dalloc((size_t)k * k);
  gemm(0, 0, k, k, r, 1.0, nd->L, k, Krsn, r, 0.0, nd->schur, k);
  nd->compressed = 1;
  free(Kss); free(Ksr); free(Krs); free(Krr); free(Krsn); free(Ksnr);
}

/* ------------------------------------------------------------------ */
/* bordered matrices: linear_solve.cpp:20-112                          */
/* ------------------------------------------------------------------ */
static void build_border(orc_solver* s) {
  int h = s->nholes, N = s->n, D = s->n * s->sd;
  if (h == 0 || s->pde == ORC_LAPLACE_NEUMANN) { s->nb = 0; return; }
  s->nb = s->pde == ORC_STOKES ? 3 * h : h;
  int nb = s->nb;
  s->U = dalloc((size_t)D * nb);
  s->Psi = dalloc((size_t)nb * D);
  for (int i = 0; i < N; ++i) {
    double x0 = s->pts[2 * i], x1 = s->pts[2 * i + 1];
    for (int hi = 0; hi < h; ++hi) {
      double r0 = x0 - s->hc[2 * hi], r1 = x1 - s->hc[2 * hi + 1];
      double rn = sqrt(r0 * r0 + r1 * r1);
      if (s->pde == ORC_LAPLACE) {
        s->U[i + (size_t)D * hi] = log(rn);
      } else {
        double scale = 1.0 / (4 * M_PI);
        double* U = s->U;
        U[2 * i + (size_t)D * (3 * hi)] = scale * (log(1 / rn) + (1.0 / pow(rn, 2)) * r0 * r0);
        U[2 * i + 1 + (size_t)D * (3 * hi)] = scale * ((1.0 / pow(rn, 2)) * r1 * r0);
        U[2 * i + (size_t)D * (3 * hi + 1)] = scale * ((1.0 / pow(rn, 2)) * r0 * r1);
        U[2 * i + 1 + (size_t)D * (3 * hi + 1)] = scale * (log(1 / rn) + (1.0 / pow(rn, 2)) * r1 * r1);
        U[2 * i + (size_t)D * (3 * hi + 2)] = r1 * (scale / pow(rn, 2));
        U[2 * i + 1 + (size_t)D * (3 * hi + 2)] = -r0 * (scale / pow(rn, 2));
      }
    }
    for (int hi = 0; hi < h; ++hi) {
      double r0 = x0 - s->hc[2 * hi], r1 = x1 - s->hc[2 * hi + 1];
      if (sqrt(r0 * r0 + r1 * r1) < s->hr[hi] + 1e-8) {
        double wi = s->w[i];
        if (s->pde == ORC_LAPLACE) {
          s->Psi[hi + (size_t)nb * i] = wi;
        } else {
          s->Psi[3 * hi + (size_t)nb * (2 * i)] = wi;
          s->Psi[3 * hi + 1 + (size_t)nb * (2 * i + 1)] = wi;
          s->Psi[3 * hi + 2 + (size_t)nb * (2 * i)] = wi * x1;
          s->Psi[3 * hi + 2 + (size_t)nb * (2 * i + 1)] = -wi * x0;
        }
        break;
      }
    }
  }
}

int orc_border_dims(const orc_solver* s) { return s->nb; }
void orc_border_mats(const orc_solver* s, double* U, double* Psi) {
  size_t D = (size_t)s->n * s->sd;
  if (!s->nb) return;
  if (U) memcpy(U, s->U, sizeof(double) * D * s->nb);
  if (Psi) memcpy(Psi, s->Psi, sizeof(double) * D * s->nb);
}

/* ------------------------------------------------------------------ */
/* sweeps: skel_factorization.cpp:388-426                              */
/* ------------------------------------------------------------------ */
/* vec(b) += mat * vec(a)  (or mat^T * vec(a) when trans) ; vec is D x w */
static void sweep(const double* mat, int rows, int cols, int trans, double sign, double* vec,
                  int ld, int w, const ivec* a, const ivec* b) {
  if (a->n * b->n == 0) return;
  /* mat is rows x cols; trans -> mat^T (cols x rows) applied to a (rows) */
  int out = b->n, in = a->n;
  double* xa = dalloc((size_t)in * w);
  double* prod = dalloc((size_t)out * w);
  for (int c = 0; c < w; ++c)
    for (int i = 0; i < in; ++i) xa[i + (size_t)in * c] = vec[a->v[i] + (size_t)ld * c];
  gemm(trans, 0, out, w, in, sign, mat, rows, xa, in, 0.0, prod, out);
  (void)cols;
  for (int c = 0; c < w; ++c)
    for (int i = 0; i < out; ++i) vec[b->v[i] + (size_t)ld * c] = prod[i + (size_t)out * c] +
                                                                 vec[b->v[i] + (size_t)ld * c];
  free(xa); free(prod);
}

static void diag_inv(const double* lu, const int* piv, int r, double* vec, int ld, int w,
                     const int* idx) {
  double* t = dalloc((size_t)r * w);
  for (int c = 0; c < w; ++c)
    for (int i = 0; i < r; ++i) t[i + (size_t)r * c] = vec[idx[i] + (size_t)ld * c];
  getrs_n(r, lu, r, piv, t, r, w);
  for (int c = 0; c < w; ++c)
    for (int i = 0; i < r; ++i) vec[idx[i] + (size_t)ld * c] = t[i + (size_t)r * c];
  free(t);
}

/* upward sweep on vec with the second operator L (use_u = 0) or U^T (use_u = 1) */
static void upward(const orc_solver* s, double* vec, int ld, int w, int use_u) {
  for (int lv = s->num_levels - 1; lv >= 0; --lv) {
    const ivec* L = &s->levels[lv];
#pragma omp parallel for num_threads(s->nthreads)
    for (int q = 0; q < L->n; ++q) {
      const node_t* nd = &s->nodes[L->v[q]];
      if (!nd->compressed) continue;
      sweep(nd->T, nd->k, nd->r, 1, -1.0, vec, ld, w, &nd->skel, &nd->red);
      if (use_u) sweep(nd->U, nd->r, nd->k, 1, -1.0, vec, ld, w, &nd->red, &nd->skel);
      else sweep(nd->L, nd->k, nd->r, 0, -1.0, vec, ld, w, &nd->red, &nd->skel);
    }
  }
}

static void downward(const orc_solver* s, double* vec, int ld, int w) {
  for (int lv = 0; lv < s->num_levels; ++lv) {
    const ivec* L = &s->levels[lv];
#pragma omp parallel for num_threads(s->nthreads)
    for (int q = L->n - 1; q >= 0; --q) {
      const node_t* nd = &s->nodes[L->v[q]];
      if (!nd->compressed) continue;
      sweep(nd->U, nd->r, nd->k, 0, -1.0, vec, ld, w, &nd->skel, &nd->red);
      sweep(nd->T, nd->k, nd->r, 0, -1.0, vec, ld, w, &nd->red, &nd->skel);
    }
  }
}

/* all compressed nodes in the reference's all_nodes order (deepest level first) */
static void diag_all(const orc_solver* s, double* vec, int ld, int w, const int* map) {
  int total = 0;
  for (int lv = s->num_levels - 1; lv >= 0; --lv) total += s->levels[lv].n;
  int* order = (int*)malloc(sizeof(int) * (size_t)total);
  int t = 0;
  for (int lv = s->num_levels - 1; lv >= 0; --lv)
    for (int q = 0; q < s->levels[lv].n; ++q) order[t++] = s->levels[lv].v[q];
#pragma omp parallel for num_threads(s->nthreads)
  for (int q = 0; q < total; ++q) {
    const node_t* nd = &s->nodes[order[q]];
    if (nd->red.n == 0 || !nd->compressed) continue;
    int* idx = (int*)malloc(sizeof(int) * (size_t)nd->r);
    for (int i = 0; i < nd->r; ++i) idx[i] = map ? map[nd->red.v[i]] : nd->red.v[i];
    diag_inv(nd->Xlu, nd->piv, nd->r, vec, ld, w, idx);
    free(idx);
  }
  free(order);
}

/* ------------------------------------------------------------------ */
/* skeletonize: skel_factorization.cpp:140-310                         */
/* ------------------------------------------------------------------ */
static int* redundant_list(const orc_solver* s, int* nred, int** map_out) {
  int D = s->n * s->sd;
  char* is_skel = (char*)calloc((size_t)D, 1);
  for (int i = 0; i < s->ns; ++i) is_skel[s->allskel[i]] = 1;
  int* red = (int*)malloc(sizeof(int) * (size_t)D);
  int* map = (int*)malloc(sizeof(int) * (size_t)D);
  int c = 0;
  for (int i = 0; i < D; ++i) {
    map[i] = -1;
    if (!is_skel[i]) { map[i] = c; red[c++] = i; }
  }
  free(is_skel);
  *nred = c;
  *map_out = map;
  return red;
}

int orc_factor(orc_solver* s) {
  if (!s->tree_built) {
    int rc = orc_build_tree(s);
    if (rc) return rc;
  }
  double t0 = omp_get_wtime();
  build_border(s);
  for (int lv = s->num_levels - 1; lv > 0; --lv) {
    remove_inactive_dofs_at_level(s, lv);
    const ivec* L = &s->levels[lv];
#pragma omp parallel for num_threads(s->nthreads)
    for (int q = 0; q < L->n; ++q) {
      int ni = L->v[q];
      node_t* nd = &s->nodes[ni];
      if (nd->compressed || nd->active.n < MIN_DOFS_TO_COMPRESS) continue;
      if (id_compress(s, ni) == 0) continue;
      decouple(s, ni);
    }
  }
  for (int lv = s->num_levels - 1; lv >= 0; --lv) remove_inactive_dofs_at_level(s, lv);
  node_t* root = &s->nodes[s->root];
  s->ns = root->active.n;
  s->allskel = (int*)malloc(sizeof(int) * (size_t)(s->ns ? s->ns : 1));
  memcpy(s->allskel, root->active.v, sizeof(int) * (size_t)s->ns);
  int ns = s->ns;
  s->allskel_mat = dalloc((size_t)ns * ns);
  if (ns > 0) {
    orc_kernel_block(s, s->allskel, ns, s->allskel, ns, s->allskel_mat);
    double* upd = dalloc((size_t)ns * ns);
    if (!root->is_leaf) get_descendents_updates(s, upd, &root->active, s->root);
    for (size_t i = 0; i < (size_t)ns * ns; ++i) s->allskel_mat[i] -= upd[i];
    free(upd);
  }
  if (s->nb == 0) {
    s->allskel_lu = dalloc((size_t)ns * ns);
    memcpy(s->allskel_lu, s->allskel_mat, sizeof(double) * (size_t)ns * ns);
    s->allskel_piv = (int*)malloc(sizeof(int) * (size_t)(ns ? ns : 1));
    getrf(ns, s->allskel_lu, ns, s->allskel_piv);
    s->t_factor = omp_get_wtime() - t0;
    s->factored = 1;
    return 0;
  }
  /* bordered system, skel_factorization.cpp:188-305 */
  int D = s->n * s->sd, nb = s->nb;
  int nred;
  int* map;
  int* red = redundant_list(s, &nred, &map);
  if (nred == 0) { free(red); free(map); return 5; } /* "No compression possible" */
  double* mU = dalloc((size_t)D * nb);
  memcpy(mU, s->U, sizeof(double) * (size_t)D * nb);
  double* mP = dalloc((size_t)D * nb); /* Psi^T, D x nb */
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < D; ++j) mP[j + (size_t)D * i] = s->Psi[i + (size_t)nb * j];
  upward(s, mU, D, nb, 0);
  upward(s, mP, D, nb, 1);
  double* DC = dalloc((size_t)nred * nb);
  for (int c = 0; c < nb; ++c)
    for (int i = 0; i < nred; ++i) DC[i + (size_t)nred * c] = mU[red[i] + (size_t)D * c];
  diag_all(s, DC, nred, nb, map);
  int SN = ns + nb;
  double* S = dalloc((size_t)SN * SN);
  for (int j = 0; j < ns; ++j)
    for (int i = 0; i < ns; ++i) S[i + (size_t)SN * j] = s->allskel_mat[i + (size_t)ns * j];
  for (int j = 0; j < ns; ++j)
    for (int i = 0; i < nb; ++i) S[ns + i + (size_t)SN * j] = mP[s->allskel[j] + (size_t)D * i];
  for (int j = 0; j < nb; ++j)
    for (int i = 0; i < ns; ++i) S[i + (size_t)SN * (ns + j)] = mU[s->allskel[i] + (size_t)D * j];
  double* pr = dalloc((size_t)nb * nb); /* Psi(:, red) * DC */
  for (int j = 0; j < nb; ++j)
    for (int l = 0; l < nred; ++l) {
      double b = DC[l + (size_t)nred * j];
      if (b == 0.0) continue;
      for (int i = 0; i < nb; ++i) pr[i + (size_t)nb * j] += mP[red[l] + (size_t)D * i] * b;
    }
  for (int j = 0; j < nb; ++j)
    for (int i = 0; i < nb; ++i)
      S[ns + i + (size_t)SN * (ns + j)] = (i == j ? -1.0 : -0.0) - pr[i + (size_t)nb * j];
  s->S_lu = S;
  s->S_piv = (int*)malloc(sizeof(int) * (size_t)SN);
  getrf(SN, S, SN, s->S_piv);
  free(pr); free(DC); free(mU); free(mP); free(red); free(map);
  s->t_factor = omp_get_wtime() - t0;
  s->factored = 1;
  return 0;
}

/* ------------------------------------------------------------------ */
/* solves                                                              */
/* ------------------------------------------------------------------ */
int orc_solve(orc_solver* s, const double* f, int nrhs, double* mu, double* alpha) {
  if (!s->factored) return 1;
  double t0 = omp_get_wtime();
  int D = s->n * s->sd, ns = s->ns;
  if (s->nb == 0) {
    memcpy(mu, f, sizeof(double) * (size_t)D * nrhs);
    upward(s, mu, D, nrhs, 0);
    diag_all(s, mu, D, nrhs, NULL);
    if (ns > 0) diag_inv(s->allskel_lu, s->allskel_piv, ns, mu, D, nrhs, s->allskel);
    downward(s, mu, D, nrhs);
    s->t_solve = omp_get_wtime() - t0;
    return 0;
  }
  if (nrhs != 1) return 2; /* skel_factorization.cpp:669-670: single RHS */
  int nb = s->nb, nred, *map;
  int* red = redundant_list(s, &nred, &map);
  memcpy(mu, f, sizeof(double) * (size_t)D);
  double* mU = dalloc((size_t)D * nb);
  memcpy(mU, s->U, sizeof(double) * (size_t)D * nb);
  upward(s, mu, D, 1, 0);
  upward(s, mU, D, nb, 0);
  double* w = dalloc(nred);
  double* z = dalloc(ns);
  for (int i = 0; i < nred; ++i) w[i] = mu[red[i]];
  for (int i = 0; i < ns; ++i) z[i] = mu[s->allskel[i]];
  double* mP = dalloc((size_t)D * nb);
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < D; ++j) mP[j + (size_t)D * i] = s->Psi[i + (size_t)nb * j];
  upward(s, mP, D, nb, 1);
  double* Dw = dalloc(nred);
  memcpy(Dw, w, sizeof(double) * (size_t)nred);
  diag_all(s, Dw, nred, 1, map);
  int SN = ns + nb;
  double* M = dalloc(SN);
  for (int i = 0; i < ns; ++i) M[i] = z[i];
  for (int i = 0; i < nb; ++i) {
    double v = 0.0;
    for (int l = 0; l < nred; ++l) v += mP[red[l] + (size_t)D * i] * Dw[l];
    M[ns + i] = -v;
  }
  getrs_n(SN, s->S_lu, SN, s->S_piv, M, SN, 1);
  for (int i = 0; i < nb; ++i) alpha[i] = M[ns + i];
  double* Nv = dalloc(nred);
  for (int l = 0; l < nred; ++l) {
    double v = 0.0;
    for (int j = 0; j < nb; ++j) v += mU[red[l] + (size_t)D * j] * alpha[j];
    Nv[l] = w[l] - v;
  }
  diag_all(s, Nv, nred, 1, map);
  for (int l = 0; l < nred; ++l) mu[red[l]] = Nv[l];
  for (int i = 0; i < ns; ++i) mu[s->allskel[i]] = M[i];
  downward(s, mu, D, 1);
  free(red); free(map); free(mU); free(w); free(z); free(mP); free(Dw); free(M); free(Nv);
  s->t_solve = omp_get_wtime() - t0;
  return 0;
}

void orc_matvec(const orc_solver* s, const double* x, int nrhs, double* y) {
  int D = s->n * s->sd;
#pragma omp parallel for schedule(static) num_threads(s->nthreads)
  for (int i = 0; i < D; ++i) {
    for (int c = 0; c < nrhs; ++c) {
      double acc = 0.0;
      for (int j = 0; j < D; ++j) acc += kentry(s, i, j) * x[j + (size_t)D * c];
      y[i + (size_t)D * c] = acc;
    }
  }
}

/* ------------------------------------------------------------------ */
/* lifecycle / introspection                                           */
/* ------------------------------------------------------------------ */
static double* dup(const double* x, size_t n) {
  double* p = dalloc(n);
  if (n) memcpy(p, x, sizeof(double) * n);
  return p;
}

orc_solver* orc_create(int pde, int sd, int n, const double* points, const double* normals,
                       const double* weights, const double* curvatures, int num_holes,
                       const double* hole_centers, const double* hole_radii, double id_tol,
                       int max_leaf_dofs, int num_proxy_points, int num_threads) {
  orc_solver* s = (orc_solver*)calloc(1, sizeof(orc_solver));
  s->pde = pde; s->sd = sd; s->n = n; s->nholes = num_holes;
  s->tol = id_tol; s->leaf = max_leaf_dofs; s->npp = num_proxy_points;
  s->nthreads = num_threads > 0 ? num_threads : 1;
  s->pts = dup(points, 2 * (size_t)n);
  s->nrm = dup(normals, 2 * (size_t)n);
  s->w = dup(weights, n);
  s->curv = dup(curvatures, n);
  s->hc = dup(hole_centers, 2 * (size_t)num_holes);
  s->hr = dup(hole_radii, num_holes);
  s->root = -1;
  return s;
}

void orc_destroy(orc_solver* s) {
  if (!s) return;
  for (int i = 0; i < s->num_nodes; ++i) {
    node_t* nd = &s->nodes[i];
    iv_free(&nd->nbr); iv_free(&nd->orig); iv_free(&nd->active); iv_free(&nd->skel);
    iv_free(&nd->red); iv_free(&nd->near); iv_free(&nd->perm);
    free(nd->T); free(nd->L); free(nd->U); free(nd->Xrr); free(nd->Xlu); free(nd->schur);
    free(nd->piv);
  }
  for (int l = 0; l < s->num_levels; ++l) iv_free(&s->levels[l]);
  free(s->levels); free(s->nodes);
  free(s->pts); free(s->nrm); free(s->w); free(s->curv); free(s->hc); free(s->hr);
  free(s->allskel); free(s->allskel_mat); free(s->allskel_lu); free(s->allskel_piv);
  free(s->U); free(s->Psi); free(s->S_lu); free(s->S_piv);
  free(s);
}

int orc_num_levels(const orc_solver* s) { return s->num_levels; }
int orc_num_nodes(const orc_solver* s) { return s->num_nodes; }

static int level_order_node(const orc_solver* s, int idx) {
  for (int l = 0; l < s->num_levels; ++l) {
    if (idx < s->levels[l].n) return s->levels[l].v[idx];
    idx -= s->levels[l].n;
  }
  return -1;
}

static int* level_order_rank(const orc_solver* s) {
  int* rk = (int*)malloc(sizeof(int) * (size_t)(s->num_nodes ? s->num_nodes : 1));
  int c = 0;
  for (int l = 0; l < s->num_levels; ++l)
    for (int q = 0; q < s->levels[l].n; ++q) rk[s->levels[l].v[q]] = c++;
  return rk;
}

void orc_node_info(const orc_solver* s, int node, int* info, double* corners8, double* side) {
  int ni = level_order_node(s, node);
  const node_t* nd = &s->nodes[ni];
  int* rk = level_order_rank(s);
  info[0] = nd->level;
  info[1] = nd->is_leaf;
  info[2] = nd->parent >= 0 ? rk[nd->parent] : -1;
  for (int c = 0; c < 4; ++c) info[3 + c] = nd->children[c] >= 0 ? rk[nd->children[c]] : -1;
  info[7] = nd->compressed;
  info[8] = nd->skel.n;
  info[9] = nd->red.n;
  if (corners8) memcpy(corners8, nd->corners, sizeof(double) * 8);
  if (side) *side = nd->side;
  free(rk);
}

int orc_node_list(const orc_solver* s, int node, int which, int* out, int cap) {
  int ni = level_order_node(s, node);
  const node_t* nd = &s->nodes[ni];
  const ivec* src = NULL;
  switch (which) {
    case 0: src = &nd->orig; break;
    case 1: src = &nd->active; break;
    case 2: src = &nd->skel; break;
    case 3: src = &nd->red; break;
    case 4: src = &nd->near; break;
    case 5: src = &nd->nbr; break;
    case 6: src = &nd->perm; break;
    default: return -1;
  }
  if (which == 5) {
    int* rk = level_order_rank(s);
    for (int i = 0; i < src->n && i < cap; ++i) out[i] = rk[src->v[i]];
    free(rk);
  } else {
    for (int i = 0; i < src->n && i < cap; ++i) out[i] = src->v[i];
  }
  return src->n;
}

int orc_allskel(const orc_solver* s, int* out, int cap) {
  for (int i = 0; i < s->ns && i < cap; ++i) out[i] = s->allskel[i];
  return s->ns;
}

double orc_tree_min(const orc_solver* s) { return s->tmin; }
double orc_tree_max(const orc_solver* s) { return s->tmax; }

int orc_node_factors(const orc_solver* s, int node, double* T, double* L, double* U,
                     double* Xrr, double* schur) {
  int ni = level_order_node(s, node);
  const node_t* nd = &s->nodes[ni];
  if (!nd->compressed) return 1;
  size_t kr = (size_t)nd->k * nd->r;
  if (T) memcpy(T, nd->T, sizeof(double) * kr);
  if (L) memcpy(L, nd->L, sizeof(double) * kr);
  if (U) memcpy(U, nd->U, sizeof(double) * kr);
  if (Xrr) memcpy(Xrr, nd->Xrr, sizeof(double) * (size_t)nd->r * nd->r);
  if (schur) memcpy(schur, nd->schur, sizeof(double) * (size_t)nd->k * nd->k);
  return 0;
}

double orc_last_factor_seconds(const orc_solver* s) { return s->t_factor; }
double orc_last_solve_seconds(const orc_solver* s) { return s->t_solve; }
