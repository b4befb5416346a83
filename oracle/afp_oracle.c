/* CPU oracle for the AFEPack elliptic-solve path -- TEST INFRASTRUCTURE.
 * See afp_oracle.h.  Each function names the reference code it restates;
 * loops and floating-point operation order follow the reference so that
 * results agree with AFEPack compiled from source, bit for bit wherever no
 * BLAS/LAPACK call is involved. */
#include "afp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../afepack_gb300/csrc/quadrature_tables.h"

#define INVALID (-1)

void orc_csr_free(orc_csr *a) {
  if (!a) return;
  free(a->rowptr);
  free(a->cols);
  free(a->vals);
  memset(a, 0, sizeof(*a));
}

/* ------------------------------------------------------------------------ */
/* Template-element math, restated from the plugin sources:                  */
/*   template/triangle/triangle.crd_trs.c, triangle.volume.c,               */
/*   triangle.1/triangle.1.bas_fun.c, triangle.2/triangle.2.bas_fun.c,       */
/*   template/tetrahedron/tetrahedron.crd_trs.c, tetrahedron.volume.c,       */
/*   tetrahedron.1/tetrahedron.1.bas_fun.c, tetrahedron.2/tetrahedron.2.bas_fun.c */
/* ------------------------------------------------------------------------ */
static double area2(const double *a, const double *b, const double *c) {
  return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
}

static double det6(const double *v0, const double *v1, const double *v2, const double *v3) {
  return ((v1[0] - v0[0]) * (v2[1] - v0[1]) * (v3[2] - v0[2]) +
          (v1[1] - v0[1]) * (v2[2] - v0[2]) * (v3[0] - v0[0]) +
          (v1[2] - v0[2]) * (v2[0] - v0[0]) * (v3[1] - v0[1]) -
          (v1[0] - v0[0]) * (v2[2] - v0[2]) * (v3[1] - v0[1]) -
          (v1[1] - v0[1]) * (v2[0] - v0[0]) * (v3[2] - v0[2]) -
          (v1[2] - v0[2]) * (v2[1] - v0[1]) * (v3[0] - v0[0]));
}

static double co_det(const double v[4][3], int m, int n) {
  double s = (m % 2 == 0) ? -1. : 1.;
  return s * ((v[(m + 2) % 4][(n + 1) % 3] - v[(m + 1) % 4][(n + 1) % 3]) *
                  (v[(m + 3) % 4][(n + 2) % 3] - v[(m + 1) % 4][(n + 2) % 3]) -
              (v[(m + 2) % 4][(n + 2) % 3] - v[(m + 1) % 4][(n + 2) % 3]) *
                  (v[(m + 3) % 4][(n + 1) % 3] - v[(m + 1) % 4][(n + 1) % 3]));
}

static const double TRI_REF[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
static const double TET_REF[4][3] = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};

/* local_to_global / local_to_global_jacobian (crd_trs plugins) */
static void tri_l2g(const double *lp, const double gv[3][2], double *gp, double *jac) {
  double area = area2(TRI_REF[0], TRI_REF[1], TRI_REF[2]);
  double l0 = area2(lp, TRI_REF[1], TRI_REF[2]) / area;
  double l1 = area2(lp, TRI_REF[2], TRI_REF[0]) / area;
  double l2 = area2(lp, TRI_REF[0], TRI_REF[1]) / area;
  gp[0] = l0 * gv[0][0] + l1 * gv[1][0] + l2 * gv[2][0];
  gp[1] = l0 * gv[0][1] + l1 * gv[1][1] + l2 * gv[2][1];
  *jac = area2(gv[0], gv[1], gv[2]) / area;
}

static void tet_l2g(const double *lp, const double gv[4][3], double *gp, double *jac) {
  double vol = det6(TET_REF[0], TET_REF[1], TET_REF[2], TET_REF[3]) / 6.;
  double l0 = det6(lp, TET_REF[1], TET_REF[2], TET_REF[3]) / 6. / vol;
  double l1 = det6(TET_REF[0], lp, TET_REF[2], TET_REF[3]) / 6. / vol;
  double l2 = det6(TET_REF[0], TET_REF[1], lp, TET_REF[3]) / 6. / vol;
  double l3 = det6(TET_REF[0], TET_REF[1], TET_REF[2], lp) / 6. / vol;
  for (int d = 0; d < 3; ++d) gp[d] = l0 * gv[0][d] + l1 * gv[1][d] + l2 * gv[2][d] + l3 * gv[3][d];
  *jac = (det6(gv[0], gv[1], gv[2], gv[3]) / 6.) / vol;
}

/* basis values (nd) and gradients (nd x dim) at a global point p */
static void tri_basis(int degree, const double v[3][2], const double *p, double *val, double grad[][3]) {
  double area = area2(v[0], v[1], v[2]);
  if (degree == 1) {
    val[0] = area2(p, v[1], v[2]) / area;
    val[1] = area2(v[0], p, v[2]) / area;
    val[2] = area2(v[0], v[1], p) / area;
    grad[0][0] = (v[1][1] - v[2][1]) / area; grad[0][1] = (v[2][0] - v[1][0]) / area;
    grad[1][0] = (v[2][1] - v[0][1]) / area; grad[1][1] = (v[0][0] - v[2][0]) / area;
    grad[2][0] = (v[0][1] - v[1][1]) / area; grad[2][1] = (v[1][0] - v[0][0]) / area;
    return;
  }
  double l[3] = {area2(p, v[1], v[2]) / area, area2(p, v[2], v[0]) / area, area2(p, v[0], v[1]) / area};
  double dx[3] = {(v[1][1] - v[2][1]) / area, (v[2][1] - v[0][1]) / area, (v[0][1] - v[1][1]) / area};
  double dy[3] = {(v[2][0] - v[1][0]) / area, (v[0][0] - v[2][0]) / area, (v[1][0] - v[0][0]) / area};
  for (int k = 0; k < 3; ++k) {
    val[k] = l[k] * (2 * l[k] - 1.0);
    grad[k][0] = (4.0 * l[k] - 1.0) * dx[k];
    grad[k][1] = (4.0 * l[k] - 1.0) * dy[k];
  }
  /* edge j is opposite vertex j: psi = 4 l_a l_b on edge (a,b) */
  val[3] = 4.0 * l[1] * l[2];
  val[4] = 4.0 * l[0] * l[2];
  val[5] = 4.0 * l[0] * l[1];
  grad[3][0] = 4.0 * (l[2] * dx[1] + l[1] * dx[2]); grad[3][1] = 4.0 * (l[2] * dy[1] + l[1] * dy[2]);
  grad[4][0] = 4.0 * (l[0] * dx[2] + l[2] * dx[0]); grad[4][1] = 4.0 * (l[0] * dy[2] + l[2] * dy[0]);
  grad[5][0] = 4.0 * (l[1] * dx[0] + l[0] * dx[1]); grad[5][1] = 4.0 * (l[1] * dy[0] + l[0] * dy[1]);
}

static void tet_basis(int degree, const double v[4][3], const double *p, double *val, double grad[][3]) {
  double vol = det6(v[0], v[1], v[2], v[3]);
  double l[4] = {det6(p, v[1], v[2], v[3]) / vol, det6(v[0], p, v[2], v[3]) / vol,
                 det6(v[0], v[1], p, v[3]) / vol, det6(v[0], v[1], v[2], p) / vol};
  if (degree == 1) {
    for (int m = 0; m < 4; ++m) {
      val[m] = l[m];
      for (int n = 0; n < 3; ++n) grad[m][n] = co_det(v, m, n) / vol;
    }
    return;
  }
  for (int m = 0; m < 4; ++m) {
    val[m] = l[m] * (2 * l[m] - 1);
    for (int n = 0; n < 3; ++n) grad[m][n] = co_det(v, m, n) / vol * (4. * l[m] - 1.);
  }
  /* template edges 0:(0,1) 1:(0,2) 2:(0,3) 3:(2,3) 4:(1,3) 5:(1,2); the .bas_fun
   * file attaches psi_1..psi_6 to edges 0,1,2,5,4,3.  Each gradient keeps the
   * plugin's operand order: 4*(co(a)/vol*l[b] + co(b)/vol*l[a]) with the
   * (first, second) pair below. */
  static const int first[6] = {1, 2, 3, 2, 1, 1};
  static const int second[6] = {0, 0, 0, 3, 3, 2};
  static const int la[6] = {0, 0, 0, 3, 3, 2};
  static const int lb[6] = {1, 2, 3, 2, 1, 1};
  /* psi values: 4*l_a*l_b with the plugin's factor order */
  val[4] = 4.0 * l[0] * l[1];
  val[5] = 4.0 * l[0] * l[2];
  val[6] = 4.0 * l[0] * l[3];
  val[7] = 4.0 * l[2] * l[3];
  val[8] = 4.0 * l[1] * l[3];
  val[9] = 4.0 * l[1] * l[2];
  for (int e = 0; e < 6; ++e)
    for (int n = 0; n < 3; ++n)
      grad[4 + e][n] = 4 * (co_det(v, first[e], n) / vol * l[la[e]] + co_det(v, second[e], n) / vol * l[lb[e]]);
}

static int quad_rule(int dim, int acc, const double **pts, int *npts) {
  if (dim == 2) {
    if (acc < 0 || acc > AFP_TRI_QUAD_MAX_ACC) return -1;
    int r = AFP_TRI_QUAD_RULE_OF_ACC[acc];
    *pts = AFP_TRI_QUAD_POINTS[AFP_TRI_QUAD_OFFSET[r]];
    *npts = AFP_TRI_QUAD_OFFSET[r + 1] - AFP_TRI_QUAD_OFFSET[r];
  } else {
    if (acc < 0 || acc > AFP_TET_QUAD_MAX_ACC) return -1;
    int r = AFP_TET_QUAD_RULE_OF_ACC[acc];
    *pts = AFP_TET_QUAD_POINTS[AFP_TET_QUAD_OFFSET[r]];
    *npts = AFP_TET_QUAD_OFFSET[r + 1] - AFP_TET_QUAD_OFFSET[r];
  }
  return 0;
}

/* StiffMatrix / MassMatrix ::getElementMatrix (BilinearOperator.templates.h:343-406) */
static int element_matrix(int dim, int degree, const double *vx, int acc, int mass, double *K) {
  const int nd = dim == 2 ? 3 * degree : (degree == 1 ? 4 : 10);
  const double *pts;
  int nq;
  if (quad_rule(dim, acc, &pts, &nq)) return -1;
  const int stride = dim + 1;
  double tv[4][3] = {{0}};
  for (int a = 0; a <= dim; ++a)
    for (int d = 0; d < dim; ++d) tv[a][d] = vx[a * dim + d];
  double tmpl_volume = dim == 2 ? .5 * area2(TRI_REF[0], TRI_REF[1], TRI_REF[2])
                                : det6(TET_REF[0], TET_REF[1], TET_REF[2], TET_REF[3]) / 6.;
  memset(K, 0, sizeof(double) * nd * nd);
  for (int l = 0; l < nq; ++l) {
    const double *lp = pts + l * stride;
    double gp[3], jac, val[10], grad[10][3];
    if (dim == 2) {
      double gv[3][2] = {{tv[0][0], tv[0][1]}, {tv[1][0], tv[1][1]}, {tv[2][0], tv[2][1]}};
      tri_l2g(lp, gv, gp, &jac);
      tri_basis(degree, gv, gp, val, grad);
    } else {
      tet_l2g(lp, (const double(*)[3])tv, gp, &jac);
      tet_basis(degree, (const double(*)[3])tv, gp, val, grad);
    }
    double Jxw = lp[dim] * jac * tmpl_volume;
    for (int j = 0; j < nd; ++j)
      for (int k = 0; k < nd; ++k) {
        if (mass) {
          K[j * nd + k] += Jxw * val[j] * val[k];
        } else {
          double ip = 0;
          for (int d = 0; d < dim; ++d) ip += grad[j][d] * grad[k][d];
          K[j * nd + k] += Jxw * ip;
        }
      }
  }
  return 0;
}

static int cmp_i64(const void *a, const void *b) {
  int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

/* SparsityPattern::add -- first free slot of the row, or nothing if present */
static void pattern_add(int64_t *slots, int64_t start, int64_t end, int64_t j) {
  for (int64_t k = start; k < end; ++k) {
    if (slots[k] == j) return;
    if (slots[k] == INVALID) { slots[k] = j; return; }
  }
}

/* SparsityPattern::compress: keep each row's valid slots, sort all but the
 * first when the pattern is square, and pack. */
static void pattern_compress(int64_t m, int square, const int64_t *slot_start, int64_t *slots, orc_csr *out) {
  out->rowptr = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
  int64_t nnz = 0;
  for (int64_t i = 0; i < m; ++i) {
    int64_t k = slot_start[i];
    while (k < slot_start[i + 1] && slots[k] != INVALID) ++k;
    nnz += k - slot_start[i];
  }
  out->cols = (int64_t *)malloc(sizeof(int64_t) * (nnz ? nnz : 1));
  out->vals = (double *)calloc(nnz ? nnz : 1, sizeof(double));
  int64_t pos = 0;
  for (int64_t i = 0; i < m; ++i) {
    out->rowptr[i] = pos;
    int64_t k = slot_start[i];
    while (k < slot_start[i + 1] && slots[k] != INVALID) out->cols[pos++] = slots[k++];
    int64_t first = out->rowptr[i] + (square ? 1 : 0);
    if (pos > first) qsort(out->cols + first, pos - first, sizeof(int64_t), cmp_i64);
  }
  out->rowptr[m] = pos;
}

/* position of column j in row i, -1 when absent.  Rows are [diagonal,
 * ascending others] (square) or ascending (rectangular), so checking the
 * first entry and binary-searching the rest finds what the reference's
 * linear scans (SparseMatrix::add / el) find. */
static int64_t row_find(const orc_csr *a, int64_t i, int64_t j) {
  int64_t b = a->rowptr[i], e = a->rowptr[i + 1];
  if (b == e) return -1;
  if (a->cols[b] == j) return b;
  int64_t lo = b + 1, hi = e;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (a->cols[mid] < j) lo = mid + 1; else hi = mid;
  }
  return (lo < e && a->cols[lo] == j) ? lo : -1;
}

/* SparseMatrix::add: adds v to entry (i, j) when it is in the pattern */
static void matrix_add(orc_csr *a, int64_t i, int64_t j, double v) {
  int64_t k = row_find(a, i, j);
  if (k >= 0) a->vals[k] += v;
}

/* SparseMatrix::el -- 0 when (i,j) is not in the pattern */
static double matrix_el(const orc_csr *a, int64_t i, int64_t j) {
  /* rows are [diagonal, ascending others] (square) or ascending (rectangular):
   * a binary search over the sorted part finds the entry the reference's
   * linear scan finds */
  int64_t b = a->rowptr[i], e = a->rowptr[i + 1];
  if (b == e) return 0;
  if (a->cols[b] == j) return a->vals[b];
  int64_t lo = b + 1, hi = e;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (a->cols[mid] < j) lo = mid + 1; else hi = mid;
  }
  return (lo < e && a->cols[lo] == j) ? a->vals[lo] : 0;
}

int orc_assemble(int dim, int degree, const double *coords, int64_t n_cell, const int64_t *cells,
                 const int32_t *elem_dof, int64_t n_dof, int acc_stiff, int acc_mass,
                 const double *coef, orc_csr *stiff, double *mass_vals) {
  if ((dim != 2 && dim != 3) || (degree != 1 && degree != 2)) return -1;
  const int nv = dim + 1;
  const int nd = dim == 2 ? 3 * degree : (degree == 1 ? 4 : 10);
  /* buildDofInfo (BilinearOperator.templates.h:116-172) */
  int64_t *ncpl = (int64_t *)calloc(n_dof, sizeof(int64_t));
  for (int64_t e = 0; e < n_cell; ++e)
    for (int j = 0; j < nd; ++j) ncpl[elem_dof[e * nd + j]] += nd;
  int64_t maxc = 0;
  for (int64_t i = 0; i < n_dof; ++i) maxc = ncpl[i] > maxc ? ncpl[i] : maxc;
  if (maxc > n_dof) maxc = n_dof;
  free(ncpl);
  /* SparsityPattern::reinit(n, n, maxc) with the diagonal in slot 0 */
  int64_t *slot_start = (int64_t *)malloc(sizeof(int64_t) * (n_dof + 1));
  int64_t *slots = (int64_t *)malloc(sizeof(int64_t) * n_dof * maxc);
  for (int64_t i = 0; i <= n_dof; ++i) slot_start[i] = i * maxc;
  for (int64_t k = 0; k < n_dof * maxc; ++k) slots[k] = INVALID;
  for (int64_t i = 0; i < n_dof; ++i) slots[i * maxc] = i;
  /* addElementPattern in element order, then compress */
  for (int64_t e = 0; e < n_cell; ++e)
    for (int j = 0; j < nd; ++j)
      for (int k = 0; k < nd; ++k) {
        int64_t r = elem_dof[e * nd + j];
        pattern_add(slots, slot_start[r], slot_start[r + 1], elem_dof[e * nd + k]);
      }
  stiff->m = stiff->n = n_dof;
  pattern_compress(n_dof, 1, slot_start, slots, stiff);
  free(slots);
  free(slot_start);
  /* buildSparseMatrix: element matrices scattered in element order */
  orc_csr mass = *stiff;
  int64_t nnz = stiff->rowptr[n_dof];
  if (mass_vals) {
    mass.vals = mass_vals;
    memset(mass_vals, 0, sizeof(double) * nnz);
  }
  double vx[12], K[100];
  for (int64_t e = 0; e < n_cell; ++e) {
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < dim; ++d) vx[a * dim + d] = coords[cells[e * nv + a] * dim + d];
    if (element_matrix(dim, degree, vx, acc_stiff, 0, K)) return -2;
    if (coef)
      for (int q = 0; q < nd * nd; ++q) K[q] *= coef[e];
    for (int j = 0; j < nd; ++j)
      for (int k = 0; k < nd; ++k) matrix_add(stiff, elem_dof[e * nd + j], elem_dof[e * nd + k], K[j * nd + k]);
    if (mass_vals) {
      if (element_matrix(dim, degree, vx, acc_mass, 1, K)) return -2;
      for (int j = 0; j < nd; ++j)
        for (int k = 0; k < nd; ++k) matrix_add(&mass, elem_dof[e * nd + j], elem_dof[e * nd + k], K[j * nd + k]);
    }
  }
  return 0;
}

/* the global point, Jxw and basis values of quadrature point l of cell vx */
static void quad_point(int dim, int degree, const double *vx, const double *lp, double *gp, double *Jxw,
                       double *val) {
  double tv[4][3] = {{0}}, jac, grad[10][3];
  for (int a = 0; a <= dim; ++a)
    for (int d = 0; d < dim; ++d) tv[a][d] = vx[a * dim + d];
  double tmpl_volume = dim == 2 ? .5 * area2(TRI_REF[0], TRI_REF[1], TRI_REF[2])
                                : det6(TET_REF[0], TET_REF[1], TET_REF[2], TET_REF[3]) / 6.;
  if (dim == 2) {
    double gv[3][2] = {{tv[0][0], tv[0][1]}, {tv[1][0], tv[1][1]}, {tv[2][0], tv[2][1]}};
    tri_l2g(lp, gv, gp, &jac);
    tri_basis(degree, gv, gp, val, grad);
  } else {
    tet_l2g(lp, (const double(*)[3])tv, gp, &jac);
    tet_basis(degree, (const double(*)[3])tv, gp, val, grad);
  }
  *Jxw = lp[dim] * jac * tmpl_volume;
}

int orc_quadrature_points(int dim, const double *coords, int64_t n_cell, const int64_t *cells, int acc,
                          double *points) {
  const double *pts;
  int nq;
  if ((dim != 2 && dim != 3) || quad_rule(dim, acc, &pts, &nq)) return -1;
  const int nv = dim + 1;
  double vx[12], gp[3], Jxw, val[10];
  for (int64_t e = 0; points && e < n_cell; ++e) {
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < dim; ++d) vx[a * dim + d] = coords[cells[e * nv + a] * dim + d];
    for (int l = 0; l < nq; ++l) {
      quad_point(dim, 1, vx, pts + l * nv, gp, &Jxw, val);
      for (int d = 0; d < dim; ++d) points[(e * nq + l) * dim + d] = gp[d];
    }
  }
  return nq;
}

/* Operator::L2Discretize (Operator.discretize.templates.h): of a point
 * function given by its values fq [n_cell*nq] at the quadrature points
 * (lines 151-183), or of a FEM function u [n_dof] on the same space
 * (lines 18-47, FEMFunction::value of FEMSpace.templates.h:1087-1100) */
int orc_l2_discretize(int dim, int degree, const double *coords, int64_t n_cell, const int64_t *cells,
                      const int32_t *elem_dof, int64_t n_dof, int acc, const double *fq, const double *u,
                      double *f1) {
  const double *pts;
  int nq;
  if ((dim != 2 && dim != 3) || (degree != 1 && degree != 2) || quad_rule(dim, acc, &pts, &nq)) return -1;
  if ((fq == NULL) == (u == NULL)) return -1;
  const int nv = dim + 1, nd = dim == 2 ? 3 * degree : (degree == 1 ? 4 : 10);
  memset(f1, 0, sizeof(double) * n_dof);
  double vx[12], gp[3], Jxw, val[10];
  for (int64_t e = 0; e < n_cell; ++e) {
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < dim; ++d) vx[a * dim + d] = coords[cells[e * nv + a] * dim + d];
    const int32_t *dof = elem_dof + e * nd;
    for (int l = 0; l < nq; ++l) {
      quad_point(dim, degree, vx, pts + l * nv, gp, &Jxw, val);
      double f = 0;
      if (fq) f = fq[e * nq + l];
      else
        for (int j = 0; j < nd; ++j) f += u[dof[j]] * val[j];
      for (int j = 0; j < nd; ++j) f1[dof[j]] += Jxw * f * val[j];
    }
  }
  return 0;
}

void orc_vmult(const orc_csr *a, const double *src, double *dst) {
  for (int64_t i = 0; i < a->m; ++i) {
    dst[i] = 0;
    for (int64_t k = a->rowptr[i]; k < a->rowptr[i + 1]; ++k) dst[i] += a->vals[k] * src[a->cols[k]];
  }
}

/* SparseMatrix::Tvmult (SparseMatrix.h:116-132) */
static void orc_tvmult(const orc_csr *a, const double *src, double *dst) {
  for (int64_t j = 0; j < a->n; ++j) dst[j] = 0;
  for (int64_t i = 0; i < a->m; ++i)
    for (int64_t k = a->rowptr[i]; k < a->rowptr[i + 1]; ++k) dst[a->cols[k]] += a->vals[k] * src[i];
}

void orc_apply_dirichlet(orc_csr *a, double *f, const int32_t *dirichlet, const double *g) {
  const int64_t *rs = a->rowptr, *cn = a->cols;
  for (int64_t i = 0; i < a->m; ++i) {
    if (!dirichlet[i]) continue;
    f[i] = a->vals[rs[i]] * (g ? g[i] : 0.0);
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) a->vals[j] = 0.0;
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) {
      int64_t k = cn[j];
      for (int64_t l = rs[k] + 1; l < rs[k + 1]; ++l) {
        if (cn[l] == i) {
          f[k] -= a->vals[l] * f[i] / a->vals[rs[i]];
          a->vals[l] = 0.;
          break;
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* AMG (src/AMGSolver.cpp)                                                  */
/* ------------------------------------------------------------------------ */

/* getPMPt (src/AMGSolver.cpp:288-358).  Rows are independent: each row's
 * column set is the reference's (diagonal first, then ascending after
 * SparsityPattern::compress) and each entry is accumulated serially in the
 * reference's (j, k, l) order, so running rows on several threads (OpenMP)
 * changes nothing in the result. */
static int rap_with_pt(const orc_csr *P, const orc_csr *M, const orc_csr *Pt, orc_csr *A) {
  const int64_t nc = P->m, nf = M->m;
  A->m = A->n = nc;
  A->rowptr = (int64_t *)calloc(nc + 1, sizeof(int64_t));
  /* pass 1: row lengths.  Only the column SET of a row is needed here, so it
   * is formed from the pattern of B = M Pt (row a of B = the union of the Pt
   * rows of a's neighbours), built once: row i of the product is the union of
   * the B rows of P row i's columns. */
  int64_t *brp = (int64_t *)calloc(nf + 1, sizeof(int64_t));
  int64_t *bci = NULL;
  for (int pass = 0; pass < 2; ++pass) {
#pragma omp parallel
    {
      char *flag = (char *)calloc(nc ? nc : 1, 1);
      int64_t *index = (int64_t *)malloc(sizeof(int64_t) * (nc ? nc : 1));
#pragma omp for schedule(dynamic, 256)
      for (int64_t a = 0; a < nf; ++a) {
        int64_t len = 0;
        for (int64_t k = M->rowptr[a]; k < M->rowptr[a + 1]; ++k) {
          int64_t b = M->cols[k];
          for (int64_t l = Pt->rowptr[b]; l < Pt->rowptr[b + 1]; ++l) {
            int64_t c = Pt->cols[l];
            if (!flag[c]) { index[len++] = c; flag[c] = 1; }
          }
        }
        for (int64_t q = 0; q < len; ++q) {
          flag[index[q]] = 0;
          if (pass == 1) bci[brp[a] + q] = index[q];
        }
        if (pass == 0) brp[a + 1] = len;
      }
      free(flag);
      free(index);
    }
    if (pass == 0) {
      for (int64_t a = 0; a < nf; ++a) brp[a + 1] += brp[a];
      bci = (int64_t *)malloc(sizeof(int64_t) * (brp[nf] ? brp[nf] : 1));
    }
  }
#pragma omp parallel
  {
    char *flag = (char *)calloc(nc ? nc : 1, 1);
    int64_t *index = (int64_t *)malloc(sizeof(int64_t) * (nc ? nc : 1));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < nc; ++i) {
      int64_t len = 1;
      flag[i] = 1;
      index[0] = i;
      for (int64_t j = P->rowptr[i]; j < P->rowptr[i + 1]; ++j) {
        int64_t a = P->cols[j];
        for (int64_t q = brp[a]; q < brp[a + 1]; ++q) {
          int64_t c = bci[q];
          if (!flag[c]) { index[len++] = c; flag[c] = 1; }
        }
      }
      for (int64_t q = 0; q < len; ++q) flag[index[q]] = 0;
      A->rowptr[i + 1] = len;
    }
    free(flag);
    free(index);
  }
  free(brp);
  free(bci);
  for (int64_t i = 0; i < nc; ++i) A->rowptr[i + 1] += A->rowptr[i];
  const int64_t nnz = A->rowptr[nc];
  A->cols = (int64_t *)malloc(sizeof(int64_t) * (nnz ? nnz : 1));
  A->vals = (double *)calloc(nnz ? nnz : 1, sizeof(double));
  /* pass 2: pattern [i, ascending others] and values */
#pragma omp parallel
  {
    char *flag = (char *)calloc(nc ? nc : 1, 1);
    double *row_entry = (double *)calloc(nc ? nc : 1, sizeof(double));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < nc; ++i) {
      int64_t *out = A->cols + A->rowptr[i];
      int64_t len = 1;
      out[0] = i;
      flag[i] = 1;
      for (int64_t j = P->rowptr[i]; j < P->rowptr[i + 1]; ++j) {
        int64_t a = P->cols[j];
        for (int64_t k = M->rowptr[a]; k < M->rowptr[a + 1]; ++k) {
          int64_t b = M->cols[k];
          for (int64_t l = Pt->rowptr[b]; l < Pt->rowptr[b + 1]; ++l) {
            int64_t c = Pt->cols[l];
            row_entry[c] += P->vals[j] * M->vals[k] * Pt->vals[l];
            if (!flag[c]) { out[len++] = c; flag[c] = 1; }
          }
        }
      }
      if (len > 2) qsort(out + 1, len - 1, sizeof(int64_t), cmp_i64);
      double *vo = A->vals + A->rowptr[i];
      for (int64_t q = 0; q < len; ++q) {
        vo[q] = 0.0 + row_entry[out[q]];
        row_entry[out[q]] = 0.0;
        flag[out[q]] = 0;
      }
    }
    free(flag);
    free(row_entry);
  }
  return 0;
}

/* Transpose of a CSR with sorted output rows (the P^T the reference keeps). */
static void csr_transpose(const orc_csr *a, orc_csr *t) {
  t->m = a->n;
  t->n = a->m;
  int64_t nnz = a->rowptr[a->m];
  t->rowptr = (int64_t *)calloc(t->m + 1, sizeof(int64_t));
  t->cols = (int64_t *)malloc(sizeof(int64_t) * (nnz ? nnz : 1));
  t->vals = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  for (int64_t k = 0; k < nnz; ++k) t->rowptr[a->cols[k] + 1]++;
  for (int64_t i = 0; i < t->m; ++i) t->rowptr[i + 1] += t->rowptr[i];
  int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (t->m ? t->m : 1));
  memcpy(cur, t->rowptr, sizeof(int64_t) * t->m);
  for (int64_t i = 0; i < a->m; ++i)
    for (int64_t k = a->rowptr[i]; k < a->rowptr[i + 1]; ++k) {
      int64_t p = cur[a->cols[k]]++;
      t->cols[p] = i;
      t->vals[p] = a->vals[k];
    }
  free(cur);
}

int orc_rap(const orc_csr *p, const orc_csr *m, orc_csr *out) {
  orc_csr pt;
  csr_transpose(p, &pt);
  int r = rap_with_pt(p, m, &pt, out);
  orc_csr_free(&pt);
  return r;
}

/* Project (src/AMGSolver.cpp:18-226); P is n_core x n, Pt is n x n_core. */
static int project(const orc_csr *M, double alpha, orc_csr *P, orc_csr *Pt, int32_t *cf_out) {
  const int64_t m = M->m;
  const int64_t *rs = M->rowptr, *cn = M->cols;
  const double *v = M->vals;
  int *flag = (int *)calloc(m, sizeof(int));
  double *beta = (double *)calloc(m, sizeof(double));
  int64_t *dep = (int64_t *)malloc(sizeof(int64_t) * (m ? m : 1));
  int64_t n_core = 0;
  for (int64_t i = 0; i < m; ++i) {
    beta[i] = 0.0;
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) {
      double a = fabs(v[j]);
      beta[i] = (a < beta[i]) ? beta[i] : a; /* std::max(fabs(a_ij), beta_i) */
    }
    beta[i] *= alpha;
    if (flag[i] != 0) continue;
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) {
      int64_t k = cn[j];
      if (flag[k] == -1) continue;
      if (fabs(v[j]) < beta[i]) continue;
      flag[k] = 1;
    }
    flag[i] = -1;
    n_core++;
  }
  /* dep[c] == i marks the strong C neighbours of F point i (the reference
   * keeps them in a std::list and searches it; membership is the same) */
  for (int64_t i = 0; i < m; ++i) dep[i] = -1;
  for (int64_t i = 0; i < m; ++i) {
    if (flag[i] != 1) continue;
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) {
      if (fabs(v[j]) < beta[i]) continue;
      if (flag[cn[j]] == -1) dep[cn[j]] = i;
    }
    int is_FF = 0;
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) {
      int64_t k = cn[j];
      if (flag[k] == -1 || k < i || fabs(v[j]) < beta[i]) continue;
      is_FF = 1;
      for (int64_t j1 = rs[k] + 1; j1 < rs[k + 1]; ++j1) {
        int64_t k1 = cn[j1];
        if (flag[k1] != -1) continue;
        if (dep[k1] == i) { is_FF = 0; break; }
      }
      if (is_FF) break;
    }
    if (!is_FF) continue;
    flag[i] = -1;
    n_core++;
  }
  int64_t *core_point = (int64_t *)malloc(sizeof(int64_t) * (n_core ? n_core : 1));
  int64_t *core_at = (int64_t *)malloc(sizeof(int64_t) * (m ? m : 1));
  int64_t *row_length = (int64_t *)calloc(n_core ? n_core : 1, sizeof(int64_t));
  int64_t *col_length = (int64_t *)calloc(m ? m : 1, sizeof(int64_t));
  for (int64_t i = 0; i < m; ++i) core_at[i] = -1;
  for (int64_t i = 0, n = 0; i < m; ++i) {
    if (flag[i] != -1) continue;
    core_point[n] = i;
    core_at[i] = n;
    for (int64_t j = rs[i]; j < rs[i + 1]; ++j) { row_length[n]++; col_length[cn[j]]++; }
    n++;
  }
  if (cf_out)
    for (int64_t i = 0; i < m; ++i) cf_out[i] = flag[i];
  /* patterns of P (n_core x m) and Pt (m x n_core) */
  int64_t *ps = (int64_t *)malloc(sizeof(int64_t) * (n_core + 1));
  int64_t *ts = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
  ps[0] = 0;
  for (int64_t i = 0; i < n_core; ++i) ps[i + 1] = ps[i] + row_length[i];
  ts[0] = 0;
  for (int64_t i = 0; i < m; ++i) ts[i + 1] = ts[i] + col_length[i];
  int64_t *pslots = (int64_t *)malloc(sizeof(int64_t) * (ps[n_core] ? ps[n_core] : 1));
  int64_t *tslots = (int64_t *)malloc(sizeof(int64_t) * (ts[m] ? ts[m] : 1));
  for (int64_t k = 0; k < ps[n_core]; ++k) pslots[k] = INVALID;
  for (int64_t k = 0; k < ts[m]; ++k) tslots[k] = INVALID;
  const int square = (n_core == m);
  if (square) {
    for (int64_t i = 0; i < n_core; ++i) if (ps[i + 1] > ps[i]) pslots[ps[i]] = i;
    for (int64_t i = 0; i < m; ++i) if (ts[i + 1] > ts[i]) tslots[ts[i]] = i;
  }
  for (int64_t i = 0; i < n_core; ++i) {
    int64_t k = core_point[i];
    pattern_add(pslots, ps[i], ps[i + 1], k);
    pattern_add(tslots, ts[k], ts[k + 1], i);
    for (int64_t j = rs[k] + 1; j < rs[k + 1]; ++j) {
      int64_t l = cn[j];
      if (flag[l] == -1) continue;
      pattern_add(pslots, ps[i], ps[i + 1], l);
      pattern_add(tslots, ts[l], ts[l + 1], i);
    }
  }
  P->m = n_core; P->n = m;
  Pt->m = m; Pt->n = n_core;
  pattern_compress(n_core, square, ps, pslots, P);
  pattern_compress(m, square, ts, tslots, Pt);
  free(pslots); free(tslots); free(ps); free(ts);
  /* a_lc[q] = M(l, core_point[c]) for the Pt entry q = (l, c), looked up once
   * (it does not depend on the fine point i being interpolated); dep_row[c]
   * == i marks the Pt row of i, the reference's "dep" list of i, whose
   * std::find membership it answers. */
  const int64_t nnz_t = Pt->rowptr[m];
  double *a_lc = (double *)malloc(sizeof(double) * (nnz_t ? nnz_t : 1));
  int64_t *dep_row = (int64_t *)malloc(sizeof(int64_t) * (n_core ? n_core : 1));
  for (int64_t l = 0; l < m; ++l)
    for (int64_t q = Pt->rowptr[l]; q < Pt->rowptr[l + 1]; ++q) a_lc[q] = matrix_el(M, l, core_point[Pt->cols[q]]);
  for (int64_t c = 0; c < n_core; ++c) dep_row[c] = -1;
  for (int64_t i = 0; i < m; ++i) {
    for (int64_t q = Pt->rowptr[i]; q < Pt->rowptr[i + 1]; ++q) dep_row[Pt->cols[q]] = i;
    int64_t k = core_at[i];
    if (k >= 0) {
      matrix_add(Pt, i, k, 1.0);
      matrix_add(P, k, i, 1.0);
      continue;
    }
    double aii = v[rs[i]];
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j)
      if (fabs(v[j]) < beta[i]) aii += v[j];
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) {
      int64_t l = cn[j];
      if (fabs(v[j]) < beta[i]) continue;
      if (core_at[l] >= 0) {
        matrix_add(Pt, i, core_at[l], fabs(v[j] / aii));
        matrix_add(P, core_at[l], i, fabs(v[j] / aii));
      } else {
        double d = 0.0;
        for (int64_t i1 = Pt->rowptr[l]; i1 < Pt->rowptr[l + 1]; ++i1)
          if (dep_row[Pt->cols[i1]] == i) d += a_lc[i1];
        if (fabs(d * aii) < 1e-16) continue;
        for (int64_t i1 = Pt->rowptr[l]; i1 < Pt->rowptr[l + 1]; ++i1) {
          int64_t c1 = Pt->cols[i1];
          if (dep_row[c1] == i) {
            /* v[j] is M(i, l): rows hold each column once */
            double w = fabs(v[j] * a_lc[i1] / (d * aii));
            matrix_add(Pt, i, c1, w);
            matrix_add(P, c1, i, w);
          }
        }
      }
    }
  }
  free(a_lc); free(dep_row);
  free(flag); free(beta); free(dep); free(core_point); free(core_at); free(row_length); free(col_length);
  return 0;
}

int orc_project(const orc_csr *m, double alpha, orc_csr *p, int32_t *cf_out) {
  orc_csr pt;
  int r = project(m, alpha, p, &pt, cf_out);
  orc_csr_free(&pt);
  return r;
}

static void csr_copy(const orc_csr *a, orc_csr *b) {
  int64_t nnz = a->rowptr[a->m];
  b->m = a->m; b->n = a->n;
  b->rowptr = (int64_t *)malloc(sizeof(int64_t) * (a->m + 1));
  b->cols = (int64_t *)malloc(sizeof(int64_t) * (nnz ? nnz : 1));
  b->vals = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  memcpy(b->rowptr, a->rowptr, sizeof(int64_t) * (a->m + 1));
  memcpy(b->cols, a->cols, sizeof(int64_t) * nnz);
  memcpy(b->vals, a->vals, sizeof(double) * nnz);
}

/* Gauss-Jordan inverse with partial pivoting (stands in for LAPACK getrf+getri,
 * DenseMatrix.h:131-172).  Returns -1 when the matrix is singular. */
static int dense_inverse(int64_t n, double *a) {
  int64_t *piv = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));
  double *inv = (double *)calloc(n * n ? n * n : 1, sizeof(double));
  for (int64_t i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int64_t c = 0; c < n; ++c) {
    int64_t p = c;
    for (int64_t r = c + 1; r < n; ++r)
      if (fabs(a[r * n + c]) > fabs(a[p * n + c])) p = r;
    if (a[p * n + c] == 0.0) { free(piv); free(inv); return -1; }
    if (p != c)
      for (int64_t k = 0; k < n; ++k) {
        double t = a[c * n + k]; a[c * n + k] = a[p * n + k]; a[p * n + k] = t;
        t = inv[c * n + k]; inv[c * n + k] = inv[p * n + k]; inv[p * n + k] = t;
      }
    double d = a[c * n + c];
    for (int64_t k = 0; k < n; ++k) { a[c * n + k] /= d; inv[c * n + k] /= d; }
    for (int64_t r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = a[r * n + c];
      if (f == 0.0) continue;
      for (int64_t k = 0; k < n; ++k) { a[r * n + k] -= f * a[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
    }
  }
  memcpy(a, inv, sizeof(double) * n * n);
  free(piv); free(inv);
  return 0;
}

int orc_amg_setup(const orc_csr *a, int smooth_step, int64_t max_coarse, double min_density,
                  double alpha, orc_amg *h) {
  memset(h, 0, sizeof(*h));
  h->smooth_step = smooth_step;
  h->alpha = alpha;
  int cap = 8;
  h->A = (orc_csr *)calloc(cap + 1, sizeof(orc_csr));
  h->P = (orc_csr *)calloc(cap, sizeof(orc_csr));
  csr_copy(a, &h->A[0]);
  uint64_t k = (uint64_t)a->m, m = (uint64_t)a->m;
  float sparse_degree = (float)a->rowptr[a->m] / ((float)m * m);
  h->most_project_full = 1;
  while (m > (uint64_t)max_coarse || sparse_degree < min_density) {
    orc_csr P, Pt, Ac;
    project(&h->A[h->n_level], alpha, &P, &Pt, NULL);
    rap_with_pt(&P, &h->A[h->n_level], &Pt, &Ac);
    orc_csr_free(&Pt);
    m = (uint64_t)Ac.m;
    if (k == m) {
      h->most_project_full = 0;
      orc_csr_free(&P);
      orc_csr_free(&Ac);
      break;
    }
    k = m;
    if (h->n_level == cap) {
      cap *= 2;
      h->A = (orc_csr *)realloc(h->A, sizeof(orc_csr) * (cap + 1));
      h->P = (orc_csr *)realloc(h->P, sizeof(orc_csr) * cap);
    }
    h->P[h->n_level] = P;
    h->A[h->n_level + 1] = Ac;
    sparse_degree = (float)Ac.rowptr[Ac.m] / ((float)m * m);
    h->n_level++;
  }
  const orc_csr *c = &h->A[h->n_level];
  h->n_coarse = c->m;
  if (h->most_project_full) {
    h->coarse_inv = (double *)calloc(c->m * c->m ? c->m * c->m : 1, sizeof(double));
    for (int64_t i = 0; i < c->m; ++i)
      for (int64_t q = c->rowptr[i]; q < c->rowptr[i + 1]; ++q) h->coarse_inv[i * c->m + c->cols[q]] = c->vals[q];
    if (dense_inverse(c->m, h->coarse_inv)) return -1;
  }
  return 0;
}

int orc_amg_from_levels(int n_level, const orc_csr *A, const orc_csr *P, int most_project_full,
                        int smooth_step, orc_amg *h) {
  memset(h, 0, sizeof(*h));
  h->smooth_step = smooth_step;
  h->alpha = 0.25;
  h->n_level = n_level;
  h->most_project_full = most_project_full;
  h->A = (orc_csr *)calloc(n_level + 1, sizeof(orc_csr));
  h->P = (orc_csr *)calloc(n_level > 0 ? n_level : 1, sizeof(orc_csr));
  for (int l = 0; l <= n_level; ++l) csr_copy(&A[l], &h->A[l]);
  for (int l = 0; l < n_level; ++l) csr_copy(&P[l], &h->P[l]);
  const orc_csr *c = &h->A[n_level];
  h->n_coarse = c->m;
  if (most_project_full) {
    h->coarse_inv = (double *)calloc(c->m * c->m ? c->m * c->m : 1, sizeof(double));
    for (int64_t i = 0; i < c->m; ++i)
      for (int64_t q = c->rowptr[i]; q < c->rowptr[i + 1]; ++q) h->coarse_inv[i * c->m + c->cols[q]] = c->vals[q];
    if (dense_inverse(c->m, h->coarse_inv)) return -1;
  }
  return 0;
}

int orc_amg_set_coarse_inverse(orc_amg *h, const double *inv) {
  const int64_t n = h->n_coarse;
  free(h->coarse_inv);
  h->coarse_inv = (double *)malloc(sizeof(double) * (n * n ? n * n : 1));
  if (!h->coarse_inv) return -1;
  memcpy(h->coarse_inv, inv, sizeof(double) * n * n);
  h->most_project_full = 1;
  return 0;
}

int orc_lazy_project(const orc_csr *M, orc_csr *P, orc_csr *Pt) {
  const int64_t m = M->m;
  const int64_t *rs = M->rowptr, *cn = M->cols;
  int64_t *counter = (int64_t *)calloc(m ? m : 1, sizeof(int64_t));
  int64_t *core = (int64_t *)malloc(sizeof(int64_t) * (m ? m : 1));
  int64_t nc = 0;
  for (int64_t i = 0; i < m; ++i) {
    if (counter[i] > 0) continue;
    for (int64_t j = rs[i] + 1; j < rs[i + 1]; ++j) counter[cn[j]]++;
    core[nc++] = i;
  }
  /* SparsityPattern::max_entries_per_row() of a compressed pattern: rows 1..m-1 */
  int64_t cap = 0;
  for (int64_t i = 1; i < m; ++i) cap = (rs[i] - rs[i - 1]) > cap ? (rs[i] - rs[i - 1]) : cap;
  const int square = (nc == m);
  int64_t *ps = (int64_t *)malloc(sizeof(int64_t) * (nc + 1));
  int64_t *ts = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
  for (int64_t i = 0; i <= nc; ++i) ps[i] = i * cap;
  for (int64_t i = 0; i <= m; ++i) ts[i] = i * cap;
  int64_t *pslots = (int64_t *)malloc(sizeof(int64_t) * (nc * cap ? nc * cap : 1));
  int64_t *tslots = (int64_t *)malloc(sizeof(int64_t) * (m * cap ? m * cap : 1));
  for (int64_t k = 0; k < nc * cap; ++k) pslots[k] = INVALID;
  for (int64_t k = 0; k < m * cap; ++k) tslots[k] = INVALID;
  if (square && cap > 0) {
    for (int64_t i = 0; i < nc; ++i) pslots[i * cap] = i;
    for (int64_t i = 0; i < m; ++i) tslots[i * cap] = i;
  }
  for (int64_t i = 0; i < nc; ++i) {
    const int64_t k = core[i];
    pattern_add(pslots, ps[i], ps[i + 1], k);
    pattern_add(tslots, ts[k], ts[k + 1], i);
    for (int64_t j = rs[k] + 1; j < rs[k + 1]; ++j) {
      pattern_add(pslots, ps[i], ps[i + 1], cn[j]);
      pattern_add(tslots, ts[cn[j]], ts[cn[j] + 1], i);
    }
  }
  P->m = nc; P->n = m;
  Pt->m = m; Pt->n = nc;
  pattern_compress(nc, square, ps, pslots, P);
  pattern_compress(m, square, ts, tslots, Pt);
  for (int64_t i = 0; i < nc; ++i) {
    const int64_t k = core[i];
    matrix_add(P, i, k, 1.0);
    matrix_add(Pt, k, i, 1.0);
    for (int64_t j = rs[k] + 1; j < rs[k + 1]; ++j) {
      const int64_t l = cn[j];
      matrix_add(P, i, l, 1.0 / counter[l]);
      matrix_add(Pt, l, i, 1.0 / counter[l]);
    }
  }
  free(counter); free(core); free(ps); free(ts); free(pslots); free(tslots);
  return 0;
}

static int coarse_inverse(orc_amg *h) {
  const orc_csr *c = &h->A[h->n_level];
  h->n_coarse = c->m;
  free(h->coarse_inv);
  h->coarse_inv = NULL;
  if (!h->most_project_full) return 0;
  h->coarse_inv = (double *)calloc(c->m * c->m ? c->m * c->m : 1, sizeof(double));
  for (int64_t i = 0; i < c->m; ++i)
    for (int64_t q = c->rowptr[i]; q < c->rowptr[i + 1]; ++q) h->coarse_inv[i * c->m + c->cols[q]] = c->vals[q];
  return dense_inverse(c->m, h->coarse_inv);
}

int orc_amg_setup_lazy(const orc_csr *a, int smooth_step, int64_t max_coarse, double min_density, orc_amg *h) {
  memset(h, 0, sizeof(*h));
  h->smooth_step = smooth_step;
  h->alpha = 0.25;
  int cap = 8;
  h->A = (orc_csr *)calloc(cap + 1, sizeof(orc_csr));
  h->P = (orc_csr *)calloc(cap, sizeof(orc_csr));
  h->Pt = (orc_csr *)calloc(cap, sizeof(orc_csr));
  csr_copy(a, &h->A[0]);
  uint64_t k = (uint64_t)a->m, m = k;
  float sparse_degree = (float)a->rowptr[a->m] / ((float)m * m);
  h->most_project_full = 1;
  while (m > (uint64_t)max_coarse || sparse_degree < min_density) {
    orc_csr P, Pt, Ac;
    orc_lazy_project(&h->A[h->n_level], &P, &Pt);
    rap_with_pt(&P, &h->A[h->n_level], &Pt, &Ac);
    m = (uint64_t)Ac.m;
    if (k == m) {
      h->most_project_full = 0;
      orc_csr_free(&P); orc_csr_free(&Pt); orc_csr_free(&Ac);
      break;
    }
    k = m;
    if (h->n_level == cap) {
      cap *= 2;
      h->A = (orc_csr *)realloc(h->A, sizeof(orc_csr) * (cap + 1));
      h->P = (orc_csr *)realloc(h->P, sizeof(orc_csr) * cap);
      h->Pt = (orc_csr *)realloc(h->Pt, sizeof(orc_csr) * cap);
    }
    h->P[h->n_level] = P;
    h->Pt[h->n_level] = Pt;
    h->A[h->n_level + 1] = Ac;
    sparse_degree = (float)Ac.rowptr[Ac.m] / ((float)m * m);
    h->n_level++;
  }
  return coarse_inverse(h);
}

int orc_amg_lazy_reinit(orc_amg *h, const orc_csr *a) {
  if (h->Pt == NULL) return -1;
  orc_csr_free(&h->A[0]);
  csr_copy(a, &h->A[0]);
  for (int l = 0; l < h->n_level; ++l) {
    orc_csr Ac;
    rap_with_pt(&h->P[l], &h->A[l], &h->Pt[l], &Ac);
    orc_csr_free(&h->A[l + 1]);
    h->A[l + 1] = Ac;
  }
  return coarse_inverse(h);
}

void orc_amg_free(orc_amg *h) {
  for (int l = 0; l <= h->n_level; ++l) orc_csr_free(&h->A[l]);
  for (int l = 0; l < h->n_level; ++l) orc_csr_free(&h->P[l]);
  if (h->Pt) {
    for (int l = 0; l < h->n_level; ++l) orc_csr_free(&h->Pt[l]);
    free(h->Pt);
  }
  free(h->A);
  free(h->P);
  free(h->coarse_inv);
  memset(h, 0, sizeof(*h));
}

/* GaussSidel (src/AMGSolver.cpp:362-381): forward lexicographic sweeps */
static void gauss_seidel(const orc_csr *M, double *x, const double *r, int s) {
  for (int i = 0; i < s; ++i)
    for (int64_t j = 0; j < M->m; ++j) {
      double r0 = r[j];
      for (int64_t k = M->rowptr[j] + 1; k < M->rowptr[j + 1]; ++k) r0 -= x[M->cols[k]] * M->vals[k];
      x[j] = r0 / M->vals[M->rowptr[j]];
    }
}

/* AMGSolver::solve (src/AMGSolver.cpp:549-639), exactly `cycles` V-cycles */
void orc_amg_vcycles(const orc_amg *h, double *x, const double *r, int cycles) {
  const int L = h->n_level;
  double **px = (double **)malloc(sizeof(double *) * (L + 1));
  double **pr = (double **)malloc(sizeof(double *) * (L + 1));
  int64_t n0 = h->A[0].m;
  px[0] = x;
  pr[0] = (double *)malloc(sizeof(double) * n0);
  memcpy(pr[0], r, sizeof(double) * n0);
  for (int l = 1; l <= L; ++l) {
    px[l] = (double *)calloc(h->A[l].m, sizeof(double));
    pr[l] = (double *)calloc(h->A[l].m, sizeof(double));
  }
  double *v0 = (double *)malloc(sizeof(double) * n0);
  double *v1 = (double *)malloc(sizeof(double) * n0);
  for (int it = 0; it < cycles; ++it) {
    for (int l = 0; l < L; ++l) {
      const orc_csr *A = &h->A[l];
      gauss_seidel(A, px[l], pr[l], h->smooth_step);
      orc_vmult(A, px[l], v0);
      for (int64_t i = 0; i < A->m; ++i) v1[i] = pr[l][i] + (-1.0) * v0[i];
      orc_vmult(&h->P[l], v1, pr[l + 1]);
      memset(px[l + 1], 0, sizeof(double) * h->A[l + 1].m);
    }
    const orc_csr *C = &h->A[L];
    if (h->most_project_full) {
      for (int64_t i = 0; i < C->m; ++i) {
        double s = 0.0;
        for (int64_t j = 0; j < C->m; ++j) s += h->coarse_inv[i * C->m + j] * pr[L][j];
        px[L][i] = s;
      }
    } else {
      for (int64_t i = 0; i < C->m; ++i) px[L][i] = pr[L][i] / C->vals[C->rowptr[i]];
    }
    for (int l = L - 1; l >= 0; --l) {
      orc_tvmult(&h->P[l], px[l + 1], v0);
      for (int64_t i = 0; i < h->A[l].m; ++i) px[l][i] += v0[i];
      gauss_seidel(&h->A[l], px[l], pr[l], h->smooth_step);
    }
  }
  for (int l = 1; l <= L; ++l) { free(px[l]); free(pr[l]); }
  free(pr[0]); free(px); free(pr); free(v0); free(v1);
}

static double dot(int64_t n, const double *a, const double *b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

int orc_pcg(const orc_csr *a, const orc_amg *h, const double *b, double *x, double tol, int maxit,
            double *relres) {
  const int64_t n = a->m;
  double *r = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
  double *p = (double *)malloc(sizeof(double) * n), *ap = (double *)malloc(sizeof(double) * n);
  orc_vmult(a, x, ap);
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - ap[i];
  double bn = sqrt(dot(n, b, b));
  if (bn < 1e-30) bn = 1e-30;
  double rel = sqrt(dot(n, r, r)) / bn;
  int it = 0;
  if (rel > tol) {
    memset(z, 0, sizeof(double) * n);
    orc_amg_vcycles(h, z, r, 1);
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z);
    for (it = 1; it <= maxit; ++it) {
      orc_vmult(a, p, ap);
      double alpha = rz / dot(n, p, ap);
      for (int64_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * ap[i]; }
      rel = sqrt(dot(n, r, r)) / bn;
      if (rel <= tol) break;
      memset(z, 0, sizeof(double) * n);
      orc_amg_vcycles(h, z, r, 1);
      double rz2 = dot(n, r, z);
      for (int64_t i = 0; i < n; ++i) p[i] = z[i] + (rz2 / rz) * p[i];
      rz = rz2;
    }
    if (it > maxit) it = maxit;
  }
  if (relres) *relres = rel;
  free(r); free(z); free(p); free(ap);
  return it;
}
