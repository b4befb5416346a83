// Finite element assembly on the GPU: element matrices, AFEPack's CSR
// sparsity pattern, the scatter of element matrices into it, and Dirichlet
// elimination.
//
// Compiled with -fmad=false: the element-matrix arithmetic repeats the
// reference's operations in the reference's order (template plugins
// triangle.{1,2}.bas_fun.c, tetrahedron.{1,2}.bas_fun.c, *.crd_trs.c and
// BilinearOperator.templates.h:343-406) and the scatter adds element
// contributions to each entry in ascending element order exactly as
// buildSparseMatrix does (:177-255), so the assembled values are bitwise
// those of AFEPack.
//
// Layout: the pattern is built "pull" style -- one warp per matrix row
// gathers the DOFs of the cells around its DOF from a DOF->cell incidence
// list, sorts and de-duplicates them in shared memory and writes the row as
// [diagonal, ascending others] (SparsityPattern::compress, SparsityPattern.h:193-237).
// The values pass walks the same incidence list in ascending cell order,
// so no atomics are needed and the result is deterministic.
#include <algorithm>
#include <climits>

#include "common.cuh"
#include "kernels.cuh"
#include "quadrature_tables.h"

struct afp_space {
  afp_context* ctx = nullptr;
  int dim = 0, degree = 0, nd = 0, nv = 0;
  int64_t n_vertex = 0, n_cell = 0, n_dof = 0;
  afp::DevBuf<double> coords;
  afp::DevBuf<int> cells;
  afp::DevBuf<int> elem_dof;
  afp::DevBuf<int> inc_ptr;  // n_dof+1
  afp::DevBuf<int> inc;      // cell*nd + local, ascending per DOF
  int max_inc = 0;
  // spaces numbered on the device (afp_space_create_numbered) also keep
  // each DOF's boundary mark and interpolation point
  afp::DevBuf<int> dof_bmark;
  afp::DevBuf<double> dof_point;
};

namespace afp {
namespace {

constexpr int BLOCK = 256;

// ------------------------------------------------------------ utilities
__global__ void k_check_range(const int* __restrict__ a, int64_t n, int64_t hi, int* __restrict__ bad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && (a[i] < 0 || a[i] >= hi)) atomicExch(bad, 1);
}

__global__ void k_count(const int* __restrict__ a, int64_t n, int* __restrict__ cnt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[a[i]], 1);
}

__global__ void k_fill_incidence(const int* __restrict__ elem_dof, int64_t n, const int* __restrict__ ptr,
                                 int* __restrict__ cursor, int* __restrict__ inc) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    int d = elem_dof[t];
    inc[ptr[d] + atomicAdd(&cursor[d], 1)] = (int)t;
  }
}

__global__ void k_sort_lists(const int* __restrict__ ptr, int* __restrict__ list, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int b = ptr[i], e = ptr[i + 1];
  for (int p = b + 1; p < e; ++p) {
    int v = list[p];
    int q = p - 1;
    while (q >= b && list[q] > v) {
      list[q + 1] = list[q];
      --q;
    }
    list[q + 1] = v;
  }
}

// ---------------------------------------------------- DOF numbering
// FEMSpace::buildDof (include/AFEPack/FEMSpace.templates.h:884-1003) numbers
// the DOFs in the order the element loop first touches their geometries:
// elements in order, inside an element the template's vertices, then its
// edges.  A "touch" is slot s of element e, t = e*T + s (T = slots per
// element, vertices first), so a geometry's DOF number is the number of
// first touches before its own first touch: an exclusive scan over first-touch
// flags.  The first touch of a vertex is the lowest (cell, local vertex) of
// its incidence list; that of an edge (a, b) is the lowest cell holding both,
// found by walking a's incidence list in ascending cell order.

// template edges as local vertex pairs, in template order
__constant__ int c_tri_edge[3][2] = {{1, 2}, {0, 2}, {0, 1}};
__constant__ int c_tet_edge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {2, 3}, {1, 3}, {1, 2}};

__device__ __forceinline__ void edge_verts(int dim, int j, int& a, int& b) {
  if (dim == 2) {
    a = c_tri_edge[j][0];
    b = c_tri_edge[j][1];
  } else {
    a = c_tet_edge[j][0];
    b = c_tet_edge[j][1];
  }
}

// first[t] = flat touch index of the first touch of slot t's geometry
__global__ void k_first_touch(int dim, int degree, int64_t n_cell, const int* __restrict__ cells,
                              const int* __restrict__ vptr, const int* __restrict__ vinc, int* __restrict__ first,
                              int* __restrict__ is_first) {
  const int nv = dim + 1, ne = degree == 2 ? (dim == 2 ? 3 : 6) : 0, T = nv + ne;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_cell * T) return;
  const int64_t e = t / T;
  const int s = (int)(t - e * T);
  int64_t f;
  if (s < nv) {
    const int v = cells[e * nv + s];
    const int g = vinc[vptr[v]];  // lowest cell*nv + local of vertex v
    f = (int64_t)(g / nv) * T + g % nv;
  } else {
    int la, lb;
    edge_verts(dim, s - nv, la, lb);
    const int a = cells[e * nv + la], b = cells[e * nv + lb];
    f = t;
    for (int q = vptr[a]; q < vptr[a + 1]; ++q) {
      const int c = vinc[q] / nv;
      if (c >= e) break;  // the cell itself holds the edge
      int jb = -1;
      for (int k = 0; k < nv; ++k)
        if (cells[(int64_t)c * nv + k] == b) jb = k;
      if (jb < 0) continue;
      const int ja = vinc[q] % nv;
      for (int j = 0; j < ne; ++j) {
        int x, y;
        edge_verts(dim, j, x, y);
        if ((x == ja && y == jb) || (x == jb && y == ja)) f = (int64_t)c * T + nv + j;
      }
      break;
    }
  }
  first[t] = (int)f;
  is_first[t] = f == t ? 1 : 0;
}

__global__ void k_number_dofs(int dim, int degree, int64_t n_cell, const int* __restrict__ cells,
                              const double* __restrict__ coords, const int* __restrict__ vmark,
                              const int* __restrict__ first, const int* __restrict__ rank, int* __restrict__ elem_dof,
                              int* __restrict__ dof_bmark, double* __restrict__ dof_point) {
  const int nv = dim + 1, ne = degree == 2 ? (dim == 2 ? 3 : 6) : 0, T = nv + ne;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_cell * T) return;
  const int d = rank[first[t]];
  elem_dof[t] = d;
  if (first[t] != t) return;
  const int64_t e = t / T;
  const int s = (int)(t - e * T);
  if (s < nv) {
    const int v = cells[e * nv + s];
    dof_bmark[d] = (vmark != nullptr && vmark[v] != 0) ? 1 : 0;
    for (int k = 0; k < dim; ++k) dof_point[(int64_t)d * dim + k] = coords[(int64_t)v * dim + k];
  } else {
    int la, lb;
    edge_verts(dim, s - nv, la, lb);
    const int a = cells[e * nv + la], b = cells[e * nv + lb];
    dof_bmark[d] = (vmark != nullptr && (vmark[a] & vmark[b]) != 0) ? 1 : 0;
    for (int k = 0; k < dim; ++k)
      dof_point[(int64_t)d * dim + k] = 0.5 * (coords[(int64_t)a * dim + k] + coords[(int64_t)b * dim + k]);
  }
}

__global__ void k_max_diff(const int* __restrict__ ptr, int64_t n, int* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int v = i < n ? ptr[i + 1] - ptr[i] : 0;
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, v);
}

// --------------------------------------------- template-element arithmetic
__device__ __forceinline__ double area2(const double* a, const double* b, const double* c) {
  return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
}

__device__ __forceinline__ double det6(const double* v0, const double* v1, const double* v2, const double* v3) {
  return ((v1[0] - v0[0]) * (v2[1] - v0[1]) * (v3[2] - v0[2]) + (v1[1] - v0[1]) * (v2[2] - v0[2]) * (v3[0] - v0[0]) +
          (v1[2] - v0[2]) * (v2[0] - v0[0]) * (v3[1] - v0[1]) - (v1[0] - v0[0]) * (v2[2] - v0[2]) * (v3[1] - v0[1]) -
          (v1[1] - v0[1]) * (v2[0] - v0[0]) * (v3[2] - v0[2]) - (v1[2] - v0[2]) * (v2[1] - v0[1]) * (v3[0] - v0[0]));
}

__device__ __forceinline__ double co_det(const double (*v)[3], int m, int n) {
  double s = (m % 2 == 0) ? -1. : 1.;
  return s * ((v[(m + 2) % 4][(n + 1) % 3] - v[(m + 1) % 4][(n + 1) % 3]) *
                  (v[(m + 3) % 4][(n + 2) % 3] - v[(m + 1) % 4][(n + 2) % 3]) -
              (v[(m + 2) % 4][(n + 2) % 3] - v[(m + 1) % 4][(n + 2) % 3]) *
                  (v[(m + 3) % 4][(n + 1) % 3] - v[(m + 1) % 4][(n + 1) % 3]));
}

struct QuadRule {
  int n;
  double p[64][4];  // local coordinates, then the weight
};

template <int DIM, int DEG>
struct Elem {
  static constexpr int NV = DIM + 1;
  static constexpr int ND = DIM == 2 ? 3 * DEG : (DEG == 1 ? 4 : 10);
};

// Quadrature point l of a triangle: its global point p and the basis values
// of triangle.{1,2}.bas_fun.c there (lam: barycentric coordinates, P2 only).
template <int DEG>
__device__ __forceinline__ void tri_values(const double (&gv)[3][2], double area, const double (&R)[3][2],
                                           double larea, const QuadRule& q, int l, double (&p)[2], double (&lam)[3],
                                           double* val) {
  const double lp[2] = {q.p[l][0], q.p[l][1]};
  const double l0 = area2(lp, R[1], R[2]) / larea;
  const double l1 = area2(lp, R[2], R[0]) / larea;
  const double l2 = area2(lp, R[0], R[1]) / larea;
  p[0] = l0 * gv[0][0] + l1 * gv[1][0] + l2 * gv[2][0];
  p[1] = l0 * gv[0][1] + l1 * gv[1][1] + l2 * gv[2][1];
  if constexpr (DEG == 1) {
    val[0] = area2(p, gv[1], gv[2]) / area;
    val[1] = area2(gv[0], p, gv[2]) / area;
    val[2] = area2(gv[0], gv[1], p) / area;
  } else {
    lam[0] = area2(p, gv[1], gv[2]) / area;
    lam[1] = area2(p, gv[2], gv[0]) / area;
    lam[2] = area2(p, gv[0], gv[1]) / area;
#pragma unroll
    for (int k = 0; k < 3; ++k) val[k] = lam[k] * (2 * lam[k] - 1.0);
    val[3] = 4.0 * lam[1] * lam[2];
    val[4] = 4.0 * lam[0] * lam[2];
    val[5] = 4.0 * lam[0] * lam[1];
  }
}

// the same for a tetrahedron (tetrahedron.{1,2}.bas_fun.c); vol = det6 of the cell
template <int DEG>
__device__ __forceinline__ void tet_values(const double (&v)[4][3], double vol, const double (&R)[4][3], double lvol,
                                           const QuadRule& q, int l, double (&p)[3], double (&lam)[4],
                                           double* val) {
  const double lp[3] = {q.p[l][0], q.p[l][1], q.p[l][2]};
  const double l0 = det6(lp, R[1], R[2], R[3]) / 6. / lvol;
  const double l1 = det6(R[0], lp, R[2], R[3]) / 6. / lvol;
  const double l2 = det6(R[0], R[1], lp, R[3]) / 6. / lvol;
  const double l3 = det6(R[0], R[1], R[2], lp) / 6. / lvol;
#pragma unroll
  for (int d = 0; d < 3; ++d) p[d] = l0 * v[0][d] + l1 * v[1][d] + l2 * v[2][d] + l3 * v[3][d];
  lam[0] = det6(p, v[1], v[2], v[3]) / vol;
  lam[1] = det6(v[0], p, v[2], v[3]) / vol;
  lam[2] = det6(v[0], v[1], p, v[3]) / vol;
  lam[3] = det6(v[0], v[1], v[2], p) / vol;
  if constexpr (DEG == 1) {
#pragma unroll
    for (int m = 0; m < 4; ++m) val[m] = lam[m];
  } else {
#pragma unroll
    for (int m = 0; m < 4; ++m) val[m] = lam[m] * (2 * lam[m] - 1);
    // template edges 0:(0,1) 1:(0,2) 2:(0,3) 3:(2,3) 4:(1,3) 5:(1,2)
    val[4] = 4.0 * lam[0] * lam[1];
    val[5] = 4.0 * lam[0] * lam[2];
    val[6] = 4.0 * lam[0] * lam[3];
    val[7] = 4.0 * lam[2] * lam[3];
    val[8] = 4.0 * lam[1] * lam[3];
    val[9] = 4.0 * lam[1] * lam[2];
  }
}

// Element matrix of one cell, reference arithmetic (see file comment).
template <int DIM, int DEG, bool MASS>
__global__ void __launch_bounds__(128) k_element_matrix(const double* __restrict__ coords, const int* __restrict__ cells,
                                                        int64_t n_cell, QuadRule q, const double* __restrict__ coef,
                                                        double* __restrict__ out) {
  constexpr int NV = Elem<DIM, DEG>::NV, ND = Elem<DIM, DEG>::ND;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_cell) return;
  double v[4][3] = {{0}};
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    int vi = cells[e * NV + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) v[a][d] = coords[(int64_t)vi * DIM + d];
  }
  double K[ND * ND];
#pragma unroll
  for (int t = 0; t < ND * ND; ++t) K[t] = 0.0;

  if constexpr (DIM == 2) {
    const double R[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
    const double larea = area2(R[0], R[1], R[2]);
    const double tmpl_volume = .5 * area2(R[0], R[1], R[2]);
    const double gv[3][2] = {{v[0][0], v[0][1]}, {v[1][0], v[1][1]}, {v[2][0], v[2][1]}};
    const double garea = area2(gv[0], gv[1], gv[2]);
    const double jac = garea / larea;
    const double area = garea;  // AREA(v[0], v[1], v[2]) of the basis plugins
    double dx[3], dy[3];
    dx[0] = (gv[1][1] - gv[2][1]) / area; dy[0] = (gv[2][0] - gv[1][0]) / area;
    dx[1] = (gv[2][1] - gv[0][1]) / area; dy[1] = (gv[0][0] - gv[2][0]) / area;
    dx[2] = (gv[0][1] - gv[1][1]) / area; dy[2] = (gv[1][0] - gv[0][0]) / area;
    for (int l = 0; l < q.n; ++l) {
      double p[2], lam[3], val[ND], g[ND][2];
      tri_values<DEG>(gv, area, R, larea, q, l, p, lam, val);
      const double Jxw = q.p[l][2] * jac * tmpl_volume;
      if constexpr (DEG == 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) { g[k][0] = dx[k]; g[k][1] = dy[k]; }
      } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          g[k][0] = (4.0 * lam[k] - 1.0) * dx[k];
          g[k][1] = (4.0 * lam[k] - 1.0) * dy[k];
        }
        g[3][0] = 4.0 * (lam[2] * dx[1] + lam[1] * dx[2]); g[3][1] = 4.0 * (lam[2] * dy[1] + lam[1] * dy[2]);
        g[4][0] = 4.0 * (lam[0] * dx[2] + lam[2] * dx[0]); g[4][1] = 4.0 * (lam[0] * dy[2] + lam[2] * dy[0]);
        g[5][0] = 4.0 * (lam[1] * dx[0] + lam[0] * dx[1]); g[5][1] = 4.0 * (lam[1] * dy[0] + lam[0] * dy[1]);
      }
#pragma unroll
      for (int j = 0; j < ND; ++j)
#pragma unroll
        for (int k = 0; k < ND; ++k) {
          if constexpr (MASS) {
            K[j * ND + k] += Jxw * val[j] * val[k];
          } else {
            double ip = 0;
            ip += g[j][0] * g[k][0];
            ip += g[j][1] * g[k][1];
            K[j * ND + k] += Jxw * ip;
          }
        }
    }
  } else {
    const double R[4][3] = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
    const double lvol = det6(R[0], R[1], R[2], R[3]) / 6.;
    const double tmpl_volume = det6(R[0], R[1], R[2], R[3]) / 6.;
    const double jac = (det6(v[0], v[1], v[2], v[3]) / 6.) / lvol;
    const double vol = det6(v[0], v[1], v[2], v[3]);  // det3 / get_volume of the basis plugins
    double gl[4][3];  // co_det(v, m, n) / volume
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int n = 0; n < 3; ++n) gl[m][n] = co_det(v, m, n) / vol;
    for (int l = 0; l < q.n; ++l) {
      double p[3], lam[4], val[ND], g[ND][3];
      tet_values<DEG>(v, vol, R, lvol, q, l, p, lam, val);
      const double Jxw = q.p[l][3] * jac * tmpl_volume;
      if constexpr (DEG == 1) {
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n) g[m][n] = gl[m][n];
      } else {
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n) g[m][n] = gl[m][n] * (4. * lam[m] - 1.);
        // template edges 0:(0,1) 1:(0,2) 2:(0,3) 3:(2,3) 4:(1,3) 5:(1,2);
        // the gradient of 4 l_a l_b is 4*(gl[first]*l[la] + gl[second]*l[lb])
        // with the operand order of the plugin function attached to the edge.
        constexpr int first[6] = {1, 2, 3, 2, 1, 1};
        constexpr int second[6] = {0, 0, 0, 3, 3, 2};
        constexpr int la[6] = {0, 0, 0, 3, 3, 2};
        constexpr int lb[6] = {1, 2, 3, 2, 1, 1};
#pragma unroll
        for (int t = 0; t < 6; ++t)
#pragma unroll
          for (int n = 0; n < 3; ++n) g[4 + t][n] = 4 * (gl[first[t]][n] * lam[la[t]] + gl[second[t]][n] * lam[lb[t]]);
      }
#pragma unroll
      for (int j = 0; j < ND; ++j)
#pragma unroll
        for (int k = 0; k < ND; ++k) {
          if constexpr (MASS) {
            K[j * ND + k] += Jxw * val[j] * val[k];
          } else {
            double ip = 0;
            ip += g[j][0] * g[k][0];
            ip += g[j][1] * g[k][1];
            ip += g[j][2] * g[k][2];
            K[j * ND + k] += Jxw * ip;
          }
        }
    }
  }
  if (!MASS && coef != nullptr) {
    const double a = coef[e];
#pragma unroll
    for (int t = 0; t < ND * ND; ++t) K[t] *= a;
  }
  double* o = out + e * (ND * ND);
#pragma unroll
  for (int t = 0; t < ND * ND; ++t) o[t] = K[t];
}

// ---------------------------------------------------- L2Discretize
// Operator::L2Discretize (include/AFEPack/Operator.discretize.templates.h)
// adds Jxw f(q_l) phi_j(q_l) into f1[dof_j] element by element, point by
// point.  Each DOF therefore receives its terms in (cell, point) order; the
// terms are formed per cell here and summed per DOF in that order by
// k_gather_rhs, which gives the reference's sums bit for bit.
enum RhsSource { SRC_POINT_VALUES = 0, SRC_FEM_FUNCTION = 1, SRC_GAUSSIANS = 2 };

template <int DIM, int DEG, int SRC>
__global__ void __launch_bounds__(128) k_element_rhs(const double* __restrict__ coords, const int* __restrict__ cells,
                                                     const int* __restrict__ elem_dof, int64_t c0, int64_t c1,
                                                     QuadRule q, const double* __restrict__ data, int n_gauss,
                                                     double* __restrict__ terms, double* __restrict__ points) {
  constexpr int NV = Elem<DIM, DEG>::NV, ND = Elem<DIM, DEG>::ND;
  const int64_t e = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= c1) return;
  double v[4][3] = {{0}};
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    const int vi = cells[e * NV + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) v[a][d] = coords[(int64_t)vi * DIM + d];
  }
  for (int l = 0; l < q.n; ++l) {
    double p[DIM], val[ND], Jxw;
    if constexpr (DIM == 2) {
      const double R[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
      const double larea = area2(R[0], R[1], R[2]);
      const double tmpl_volume = .5 * area2(R[0], R[1], R[2]);
      const double gv[3][2] = {{v[0][0], v[0][1]}, {v[1][0], v[1][1]}, {v[2][0], v[2][1]}};
      const double garea = area2(gv[0], gv[1], gv[2]);
      double lam[3];
      tri_values<DEG>(gv, garea, R, larea, q, l, p, lam, val);
      Jxw = q.p[l][2] * (garea / larea) * tmpl_volume;
    } else {
      const double R[4][3] = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
      const double lvol = det6(R[0], R[1], R[2], R[3]) / 6.;
      const double tmpl_volume = det6(R[0], R[1], R[2], R[3]) / 6.;
      const double jac = (det6(v[0], v[1], v[2], v[3]) / 6.) / lvol;
      double lam[4];
      tet_values<DEG>(v, det6(v[0], v[1], v[2], v[3]), R, lvol, q, l, p, lam, val);
      Jxw = q.p[l][3] * jac * tmpl_volume;
    }
    const int64_t ql = (e - c0) * q.n + l;
    if (points != nullptr) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) points[(e * q.n + l) * DIM + d] = p[d];
    }
    if (terms == nullptr) continue;
    double f = 0;
    if constexpr (SRC == SRC_POINT_VALUES) {
      f = data[e * q.n + l];
    } else if constexpr (SRC == SRC_FEM_FUNCTION) {
      // FEMFunction::value (include/AFEPack/FEMSpace.templates.h:1087-1100)
#pragma unroll
      for (int j = 0; j < ND; ++j) f += data[elem_dof[e * ND + j]] * val[j];
    } else {
      // sum of amp * exp(-|p - c|^2 / (2 s^2)); data: [c (DIM), s, amp] per Gaussian
      for (int g = 0; g < n_gauss; ++g) {
        const double* c = data + g * (DIM + 2);
        double r2 = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const double t = p[d] - c[d];
          r2 += t * t;
        }
        const double s = c[DIM];
        f += c[DIM + 1] * exp(-r2 / (2.0 * s * s));
      }
    }
#pragma unroll
    for (int j = 0; j < ND; ++j) terms[ql * ND + j] = Jxw * f * val[j];
  }
}

// f1[i] += the terms of the cells [c0, c1) around DOF i, ascending cell, then point
__global__ void k_gather_rhs(int64_t n_dof, const int* __restrict__ inc_ptr, const int* __restrict__ inc, int nd,
                             int nq, int64_t c0, int64_t c1, const double* __restrict__ terms,
                             double* __restrict__ f1) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_dof) return;
  double acc = f1[i];
  for (int p = inc_ptr[i]; p < inc_ptr[i + 1]; ++p) {
    const int qd = inc[p];
    const int64_t c = qd / nd;
    if (c < c0) continue;
    if (c >= c1) break;
    const double* t = terms + ((c - c0) * nq) * nd + qd % nd;
    for (int l = 0; l < nq; ++l) acc += t[(int64_t)l * nd];
  }
  f1[i] = acc;
}

// ------------------------------------------------------------ pattern
__device__ __forceinline__ void warp_bitonic_sort(int* buf, int P, int lane) {
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < P; t += 32) {
        int ixj = t ^ j;
        if (ixj > t) {
          int a = buf[t], b = buf[ixj];
          bool up = (t & k) == 0;
          if ((a > b) == up) {
            buf[t] = b;
            buf[ixj] = a;
          }
        }
      }
      __syncwarp();
    }
  }
}

// One warp per row: gather the DOFs of the cells around DOF `row`, sort,
// de-duplicate.  count pass: row_len[row] = #unique; fill pass: write the
// row as [row, ascending others].
template <int ND>
__global__ void k_pattern(int64_t n_dof, const int* __restrict__ inc_ptr, const int* __restrict__ inc,
                          const int* __restrict__ elem_dof, int cap, int* __restrict__ row_len,
                          const int* __restrict__ rowptr, int* __restrict__ cols) {
  extern __shared__ int sm_pat[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  int* buf = sm_pat + warp * cap;
  for (int64_t row = (int64_t)blockIdx.x * wpb + warp; row < n_dof; row += (int64_t)gridDim.x * wpb) {
    const int b = inc_ptr[row], S = (inc_ptr[row + 1] - b) * ND;
    int P = 1;
    while (P < S) P <<= 1;
    for (int t = lane; t < P; t += 32) {
      int val = INT_MAX;
      if (t < S) {
        int qd = inc[b + t / ND];
        val = elem_dof[(int64_t)(qd / ND) * ND + t % ND];
      }
      buf[t] = val;
    }
    __syncwarp();
    warp_bitonic_sort(buf, P, lane);
    if (rowptr == nullptr) {
      int cnt = 0;
      for (int t = lane; t < S; t += 32) cnt += (t == 0 || buf[t] != buf[t - 1]);
      for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
      if (lane == 0) row_len[row] = cnt;
    } else {
      int* out = cols + rowptr[row];
      if (lane == 0) out[0] = (int)row;
      int base = 1;
      for (int t0 = 0; t0 < S; t0 += 32) {
        int t = t0 + lane;
        bool keep = t < S && (t == 0 || buf[t] != buf[t - 1]) && buf[t] != (int)row;
        unsigned mask = __ballot_sync(0xffffffffu, keep);
        if (keep) out[base + __popc(mask & ((1u << lane) - 1u))] = buf[t];
        base += __popc(mask);
      }
    }
    __syncwarp();
  }
}

// One warp per row: add the element matrices' rows into the CSR row in
// ascending cell order (one cell at a time, one lane per element column).
template <int ND>
__global__ void k_gather_values(int64_t n_dof, const int* __restrict__ inc_ptr, const int* __restrict__ inc,
                                const int* __restrict__ elem_dof, const int* __restrict__ rowptr,
                                const int* __restrict__ cols, const double* __restrict__ eK,
                                const double* __restrict__ eM, double* __restrict__ vK, double* __restrict__ vM,
                                int rcap) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  double* accK = reinterpret_cast<double*>(sm_raw) + (size_t)warp * 2 * rcap;
  double* accM = accK + rcap;
  int* ucol = reinterpret_cast<int*>(reinterpret_cast<double*>(sm_raw) + (size_t)wpb * 2 * rcap) + warp * rcap;
  for (int64_t row = (int64_t)blockIdx.x * wpb + warp; row < n_dof; row += (int64_t)gridDim.x * wpb) {
    const int r0 = rowptr[row], R = rowptr[row + 1] - r0;
    for (int t = lane; t < R; t += 32) {
      ucol[t] = cols[r0 + t];
      accK[t] = 0.0;
      accM[t] = 0.0;
    }
    __syncwarp();
    const int b = inc_ptr[row], e = inc_ptr[row + 1];
    for (int p = b; p < e; ++p) {
      const int qd = inc[p];
      const int64_t c = qd / ND;
      const int li = qd % ND;
      if (lane < ND) {
        const int dof = elem_dof[c * ND + lane];
        int slot = 0;
        if (dof != (int)row) {
          int lo = 1, hi = R;  // first position >= dof in the sorted part
          while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (ucol[mid] < dof) lo = mid + 1; else hi = mid;
          }
          slot = lo;
        }
        const int64_t src = (c * ND + li) * ND + lane;
        accK[slot] += eK[src];
        if (eM != nullptr) accM[slot] += eM[src];
      }
      __syncwarp();
    }
    for (int t = lane; t < R; t += 32) {
      vK[r0 + t] = accK[t];
      if (vM != nullptr) vM[r0 + t] = accM[t];
    }
    __syncwarp();
  }
}

// ---------------------------------------------------- Dirichlet elimination
// Pull form of BoundaryConditionAdmin::apply: a Dirichlet row gets
// f_i = a_ii g_i and zero off-diagonals; every other row subtracts
// a_ki (a_ii g_i) / a_ii for its Dirichlet columns in ascending column order
// (the order the reference's loop over i visits them) and zeroes them.
__global__ void k_apply_dirichlet(int64_t n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                  double* __restrict__ vals, double* __restrict__ f, const int* __restrict__ dir,
                                  const double* __restrict__ g, int symmetric) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int b = rowptr[k], e = rowptr[k + 1];
  if (dir[k]) {
    f[k] = vals[b] * (g ? g[k] : 0.0);
    for (int j = b + 1; j < e; ++j) vals[j] = 0.0;
    return;
  }
  if (!symmetric) return;
  double fk = f[k];
  for (int j = b + 1; j < e; ++j) {
    const int i = cols[j];
    if (!dir[i]) continue;
    const double aii = vals[rowptr[i]];
    const double fi = aii * (g ? g[i] : 0.0);
    fk -= vals[j] * fi / aii;
    vals[j] = 0.;
  }
  f[k] = fk;
}

QuadRule make_rule(int dim, int acc) {
  QuadRule q{};
  const double* pts;
  int n, stride = dim + 1;
  if (dim == 2) {
    AFP_REQUIRE(acc >= 0 && acc <= AFP_TRI_QUAD_MAX_ACC, AFP_ERR_UNSUPPORTED, "triangle quadrature accuracy out of range");
    int r = AFP_TRI_QUAD_RULE_OF_ACC[acc];
    pts = AFP_TRI_QUAD_POINTS[AFP_TRI_QUAD_OFFSET[r]];
    n = AFP_TRI_QUAD_OFFSET[r + 1] - AFP_TRI_QUAD_OFFSET[r];
  } else {
    AFP_REQUIRE(acc >= 0 && acc <= AFP_TET_QUAD_MAX_ACC, AFP_ERR_UNSUPPORTED, "tetrahedron quadrature accuracy out of range");
    int r = AFP_TET_QUAD_RULE_OF_ACC[acc];
    pts = AFP_TET_QUAD_POINTS[AFP_TET_QUAD_OFFSET[r]];
    n = AFP_TET_QUAD_OFFSET[r + 1] - AFP_TET_QUAD_OFFSET[r];
  }
  AFP_REQUIRE(n <= 64, AFP_ERR_UNSUPPORTED, "quadrature rule too large");
  q.n = n;
  for (int l = 0; l < n; ++l)
    for (int c = 0; c < stride; ++c) q.p[l][c] = pts[l * stride + c];
  return q;
}

template <int DIM, int DEG>
void element_matrices(const afp_space* sp, const QuadRule& q, const double* coef, bool mass, double* out) {
  const afp_context* ctx = sp->ctx;
  unsigned grid = grid_for(sp->n_cell, 128);
  if (mass)
    k_element_matrix<DIM, DEG, true><<<grid, 128, 0, ctx->stream>>>(sp->coords.get(), sp->cells.get(), sp->n_cell, q,
                                                                    nullptr, out);
  else
    k_element_matrix<DIM, DEG, false><<<grid, 128, 0, ctx->stream>>>(sp->coords.get(), sp->cells.get(), sp->n_cell, q,
                                                                     coef, out);
  check_launch(ctx, "element matrices");
}

void element_matrices(const afp_space* sp, int acc, const double* coef, bool mass, double* out) {
  QuadRule q = make_rule(sp->dim, acc);
  if (sp->dim == 2 && sp->degree == 1) element_matrices<2, 1>(sp, q, coef, mass, out);
  else if (sp->dim == 2 && sp->degree == 2) element_matrices<2, 2>(sp, q, coef, mass, out);
  else if (sp->dim == 3 && sp->degree == 1) element_matrices<3, 1>(sp, q, coef, mass, out);
  else element_matrices<3, 2>(sp, q, coef, mass, out);
}

template <int DIM, int DEG>
void element_rhs(const afp_space* sp, int src, int64_t c0, int64_t c1, const QuadRule& q, const double* data,
                 int n_gauss, double* terms, double* points) {
  const afp_context* ctx = sp->ctx;
  const unsigned grid = grid_for(c1 - c0, 128);
  const double* co = sp->coords.get();
  const int* ce = sp->cells.get();
  const int* ed = sp->elem_dof.get();
  if (src == SRC_POINT_VALUES)
    k_element_rhs<DIM, DEG, SRC_POINT_VALUES><<<grid, 128, 0, ctx->stream>>>(co, ce, ed, c0, c1, q, data, n_gauss,
                                                                             terms, points);
  else if (src == SRC_FEM_FUNCTION)
    k_element_rhs<DIM, DEG, SRC_FEM_FUNCTION><<<grid, 128, 0, ctx->stream>>>(co, ce, ed, c0, c1, q, data, n_gauss,
                                                                             terms, points);
  else
    k_element_rhs<DIM, DEG, SRC_GAUSSIANS><<<grid, 128, 0, ctx->stream>>>(co, ce, ed, c0, c1, q, data, n_gauss,
                                                                          terms, points);
  check_launch(ctx, "element right-hand sides");
}

void element_rhs(const afp_space* sp, int src, int64_t c0, int64_t c1, const QuadRule& q, const double* data,
                 int n_gauss, double* terms, double* points) {
  if (sp->dim == 2 && sp->degree == 1) element_rhs<2, 1>(sp, src, c0, c1, q, data, n_gauss, terms, points);
  else if (sp->dim == 2 && sp->degree == 2) element_rhs<2, 2>(sp, src, c0, c1, q, data, n_gauss, terms, points);
  else if (sp->dim == 3 && sp->degree == 1) element_rhs<3, 1>(sp, src, c0, c1, q, data, n_gauss, terms, points);
  else element_rhs<3, 2>(sp, src, c0, c1, q, data, n_gauss, terms, points);
}

template <int ND>
void build_pattern_nd(const afp_space* sp, Pattern& pat) {
  const afp_context* ctx = sp->ctx;
  int cap = 1;
  while (cap < sp->max_inc * ND) cap <<= 1;
  int wpb = 4;
  while (wpb > 1 && (size_t)wpb * cap * sizeof(int) > 96 * 1024) wpb >>= 1;
  size_t smem = (size_t)wpb * cap * sizeof(int);
  AFP_REQUIRE(smem <= 200 * 1024, AFP_ERR_UNSUPPORTED, "a DOF touches too many cells for the pattern kernel");
  AFP_CUDA(cudaFuncSetAttribute(k_pattern<ND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  unsigned grid = (unsigned)std::min<int64_t>((sp->n_dof + wpb - 1) / wpb, (int64_t)ctx->sm_count * 32);
  DevBuf<int> row_len(ctx, sp->n_dof);
  k_pattern<ND><<<grid, wpb * 32, smem, ctx->stream>>>(sp->n_dof, sp->inc_ptr.get(), sp->inc.get(), sp->elem_dof.get(),
                                                       cap, row_len.get(), nullptr, nullptr);
  check_launch(ctx, "pattern count");
  pat.m = pat.n = sp->n_dof;
  pat.rowptr.alloc(ctx, sp->n_dof + 1);
  pat.nnz = exclusive_scan(ctx, row_len.get(), pat.rowptr.get(), sp->n_dof);
  pat.cols.alloc(ctx, pat.nnz);
  k_pattern<ND><<<grid, wpb * 32, smem, ctx->stream>>>(sp->n_dof, sp->inc_ptr.get(), sp->inc.get(), sp->elem_dof.get(),
                                                       cap, nullptr, pat.rowptr.get(), pat.cols.get());
  check_launch(ctx, "pattern fill");
}

template <int ND>
void gather_values_nd(const afp_space* sp, const Pattern& pat, const double* eK, const double* eM, double* vK,
                      double* vM) {
  const afp_context* ctx = sp->ctx;
  DevBuf<int> mx(ctx, 1);
  mx.zero();
  k_max_diff<<<grid_for(pat.m, BLOCK), BLOCK, 0, ctx->stream>>>(pat.rowptr.get(), pat.m, mx.get());
  check_launch(ctx, "max row");
  int rcap = 0;
  mx.download(&rcap, 1);
  sync(ctx);
  const int wpb = 4;
  size_t smem = (size_t)wpb * rcap * (2 * sizeof(double) + sizeof(int));
  AFP_REQUIRE(smem <= 200 * 1024, AFP_ERR_UNSUPPORTED, "matrix row too long for the scatter kernel");
  AFP_CUDA(cudaFuncSetAttribute(k_gather_values<ND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  unsigned grid = (unsigned)std::min<int64_t>((pat.m + wpb - 1) / wpb, (int64_t)ctx->sm_count * 32);
  k_gather_values<ND><<<grid, wpb * 32, smem, ctx->stream>>>(pat.m, sp->inc_ptr.get(), sp->inc.get(),
                                                             sp->elem_dof.get(), pat.rowptr.get(), pat.cols.get(), eK,
                                                             eM, vK, vM, rcap);
  check_launch(ctx, "scatter values");
}

void build_pattern(const afp_space* sp, Pattern& pat) {
  switch (sp->nd) {
    case 3: build_pattern_nd<3>(sp, pat); break;
    case 4: build_pattern_nd<4>(sp, pat); break;
    case 6: build_pattern_nd<6>(sp, pat); break;
    default: build_pattern_nd<10>(sp, pat); break;
  }
}

void gather_values(const afp_space* sp, const Pattern& pat, const double* eK, const double* eM, double* vK,
                   double* vM) {
  switch (sp->nd) {
    case 3: gather_values_nd<3>(sp, pat, eK, eM, vK, vM); break;
    case 4: gather_values_nd<4>(sp, pat, eK, eM, vK, vM); break;
    case 6: gather_values_nd<6>(sp, pat, eK, eM, vK, vM); break;
    default: gather_values_nd<10>(sp, pat, eK, eM, vK, vM); break;
  }
}

}  // namespace
}  // namespace afp

using namespace afp;

extern "C" {

namespace {

// checks the index arrays and builds the DOF -> (cell, local) incidence of a
// space whose cells and elem_dof are on the device
void finish_space(afp_space* sp) {
  afp_context* ctx = sp->ctx;
  const int64_t n_cell = sp->n_cell, n_dof = sp->n_dof;
  DevBuf<int> bad(ctx, 2);
  bad.zero();
  const int64_t ncd = n_cell * sp->nd, ncv = n_cell * sp->nv;
  k_check_range<<<grid_for(ncv, BLOCK), BLOCK, 0, ctx->stream>>>(sp->cells.get(), ncv, sp->n_vertex, bad.get());
  check_launch(ctx, "check cells");
  k_check_range<<<grid_for(ncd, BLOCK), BLOCK, 0, ctx->stream>>>(sp->elem_dof.get(), ncd, n_dof, bad.get() + 1);
  check_launch(ctx, "check dofs");
  int hb[2];
  bad.download(hb, 2);
  sync(ctx);
  AFP_REQUIRE(!hb[0], AFP_ERR_INVALID, "cell vertex index out of range");
  AFP_REQUIRE(!hb[1], AFP_ERR_INVALID, "element DOF index out of range");
  // DOF -> (cell, local) incidence, ascending cell order per DOF
  DevBuf<int> cnt(ctx, n_dof);
  cnt.zero();
  k_count<<<grid_for(ncd, BLOCK), BLOCK, 0, ctx->stream>>>(sp->elem_dof.get(), ncd, cnt.get());
  check_launch(ctx, "incidence count");
  sp->inc_ptr.alloc(ctx, n_dof + 1);
  exclusive_scan(ctx, cnt.get(), sp->inc_ptr.get(), n_dof);
  sp->inc.alloc(ctx, ncd);
  cnt.zero();
  k_fill_incidence<<<grid_for(ncd, BLOCK), BLOCK, 0, ctx->stream>>>(sp->elem_dof.get(), ncd, sp->inc_ptr.get(),
                                                                    cnt.get(), sp->inc.get());
  check_launch(ctx, "incidence fill");
  k_sort_lists<<<grid_for(n_dof, BLOCK), BLOCK, 0, ctx->stream>>>(sp->inc_ptr.get(), sp->inc.get(), n_dof);
  check_launch(ctx, "incidence sort");
  DevBuf<int> mx(ctx, 1);
  mx.zero();
  k_max_diff<<<grid_for(n_dof, BLOCK), BLOCK, 0, ctx->stream>>>(sp->inc_ptr.get(), n_dof, mx.get());
  check_launch(ctx, "max incidence");
  mx.download(&sp->max_inc, 1);
  sync(ctx);
}

std::unique_ptr<afp_space> new_space(afp_context* ctx, int dim, int degree, int64_t n_vertex, const double* coords,
                                     int64_t n_cell, const int32_t* cells) {
  AFP_REQUIRE((dim == 2 || dim == 3) && (degree == 1 || degree == 2), AFP_ERR_UNSUPPORTED,
              "only P1/P2 on triangles and tetrahedra");
  AFP_REQUIRE(n_vertex > 0 && n_cell > 0, AFP_ERR_INVALID, "empty mesh");
  auto sp = std::make_unique<afp_space>();
  sp->ctx = ctx;
  sp->dim = dim;
  sp->degree = degree;
  sp->nv = dim + 1;
  sp->nd = dim == 2 ? 3 * degree : (degree == 1 ? 4 : 10);
  sp->n_vertex = n_vertex;
  sp->n_cell = n_cell;
  AFP_REQUIRE(n_cell * sp->nd < INT32_MAX, AFP_ERR_UNSUPPORTED, "more than 2^31 cell DOFs");
  sp->coords.alloc(ctx, n_vertex * dim);
  sp->cells.alloc(ctx, n_cell * sp->nv);
  sp->coords.upload(coords, n_vertex * dim);
  sp->cells.upload(cells, n_cell * sp->nv);
  return sp;
}

}  // namespace

afp_status afp_space_create(afp_context* ctx, int dim, int degree, int64_t n_vertex, const double* coords,
                            int64_t n_cell, const int32_t* cells, int64_t n_dof, const int32_t* elem_dof,
                            afp_space** out) {
  return guarded([&] {
    AFP_REQUIRE(ctx && coords && cells && elem_dof && out, AFP_ERR_INVALID, "null argument");
    AFP_REQUIRE(n_dof > 0, AFP_ERR_INVALID, "empty mesh");
    bind(ctx);
    auto sp = new_space(ctx, dim, degree, n_vertex, coords, n_cell, cells);
    sp->n_dof = n_dof;
    sp->elem_dof.alloc(ctx, n_cell * sp->nd);
    sp->elem_dof.upload(elem_dof, n_cell * sp->nd);
    finish_space(sp.get());
    *out = sp.release();
  });
}

afp_status afp_space_create_numbered(afp_context* ctx, int dim, int degree, int64_t n_vertex, const double* coords,
                                     int64_t n_cell, const int32_t* cells, const int32_t* vertex_bmark,
                                     afp_space** out) {
  return guarded([&] {
    AFP_REQUIRE(ctx && coords && cells && out, AFP_ERR_INVALID, "null argument");
    bind(ctx);
    auto sp = new_space(ctx, dim, degree, n_vertex, coords, n_cell, cells);
    const int64_t ncv = n_cell * sp->nv, T = sp->nd, nt = n_cell * T;
    DevBuf<int> bad(ctx, 1);
    bad.zero();
    k_check_range<<<grid_for(ncv, BLOCK), BLOCK, 0, ctx->stream>>>(sp->cells.get(), ncv, n_vertex, bad.get());
    check_launch(ctx, "check cells");
    int hb = 0;
    bad.download(&hb, 1);
    sync(ctx);
    AFP_REQUIRE(!hb, AFP_ERR_INVALID, "cell vertex index out of range");
    // vertex -> (cell, local vertex) incidence, ascending cell order
    DevBuf<int> vcnt(ctx, n_vertex), vptr(ctx, n_vertex + 1), vinc(ctx, ncv);
    vcnt.zero();
    k_count<<<grid_for(ncv, BLOCK), BLOCK, 0, ctx->stream>>>(sp->cells.get(), ncv, vcnt.get());
    exclusive_scan(ctx, vcnt.get(), vptr.get(), n_vertex);
    vcnt.zero();
    k_fill_incidence<<<grid_for(ncv, BLOCK), BLOCK, 0, ctx->stream>>>(sp->cells.get(), ncv, vptr.get(), vcnt.get(),
                                                                      vinc.get());
    k_sort_lists<<<grid_for(n_vertex, BLOCK), BLOCK, 0, ctx->stream>>>(vptr.get(), vinc.get(), n_vertex);
    check_launch(ctx, "vertex incidence");
    DevBuf<int> first(ctx, nt), is_first(ctx, nt), rank(ctx, nt + 1);
    k_first_touch<<<grid_for(nt, BLOCK), BLOCK, 0, ctx->stream>>>(dim, degree, n_cell, sp->cells.get(), vptr.get(),
                                                                  vinc.get(), first.get(), is_first.get());
    check_launch(ctx, "first touch");
    sp->n_dof = exclusive_scan(ctx, is_first.get(), rank.get(), nt);
    DevBuf<int> vmark;
    if (vertex_bmark) {
      vmark.alloc(ctx, n_vertex);
      vmark.upload(vertex_bmark, n_vertex);
    }
    sp->elem_dof.alloc(ctx, nt);
    sp->dof_bmark.alloc(ctx, sp->n_dof);
    sp->dof_point.alloc(ctx, sp->n_dof * dim);
    k_number_dofs<<<grid_for(nt, BLOCK), BLOCK, 0, ctx->stream>>>(
        dim, degree, n_cell, sp->cells.get(), sp->coords.get(), vertex_bmark ? vmark.get() : nullptr, first.get(),
        rank.get(), sp->elem_dof.get(), sp->dof_bmark.get(), sp->dof_point.get());
    check_launch(ctx, "DOF numbering");
    finish_space(sp.get());
    *out = sp.release();
  });
}

afp_status afp_space_info(const afp_space* sp, int64_t* n_dof, int* nd) {
  return guarded([&] {
    AFP_REQUIRE(sp, AFP_ERR_INVALID, "null argument");
    if (n_dof) *n_dof = sp->n_dof;
    if (nd) *nd = sp->nd;
  });
}

afp_status afp_space_download_dofs(const afp_space* sp, int32_t* elem_dof, int32_t* dof_bmark, double* dof_point) {
  return guarded([&] {
    AFP_REQUIRE(sp, AFP_ERR_INVALID, "null argument");
    AFP_REQUIRE((!dof_bmark && !dof_point) || sp->dof_bmark.size() > 0, AFP_ERR_INVALID,
                "boundary marks and points exist only for spaces numbered by afp_space_create_numbered");
    bind(sp->ctx);
    if (elem_dof) sp->elem_dof.download(elem_dof, sp->n_cell * sp->nd);
    if (dof_bmark) sp->dof_bmark.download(dof_bmark, sp->n_dof);
    if (dof_point) sp->dof_point.download(dof_point, sp->n_dof * sp->dim);
    sync(sp->ctx);
  });
}

afp_status afp_quadrature_points(afp_space* sp, int acc, int* n_q, double* points) {
  return guarded([&] {
    AFP_REQUIRE(sp, AFP_ERR_INVALID, "null argument");
    bind(sp->ctx);
    const QuadRule q = make_rule(sp->dim, acc);
    if (n_q) *n_q = q.n;
    if (!points) return;
    DevBuf<double> pts(sp->ctx, sp->n_cell * q.n * sp->dim);
    element_rhs(sp, SRC_POINT_VALUES, 0, sp->n_cell, q, nullptr, 0, nullptr, pts.get());
    pts.download(points, sp->n_cell * q.n * sp->dim);
    sync(sp->ctx);
  });
}

afp_status afp_l2_discretize(afp_space* sp, int acc, int source, const double* data, int64_t n_data, double* f1) {
  return guarded([&] {
    AFP_REQUIRE(sp && data && f1, AFP_ERR_INVALID, "null argument");
    bind(sp->ctx);
    afp_context* ctx = sp->ctx;
    const QuadRule q = make_rule(sp->dim, acc);
    int n_gauss = 0;
    if (source == SRC_POINT_VALUES)
      AFP_REQUIRE(n_data == sp->n_cell * q.n, AFP_ERR_INVALID, "point values: n_data must be n_cell * n_q");
    else if (source == SRC_FEM_FUNCTION)
      AFP_REQUIRE(n_data == sp->n_dof, AFP_ERR_INVALID, "FEM function: n_data must be n_dof");
    else if (source == SRC_GAUSSIANS) {
      AFP_REQUIRE(n_data >= 0 && n_data % (sp->dim + 2) == 0, AFP_ERR_INVALID,
                  "Gaussians: n_data must be a multiple of dim + 2");
      n_gauss = (int)(n_data / (sp->dim + 2));
    } else
      fail(AFP_ERR_INVALID, "unknown source");
    DevBuf<double> d(ctx, n_data > 0 ? n_data : 1), out(ctx, sp->n_dof);
    d.upload(data, n_data);
    out.zero();
    // terms of at most ~256 MB at a time; cells in ascending chunks keep the per-DOF order
    const int64_t per_cell = (int64_t)q.n * sp->nd;
    const int64_t chunk = std::max<int64_t>(1, ((int64_t)256 << 20) / 8 / per_cell);
    DevBuf<double> terms(ctx, std::min(chunk, sp->n_cell) * per_cell);
    for (int64_t c0 = 0; c0 < sp->n_cell; c0 += chunk) {
      const int64_t c1 = std::min(sp->n_cell, c0 + chunk);
      element_rhs(sp, source, c0, c1, q, d.get(), n_gauss, terms.get(), nullptr);
      k_gather_rhs<<<grid_for(sp->n_dof, BLOCK), BLOCK, 0, ctx->stream>>>(sp->n_dof, sp->inc_ptr.get(),
                                                                          sp->inc.get(), sp->nd, q.n, c0, c1,
                                                                          terms.get(), out.get());
      check_launch(ctx, "right-hand side gather");
    }
    out.download(f1, sp->n_dof);
    sync(ctx);
  });
}

afp_status afp_space_destroy(afp_space* sp) {
  return guarded([&] {
    if (!sp) return;
    bind(sp->ctx);
    sync(sp->ctx);
    delete sp;
  });
}

afp_status afp_assemble(afp_space* sp, const afp_assemble_opts* opts, afp_matrix** stiff, afp_matrix** mass) {
  return guarded([&] {
    AFP_REQUIRE(sp && opts && stiff, AFP_ERR_INVALID, "null argument");
    afp_context* ctx = sp->ctx;
    bind(ctx);
    const int64_t esz = sp->n_cell * sp->nd * sp->nd;
    DevBuf<double> coef;
    if (opts->coef) {
      coef.alloc(ctx, sp->n_cell);
      coef.upload(opts->coef, sp->n_cell);
    }
    DevBuf<double> eK(ctx, esz), eM;
    element_matrices(sp, opts->acc_stiff, opts->coef ? coef.get() : nullptr, false, eK.get());
    if (mass) {
      eM.alloc(ctx, esz);
      element_matrices(sp, opts->acc_mass, nullptr, true, eM.get());
    }
    auto pat = std::make_shared<Pattern>();
    build_pattern(sp, *pat);
    auto K = std::make_unique<afp_matrix>();
    K->ctx = ctx;
    K->pat = pat;
    K->vals.alloc(ctx, pat->nnz);
    std::unique_ptr<afp_matrix> M;
    if (mass) {
      M = std::make_unique<afp_matrix>();
      M->ctx = ctx;
      M->pat = pat;
      M->vals.alloc(ctx, pat->nnz);
    }
    gather_values(sp, *pat, eK.get(), mass ? eM.get() : nullptr, K->vals.get(), mass ? M->vals.get() : nullptr);
    sync(ctx);
    *stiff = K.release();
    if (mass) *mass = M.release();
  });
}

afp_status afp_apply_dirichlet(afp_matrix* a, double* f, const int32_t* dirichlet, const double* g,
                               int preserve_symmetry) {
  return guarded([&] {
    AFP_REQUIRE(a && f && dirichlet, AFP_ERR_INVALID, "null argument");
    AFP_REQUIRE(a->pat->m == a->pat->n, AFP_ERR_INVALID, "matrix is not square");
    afp_context* ctx = a->ctx;
    bind(ctx);
    const int64_t n = a->pat->m;
    DevBuf<double> df(ctx, n), dg;
    DevBuf<int> dd(ctx, n);
    df.upload(f, n);
    dd.upload(dirichlet, n);
    if (g) {
      dg.alloc(ctx, n);
      dg.upload(g, n);
    }
    k_apply_dirichlet<<<grid_for(n, BLOCK), BLOCK, 0, ctx->stream>>>(n, a->pat->rowptr.get(), a->pat->cols.get(),
                                                                     a->vals.get(), df.get(), dd.get(),
                                                                     g ? dg.get() : nullptr, preserve_symmetry);
    check_launch(ctx, "dirichlet");
    df.download(f, n);
    sync(ctx);
  });
}

}  // extern "C"
