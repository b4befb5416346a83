// Drop-in replacement for AFEPack's src/BilinearOperator.cpp that assembles
// StiffMatrix and MassMatrix on a GB300 through the afepack_gb300 C ABI.  It
// is compiled inside AFEPack's own build in place of src/BilinearOperator.cpp,
// against the UNCHANGED headers (BilinearOperator.h / .templates.h), and
// linked with libafepack_gb300.so.
//
// BilinearOperator<D, double, double, D, D, D>::build() (include/AFEPack/
// BilinearOperator.templates.h:56-60) is specialised for D = 2, 3.  When the
// object's exact dynamic type is StiffMatrix<D, double>, MassMatrix<D,
// double> or VarCoeffStiffMatrix<D> (one coefficient per element,
// VarCoeffStiffMatrix.h) -- not a user subclass that overrides
// getElementMatrix -- and every
// element's template takes its basis functions from AFEPack's Lagrange P1/P2
// triangle or tetrahedron plugin (libtriangle.{1,2}.bas_fun.so,
// libtetrahedron.{1,2}.bas_fun.so, read from the template's own basis
// function records), the mesh and DOF map go to afp_space_create,
// afp_assemble builds the matrix on the GPU (pattern and values bitwise the
// reference's), and the result is copied into the object's own
// SparsityPattern and SparseMatrix storage, which then hold exactly what the
// reference's build() would have produced.  Any other scalar operator of
// these two instantiations (a user getElementMatrix, another template such as
// the discontinuous P1 triangle, which also has 3 DOFs) is refused with a
// message and abort(): this replacement has no CPU path for them.  GPU
// failures abort too (the reference's own failures assert or abort).
//
// The file also provides the explicit instantiations that the replaced file
// provides, so the library links unchanged (the vector-valued operators keep
// the header's generic build()).  AFP_DEVICE selects the GPU.
#include <AFEPack/BilinearOperator.templates.h>

#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>
#include <typeinfo>
#include <vector>

#include "VarCoeffStiffMatrix.h"
#include "afepack_gb300.h"

AFEPACK_OPEN_NAMESPACE

namespace {

afp_context* g_ctx = nullptr;

void check(afp_status s, const char* what) {
  if (s == AFP_OK) return;
  std::cerr << "afepack_gb300: " << what << " failed: " << afp_status_string(s) << " (" << afp_last_error()
            << ")" << std::endl;
  abort();
}

afp_context* context() {
  if (g_ctx == nullptr) {
    const char* dev = std::getenv("AFP_DEVICE");
    check(afp_context_create(dev ? std::atoi(dev) : 0, &g_ctx), "afp_context_create");
  }
  return g_ctx;
}

// Polynomial degree of the Lagrange template whose basis functions come from
// the plugin library `lib` on the D-simplex (0 if it is not one the GPU path
// covers).  The library name is the first field of a basis function record
// as BasisFunction's stream output writes it (TemplateElement.h:181-191).
int lagrange_degree(int D, const std::string& lib) {
  const std::string base = lib.substr(lib.find_last_of('/') == std::string::npos ? 0 : lib.find_last_of('/') + 1);
  if (D == 2) return base == "libtriangle.1.bas_fun.so" ? 1 : base == "libtriangle.2.bas_fun.so" ? 2 : 0;
  return base == "libtetrahedron.1.bas_fun.so" ? 1 : base == "libtetrahedron.2.bas_fun.so" ? 2 : 0;
}

template <class BF>
std::string plugin_library(const BF& bf) {
  std::ostringstream os;
  os << bf;  // interpolation point, then "library\tvalue\tgradient"
  std::istringstream is(os.str());
  std::string tok, lib;
  while (is >> tok)
    if (tok.size() > 3 && tok.compare(tok.size() - 3, 3, ".so") == 0) lib = tok;
  return lib;
}

// Degree of the template every element uses when it is one P1 or P2 plugin
// throughout, else 0.
template <int D, class Space>
int space_degree(const Space& sp) {
  const int ne = sp.n_element();
  int degree = -1;
  for (int e = 0; e < ne; ++e) {
    const auto& tmpl = sp.element(e).templateElement();
    const int nd = (int)tmpl.n_dof();
    int deg = -1;
    for (int i = 0; i < nd; ++i) {
      const int d = lagrange_degree(D, plugin_library(tmpl.basisFunction(i)));
      if (d == 0 || (deg >= 0 && d != deg)) return 0;
      deg = d;
    }
    const int expect = D == 2 ? (deg == 1 ? 3 : 6) : (deg == 1 ? 4 : 10);
    if (nd != expect || (degree >= 0 && deg != degree)) return 0;
    degree = deg;
  }
  return degree < 0 ? 0 : degree;
}

// Assembles `op` on the GPU when it is a plain StiffMatrix / MassMatrix on a
// P1/P2 simplex space; returns false (nothing done) otherwise.
template <int D>
bool gpu_build(BilinearOperator<D, double, double, D, D, D>& op) {
  const bool varcoef = typeid(op) == typeid(VarCoeffStiffMatrix<D>);
  const bool stiff = varcoef || typeid(op) == typeid(StiffMatrix<D, double, D, D>);
  const bool mass = typeid(op) == typeid(MassMatrix<D, double, D, D>);
  if (!stiff && !mass) return false;
  FEMSpace<double, D, D, D>* sp = op.FEMSpace0();
  if (sp == nullptr || sp != op.FEMSpace1()) return false;
  const int ne = sp->n_element();
  if (ne == 0) return false;
  const int degree = space_degree<D>(*sp);
  if (degree == 0) return false;
  const int nd = (int)sp->element(0).n_dof();
  Mesh<D, D>& mesh = sp->mesh();
  std::vector<int32_t> cells((size_t)ne * (D + 1)), elem_dof((size_t)ne * nd);
  for (int e = 0; e < ne; ++e) {
    const auto& el = sp->element(e);
    if ((int)el.n_dof() != nd) return false;  // mixed templates: not this path
    const GeometryBM& geo = el.geometry();
    if (geo.n_vertex() != D + 1) return false;
    // vertex point numbers in the element's own vertex order (as the
    // reference's Element::buildVertexArray reads them)
    for (int i = 0; i <= D; ++i) cells[(size_t)e * (D + 1) + i] = mesh.geometry(0, geo.vertex(i)).vertex(0);
    const std::vector<int>& dof = el.dof();
    for (int l = 0; l < nd; ++l) elem_dof[(size_t)e * nd + l] = dof[l];
  }
  const int nv = mesh.n_point();
  std::vector<double> coords((size_t)nv * D);
  for (int i = 0; i < nv; ++i)
    for (int k = 0; k < D; ++k) coords[(size_t)i * D + k] = mesh.point(i)[k];
  const int64_t n = sp->n_dof();

  afp_space* space = nullptr;
  check(afp_space_create(context(), D, degree, nv, coords.data(), ne, cells.data(), n, elem_dof.data(), &space),
        "afp_space_create");
  const double* coef = nullptr;
  if (varcoef) {
    const std::vector<double>& c = static_cast<VarCoeffStiffMatrix<D>&>(op).coefficient();
    if ((int64_t)c.size() != ne) {
      std::cerr << "afepack_gb300: VarCoeffStiffMatrix has " << c.size() << " coefficients for " << ne
                << " elements" << std::endl;
      abort();
    }
    coef = c.data();
  }
  afp_assemble_opts opts{op.algebricAccuracy(), op.algebricAccuracy(), coef};
  afp_matrix *K = nullptr, *M = nullptr;
  check(afp_assemble(space, &opts, &K, mass ? &M : nullptr), "afp_assemble");
  afp_matrix* A = stiff ? K : M;
  int64_t m = 0, nc = 0, nnz = 0;
  check(afp_matrix_info(A, &m, &nc, &nnz), "afp_matrix_info");
  std::vector<int32_t> rowptr(m + 1), cols(nnz);
  std::vector<double> vals(nnz);
  check(afp_matrix_download(A, rowptr.data(), cols.data(), vals.data()), "afp_matrix_download");
  afp_matrix_destroy(K);
  if (M) afp_matrix_destroy(M);
  afp_space_destroy(space);

  // the object's own storage: exact row lengths, the diagonal first (set by
  // reinit for a square pattern), the other columns added in ascending order
  op.nDof0() = (int)n;
  op.nDof1() = (int)n;
  SparsityPattern& pattern = op.getSparsityPattern();
  std::vector<unsigned int> lengths(m);
  for (int64_t i = 0; i < m; ++i) lengths[i] = (unsigned int)(rowptr[i + 1] - rowptr[i]);
  pattern.reinit(m, nc, lengths);
  for (int64_t i = 0; i < m; ++i)
    for (int32_t q = rowptr[i]; q < rowptr[i + 1]; ++q)
      if (cols[q] != i) pattern.add(i, cols[q]);
  pattern.compress();
  const size_t* cn = pattern.get_column_numbers();
  for (int64_t q = 0; q < nnz; ++q)
    if (cn[q] != (size_t)cols[q]) {
      std::cerr << "afepack_gb300: assembled pattern does not match the SparsityPattern layout" << std::endl;
      abort();
    }
  op.SparseMatrix<double>::reinit(pattern);
  for (int64_t q = 0; q < nnz; ++q) op.global_entry(q) = vals[q];
  return true;
}

}  // namespace

// An operator the GPU path does not cover: refused (this replacement has no CPU path).
[[noreturn]] static void refuse(const char* type) {
  std::cerr << "afepack_gb300: BilinearOperator::build() of " << type
            << " is not on the GPU path (StiffMatrix / MassMatrix on AFEPack's Lagrange P1/P2 triangle or "
               "tetrahedron templates); link the reference's src/BilinearOperator.cpp for other operators"
            << std::endl;
  abort();
}

template <>
void BilinearOperator<2, double, double, 2, 2, 2>::build() {
  if (!gpu_build<2>(*this)) refuse(typeid(*this).name());
}

template <>
void BilinearOperator<3, double, double, 3, 3, 3>::build() {
  if (!gpu_build<3>(*this)) refuse(typeid(*this).name());
}

// The instantiations of the replaced src/BilinearOperator.cpp: scalar
// operators (with the L2 inner product, mass and stiffness matrices) and the
// operators between scalar and 2- or 3-vector valued spaces, for D = 1, 2, 3.
#define AFP_GB300_SCALAR(D)                                  \
  template class BilinearOperator<D, double, double, D, D, D>; \
  template class L2InnerProduct<D, double, double, D, D, D>;   \
  template class MassMatrix<D, double, D, D>;                  \
  template class StiffMatrix<D, double, D, D>;
#define AFP_GB300_VECTOR(D, L)                                                          \
  template class BilinearOperator<D, nVector<L, double>, double, D, D, D>;              \
  template class BilinearOperator<D, double, nVector<L, double>, D, D, D>;              \
  template class BilinearOperator<D, nVector<L, double>, nVector<L, double>, D, D, D>;

AFP_GB300_SCALAR(1)
AFP_GB300_SCALAR(2)
AFP_GB300_SCALAR(3)
AFP_GB300_VECTOR(1, 2)
AFP_GB300_VECTOR(2, 2)
AFP_GB300_VECTOR(3, 2)
AFP_GB300_VECTOR(1, 3)
AFP_GB300_VECTOR(2, 3)
AFP_GB300_VECTOR(3, 3)

#undef AFP_GB300_VECTOR
#undef AFP_GB300_SCALAR

AFEPACK_CLOSE_NAMESPACE
