// Oracle harness around the UNMODIFIED AFEPack sources (test infrastructure:
// only tests, the smoke check and the bench's CPU-baseline leg run it).
//
// It drives the reference's own call sequence for the elliptic-solve path,
// the one of examples/poisson_equation/poisson_equation.cpp:42-74:
//   Mesh::readData -> FEMSpace::buildElement/buildDof/buildDofBoundaryMark
//   -> StiffMatrix / MassMatrix ::build  (BilinearOperator.templates.h:56-227)
//   -> b = M f  (SparseMatrix::vmult)
//   -> BoundaryConditionAdmin::apply     (FEMSpace.templates.h:1338-1366)
//   -> AMGSolver::reinit                 (src/AMGSolver.cpp:384-438)
//   -> AMGSolver::solve / example-style PCG with one V-cycle per iteration
//      (examples/FAST/src/poisson_solver_comparison_afepack.cpp:197-253)
// and writes every intermediate as .npy files so the GPU path can be compared
// entry by entry.  A variable coefficient is applied per element, as
// examples/elliptic_equation/EllipticEquation.cpp:337-383 does in its
// getElementMatrix override.
//
// usage: ref_driver key=value ...
//   mesh=FILE dim=2|3 deg=1|2 acc_stiff=N acc_mass=N out=DIR
//   [coef=FILE.f64] [f=FILE.f64] [amg=0|1] [dump_levels=0|1]
//   [vcycles=K] [pcg_tol=T] [pcg_maxit=N] [smooth=3]
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <list>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#define private public
#include <AFEPack/AMGSolver.h>
#undef private
#include <AFEPack/Geometry.h>
#include <AFEPack/TemplateElement.h>
#include <AFEPack/FEMSpace.h>
#include <AFEPack/BilinearOperator.h>
#include <AFEPack/Operator.h>

using namespace AFEPack;

namespace {

std::map<std::string, std::string> g_args;

std::string arg(const char* k, const char* def = "") {
  auto it = g_args.find(k);
  return it == g_args.end() ? std::string(def) : it->second;
}

template <class T> const char* npy_descr();
template <> const char* npy_descr<double>() { return "<f8"; }
template <> const char* npy_descr<int64_t>() { return "<i8"; }
template <> const char* npy_descr<int32_t>() { return "<i4"; }

template <class T>
void save_npy(const std::string& path, const T* data, const std::vector<size_t>& shape) {
  std::string sh = "(";
  size_t count = 1;
  for (size_t i = 0; i < shape.size(); ++i) {
    sh += std::to_string(shape[i]);
    sh += (shape.size() == 1 || i + 1 < shape.size()) ? "," : "";
    if (i + 1 < shape.size()) sh += " ";
    count *= shape[i];
  }
  sh += ")";
  std::string dict = std::string("{'descr': '") + npy_descr<T>() +
                     "', 'fortran_order': False, 'shape': " + sh + ", }";
  size_t total = 10 + dict.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  dict += std::string(pad, ' ');
  dict += '\n';
  std::ofstream os(path, std::ios::binary);
  os.write("\x93NUMPY\x01\x00", 8);
  uint16_t hl = (uint16_t)dict.size();
  os.write((const char*)&hl, 2);
  os.write(dict.data(), dict.size());
  os.write((const char*)data, sizeof(T) * count);
}

std::vector<double> load_f64(const std::string& path, size_t n) {
  std::vector<double> v(n, 0.0);
  std::ifstream is(path, std::ios::binary);
  if (!is) { std::cerr << "cannot read " << path << "\n"; std::exit(2); }
  is.read((char*)v.data(), sizeof(double) * n);
  return v;
}

void dump_csr(const std::string& dir, const std::string& name, const SparseMatrix<double>& A) {
  const SparsityPattern& sp = A.get_sparsity_pattern();
  size_t m = A.m();
  const size_t* rs = sp.get_rowstart_indices();
  const size_t* cn = sp.get_column_numbers();
  size_t nnz = rs[m];
  std::vector<int64_t> r(rs, rs + m + 1), c(cn, cn + nnz);
  std::vector<double> v(nnz);
  for (size_t k = 0; k < nnz; ++k) v[k] = A.global_entry(k);
  save_npy(dir + "/" + name + "_rowptr.npy", r.data(), {m + 1});
  save_npy(dir + "/" + name + "_cols.npy", c.data(), {nnz});
  save_npy(dir + "/" + name + "_vals.npy", v.data(), {nnz});
  int64_t shape[2] = {(int64_t)A.m(), (int64_t)A.n()};
  save_npy(dir + "/" + name + "_shape.npy", shape, {2});
}

double zero_fun(const double*) { return 0.0; }
// source of the L2Discretize fixture: a polynomial, so that any caller that
// evaluates it at the same points with the same operations gets the same bits
double poly_fun(const double* p) { return 1.0 + p[0] * p[1] - 2.0 * p[1] * p[1]; }

// Stiffness operator scaled by a per-element coefficient a_e.
template <int D>
class CoefStiff : public StiffMatrix<D, double> {
 public:
  const std::vector<double>* coef = nullptr;
  CoefStiff(FEMSpace<double, D>& sp) : StiffMatrix<D, double>(sp) {}
  void getElementMatrix(const Element<double, D>& e0, const Element<double, D>& e1,
                        const typename ActiveElementPairIterator<D>::State state) override {
    StiffMatrix<D, double>::getElementMatrix(e0, e1, state);
    if (coef == nullptr) return;
    double a = (*coef)[e0.index()];
    auto& K = this->elementMatrix();
    for (size_t j = 0; j < K.n_rows(); ++j)
      for (size_t k = 0; k < K.n_cols(); ++k) K(j, k) *= a;
  }
};

double secs(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

template <int D>
int run() {
  const std::string out = arg("out", ".");
  const int deg = std::atoi(arg("deg", "1").c_str());
  const int acc_stiff = std::atoi(arg("acc_stiff", D == 2 ? "4" : "2").c_str());
  const int acc_mass = std::atoi(arg("acc_mass", "4").c_str());
  const std::string base = D == 2 ? "triangle" : "tetrahedron";
  std::ostringstream js;
  js << "{";

  auto t0 = std::chrono::steady_clock::now();
  Mesh<D, D> mesh;
  mesh.readData(arg("mesh"));
  TemplateGeometry<D> tg;
  tg.readData(base + ".tmp_geo");
  CoordTransform<D, D> ct;
  ct.readData(base + ".crd_trs");
  TemplateDOF<D> td(tg);
  td.readData(base + "." + std::to_string(deg) + ".tmp_dof");
  BasisFunctionAdmin<double, D, D> bf(td);
  bf.readData(base + "." + std::to_string(deg) + ".bas_fun");
  std::vector<TemplateElement<double, D, D>> te(1);
  te[0].reinit(tg, td, ct, bf);
  auto t1 = std::chrono::steady_clock::now();
  FEMSpace<double, D> sp(mesh, te);
  const int ne = mesh.n_geometry(D);
  sp.element().resize(ne);
  for (int i = 0; i < ne; ++i) sp.element(i).reinit(sp, i, 0);
  sp.buildElement();
  sp.buildDof();
  sp.buildDofBoundaryMark();
  auto t2 = std::chrono::steady_clock::now();
  const size_t n = sp.n_dof();
  {
    const size_t nd = sp.element(0).dof().size();
    std::vector<int32_t> ed(ne * nd);
    for (int e = 0; e < ne; ++e)
      for (size_t l = 0; l < nd; ++l) ed[e * nd + l] = sp.element(e).dof()[l];
    save_npy(out + "/elem_dof.npy", ed.data(), {(size_t)ne, nd});
    std::vector<int32_t> bm(n);
    for (size_t i = 0; i < n; ++i) bm[i] = sp.dofBoundaryMark(i);
    save_npy(out + "/dof_bmark.npy", bm.data(), {n});
  }

  std::vector<double> coef;
  if (!arg("coef").empty()) coef = load_f64(arg("coef"), ne);
  CoefStiff<D> A(sp);
  if (!coef.empty()) A.coef = &coef;
  A.algebricAccuracy() = acc_stiff;
  A.build();
  auto t3 = std::chrono::steady_clock::now();
  MassMatrix<D, double> M(sp);
  M.algebricAccuracy() = acc_mass;
  M.build();
  auto t4 = std::chrono::steady_clock::now();
  dump_csr(out, "stiff", A);
  dump_csr(out, "mass", M);

  Vector<double> f(n), b(n);
  if (!arg("f").empty()) {
    std::vector<double> fv = load_f64(arg("f"), n);
    for (size_t i = 0; i < n; ++i) f(i) = fv[i];
  }
  M.vmult(b, f);
  save_npy(out + "/rhs_mass.npy", &b(0), {n});
  {
    // Operator::L2Discretize of a point function and of a FEM function
    Vector<double> l2;
    Operator::L2Discretize(&poly_fun, sp, l2, acc_mass);
    save_npy(out + "/l2_fun.npy", &l2(0), {n});
    FEMFunction<double, D> fu(sp);
    for (size_t i = 0; i < n; ++i) fu(i) = f(i);
    Vector<double> l2u;
    Operator::L2Discretize(fu, l2u, acc_mass);
    save_npy(out + "/l2_fem.npy", &l2u(0), {n});
  }

  FEMFunction<double, D> u(sp);
  BoundaryFunction<double, D> bc(BoundaryConditionInfo::DIRICHLET, 1, &zero_fun);
  BoundaryConditionAdmin<double, D> adm(sp);
  adm.add(bc);
  auto t5 = std::chrono::steady_clock::now();
  adm.apply(A, u, b);
  auto t6 = std::chrono::steady_clock::now();
  dump_csr(out, "system", A);
  save_npy(out + "/rhs.npy", &b(0), {n});
  js << "\"n_dof\": " << n << ", \"nnz\": " << A.n_nonzero_elements()
     << ", \"t_template\": " << secs(t0, t1) << ", \"t_femspace\": " << secs(t1, t2)
     << ", \"t_stiff_build\": " << secs(t2, t3) << ", \"t_mass_build\": " << secs(t3, t4)
     << ", \"t_apply\": " << secs(t5, t6);

  if (arg("amg", "0") == "1") {
    const int smooth = std::atoi(arg("smooth", "3").c_str());
    auto t7 = std::chrono::steady_clock::now();
    AMGSolver solver(A, 1.0e-12, smooth);
    auto t8 = std::chrono::steady_clock::now();
    js << ", \"t_amg_reinit\": " << secs(t7, t8) << ", \"n_project\": " << solver.n_project
       << ", \"most_project_full\": " << (solver.is_most_project_full ? 1 : 0) << ", \"levels\": [";
    for (u_int l = 0; l <= solver.n_project; ++l) {
      const auto* Al = solver.projected_matrix[l];
      js << (l ? ", " : "") << "[" << Al->m() << ", " << Al->n_nonzero_elements() << "]";
    }
    js << "]";
    if (arg("dump_levels", "0") == "1") {
      for (u_int l = 0; l < solver.n_project; ++l) {
        dump_csr(out, "P" + std::to_string(l), *solver.project_matrix[l]);
        dump_csr(out, "A" + std::to_string(l + 1), *solver.projected_matrix[l + 1]);
      }
      if (solver.is_most_project_full) {
        const size_t m = solver.M_n.n_rows();
        std::vector<double> inv(m * m);
        for (size_t i = 0; i < m; ++i)
          for (size_t j = 0; j < m; ++j) inv[i * m + j] = solver.M_n(i, j);
        save_npy(out + "/coarse_inverse.npy", inv.data(), {m, m});
      }
    }
    const int vcycles = std::atoi(arg("vcycles", "0").c_str());
    if (vcycles > 0) {
      Vector<double> x(n);
      auto t9 = std::chrono::steady_clock::now();
      solver.solve(x, b, 0.0, vcycles - 1, 1);  // runs step+1 cycles
      auto t10 = std::chrono::steady_clock::now();
      save_npy(out + "/x_vcycle.npy", &x(0), {n});
      js << ", \"t_vcycles\": " << secs(t9, t10) << ", \"vcycles\": " << vcycles;
    }
    const double pcg_tol = std::atof(arg("pcg_tol", "0").c_str());
    if (pcg_tol > 0) {
      const int maxit = std::atoi(arg("pcg_maxit", "500").c_str());
      auto t11 = std::chrono::steady_clock::now();
      Vector<double> x(n), r(b), z(n), p(n), ap(n);
      const double bn = std::max(b.l2_norm(), 1e-30);
      double rel = r.l2_norm() / bn;
      int it = 0;
      std::vector<double> hist{rel};
      if (rel > pcg_tol) {
        z = 0.0;
        solver.solve(z, r, 0.0, 0, 1);
        p = z;
        double rz = r.dot(z);
        for (it = 1; it <= maxit; ++it) {
          A.vmult(ap, p);
          const double alpha = rz / p.dot(ap);
          x.add(alpha, p);
          r.add(-alpha, ap);
          rel = r.l2_norm() / bn;
          hist.push_back(rel);
          if (rel <= pcg_tol) break;
          z = 0.0;
          solver.solve(z, r, 0.0, 0, 1);
          const double rz2 = r.dot(z);
          p.scale(rz2 / rz);
          p.add(1.0, z);
          rz = rz2;
        }
      }
      auto t12 = std::chrono::steady_clock::now();
      save_npy(out + "/x_pcg.npy", &x(0), {n});
      save_npy(out + "/pcg_history.npy", hist.data(), {hist.size()});
      js << ", \"t_pcg\": " << secs(t11, t12) << ", \"pcg_iters\": " << it
         << ", \"pcg_relres\": " << rel;
    }
  }
  if (arg("lazy", "0") == "1") {
    // AMGPreconditioner: lazyReinit -> lazyInit, vmult = iterate_step+1 V-cycles,
    // then a numeric re-setup for new values on the same pattern object.
    const int smooth = std::atoi(arg("smooth", "3").c_str());
    AMGPreconditioner pre(A, 2, smooth);
    js << ", \"lazy_n_project\": " << pre.n_project;
    for (u_int l = 0; l < pre.n_project; ++l) {
      dump_csr(out, "LP" + std::to_string(l), *pre.project_matrix[l]);
      dump_csr(out, "LPt" + std::to_string(l), *pre.project_matrix_r[l]);
      dump_csr(out, "LA" + std::to_string(l + 1), *pre.projected_matrix[l + 1]);
    }
    Vector<double> x(n);
    pre.vmult(x, b);
    save_npy(out + "/x_lazy.npy", &x(0), {n});
    for (size_t k = 0; k < A.n_nonzero_elements(); ++k) A.global_entry(k) *= 1.5;
    pre.reinit(A, 2);
    for (u_int l = 0; l < pre.n_project; ++l) dump_csr(out, "LRA" + std::to_string(l + 1), *pre.projected_matrix[l + 1]);
    Vector<double> x2(n);
    pre.vmult(x2, b);
    save_npy(out + "/x_lazy2.npy", &x2(0), {n});
  }
  js << "}";
  std::cout << js.str() << std::endl;
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  for (int i = 1; i < argc; ++i) {
    const char* eq = std::strchr(argv[i], '=');
    if (eq == nullptr) continue;
    g_args[std::string(argv[i], (size_t)(eq - argv[i]))] = std::string(eq + 1);
  }
  const int dim = std::atoi(arg("dim", "2").c_str());
  if (dim == 2) return run<2>();
  if (dim == 3) return run<3>();
  std::cerr << "dim must be 2 or 3\n";
  return 2;
}
