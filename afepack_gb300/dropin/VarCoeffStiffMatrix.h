// StiffMatrix with one coefficient per element: the element matrix of
// -div(a grad u) with a constant on each element, the coefficient form of the
// variable-coefficient examples (examples/elliptic_equation/
// EllipticEquation.cpp:337-383 override getElementMatrix for it).
//
// getElementMatrix is the reference's stiffness element matrix times the
// element's coefficient, so the reference's own build() assembles the same
// matrix; with the afepack_gb300 replacement of src/BilinearOperator.cpp,
// build() recognises this exact type and assembles it on the GPU
// (afp_assemble_opts.coef), bitwise the same.
#pragma once

#include <vector>

#include <AFEPack/BilinearOperator.h>

AFEPACK_OPEN_NAMESPACE

template <int D>
class VarCoeffStiffMatrix : public StiffMatrix<D, double> {
 public:
  // coef[e] is the coefficient of element e; the vector must outlive build()
  VarCoeffStiffMatrix(FEMSpace<double, D>& sp, const std::vector<double>& coef)
      : StiffMatrix<D, double>(sp), coef_(&coef) {}
  const std::vector<double>& coefficient() const { return *coef_; }
  void getElementMatrix(const Element<double, D>& e0, const Element<double, D>& e1,
                        const typename ActiveElementPairIterator<D>::State state) override {
    StiffMatrix<D, double>::getElementMatrix(e0, e1, state);
    const double a = (*coef_)[e0.index()];
    auto& K = this->elementMatrix();
    for (size_t j = 0; j < K.n_rows(); ++j)
      for (size_t k = 0; k < K.n_cols(); ++k) K(j, k) *= a;
  }

 private:
  const std::vector<double>* coef_;
};

AFEPACK_CLOSE_NAMESPACE
