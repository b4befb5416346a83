// The state behind the C++ drop-in for AFEPack's AMGSolver, without AFEPack
// types: one device solver per AFEPack object (keyed by its address, since
// AMGSolver.h has no spare member for a handle), created by reinit (the
// classical hierarchy, AMGSolver::reinit, src/AMGSolver.cpp:384-438) or by
// lazy_reinit (AMGSolver::lazyReinit, src/AMGSolver.cpp:442-545: lazyInit's
// hierarchy on first use, then a numeric re-setup when the same sparsity
// pattern comes back with new values), used by solve (AMGSolver::solve,
// :549-639) and precondition (AMGPreconditioner::vmult, AMGSolver.h:193-195),
// and released by clear.  AMGSolver_gb300.cpp maps AFEPack's classes onto it;
// it compiles and runs without AFEPack.
//
// Errors are thrown as std::runtime_error with the message the reference
// prints before it aborts (the AFEPack-side glue prints it and aborts).
// Environment: AFP_DEVICE selects the GPU (default 0), AFP_PRECISION=mixed
// the FP32 V-cycle, AFP_DENSE_TAIL the dense-tail size (default 0: the
// reference's full depth, so that solve() iterates the reference's hierarchy).
#pragma once

#include <cstdint>

#include "../../include/afepack_gb300.h"

namespace afp_dropin {

struct Matrix {  // a CSR matrix in AFEPack's layout (diagonal first in each row)
  int64_t m = 0, n = 0, nnz = 0;
  const int32_t* rowptr = nullptr;
  const int32_t* cols = nullptr;
  const double* vals = nullptr;
};

struct Options {  // the reference constructor's parameters
  double tol = 1e-12;
  int smooth_step = 3;
  int max_coarse = 50;
  double min_density = 0.382;
  double alpha = 0.25;
};

void reinit(const void* owner, const Matrix& M, const Options& o);
void lazy_reinit(const void* owner, const void* pattern, const Matrix& M, const Options& o);
afp_solve_info solve(const void* owner, double* x, const double* r, double tol, int64_t step, int mode);
void precondition(const void* owner, double* x, const double* b, int iterate_step);
void clear(const void* owner);
bool initialized(const void* owner);
int n_project(const void* owner);
afp_amg* handle(const void* owner);

}  // namespace afp_dropin
