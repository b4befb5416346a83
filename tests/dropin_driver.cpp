// Test driver for the AFEPack drop-in's core (afepack_gb300/dropin/dropin_core.cpp),
// built and run by tests/test_gpu_dropin.py.  It replays what AFEPack calls
// through the drop-in -- AMGPreconditioner's lazyReinit twice on one pattern
// (new values the second time), lazyReinit with another pattern (refused),
// AMGSolver::reinit + solve, AMGPreconditioner::vmult -- and writes what it
// got as raw arrays into the directory given as argv[1]:
//   in:  system.bin = int64 m, int64 nnz, int32 rowptr[m+1], int32 cols[nnz],
//        double vals[nnz], double rhs[m]
//   out: lazy_levels.txt (n_project), lazy{l}_{rp,ci,va}.bin (level l >= 1),
//        relazy{l}_va.bin, refused.txt, x_solve.bin, x_vmult.bin
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../afepack_gb300/dropin/dropin_core.h"

template <class T>
static void save(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), sizeof(T) * v.size());
}

static void dump_levels(afp_amg* amg, int np, const std::string& dir, const std::string& tag, bool values_only) {
  for (int l = 1; l <= np; ++l) {
    int64_t n = 0, nnz = 0;
    int colors = 0;
    afp_amg_level_info(amg, l, &n, &nnz, &colors);
    std::vector<int32_t> rp(n + 1);
    afp_amg_download_level(amg, l, rp.data(), nullptr, nullptr);
    std::vector<int32_t> ci(rp[n]);
    std::vector<double> va(rp[n]);
    afp_amg_download_level(amg, l, nullptr, ci.data(), va.data());
    const std::string p = dir + "/" + tag + std::to_string(l) + "_";
    if (!values_only) {
      save(p + "rp.bin", rp);
      save(p + "ci.bin", ci);
    }
    save(p + "va.bin", va);
  }
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  std::ifstream f(dir + "/system.bin", std::ios::binary);
  int64_t m = 0, nnz = 0;
  f.read(reinterpret_cast<char*>(&m), 8);
  f.read(reinterpret_cast<char*>(&nnz), 8);
  std::vector<int32_t> rp(m + 1), ci(nnz);
  std::vector<double> va(nnz), rhs(m);
  f.read(reinterpret_cast<char*>(rp.data()), 4 * (m + 1));
  f.read(reinterpret_cast<char*>(ci.data()), 4 * nnz);
  f.read(reinterpret_cast<char*>(va.data()), 8 * nnz);
  f.read(reinterpret_cast<char*>(rhs.data()), 8 * m);
  afp_dropin::Matrix M;
  M.m = M.n = m;
  M.nnz = nnz;
  M.rowptr = rp.data();
  M.cols = ci.data();
  M.vals = va.data();
  afp_dropin::Options o;  // the reference defaults
  int pattern_a = 0, pattern_b = 0, pre = 0, solver = 0;  // stand-ins for AFEPack objects
  try {
    // AMGPreconditioner(M, 2, 3): lazyReinit on a fresh object = lazyInit
    afp_dropin::lazy_reinit(&pre, &pattern_a, M, o);
    const int np = afp_dropin::n_project(&pre);
    std::ofstream(dir + "/lazy_levels.txt") << np << "\n";
    dump_levels(afp_dropin::handle(&pre), np, dir, "lazy", false);
    // the same pattern object with new values: numeric re-setup
    std::vector<double> va2(va);
    for (double& v : va2) v *= 1.5;
    afp_dropin::Matrix M2 = M;
    M2.vals = va2.data();
    afp_dropin::lazy_reinit(&pre, &pattern_a, M2, o);
    dump_levels(afp_dropin::handle(&pre), np, dir, "relazy", true);
    // another pattern object: refused, as the reference aborts
    std::string refused = "no";
    try {
      afp_dropin::lazy_reinit(&pre, &pattern_b, M2, o);
    } catch (const std::runtime_error& e) {
      refused = e.what();
    }
    std::ofstream(dir + "/refused.txt") << refused << "\n";
    // AMGPreconditioner::vmult(x, b) = solve(x, b, 0, iterate_step = 2, 1)
    std::vector<double> xv(m, 0.0);
    afp_dropin::precondition(&pre, xv.data(), rhs.data(), 2);
    save(dir + "/x_vmult.bin", xv);
    // AMGSolver(M) + solve(x, r, 1e-8, 4): five stationary V-cycles
    afp_dropin::reinit(&solver, M, o);
    std::vector<double> xs(m, 0.0);
    const afp_solve_info info = afp_dropin::solve(&solver, xs.data(), rhs.data(), 1e-8, 4, 1);
    save(dir + "/x_solve.bin", xs);
    std::printf("solve: %d cycles, residual %g -> %g\n", info.iterations, info.initial_residual, info.final_residual);
    afp_dropin::clear(&solver);
    afp_dropin::clear(&pre);
    if (afp_dropin::initialized(&pre)) return 3;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
