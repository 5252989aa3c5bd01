// Stand-in for amgcl::make_solver (TEST INFRASTRUCTURE for oracle/_ref).  amgcl is not vendored by the
// reference and is absent here; what the reference's sources hand to it -- the assembled matrix, the
// right-hand side, the initial guess and the tolerance -- is what the oracle is checked against.  So the
// constructor records the matrix (CSR), and operator() records rhs, x0 and tol and then calls a solve hook
// installed by oracle/ref_driver.cpp (which injects a given solution or solves to a tight tolerance).
#pragma once

#include <cstddef>
#include <tuple>
#include <vector>

namespace amgcl {
namespace backend {
template <class T> struct eigen {};
} // namespace backend
namespace coarsening {
struct smoothed_aggregation {
    struct params {};
};
} // namespace coarsening
namespace relaxation {
struct spai0 {
    struct params {};
};
} // namespace relaxation
namespace solver {
// amgcl's documented defaults: relative tolerance 1e-8, at most 100 iterations.
struct iterative_params {
    double tol = 1e-8;
    double abstol = 0.0;
    std::size_t maxiter = 100;
};
template <class Backend> struct bicgstab {
    using params = iterative_params;
    static constexpr int kind = 0;
};
template <class Backend> struct cg {
    using params = iterative_params;
    static constexpr int kind = 1;
};
} // namespace solver
template <class Backend, class Coarsening, class Relaxation> struct amg {
    struct params {};
};

namespace refshim {
struct System {
    int kind = -1; // 0 BiCGStab (pressure), 1 CG (potential)
    long long n = 0;
    std::vector<long long> rowptr;
    std::vector<int> col;
    std::vector<double> val;
    std::vector<double> rhs, x0;
    double tol = 0.0;
    long long solves = 0;
};
// (iterations, error) as amgcl returns them; x holds the initial guess on entry.
using SolveHook = std::tuple<std::size_t, double> (*)(const System &, double *x);
System &last_system();
SolveHook &solve_hook();
} // namespace refshim

template <class Precond, class IterSolver> class make_solver {
  public:
    struct params {
        typename Precond::params precond;
        typename IterSolver::params solver;
    };

    template <class Matrix> explicit make_solver(const Matrix &A, const params &prm = params()) : prm_(prm) {
        refshim::System &s = refshim::last_system();
        s.kind = IterSolver::kind;
        s.n = A.rows();
        s.rowptr.assign(A.outerIndexPtr(), A.outerIndexPtr() + A.rows() + 1);
        s.col.assign(A.innerIndexPtr(), A.innerIndexPtr() + A.nonZeros());
        s.val.assign(A.valuePtr(), A.valuePtr() + A.nonZeros());
    }

    template <class Vec1, class Vec2> std::tuple<std::size_t, double> operator()(const Vec1 &rhs, Vec2 &x) const {
        refshim::System &s = refshim::last_system();
        s.kind = IterSolver::kind;
        s.tol = prm_.solver.tol;
        s.rhs.assign(rhs.data(), rhs.data() + rhs.size());
        s.x0.assign(x.data(), x.data() + x.size());
        s.solves++;
        refshim::SolveHook h = refshim::solve_hook();
        return h ? h(s, x.data()) : std::tuple<std::size_t, double>(0, 0.0);
    }

  private:
    params prm_;
};
} // namespace amgcl
