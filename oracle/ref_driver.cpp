// ref_driver.cpp -- C entry points over the reference's own hot-path classes, compiled unmodified from their
// sources (core/Pressure.cpp, core/MagneticField.cpp, core/Collider.cpp, core/FastMarching.cpp,
// core/Extrapolation.cpp, core/Reinitialization.cpp, core/CSG.cpp and the header-only core/Advection.h, TriLerp.h,
// TriCuInterp.h) against the stand-in headers in oracle/refshim.  Built by oracle/ref.mk into
// oracle/_ref/libsfref.so.
//
// TEST INFRASTRUCTURE ONLY: this library pins the C oracle (oracle/sf_oracle.c) to the reference's code.  The
// tests and tests/golden/make_ref_golden.py call it; the product never does.
//
// amgcl is absent, so the solve is replaced (oracle/refshim/amgcl/make_solver.hpp): the matrix, right-hand
// side, initial guess and tolerance the reference hands to amgcl are recorded, and the "solution" is chosen by
// the caller: mode 0 leaves the initial guess, mode 1 injects a given vector, mode 2 solves with Jacobi-PCG to
// a given relative tolerance.  The members the reference keeps private (Pressure::m_Grid2Mat,
// Collider::m_Fraction, MagneticField::m_Coeff / m_TotalField, ...) are read and set through `private`
// redefined as `public` for the reference headers only; every standard and stand-in header is included
// before that.
#include <algorithm>
#include <array>
#include <atomic>
#include <cassert>
#include <chrono>
#include <cmath>
#include <concepts>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <initializer_list>
#include <iostream>
#include <limits>
#include <memory>
#include <numbers>
#include <optional>
#include <queue>
#include <span>
#include <string>
#include <string_view>
#include <thread>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include <Eigen/Dense>
#include <Eigen/Sparse>
#include <amgcl/make_solver.hpp>
#include <fmt/core.h>
#include <spdlog/spdlog.h>
#include <tbb/tbb.h>
#include <yaml-cpp/yaml.h>

#define private public
#include "Advection.h"
#include "CSG.h"
#include "ImplicitSurface.h"
#include "Collider.h"
#include "Extrapolation.h"
#include "FastMarching.h"
#include "MagneticField.h"
#include "Pressure.h"
#include "Reinitialization.h"
#undef private

using namespace Pivot;

namespace amgcl::refshim {
System &last_system() {
    static System s;
    return s;
}
SolveHook &solve_hook() {
    static SolveHook h = nullptr;
    return h;
}
} // namespace amgcl::refshim

namespace {

using amgcl::refshim::System;

int g_mode = 0;
std::vector<double> g_inject;
double g_tol = 1e-13;
long long g_iters = 0;

void spmv(const System &s, const double *x, double *y) {
    for (long long r = 0; r < s.n; r++) {
        double acc = 0;
        for (long long k = s.rowptr[r]; k < s.rowptr[r + 1]; k++) acc += s.val[k] * x[s.col[k]];
        y[r] = acc;
    }
}

double dot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}

// Jacobi-preconditioned CG to ||b - A x|| <= tol ||b|| from the initial guess in x.
std::tuple<std::size_t, double> pcg(const System &s, double *x) {
    const long long n = s.n;
    std::vector<double> r(n), z(n), p(n), q(n), dinv(n, 1.0);
    for (long long i = 0; i < n; i++)
        for (long long k = s.rowptr[i]; k < s.rowptr[i + 1]; k++)
            if (s.col[k] == i && s.val[k] != 0) dinv[i] = 1.0 / s.val[k];
    spmv(s, x, q.data());
    for (long long i = 0; i < n; i++) r[i] = s.rhs[i] - q[i];
    const double bn = std::sqrt(dot(s.rhs, s.rhs));
    double rn = std::sqrt(dot(r, r));
    if (bn == 0) return {0, rn};
    for (long long i = 0; i < n; i++) p[i] = z[i] = dinv[i] * r[i];
    double rz = dot(r, z);
    std::size_t it = 0;
    while (rn > g_tol * bn && it < 100000) {
        spmv(s, p.data(), q.data());
        const double alpha = rz / dot(p, q);
        for (long long i = 0; i < n; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        for (long long i = 0; i < n; i++) z[i] = dinv[i] * r[i];
        const double rz1 = dot(r, z);
        for (long long i = 0; i < n; i++) p[i] = z[i] + rz1 / rz * p[i];
        rz = rz1;
        rn = std::sqrt(dot(r, r));
        it++;
    }
    return {it, rn / bn};
}

std::tuple<std::size_t, double> hook(const System &s, double *x) {
    if (g_mode == 1) {
        std::copy(g_inject.begin(), g_inject.begin() + std::min<size_t>(g_inject.size(), s.n), x);
        return {0, 0.0};
    }
    if (g_mode == 2) {
        auto r = pcg(s, x);
        g_iters = (long long)std::get<0>(r);
        return r;
    }
    return {0, 0.0};
}

struct ref_grid {
    int nx, ny, nz;
    double h, ox, oy, oz;
};

// One simulation grid with its collider and the two solver objects, as core/Simulation.h holds them.
struct Session {
    std::unique_ptr<StaggeredGrid> sg;
    std::unique_ptr<Collider> collider;
    std::unique_ptr<Pressure> pressure;
    std::unique_ptr<MagneticField> magnetic;
};

// StaggeredGrid(bw, h, res, center) whose corner is exactly (ox, oy, oz): the reference derives the corner
// as center - res h / 2, which can differ from the intended corner by rounding, so the corner and the grids
// built from it are set to the constructor's formulas (core/StaggeredGrid.h:10-20) with the exact corner.
std::unique_ptr<StaggeredGrid> make_sgrid(const ref_grid *g, int bw) {
    Vector3i res(g->nx, g->ny, g->nz);
    Vector3d o(g->ox, g->oy, g->oz);
    auto sg = std::make_unique<StaggeredGrid>(bw, g->h, res, o + res.cast<double>() * g->h / 2);
    if (sg->m_Origin != o) {
        const double h = g->h;
        sg->m_Origin = o;
        sg->m_NodeGrid = Grid(h, res + Vector3i::Ones(), o);
        sg->m_CellGrid = Grid(h, res, o + Vector3d::Constant(h / 2));
        sg->m_FaceGrids[0] = Grid(h, res + Vector3i(1, 0, 0), o + Vector3d(0, 1, 1) * h / 2);
        sg->m_FaceGrids[1] = Grid(h, res + Vector3i(0, 1, 0), o + Vector3d(1, 0, 1) * h / 2);
        sg->m_FaceGrids[2] = Grid(h, res + Vector3i(0, 0, 1), o + Vector3d(1, 1, 0) * h / 2);
    }
    return sg;
}

template <class T> void put(GridData<T> &d, const T *src) {
    std::copy(src, src + d.GetData().size(), d.GetData().begin());
}
template <class T> void get(const GridData<T> &d, T *dst) {
    if (dst) std::copy(d.GetData().begin(), d.GetData().end(), dst);
}
void put3(SGridData<double> &d, const double *const src[3]) {
    for (int a = 0; a < 3; a++) put(d[a], src[a]);
}
void get3(const SGridData<double> &d, double *const dst[3]) {
    if (!dst) return;
    for (int a = 0; a < 3; a++) get(d[a], dst[a]);
}

void set_mode(int mode, const double *inject, long long n, double tol) {
    g_mode = mode;
    g_tol = tol;
    g_inject.assign(inject ? inject : nullptr, inject ? inject + n : nullptr);
    amgcl::refshim::solve_hook() = hook;
}

void read_system(long long *rowptr, int *col, double *val, double *rhs, double *x0, double *tol_seen) {
    const System &s = amgcl::refshim::last_system();
    if (rowptr) std::copy(s.rowptr.begin(), s.rowptr.end(), rowptr);
    if (col) std::copy(s.col.begin(), s.col.end(), col);
    if (val) std::copy(s.val.begin(), s.val.end(), val);
    if (rhs) std::copy(s.rhs.begin(), s.rhs.end(), rhs);
    if (x0) std::copy(s.x0.begin(), s.x0.end(), x0);
    if (tol_seen) *tol_seen = s.tol;
}

} // namespace

extern "C" {

int ref_version(void) { return 1; }

// Simulation grid with boundary width bw and its Collider (core/Collider.cpp:8-19: the node level set of the
// domain box, not yet finished).
void *ref_session_new(const ref_grid *g, int bw) {
    auto *s = new Session;
    s->sg = make_sgrid(g, bw);
    s->collider = std::make_unique<Collider>(*s->sg);
    s->pressure = std::make_unique<Pressure>(*s->sg);
    return s;
}

void ref_session_free(void *p) { delete static_cast<Session *>(p); }

// Collider::Finish (core/Collider.cpp:21-45): fast marching of the node level set, face fractions, normals.
void ref_collider_finish(void *p, double *node_ls, double *const frac[3], double *const normal[3]) {
    auto *s = static_cast<Session *>(p);
    s->collider->Finish(*s->sg);
    get(s->collider->LevelSet, node_ls);
    get3(s->collider->m_Fraction, frac);
    get3(s->collider->m_Normal, normal);
}

// Set the collider's face fractions, normals and velocity (NULL: leave as they are).
void ref_collider_set(void *p, const double *const frac[3], const double *const normal[3],
                      const double *const solid_vel[3]) {
    auto *s = static_cast<Session *>(p);
    if (frac) put3(s->collider->m_Fraction, frac);
    if (normal) put3(s->collider->m_Normal, normal);
    if (solid_vel) put3(s->collider->Velocity, solid_vel);
}

// Pressure::Project (reproject = 0, core/Pressure.cpp:17-26) or Pressure::Reproject (reproject = 1, :28-36)
// on this session's Pressure object, with the jump callback J(axis, face, theta) = jump[axis][face] (the
// shipped callback ignores theta; NULL: no callback).  vel is updated in place.  Returns the number of
// unknowns; fills the recorded matrix (Project only), rhs, initial guess, solution (reduced) and grid2mat.
long long ref_pressure_project(void *p, int reproject, const double *phi, const double *const jump[3],
                               double vol_error, double *const vel[3], int mode, const double *p_inject,
                               double tol, long long *rowptr, int *col, double *val, double *rhs, double *x0,
                               double *sol, int *grid2mat, double *tol_seen) {
    auto *s = static_cast<Session *>(p);
    GridData<double> ls(s->sg->GetCellGrid());
    put(ls, phi);
    SGridData<double> u(s->sg->GetFaceGrids());
    put3(u, vel);
    SGridData<double> J(s->sg->GetFaceGrids());
    if (jump) {
        put3(J, jump);
        s->pressure->SetPressureJump([&J](int axis, Vector3i const &face, double) -> double { return J[axis][face]; });
    } else {
        s->pressure->m_PressureJump = nullptr;
    }
    long long n_prev = s->pressure->m_RdP.size();
    set_mode(mode, p_inject, reproject ? n_prev : 0, tol);
    if (!reproject) {
        // the unknown count is known only after SetUnKnowns; inject after it through the recorded system
        long long n = 0;
        for (double v : ls.GetData()) n += v <= 0;
        set_mode(mode, p_inject, n, tol);
        amgcl::refshim::last_system() = System();
        s->pressure->Project(u, ls, *s->collider, vol_error);
    } else {
        amgcl::refshim::last_system().rhs.clear();
        s->pressure->Reproject(u, ls, *s->collider, vol_error);
    }
    s->pressure->m_PressureJump = nullptr;
    get3(u, vel);
    read_system(reproject ? nullptr : rowptr, reproject ? nullptr : col, reproject ? nullptr : val, rhs, x0, tol_seen);
    const long long n = s->pressure->m_RdP.size();
    if (sol) std::copy(s->pressure->m_RdP.data(), s->pressure->m_RdP.data() + n, sol);
    get(s->pressure->m_Grid2Mat, grid2mat);
    return n;
}

// MagneticField::Solve (core/MagneticField.cpp:29-35) on this session's MagneticField (created on the first
// call with chi and band_width; later calls set them as SetSusceptibility / SetBandWidth do, and keep m_Sol as
// the warm start).  Fills mu on faces, the recorded matrix, rhs, initial guess, the solution psi (cells), the
// total field H, the tolerance passed to amgcl and the corner of the field's own grid.
void ref_magnetic_solve(void *p, double chi, double band_width, const double *phi, const double *const hext[3],
                        int mode, const double *psi_inject, double tol, double *const mu[3], long long *rowptr,
                        int *col, double *val, double *rhs, double *x0, double *psi, double *const H[3],
                        double *tol_seen, double *origin_ext) {
    auto *s = static_cast<Session *>(p);
    if (!s->magnetic) s->magnetic = std::make_unique<MagneticField>(*s->sg, chi, band_width);
    MagneticField &M = *s->magnetic;
    M.SetSusceptibility(chi);
    M.SetBandWidth(band_width);
    GridData<double> ls(s->sg->GetCellGrid());
    put(ls, phi);
    SGridData<double> he(s->sg->GetFaceGrids());
    put3(he, hext);
    set_mode(mode, psi_inject, (long long)ls.GetData().size(), tol);
    M.Solve(ls, he);
    get3(M.m_Coeff, mu);
    read_system(rowptr, col, val, rhs, x0, tol_seen);
    get(M.m_Potential, psi);
    get3(M.m_TotalField, H);
    if (origin_ext) {
        Vector3d o = M.m_SGridExt.GetOrigin();
        for (int a = 0; a < 3; a++) origin_ext[a] = o[a];
    }
}

// MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48) with the total field set to H.
void ref_vertex_pressures(void *p, double chi, const double *const H[3], const double *positions,
                          const double *normals, long long nverts, double *out) {
    auto *s = static_cast<Session *>(p);
    if (!s->magnetic) s->magnetic = std::make_unique<MagneticField>(*s->sg, chi, 2 * s->sg->GetSpacing());
    s->magnetic->SetSusceptibility(chi);
    put3(s->magnetic->m_TotalField, H);
    SurfaceMesh mesh;
    for (long long v = 0; v < nverts; v++) {
        mesh.Positions.emplace_back(positions[3 * v], positions[3 * v + 1], positions[3 * v + 2]);
        mesh.Normals.emplace_back(normals[3 * v], normals[3 * v + 1], normals[3 * v + 2]);
    }
    std::vector<double> pr = s->magnetic->CalculateVertexPressures(mesh);
    std::copy(pr.begin(), pr.end(), out);
}

// Extrapolation::Solve (core/Extrapolation.cpp:4-30) of the velocity with the simulation's validity predicate
// (core/Simulation.cpp:237-240: fraction < 1 and one adjacent cell liquid).  The predicate is the simulation's
// lambda, written here because core/Simulation.cpp is not compiled; a cell outside the grid counts as not
// liquid (the reference's lambda reads outside its array there).
void ref_extrapolate_velocity(void *p, double *const vel[3], const double *phi, double clear_val, int max_steps) {
    auto *s = static_cast<Session *>(p);
    GridData<double> ls(s->sg->GetCellGrid());
    put(ls, phi);
    SGridData<double> u(s->sg->GetFaceGrids());
    put3(u, vel);
    const Grid &cg = ls.GetGrid();
    Extrapolation::Solve(u, clear_val, max_steps, [&](int axis, Vector3i const &face) {
        Vector3i const cell0 = StaggeredGrid::AdjCellOfFace(axis, face, 0);
        Vector3i const cell1 = StaggeredGrid::AdjCellOfFace(axis, face, 1);
        return s->collider->GetFraction()[axis][face] < 1 &&
               ((cg.IsValid(cell0) && ls[cell0] <= 0) || (cg.IsValid(cell1) && ls[cell1] <= 0));
    });
    get3(u, vel);
}

// Collider::Enforce (core/Collider.cpp:75-86) with the session collider's fractions, normals and velocity.
void ref_collider_enforce(void *p, double *const vel[3]) {
    auto *s = static_cast<Session *>(p);
    SGridData<double> u(s->sg->GetFaceGrids());
    put3(u, vel);
    s->collider->Enforce(u);
    get3(u, vel);
}

// Advection::Solve<2> (core/Advection.h:35-55) of the level set and of the velocity by itself.
void ref_advect_levelset(void *p, double *phi, const double *const vel[3], double dt) {
    auto *s = static_cast<Session *>(p);
    GridData<double> ls(s->sg->GetCellGrid());
    put(ls, phi);
    SGridData<double> u(s->sg->GetFaceGrids());
    put3(u, vel);
    Advection::Solve<2>(ls, u, dt);
    get(ls, phi);
}

void ref_advect_velocity(void *p, double *const vel[3], double dt) {
    auto *s = static_cast<Session *>(p);
    SGridData<double> u(s->sg->GetFaceGrids());
    put3(u, vel);
    Advection::Solve<2>(u, u, dt);
    get3(u, vel);
}

// Reinitialization::Solve (core/Reinitialization.cpp:36-46) of a cell level set.
void ref_reinitialize(void *p, double *phi, int max_steps) {
    auto *s = static_cast<Session *>(p);
    GridData<double> ls(s->sg->GetCellGrid());
    put(ls, phi);
    Reinitialization::Solve(ls, max_steps);
    get(ls, phi);
}

// FastMarching::Solve (core/FastMarching.cpp:25-62) of a node level set.
void ref_fast_marching(void *p, double *node_ls, int max_steps) {
    auto *s = static_cast<Session *>(p);
    GridData<double> ls(s->sg->GetNodeGrid());
    put(ls, node_ls);
    FastMarching::Solve(ls, max_steps);
    get(ls, node_ls);
}

long long ref_last_solve_iters(void) { return g_iters; }

// A scene's cell level set as the reference builds it (core/Simulation.cpp:17 starts from +infinity,
// demo/SimBuilder.cpp then unites surfaces with CSG::Union, core/CSG.cpp:4-9): kind 0 = ImplicitPlane(point a,
// direction b), 1 = ImplicitSphere(centre a, radius r), 2 = ImplicitBox(min corner a, lengths b).  phi is
// updated in place (pass +infinity for a fresh level set).
void ref_csg_union(void *p, double *phi, int kind, const double *a, const double *b, double r) {
    auto *s = static_cast<Session *>(p);
    GridData<double> ls(s->sg->GetCellGrid());
    put(ls, phi);
    Vector3d va(a[0], a[1], a[2]);
    if (kind == 0) {
        CSG::Union(ls, ImplicitPlane(va, Vector3d(b[0], b[1], b[2])));
    } else if (kind == 1) {
        CSG::Union(ls, ImplicitSphere(va, r));
    } else {
        CSG::Union(ls, ImplicitBox(va, Vector3d(b[0], b[1], b[2])));
    }
    get(ls, phi);
}

// StaggeredGrid::GetDomainOrigin / GetDomainLengths of the session's grid (core/StaggeredGrid.h:36-37).
void ref_domain(void *p, double *origin, double *lengths) {
    auto *s = static_cast<Session *>(p);
    Vector3d o = s->sg->GetDomainOrigin(), l = s->sg->GetDomainLengths();
    for (int a = 0; a < 3; a++) {
        origin[a] = o[a];
        lengths[a] = l[a];
    }
}

} // extern "C"
