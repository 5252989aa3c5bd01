// sfgpu.hpp -- header-only C++ mirror of the reference's solver classes over the C ABI (sfgpu.h).
//
// A caller of the reference (core/Pressure.h, core/MagneticField.h) switches by replacing
//   Pivot::Pressure / Pivot::MagneticField  ->  sfgpu::Pressure / sfgpu::MagneticField
// with the same constructor arguments and method names.  Containers are plain std::vector<double> in the
// reference's layout (GridData::GetData(), core/GridData.h:51-52), so `levelSet.GetData().data()` of the
// reference's own grids can be wrapped without copying (sfgpu::CellView / sfgpu::FaceView).
//
// Error behaviour: the reference's methods return void, ignore non-convergence (printing the iteration count)
// and exit on fatal errors.  Here non-convergence is reported in LastStats() (and printed when Verbose is
// set); every other failure (bad argument, CUDA error, no sm_103 device) throws sfgpu::Error.
#pragma once

#include <array>
#include <cmath>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "sfgpu.h"

namespace sfgpu {

struct Error : std::runtime_error {
    sf_status status;
    Error(sf_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

// StaggeredGrid(boundaryWidth, spacing, resolution, center) (core/StaggeredGrid.h:10-21).
struct StaggeredGrid {
    int BoundaryWidth;
    double Spacing;
    std::array<int, 3> Resolution;
    std::array<double, 3> Origin;  // center - resolution * spacing / 2

    StaggeredGrid(int boundaryWidth, double spacing, std::array<int, 3> resolution,
                  std::array<double, 3> center = {0, 0, 0})
        : BoundaryWidth(boundaryWidth), Spacing(spacing), Resolution(resolution) {
        for (int a = 0; a < 3; a++) Origin[a] = center[a] - resolution[a] * spacing / 2;
    }
    long long NumCells() const { return (long long)Resolution[0] * Resolution[1] * Resolution[2]; }
    long long NumFaces(int axis) const {
        long long n = 1;
        for (int b = 0; b < 3; b++) n *= Resolution[b] + (b == axis ? 1 : 0);
        return n;
    }
    std::array<int, 3> FaceSize(int axis) const {
        std::array<int, 3> s = Resolution;
        s[axis] += 1;
        return s;
    }
    sf_grid C() const {
        sf_grid g;
        g.nx = Resolution[0];
        g.ny = Resolution[1];
        g.nz = Resolution[2];
        g.h = Spacing;
        for (int a = 0; a < 3; a++) g.origin[a] = Origin[a];
        return g;
    }
    // Grid::IndexOf (core/Grid.h:28) on the cell grid / a face grid
    long long CellIndex(int i, int j, int k) const {
        return (long long)k + (long long)Resolution[2] * ((long long)j + (long long)Resolution[1] * i);
    }
    long long FaceIndex(int axis, int i, int j, int k) const {
        auto s = FaceSize(axis);
        return (long long)k + (long long)s[2] * ((long long)j + (long long)s[1] * i);
    }
};

using GridData = std::vector<double>;  // cell (or node) array, reference layout
struct SGridData {                      // three face arrays (core/SGridData.h)
    std::array<std::vector<double>, 3> Data;
    SGridData() = default;
    explicit SGridData(const StaggeredGrid &g, std::array<double, 3> value = {0, 0, 0}) {
        for (int a = 0; a < 3; a++) Data[a].assign(g.NumFaces(a), value[a]);
    }
    std::vector<double> &operator[](int a) { return Data[a]; }
    const std::vector<double> &operator[](int a) const { return Data[a]; }
};

// One CUDA stream + device workspaces shared by the solvers of a simulation.
class Context {
   public:
    explicit Context(int device = 0, void *stream = nullptr) {
        sf_status s = sf_create(device, stream, &h_);
        if (s != SF_OK) throw Error(s, std::string("sf_create: ") + sf_status_string(s));
    }
    ~Context() { sf_destroy(h_); }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    void *Handle() const { return h_; }

   private:
    void *h_ = nullptr;
};

inline void check(void *ctx, sf_status s, const sf_solve_stats &st, bool verbose) {
    if (s == SF_OK || s == SF_STALLED_FALLBACK || s == SF_NOT_CONVERGED) {
        if (verbose) std::printf("%6d iters (%.2e) ", st.iters, st.rel_residual);
        return;
    }
    throw Error(s, std::string(sf_status_string(s)) + ": " + sf_last_error(ctx));
}

// Collider inputs of the pressure solve: per-face solid fraction (1 = solid) and solid velocity
// (core/Collider.h:26-28).  Box() builds the domain-box walls as Collider(sgrid) + Finish() does.
struct Collider {
    SGridData Fraction;
    SGridData Velocity;
    SGridData Normal;  // m_Normal: face means of the node level set's derivatives (core/Collider.cpp:30-44)
    static Collider Box(const StaggeredGrid &g) {
        Collider c;
        c.Fraction = SGridData(g);
        c.Velocity = SGridData(g);
        c.Normal = SGridData(g);
        sf_grid cg = g.C();
        std::vector<double> ls((size_t)(g.Resolution[0] + 1) * (g.Resolution[1] + 1) * (g.Resolution[2] + 1));
        double *fr[3] = {c.Fraction[0].data(), c.Fraction[1].data(), c.Fraction[2].data()};
        sf_status s = sf_collider_box_fractions(&cg, g.BoundaryWidth, fr, ls.data());
        if (s != SF_OK) throw Error(s, "sf_collider_box_fractions failed");
        double *nm[3] = {c.Normal[0].data(), c.Normal[1].data(), c.Normal[2].data()};
        if ((s = sf_collider_face_normals(&cg, ls.data(), nm)) != SF_OK) throw Error(s, "sf_collider_face_normals failed");
        return c;
    }
    // Collider::Enforce (core/Collider.cpp:75-86) on the GPU.
    void Enforce(Context &ctx, const StaggeredGrid &g, SGridData &fluidVelocity) const {
        sf_grid cg = g.C();
        double *v[3] = {fluidVelocity[0].data(), fluidVelocity[1].data(), fluidVelocity[2].data()};
        const double *fr[3] = {Fraction[0].data(), Fraction[1].data(), Fraction[2].data()};
        const double *nm[3] = {Normal[0].data(), Normal[1].data(), Normal[2].data()};
        const double *us[3] = {Velocity[0].data(), Velocity[1].data(), Velocity[2].data()};
        sf_status s = sf_collider_enforce(ctx.Handle(), &cg, v, fr, nm, Velocity[0].empty() ? nullptr : us);
        if (s != SF_OK) throw Error(s, std::string("sf_collider_enforce: ") + sf_last_error(ctx.Handle()));
    }
};

// Extrapolation::Solve of the projected velocity (core/Extrapolation.cpp:4-30) with the simulation's validity
// predicate (core/Simulation.cpp:237-240), on the GPU.
struct Extrapolation {
    static void Solve(Context &ctx, const StaggeredGrid &g, SGridData &velocity, const GridData &levelSet,
                      const Collider &collider, double clearVal = 0., int maxSteps = 6) {
        sf_grid cg = g.C();
        double *v[3] = {velocity[0].data(), velocity[1].data(), velocity[2].data()};
        const double *fr[3] = {collider.Fraction[0].data(), collider.Fraction[1].data(), collider.Fraction[2].data()};
        sf_status s = sf_extrapolate_velocity(ctx.Handle(), &cg, v, levelSet.data(), fr, clearVal, maxSteps);
        if (s != SF_OK) throw Error(s, std::string("sf_extrapolate_velocity: ") + sf_last_error(ctx.Handle()));
    }
};

// The parts of core/SurfaceMesh.h the interface coupling reads, and the contour's edge marks
// (Contour::VertexIndexOf, core/Contour.h:19-21: one int per cell-grid edge along each axis, -1 = no vertex).
struct SurfaceMesh {
    std::vector<std::array<double, 3>> Positions, Normals;
    std::vector<double> MeanCurvatures;
    std::array<std::vector<int32_t>, 3> EdgeMark;
    int size() const { return (int)Positions.size(); }
};

// Pressure projection (core/Pressure.h:8-56).
class Pressure {
   public:
    using JumpFunc = std::function<double(int, const std::array<int, 3> &, double)>;

    Pressure(Context &ctx, const StaggeredGrid &sgrid) : ctx_(ctx), g_(sgrid) { sf_default_opts(&opts_, 0); }

    // Same contract as the reference: J(axis, face, theta) = p_liquid - p_air on liquid-air faces.  It is
    // evaluated on the host for those faces only (O(surface)), with theta = phi0 / (phi0 - phi1) of the face's
    // two cells, and passed to the device as a per-face array.
    template <typename Func>
    void SetPressureJump(Func &&f) {
        jump_ = JumpFunc(std::forward<Func>(f));
        jump_array_ = false;
    }
    // The simulation's jump (core/Simulation.cpp:216-235) built on the GPU from the mesh: curvature term when
    // stCoeff != 0, magnetic term from magPressures (CalculateVertexPressures) when given.
    void SetPressureJump(const StaggeredGrid &g, const SurfaceMesh &mesh, const std::vector<double> *magPressures,
                         double stCoeff, double density, double dt) {
        sf_grid cg = g.C();
        const int32_t *em[3] = {mesh.EdgeMark[0].data(), mesh.EdgeMark[1].data(), mesh.EdgeMark[2].data()};
        for (int a = 0; a < 3; a++) jarr_[a].assign(g_.NumFaces(a), 0.0);
        double *jp[3] = {jarr_[0].data(), jarr_[1].data(), jarr_[2].data()};
        sf_status s = sf_pressure_jump(ctx_.Handle(), &cg, em, stCoeff != 0 ? mesh.MeanCurvatures.data() : nullptr,
                                       magPressures ? magPressures->data() : nullptr, mesh.size(), stCoeff, density,
                                       dt, jp);
        if (s != SF_OK) throw Error(s, std::string("sf_pressure_jump: ") + sf_last_error(ctx_.Handle()));
        jump_ = nullptr;
        jump_array_ = true;
    }

    void Project(SGridData &velocity, const GridData &levelSet, const Collider &collider, double volError = 0) {
        run(velocity, levelSet, collider, volError, false);
    }
    void Reproject(SGridData &velocity, const GridData &levelSet, const Collider &collider, double volError = 0) {
        run(velocity, levelSet, collider, volError, true);
    }

    sf_solve_opts &Options() { return opts_; }
    const sf_solve_stats &LastStats() const { return stats_; }
    const GridData &PressureField() const { return p_; }  // m_RdP scattered to cells (0 in air)
    bool Verbose = false;

   private:
    void fill_jump(const GridData &phi, const Collider &col) {
        for (int a = 0; a < 3; a++) jarr_[a].assign(g_.NumFaces(a), 0.0);
        auto R = g_.Resolution;
        for (int a = 0; a < 3; a++) {
            auto s = g_.FaceSize(a);
            for (int i = 0; i < s[0]; i++)
                for (int j = 0; j < s[1]; j++)
                    for (int k = 0; k < s[2]; k++) {
                        std::array<int, 3> f{i, j, k};
                        if (f[a] <= 0 || f[a] >= R[a]) continue;
                        long long fi = g_.FaceIndex(a, i, j, k);
                        if (1. - col.Fraction[a][fi] <= 0) continue;
                        std::array<int, 3> c0 = f;
                        c0[a] -= 1;
                        double p0 = phi[g_.CellIndex(c0[0], c0[1], c0[2])], p1 = phi[g_.CellIndex(i, j, k)];
                        if ((p0 <= 0) == (p1 <= 0)) continue;  // not a liquid-air face
                        jarr_[a][fi] = jump_(a, f, p0 / (p0 - p1));
                    }
        }
    }
    void run(SGridData &vel, const GridData &phi, const Collider &col, double volError, bool re) {
        double *v[3] = {vel[0].data(), vel[1].data(), vel[2].data()};
        const double *fr[3] = {col.Fraction[0].data(), col.Fraction[1].data(), col.Fraction[2].data()};
        const double *us[3] = {col.Velocity[0].data(), col.Velocity[1].data(), col.Velocity[2].data()};
        const double *jp[3] = {nullptr, nullptr, nullptr};
        bool has_us = !col.Velocity[0].empty();
        if (jump_) fill_jump(phi, col);
        const bool has_jump = jump_ || jump_array_;
        if (has_jump)
            for (int a = 0; a < 3; a++) jp[a] = jarr_[a].data();
        p_.assign(g_.NumCells(), 0.0);
        sf_grid cg = g_.C();
        sf_status s = (re ? sf_pressure_reproject : sf_pressure_project)(
            ctx_.Handle(), &cg, v, phi.data(), fr, has_us ? us : nullptr, has_jump ? jp : nullptr, volError, p_.data(),
            &opts_, &stats_);
        check(ctx_.Handle(), s, stats_, Verbose);
    }

    Context &ctx_;
    StaggeredGrid g_;
    JumpFunc jump_;
    bool jump_array_ = false;
    std::array<std::vector<double>, 3> jarr_;
    GridData p_;
    sf_solve_opts opts_;
    sf_solve_stats stats_{};
};

// FDM magnetostatic potential (core/MagneticField.h:15-71).  Potential() and TotalField() expose what the
// reference keeps private (m_Potential, m_TotalField).
class MagneticField {
   public:
    MagneticField(Context &ctx, const StaggeredGrid &sgrid, double susceptibility, double bandWidth)
        : ctx_(ctx), g_(sgrid), chi_(susceptibility), bw_(bandWidth) {
        sf_default_opts(&opts_, 1);
        sf_magnetic_reset(ctx_.Handle());  // m_Sol starts at zero (core/MagneticField.cpp:26)
        psi_.assign(g_.NumCells(), 0.0);
        H_ = SGridData(g_);
    }
    void SetSusceptibility(double chi) { chi_ = chi; }
    void SetBandWidth(double bw) { bw_ = bw; }

    void Solve(const GridData &levelSet, const SGridData &externalField) {
        const double *he[3] = {externalField[0].data(), externalField[1].data(), externalField[2].data()};
        double *H[3] = {H_[0].data(), H_[1].data(), H_[2].data()};
        sf_grid cg = g_.C();
        sf_status s = sf_magnetic_solve(ctx_.Handle(), &cg, levelSet.data(), chi_, bw_, he, psi_.data(), H, &opts_,
                                        &stats_);
        check(ctx_.Handle(), s, stats_, Verbose);
    }

    const GridData &Potential() const { return psi_; }
    const SGridData &TotalField() const { return H_; }

    // MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48) from the last solve's total field.
    std::vector<double> CalculateVertexPressures(const SurfaceMesh &mesh) const {
        std::vector<double> p(mesh.Positions.size());
        if (p.empty()) return p;
        sf_grid cg = g_.C();
        const double *H[3] = {H_[0].data(), H_[1].data(), H_[2].data()};
        sf_status s = sf_magnetic_vertex_pressures(ctx_.Handle(), &cg, chi_, H, mesh.Positions[0].data(),
                                                   mesh.Normals[0].data(), (long long)p.size(), p.data());
        if (s != SF_OK) throw Error(s, std::string("sf_magnetic_vertex_pressures: ") + sf_last_error(ctx_.Handle()));
        return p;
    }
    sf_solve_opts &Options() { return opts_; }
    const sf_solve_stats &LastStats() const { return stats_; }
    bool Verbose = false;

   private:
    Context &ctx_;
    StaggeredGrid g_;
    double chi_, bw_;
    GridData psi_;
    SGridData H_;
    sf_solve_opts opts_;
    sf_solve_stats stats_{};
};

}  // namespace sfgpu
