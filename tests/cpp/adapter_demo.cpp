// Drives the C++ mirror of the reference classes (include/sfgpu.hpp) the way core/Simulation.cpp does:
// MagneticField::Solve, then Pressure::SetPressureJump + Project, then Extrapolation::Solve and
// Collider::Enforce; and the interface coupling from a surface mesh (CalculateVertexPressures, the jump built
// from the mesh, Project).  Reads a scene written by the test (raw arrays) and writes the results next to it.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "sfgpu.hpp"

static std::vector<double> load(const std::string &p, size_t n) {
    std::vector<double> v(n);
    std::ifstream f(p, std::ios::binary);
    f.read(reinterpret_cast<char *>(v.data()), n * sizeof(double));
    if (!f) throw std::runtime_error("cannot read " + p);
    return v;
}
static std::vector<int32_t> load_i32(const std::string &p, size_t n) {
    std::vector<int32_t> v(n);
    std::ifstream f(p, std::ios::binary);
    f.read(reinterpret_cast<char *>(v.data()), n * sizeof(int32_t));
    if (!f) throw std::runtime_error("cannot read " + p);
    return v;
}
static void save(const std::string &p, const std::vector<double> &v) {
    std::ofstream f(p, std::ios::binary);
    f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: adapter_demo DIR N CHI NVERTS\n");
        return 2;
    }
    std::string dir = argv[1];
    int n = std::stoi(argv[2]);
    double chi = std::stod(argv[3]);
    sfgpu::StaggeredGrid g(0, 1.0 / n, {n, n, n}, {0.5, 0.5, 0.5});
    sfgpu::Context ctx(0);
    auto phi = load(dir + "/phi.bin", g.NumCells());
    sfgpu::SGridData vel(g), hext(g);
    for (int a = 0; a < 3; a++) {
        vel[a] = load(dir + "/vel" + std::to_string(a) + ".bin", g.NumFaces(a));
        hext[a] = load(dir + "/hext" + std::to_string(a) + ".bin", g.NumFaces(a));
    }
    sfgpu::Collider col = sfgpu::Collider::Box(g);
    sfgpu::MagneticField mag(ctx, g, chi, 2 * g.Spacing);
    mag.Solve(phi, hext);
    sfgpu::Pressure pres(ctx, g);
    pres.SetPressureJump([](int axis, const std::array<int, 3> &face, double theta) -> double {
        return 0.01 * axis + 0.001 * face[1];  // a theta-independent jump, like the shipped callback
    });
    pres.Project(vel, phi, col, 0.0);
    save(dir + "/psi.bin", mag.Potential());
    save(dir + "/p.bin", pres.PressureField());
    for (int a = 0; a < 3; a++) {
        save(dir + "/vel_out" + std::to_string(a) + ".bin", vel[a]);
        save(dir + "/H" + std::to_string(a) + ".bin", mag.TotalField()[a]);
        save(dir + "/frac" + std::to_string(a) + ".bin", col.Fraction[a]);
    }
    // the velocity pipeline after the projection (core/Simulation.cpp:236-241)
    sfgpu::Extrapolation::Solve(ctx, g, vel, phi, col, 0., 6);
    col.Enforce(ctx, g, vel);
    for (int a = 0; a < 3; a++) {
        save(dir + "/vel_post" + std::to_string(a) + ".bin", vel[a]);
        save(dir + "/normal" + std::to_string(a) + ".bin", col.Normal[a]);
    }
    // interface coupling from the mesh written by the test (core/Simulation.cpp:204-235)
    sfgpu::SurfaceMesh mesh;
    const size_t nv = (size_t)std::stoll(argv[4]);
    auto pos = load(dir + "/pos.bin", 3 * nv), nrm = load(dir + "/nrm.bin", 3 * nv);
    mesh.Positions.resize(nv);
    mesh.Normals.resize(nv);
    for (size_t v = 0; v < nv; v++)
        for (int b = 0; b < 3; b++) {
            mesh.Positions[v][b] = pos[3 * v + b];
            mesh.Normals[v][b] = nrm[3 * v + b];
        }
    for (int a = 0; a < 3; a++) {
        size_t ne = 1;
        for (int b = 0; b < 3; b++) ne *= (size_t)(n - (a == b));
        mesh.EdgeMark[a] = load_i32(dir + "/mark" + std::to_string(a) + ".bin", ne);
    }
    std::vector<double> pm = mag.CalculateVertexPressures(mesh);
    save(dir + "/pm.bin", pm);
    sfgpu::SGridData vel2(g);
    for (int a = 0; a < 3; a++) vel2[a] = load(dir + "/vel" + std::to_string(a) + ".bin", g.NumFaces(a));
    pres.SetPressureJump(g, mesh, &pm, 0.0, 1.0, 1e-2);
    pres.Project(vel2, phi, col, 0.0);
    save(dir + "/p_mesh.bin", pres.PressureField());
    std::printf("pressure iters %d relres %.3e | magnetic iters %d relres %.3e\n", pres.LastStats().iters,
                pres.LastStats().rel_residual, mag.LastStats().iters, mag.LastStats().rel_residual);
    return 0;
}
