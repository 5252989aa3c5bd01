// Reads a checkpoint and a mag_pressure.out with include/sfgpu_io.hpp and writes them back, so the test can check
// that the C++ and Python codecs of the reference's formats agree byte for byte.
#include <cstdio>
#include <string>

#include "sfgpu_io.hpp"

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: io_roundtrip DIR NX NY NZ\n");
        return 2;
    }
    const std::string dir = argv[1];
    const size_t nx = std::stoul(argv[2]), ny = std::stoul(argv[3]), nz = std::stoul(argv[4]);
    const std::array<size_t, 3> faces = {(nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)};
    auto ck = sfgpu::io::ReadCheckpoint(dir + "/in.sav", faces, nx * ny * nz);
    sfgpu::io::WriteCheckpoint(dir + "/out.sav", ck);
    auto m = sfgpu::io::ReadMesh(dir + "/in_mag_pressure.out", true);
    sfgpu::io::WriteMesh(dir + "/out_mag_pressure.out", m);
    std::printf("%zu timings, %zu vertices, %zu indices\n", ck.Timings.size(), m.Positions.size(), m.Indices.size());
    return 0;
}
