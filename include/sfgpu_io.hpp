/*
 * sfgpu_io.hpp -- the reference's on-disk formats for C++ hosts of the library (header-only, no CUDA): resume a
 * GPU pipeline from a reference checkpoint and write outputs the reference's tools read.  Raw little-endian records
 * as IO::Write writes them (core/Common.h:70-91): a value's bytes, a contiguous range's bytes without a length.
 *
 *   <frame>.sav (Simulation::Save core/Simulation.cpp:118-125, StopWatch::Save core/StopWatch.cpp:18-26):
 *     velocity x, y, z face arrays (double), level set (double), init volume, cumulative and current volume error
 *     (double), max mesh size (int32), size_t timing count, NUL-terminated names, uint32 counts, double mean and
 *     max seconds.
 *   contour.out / curv.out / mag_pressure.out (SurfaceMesh::Export core/SurfaceMesh.cpp:10-20,
 *     core/Simulation.cpp:86-115): uint32 n, n float xyz positions, n float xyz normals, [n float values],
 *     uint32 m, m uint32 indices.
 */
#ifndef SFGPU_IO_HPP
#define SFGPU_IO_HPP

#include <array>
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace sfgpu {
namespace io {

template <class T>
inline void put(std::ostream &o, const T &v) {
    o.write(reinterpret_cast<const char *>(&v), sizeof(T));
}
template <class T>
inline void put(std::ostream &o, const std::vector<T> &v) {
    o.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}
template <class T>
inline void get(std::istream &i, T &v) {
    i.read(reinterpret_cast<char *>(&v), sizeof(T));
    if (!i) throw std::runtime_error("truncated record");
}
template <class T>
inline void get(std::istream &i, std::vector<T> &v) {  // v sized by the caller
    i.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
    if (!i) throw std::runtime_error("truncated record");
}

struct Timing {
    std::string Name;
    uint32_t Count = 0;
    double Mean = 0, Max = 0;
};

struct Checkpoint {
    std::array<std::vector<double>, 3> Velocity;  // face arrays in the reference layout
    std::vector<double> LevelSet;                 // cell array in the reference layout
    double InitVolume = 0, CumulVolError = 0, VolError = 0;
    int32_t MaxMeshSize = 0;
    std::vector<Timing> Timings;
};

inline void WriteCheckpoint(const std::string &path, const Checkpoint &c) {
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("cannot write " + path);
    for (int a = 0; a < 3; a++) put(o, c.Velocity[a]);
    put(o, c.LevelSet);
    put(o, c.InitVolume);
    put(o, c.CumulVolError);
    put(o, c.VolError);
    put(o, c.MaxMeshSize);
    put(o, (uint64_t)c.Timings.size());
    for (const auto &t : c.Timings) o.write(t.Name.c_str(), (std::streamsize)t.Name.size() + 1);
    for (const auto &t : c.Timings) put(o, t.Count);
    for (const auto &t : c.Timings) put(o, t.Mean);
    for (const auto &t : c.Timings) put(o, t.Max);
}

// face_counts / cells: the grid's sizes (res + e_a per face grid, res product for cells)
inline Checkpoint ReadCheckpoint(const std::string &path, const std::array<size_t, 3> &face_counts, size_t cells) {
    std::ifstream i(path, std::ios::binary);
    if (!i) throw std::runtime_error("cannot read " + path);
    Checkpoint c;
    for (int a = 0; a < 3; a++) {
        c.Velocity[a].resize(face_counts[a]);
        get(i, c.Velocity[a]);
    }
    c.LevelSet.resize(cells);
    get(i, c.LevelSet);
    get(i, c.InitVolume);
    get(i, c.CumulVolError);
    get(i, c.VolError);
    get(i, c.MaxMeshSize);
    uint64_t n = 0;
    if (i.peek() == std::char_traits<char>::eof()) return c;  // written without the timing table
    get(i, n);
    c.Timings.resize(n);
    for (auto &t : c.Timings) std::getline(i, t.Name, '\0');
    for (auto &t : c.Timings) get(i, t.Count);
    for (auto &t : c.Timings) get(i, t.Mean);
    for (auto &t : c.Timings) get(i, t.Max);
    return c;
}

struct MeshRecord {
    std::vector<std::array<float, 3>> Positions, Normals;
    std::vector<float> Values;  // empty for contour.out
    std::vector<uint32_t> Indices;
};

inline void WriteMesh(const std::string &path, const MeshRecord &m) {
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("cannot write " + path);
    put(o, (uint32_t)m.Positions.size());
    put(o, m.Positions);
    put(o, m.Normals);
    if (!m.Values.empty()) put(o, m.Values);
    put(o, (uint32_t)m.Indices.size());
    put(o, m.Indices);
}

inline MeshRecord ReadMesh(const std::string &path, bool with_values) {
    std::ifstream i(path, std::ios::binary);
    if (!i) throw std::runtime_error("cannot read " + path);
    MeshRecord m;
    uint32_t n = 0, k = 0;
    get(i, n);
    m.Positions.resize(n);
    m.Normals.resize(n);
    get(i, m.Positions);
    get(i, m.Normals);
    if (with_values) {
        m.Values.resize(n);
        get(i, m.Values);
    }
    get(i, k);
    m.Indices.resize(k);
    get(i, m.Indices);
    return m;
}

}  // namespace io
}  // namespace sfgpu

#endif  // SFGPU_IO_HPP
