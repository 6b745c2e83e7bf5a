// VTK legacy IO with the layouts of miniIsosurface:
//   reader: util::loadHeader / util::loadImage (flyingEdges/util/LoadImage.h:27-198)
//           + convertBufferWithTypeInfo (ConvertBuffer.h:45-72)
//   writer: util::saveTriangleMesh (flyingEdges/util/SaveTriangleMesh.h:33-118),
//           reproduced byte for byte (big-endian floats, POLYGONS records of
//           four 8-byte big-endian words [3, a, b, c]).
// Byte-order conversion runs on all host threads (OpenMP); the file is read
// and written in one block each.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/miniiso.h"

namespace {

// Byte order: the files are big-endian, the hosts (x86-64, Arm64) little-endian.
inline uint16_t bswap(uint16_t v) { return __builtin_bswap16(v); }
inline uint32_t bswap(uint32_t v) { return __builtin_bswap32(v); }
inline uint64_t bswap(uint64_t v) { return __builtin_bswap64(v); }

template <typename T>
T from_big_endian(const unsigned char* p)
{
    using U = typename std::conditional<sizeof(T) == 2, uint16_t,
                                        typename std::conditional<sizeof(T) == 4, uint32_t, uint64_t>::type>::type;
    U u;
    std::memcpy(&u, p, sizeof(U));
    u = bswap(u);
    T v;
    std::memcpy(&v, &u, sizeof(T));
    return v;
}

template <typename T>
void to_big_endian(T v, unsigned char* p)
{
    using U = typename std::conditional<sizeof(T) == 2, uint16_t,
                                        typename std::conditional<sizeof(T) == 4, uint32_t, uint64_t>::type>::type;
    U u;
    std::memcpy(&u, &v, sizeof(U));
    u = bswap(u);
    std::memcpy(p, &u, sizeof(U));
}

// Big-endian samples of type T -> float, on all host threads.
template <typename T>
void convert_samples(const unsigned char* raw, int64_t n, float* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) out[q] = (float)from_big_endian<T>(raw + (size_t)q * sizeof(T));
}

// float[n] -> big-endian bytes, on all host threads.
void floats_to_big_endian(const float* v, int64_t n, unsigned char* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) to_big_endian<float>(v[q], out + (size_t)q * 4);
}

struct Header {
    int64_t dims[3] = {0, 0, 0};
    float spacing[3] = {1, 1, 1};
    float origin[3] = {0, 0, 0};
    int64_t npoints = 0;
    std::string type;
};

// Same acceptance rules as util::loadHeader: two discarded lines, "BINARY",
// "DATASET STRUCTURED_POINTS", DIMENSIONS/SPACING/ORIGIN in any order,
// POINT_DATA, SCALARS <name> <type>, LOOKUP_TABLE <name>.
iso_status read_header(std::ifstream& in, Header& h)
{
    std::string line, tag;
    if (!std::getline(in, line) || !std::getline(in, line)) return ISO_ERR_FORMAT;
    if (!std::getline(in, line) || line != "BINARY") return ISO_ERR_FORMAT;
    {
        if (!std::getline(in, line)) return ISO_ERR_FORMAT;
        std::stringstream ls(line);
        std::string ds;
        ls >> tag >> ds;
        if (tag != "DATASET" || ds != "STRUCTURED_POINTS" || ls.bad()) return ISO_ERR_FORMAT;
    }
    for (int q = 0; q < 3; ++q) {
        if (!std::getline(in, line)) return ISO_ERR_FORMAT;
        std::stringstream ls(line);
        ls >> tag;
        if (tag == "DIMENSIONS") {
            ls >> h.dims[0] >> h.dims[1] >> h.dims[2];
        } else if (tag == "SPACING") {
            ls >> h.spacing[0] >> h.spacing[1] >> h.spacing[2];
        } else if (tag == "ORIGIN") {
            ls >> h.origin[0] >> h.origin[1] >> h.origin[2];
        } else {
            return ISO_ERR_FORMAT;
        }
        if (ls.bad()) return ISO_ERR_FORMAT;
    }
    {
        if (!std::getline(in, line)) return ISO_ERR_FORMAT;
        std::stringstream ls(line);
        ls >> tag >> h.npoints;
        if (tag != "POINT_DATA" || ls.bad()) return ISO_ERR_FORMAT;
    }
    {
        if (!std::getline(in, line)) return ISO_ERR_FORMAT;
        std::stringstream ls(line);
        std::string name;
        ls >> tag >> name >> h.type;
        if (tag != "SCALARS" || ls.bad()) return ISO_ERR_FORMAT;
    }
    {
        if (!std::getline(in, line)) return ISO_ERR_FORMAT;
        std::stringstream ls(line);
        std::string name;
        ls >> tag >> name;
        if (tag != "LOOKUP_TABLE" || ls.bad()) return ISO_ERR_FORMAT;
    }
    return ISO_OK;
}

int type_size(const std::string& t)
{
    if (t == "char") return 1;
    if (t == "short" || t == "unsigned_short") return 2;
    if (t == "int" || t == "float") return 4;
    if (t == "double") return 8;
    return 0;
}

}  // namespace

extern "C" {

iso_status iso_vtk_read_image(const char* path, iso_grid* grid, float* data)
{
    if (!path || !grid) return ISO_ERR_INVALID_ARG;
    std::ifstream in(path, std::ios::binary);
    if (!in) return ISO_ERR_IO;
    Header h;
    iso_status st = read_header(in, h);
    if (st != ISO_OK) return st;
    const int ts = type_size(h.type);
    if (ts == 0) return ISO_ERR_FORMAT;
    for (int a = 0; a < 3; ++a) {
        grid->dims[a] = h.dims[a];
        grid->spacing[a] = h.spacing[a];
        grid->origin[a] = h.origin[a];
    }
    if (!data) return ISO_OK;
    const int64_t n = h.dims[0] * h.dims[1] * h.dims[2];
    if (h.npoints < n) return ISO_ERR_FORMAT;
    std::vector<unsigned char> raw((size_t)n * ts);
    in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)raw.size());
    if ((size_t)in.gcount() != raw.size()) return ISO_ERR_FORMAT;
    const unsigned char* p = raw.data();
    // "char" is read as a signed byte, as the reference does on its x86 hosts
    if (h.type == "char") {
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n; ++q) data[q] = (float)(int8_t)p[q];
    } else if (h.type == "short") {
        convert_samples<int16_t>(p, n, data);
    } else if (h.type == "unsigned_short") {
        convert_samples<uint16_t>(p, n, data);
    } else if (h.type == "int") {
        convert_samples<int32_t>(p, n, data);
    } else if (h.type == "float") {
        convert_samples<float>(p, n, data);
    } else {
        convert_samples<double>(p, n, data);
    }
    return ISO_OK;
}

iso_status iso_vtk_write_mesh(const char* path, const iso_mesh* mesh)
{
    if (!path || !mesh) return ISO_ERR_INVALID_ARG;
    if (mesh->index_bytes != 4 && mesh->index_bytes != 8) return ISO_ERR_INVALID_ARG;
    std::ofstream out(path, std::ios::binary);
    if (!out) return ISO_ERR_IO;
    const int64_t nv = mesh->n_points, nt = mesh->n_tris;
    out << "# vtk DataFile Version 3.0\n";
    out << "Isosurface Mesh\n";
    out << "BINARY\n";
    out << "DATASET POLYDATA\n";
    out << "POINTS " << nv << " float\n";
    std::vector<unsigned char> buf((size_t)nv * 12);
    floats_to_big_endian(mesh->points, 3 * nv, buf.data());
    out.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
    out << "\n";
    buf.assign((size_t)nt * 32, 0);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < nt; ++t) {
        unsigned char* p = &buf[(size_t)t * 32];
        to_big_endian<uint64_t>(3, p);
        for (int c = 0; c < 3; ++c) {
            uint64_t v = mesh->index_bytes == 8 ? static_cast<const uint64_t*>(mesh->tris)[3 * t + c]
                                                : static_cast<const uint32_t*>(mesh->tris)[3 * t + c];
            to_big_endian<uint64_t>(v, p + 8 * (c + 1));
        }
    }
    out << "POLYGONS " << nt << " " << nt * 4 << "\n";
    out.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
    out << "\n";
    buf.resize((size_t)nv * 12);
    floats_to_big_endian(mesh->normals, 3 * nv, buf.data());
    out << "POINT_DATA " << nv << "\n";
    out << "NORMALS Normals float\n";
    out.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
    out << "\n";
    return out.good() ? ISO_OK : ISO_ERR_IO;
}

iso_status iso_vtk_write_image(const char* path, const iso_grid* grid, const float* data)
{
    if (!path || !grid || !data) return ISO_ERR_INVALID_ARG;
    std::ofstream out(path, std::ios::binary);
    if (!out) return ISO_ERR_IO;
    const int64_t n = grid->dims[0] * grid->dims[1] * grid->dims[2];
    char line[256];
    out << "# vtk DataFile Version 3.0\n";
    out << "miniiso volume\n";
    out << "BINARY\n";
    out << "DATASET STRUCTURED_POINTS\n";
    std::snprintf(line, sizeof line, "DIMENSIONS %lld %lld %lld\n", (long long)grid->dims[0],
                  (long long)grid->dims[1], (long long)grid->dims[2]);
    out << line;
    std::snprintf(line, sizeof line, "SPACING %.9g %.9g %.9g\n", grid->spacing[0], grid->spacing[1],
                  grid->spacing[2]);
    out << line;
    std::snprintf(line, sizeof line, "ORIGIN %.9g %.9g %.9g\n", grid->origin[0], grid->origin[1], grid->origin[2]);
    out << line;
    out << "POINT_DATA " << n << "\n";
    out << "SCALARS scalars float\n";
    out << "LOOKUP_TABLE default\n";
    std::vector<unsigned char> buf((size_t)n * 4);
    floats_to_big_endian(data, n, buf.data());
    out.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
    return out.good() ? ISO_OK : ISO_ERR_IO;
}

}  // extern "C"
