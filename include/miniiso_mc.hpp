/*
 * Marching Cubes over the miniiso C ABI, for marchingCubes/serial/main.cpp.
 *
 * The reference defines MarchingCubes<T>(util::Image3D<T> const&, T const&)
 * inside its main.cpp (marchingCubes/serial/main.cpp:42-192), so it cannot
 * be replaced by a header alone: the integration makes that function's body
 *
 *     return miniiso::marching_cubes<util::TriangleMesh<T> >(image, isoval);
 *
 * The result is the serial reference's mesh, bit for bit: vertices in
 * owner-cell / first-appearance order, size_t triangle indices.
 *
 * The image type must expose its samples, spacing and origin.  The
 * reference's marchingCubes util::Image3D<T> keeps them private, so the
 * integration adds three one-line accessors to it, the ones its Flying Edges
 * counterpart already has (flyingEdges/util/Image3D.h):
 *     const T* pointer() const { return data.data(); }
 *     std::array<T, 3> getSpacing() const { return spacing; }
 *     std::array<T, 3> getZeroPos() const { return zeroPos; }
 * Failures of the GPU path throw std::runtime_error.
 */
#ifndef MINIISO_MC_HPP
#define MINIISO_MC_HPP

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "miniiso.h"

namespace miniiso {

inline iso_ctx* mc_context()
{
    static iso_ctx* ctx = nullptr;
    static const iso_status st = iso_ctx_create(0, &ctx);  // thread-safe static init
    if (st != ISO_OK) throw std::runtime_error(std::string("miniiso: context: ") + iso_status_string(st));
    return ctx;
}

template <class Mesh, class Image, class T>
Mesh marching_cubes(Image const& image, T const& isoval)
{
    static_assert(std::is_same<T, float>::value, "the GPU path computes in float32");
    iso_ctx* ctx = mc_context();
    iso_grid g;
    g.dims[0] = (int64_t)image.xdimension();
    g.dims[1] = (int64_t)image.ydimension();
    g.dims[2] = (int64_t)image.zdimension();
    const std::array<T, 3> sp = image.getSpacing(), zp = image.getZeroPos();
    for (int a = 0; a < 3; ++a) {
        g.spacing[a] = sp[a];
        g.origin[a] = zp[a];
    }
    std::vector<std::array<T, 3> > points, normals;
    std::vector<std::array<size_t, 3> > tris;
    iso_mesh m = {};
    m.index_bytes = (int32_t)sizeof(size_t);
    // first call sizes the mesh (nothing is written), the second fills it
    iso_status st = iso_extract_host(ctx, ISO_MARCHING_CUBES, image.pointer(), &g, isoval, &m, nullptr);
    if (st == ISO_ERR_CAPACITY) {
        points.resize((size_t)m.n_points);
        normals.resize((size_t)m.n_points);
        tris.resize((size_t)m.n_tris);
        m.points = m.n_points ? points[0].data() : nullptr;
        m.normals = m.n_points ? normals[0].data() : nullptr;
        m.tris = m.n_tris ? tris[0].data() : nullptr;
        m.cap_points = m.n_points;
        m.cap_tris = m.n_tris;
        st = iso_extract_host(ctx, ISO_MARCHING_CUBES, image.pointer(), &g, isoval, &m, nullptr);
    }
    if (st != ISO_OK) {
        throw std::runtime_error(std::string("miniiso: MarchingCubes: ") + iso_status_string(st) + " (" +
                                 iso_ctx_last_error(ctx) + ")");
    }
    return Mesh(points, normals, tris);
}

}  // namespace miniiso

#endif /* MINIISO_MC_HPP */
