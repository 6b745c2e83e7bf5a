/*
 * Drop-in FlyingEdgesAlgorithm over the miniiso C ABI.
 *
 * Replaces flyingEdges/serial/FlyingEdgesAlgorithm.h:29-49 (and the matching
 * .cpp): same constructor (util::Image3D const&, scalar_t const&), same
 * pass1() .. pass4() and moveOutput() returning util::TriangleMesh with
 * size_t triangle indices.  The passes run on the GPU; the output is the
 * serial reference's, bit for bit.
 *
 * The header uses the reference header's include guard, so a translation
 * unit that includes this one first (e.g. `g++ -include miniiso_fe.hpp`)
 * compiles the reference's flyingEdges/serial/main.cpp unchanged: its own
 * #include "FlyingEdgesAlgorithm.h" then expands to nothing.  It needs the
 * reference's util headers on the include path (FlyingEdges_Config.h,
 * Image3D.h, TriangleMesh.h) and links against libminiiso.so.
 *
 * The reference has no error path in the extraction; failures of the GPU
 * path (no device, out of memory) throw std::runtime_error here.
 */
#ifndef FLYINGEDGESALGORITHM_H_
#define FLYINGEDGESALGORITHM_H_

#include <array>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "FlyingEdges_Config.h"
#include "Image3D.h"
#include "TriangleMesh.h"
#include "miniiso.h"

namespace miniiso_compat {

// One context per process on device 0 (created on first use, kept until
// exit, like a CUDA primary context).
inline iso_ctx* shared_context()
{
    static std::once_flag once;
    static iso_ctx* ctx = nullptr;
    static iso_status st = ISO_OK;
    std::call_once(once, [] { st = iso_ctx_create(0, &ctx); });
    if (st != ISO_OK) throw std::runtime_error(std::string("miniiso: context: ") + iso_status_string(st));
    return ctx;
}

inline void check(iso_status st, const char* what)
{
    if (st == ISO_OK) return;
    std::string msg = std::string("miniiso: ") + what + ": " + iso_status_string(st);
    const char* detail = iso_ctx_last_error(shared_context());
    if (detail && *detail) msg += std::string(" (") + detail + ")";
    throw std::runtime_error(msg);
}

}  // namespace miniiso_compat

struct FlyingEdgesAlgorithm
{
    FlyingEdgesAlgorithm(util::Image3D const& image, scalar_t const& isoval)
    {
        static_assert(sizeof(scalar_t) == 4, "the GPU path computes in float32");
        iso_grid g;
        g.dims[0] = (int64_t)image.xdimension();
        g.dims[1] = (int64_t)image.ydimension();
        g.dims[2] = (int64_t)image.zdimension();
        const std::array<scalar_t, 3> sp = image.getSpacing(), zp = image.getZeroPos();
        for (int a = 0; a < 3; ++a) {
            g.spacing[a] = sp[a];
            g.origin[a] = zp[a];
        }
        // the image must outlive pass 4, as it must outlive the reference's object
        miniiso_compat::check(iso_fe_create(miniiso_compat::shared_context(), image.pointer(), &g, isoval, &fe),
                              "iso_fe_create");
    }

    ~FlyingEdgesAlgorithm()
    {
        if (fe) iso_fe_destroy(fe);
    }

    FlyingEdgesAlgorithm(FlyingEdgesAlgorithm const&) = delete;
    FlyingEdgesAlgorithm& operator=(FlyingEdgesAlgorithm const&) = delete;

    void pass1() { miniiso_compat::check(iso_fe_pass1(fe), "pass1"); }
    void pass2() { miniiso_compat::check(iso_fe_pass2(fe), "pass2"); }
    void pass3() { miniiso_compat::check(iso_fe_pass3(fe), "pass3"); }
    void pass4() { miniiso_compat::check(iso_fe_pass4(fe), "pass4"); }

    util::TriangleMesh moveOutput()
    {
        int64_t np = 0, nt = 0;
        miniiso_compat::check(iso_fe_sizes(fe, &np, &nt), "iso_fe_sizes");
        std::vector<std::array<scalar_t, 3> > points((size_t)np), normals((size_t)np);
        std::vector<std::array<size_t, 3> > tris((size_t)nt);
        iso_mesh m;
        m.points = np ? points[0].data() : nullptr;
        m.normals = np ? normals[0].data() : nullptr;
        m.tris = nt ? tris[0].data() : nullptr;
        m.index_bytes = (int32_t)sizeof(size_t);
        m.cap_points = np;
        m.cap_tris = nt;
        m.n_points = 0;
        m.n_tris = 0;
        miniiso_compat::check(iso_fe_move_output(fe, &m), "moveOutput");
        return util::TriangleMesh(std::move(points), std::move(normals), std::move(tris));
    }

private:
    iso_fe* fe = nullptr;
};

#endif /* FLYINGEDGESALGORITHM_H_ */
