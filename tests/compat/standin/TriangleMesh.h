// Stand-in for the reference's util::TriangleMesh (flyingEdges/util/TriangleMesh.h)
// in the shim test: the moving constructor and read access.
#pragma once
#include <array>
#include <vector>

#include "FlyingEdges_Config.h"

namespace util {

class TriangleMesh
{
public:
    TriangleMesh(std::vector<std::array<scalar_t, 3> >&& p, std::vector<std::array<scalar_t, 3> >&& n,
                 std::vector<std::array<size_t, 3> >&& t)
      : points(std::move(p)), normals(std::move(n)), tris(std::move(t))
    {}
    std::vector<std::array<scalar_t, 3> > points, normals;
    std::vector<std::array<size_t, 3> > tris;
};

}  // namespace util
