// Runs the C++ integration headers the way the reference's programs would:
// FlyingEdgesAlgorithm (pass1..pass4, moveOutput) and
// miniiso::marching_cubes on a seeded blob volume, and dumps both meshes as
//   int64 V, int64 T, float32 points[V][3], float32 normals[V][3], uint64 tris[T][3]
// for the test to compare with the oracle.
// Usage: shim_check nx ny nz iso out_fe.bin out_mc.bin
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "miniiso_fe.hpp"
#include "miniiso_mc.hpp"

namespace {

struct McMesh {  // the shape of marchingCubes' util::TriangleMesh<float>
    McMesh(std::vector<std::array<float, 3> > p, std::vector<std::array<float, 3> > n,
           std::vector<std::array<size_t, 3> > t)
      : points(std::move(p)), normals(std::move(n)), tris(std::move(t))
    {}
    std::vector<std::array<float, 3> > points, normals;
    std::vector<std::array<size_t, 3> > tris;
};

template <class M>
void dump(const char* path, const M& m)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) std::exit(2);
    const int64_t V = (int64_t)m.points.size(), T = (int64_t)m.tris.size();
    std::fwrite(&V, 8, 1, f);
    std::fwrite(&T, 8, 1, f);
    if (V) {
        std::fwrite(m.points.data(), 12, (size_t)V, f);
        std::fwrite(m.normals.data(), 12, (size_t)V, f);
    }
    for (const auto& t : m.tris) {
        const uint64_t w[3] = {t[0], t[1], t[2]};
        std::fwrite(w, 8, 3, f);
    }
    std::fclose(f);
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 7) return 1;
    const int64_t dims[3] = {std::atoll(argv[1]), std::atoll(argv[2]), std::atoll(argv[3])};
    const float iso = (float)std::atof(argv[4]);
    std::vector<float> vol((size_t)(dims[0] * dims[1] * dims[2]));
    if (iso_generate_blobs(dims, 6, 21, vol.data()) != ISO_OK) return 3;
    util::Image3D image(vol, {0.5f, 1.0f, 2.0f}, {-1.0f, 0.25f, 3.0f},
                        {(size_t)dims[0], (size_t)dims[1], (size_t)dims[2]});
    FlyingEdgesAlgorithm algo(image, iso);
    algo.pass1();
    algo.pass2();
    algo.pass3();
    algo.pass4();
    util::TriangleMesh fe = algo.moveOutput();
    dump(argv[5], fe);
    McMesh mc = miniiso::marching_cubes<McMesh>(image, iso);
    dump(argv[6], mc);
    std::printf("%zu %zu %zu %zu\n", fe.points.size(), fe.tris.size(), mc.points.size(), mc.tris.size());
    return 0;
}
