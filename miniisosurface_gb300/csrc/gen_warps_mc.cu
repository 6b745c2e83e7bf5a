// Marching Cubes pass 4 (the kernels of gen_pairs.cuh for rows of up to 16
// words, else the warp-per-row kernels of gen_warps.cuh): vertex records
// in owner order with the Flying Edges -> MC index map, the vertices from the
// records (vertices.cuh), then the triangles with their corners mapped; and
// the duplicate-free order in one pass.
#include "gen_pairs.cuh"
#include "gen_warps.cuh"
#include "vertices.cuh"

namespace iso {

void launch_mc_gen_warps(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                         const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                         float* normals, int reverse, cudaStream_t s)
{
    if (g.W <= 16 && p.nsm > 0)  // several rows per warp
        launch_gen_pairs_impl<uint32_t, kGenMC>(g, cases, b, cp, p, p.nsm, capV, capT, points, nullptr, reverse, s);
    else
        launch_gen_warps_impl<kGenMC, uint32_t>(vol, g, iso, cases, b, cp, p, capV, capT, points, normals, nullptr,
                                                reverse, s);
}

bool launch_mc_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                        long long capV, long long capT, float* points, float* normals, cudaStream_t s)
{
    if (p.nsm <= 0) return false;
    launch_vertices_impl<true, 2>(vol, g, iso, b, p.kemit, p.kend, p.nsm, capV, capT, points, normals, s);
    return true;
}

bool launch_dup_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                         long long capV, long long capT, float* points, float* normals, cudaStream_t s)
{
    if (p.nsm <= 0) return false;
    launch_vertices_impl<true, 0>(vol, g, iso, b, g.kr, g.ke, p.nsm, capV, capT, points, normals, s);
    return true;
}

template <typename IndexT>
void launch_mc_tri_warps(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                         const GenPlan& p, long long capV, long long capT, IndexT* tris, cudaStream_t s)
{
    if (g.W <= 16 && p.nsm > 0)  // several rows per warp
        launch_gen_pairs_impl<IndexT, kGenTri>(g, cases, b, cp, p, p.nsm, capV, capT, nullptr, tris, 0, s);
    else
        launch_gen_warps_impl<kGenTri, IndexT>(nullptr, g, 0.f, cases, b, cp, p, capV, capT, nullptr, nullptr, tris,
                                               0, s);
}

template <typename IndexT>
void launch_dup_gen_warps(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                          const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                          float* normals, IndexT* tris, int reverse, cudaStream_t s)
{
    launch_gen_warps_impl<kGenDup, IndexT>(vol, g, iso, cases, b, cp, p, capV, capT, points, normals, tris, reverse,
                                           s);
}

template void launch_dup_gen_warps<uint32_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                             const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                             uint32_t*, int, cudaStream_t);
template void launch_dup_gen_warps<uint64_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                             const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                             uint64_t*, int, cudaStream_t);
template void launch_mc_tri_warps<uint32_t>(const Grid&, const CaseTables*, const FeBuffers&, const CountPlan&,
                                            const GenPlan&, long long, long long, uint32_t*, cudaStream_t);
template void launch_mc_tri_warps<uint64_t>(const Grid&, const CaseTables*, const FeBuffers&, const CountPlan&,
                                            const GenPlan&, long long, long long, uint64_t*, cudaStream_t);

}  // namespace iso
