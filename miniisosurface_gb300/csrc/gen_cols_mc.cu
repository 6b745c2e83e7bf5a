// Marching Cubes vertices, column-marching kernel instantiation (gen_cols.cuh).
#include "gen_cols.cuh"

namespace iso {

void launch_mc_gen_cols(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                        const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                        float* normals, int reverse, cudaStream_t s)
{
    launch_gen_cols_impl<true, uint32_t>(vol, g, iso, cases, b, cp, p, capV, capT, points, normals, nullptr, reverse,
                                         s);
}

}  // namespace iso
