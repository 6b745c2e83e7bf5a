// Flying Edges pass 4, column-marching kernel instantiations (gen_cols.cuh).
#include "gen_cols.cuh"

namespace iso {

// Column kernels run 2 CTAs per SM when their shared memory stays under
// kTwoPerSm bytes; rows too wide for kOnePerSm take the row-wise kernels.
constexpr size_t kTwoPerSm = 104 * 1024;
constexpr size_t kOnePerSm = 200 * 1024;

GenPlan gen_plan(const Grid& g, int nsm)
{
    GenPlan p;
    int G = lanes_per_row(g.W);
    if (G < 4) G = 4;
    size_t smem = 0;
    for (;;) {
        smem = GenLayout(kThreads / G, g.W, g.nx).total;
        if (smem <= kTwoPerSm || G == 32) break;
        G *= 2;
    }
    if (smem > kOnePerSm) return p;
    p.fits = true;
    p.G = G;
    p.J = kThreads / G;
    p.smem = smem;
    p.nyb = (g.ny + p.J - 1) / p.J;
    const long long resident = (long long)nsm * (smem <= kTwoPerSm ? 2 : 1);
    int nkc = (int)((4 * resident + p.nyb - 1) / p.nyb);
    if (nkc < 1) nkc = 1;
    p.KC = (g.nz + nkc - 1) / nkc;
    if (p.KC < 4) p.KC = 4;
    if (p.KC > g.nz) p.KC = g.nz;
    p.nkc = (g.nz + p.KC - 1) / p.KC;
    return p;
}

template <typename IndexT>
void launch_fe_gen_cols(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                        const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                        float* normals, IndexT* tris, int reverse, cudaStream_t s)
{
    launch_gen_cols_impl<false, IndexT>(vol, g, iso, cases, b, cp, p, capV, capT, points, normals, tris, reverse, s);
}

template void launch_fe_gen_cols<uint32_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                           const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                           uint32_t*, int, cudaStream_t);
template void launch_fe_gen_cols<uint64_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                           const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                           uint64_t*, int, cudaStream_t);

}  // namespace iso
