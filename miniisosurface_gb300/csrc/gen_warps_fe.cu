// Flying Edges pass 4 (two or four rows per warp, gen_pairs.cuh, for rows of up to 16
// words; else one row per warp, gen_warps.cuh) and the plan of the
// warp-per-row kernels.
#include "../../include/miniiso.h"
#include "gen_pairs.cuh"
#include "gen_warps.cuh"

namespace iso {

// Warp-per-row kernels take rows of up to 32 words (1024 points) whose cell
// rows number their vertices in 32 bits relative to the row's first one;
// wider grids use the row-wise kernels.
// Columns of KC planes over [kbeg, kend): about 4 waves of resident CTAs,
// at least 4 planes per column.
void gen_split(GenPlan& p, int nsm)
{
    p.nsm = nsm;
    const int nzw = p.kend - p.kbeg;
    const long long resident = (long long)nsm * kGenCtasPerSm;
    int nkc = (int)((4 * resident + p.nyb - 1) / p.nyb);
    if (nkc < 1) nkc = 1;
    p.KC = (nzw + nkc - 1) / nkc;
    if (p.KC < 4) p.KC = 4;
    if (p.KC > nzw) p.KC = nzw;
    if (p.KC < 1) p.KC = 1;
    p.nkc = nzw > 0 ? (nzw + p.KC - 1) / p.KC : 0;
}

GenPlan gen_plan(const Grid& g, int nsm)
{
    GenPlan p;
    p.J = kGenRows;
    p.nyb = (g.ny + p.J - 1) / p.J;
    p.smem = (size_t)kGenRows * gen_warp_scratch_bytes(g.W, kGenMC);
    const bool rel32 = 6.0 * g.nx * g.ny < 4294967295.0;  // two planes of vertices
    // vertex records pack i < 2^10, j < 2^27, k < 2^22
    p.fits = g.W <= 32 && rel32 && g.ny < (1 << 27) && g.nz < (1 << 22);
    p.kbeg = g.kr;
    p.kend = g.ke;
    p.kemit = g.kr;
    gen_split(p, nsm);
    return p;
}

// Grids whose pass 4 runs as k_gen_pairs + k_vertices.
static bool fe_writes_records(const Grid& g, const GenPlan& p)
{
    return g.W <= 16 && p.nsm > 0;
}

template <typename IndexT>
void launch_fe_gen_warps(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                         const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                         float* normals, IndexT* tris, int reverse, cudaStream_t s)
{
    if (fe_writes_records(g, p))  // several rows per warp
        launch_gen_pairs_impl<IndexT, kGenFE>(g, cases, b, cp, p, p.nsm, capV, capT, points, tris, reverse, s);
    else
        launch_gen_warps_impl<kGenFE, IndexT>(vol, g, iso, cases, b, cp, p, capV, capT, points, normals, tris,
                                              reverse, s);
}

bool launch_fe_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                        long long capV, long long capT, float* points, float* normals, cudaStream_t s)
{
    if (!fe_writes_records(g, p)) return false;
    launch_vertices_impl<false, 0>(vol, g, iso, b, p.kbeg, p.kend, p.nsm, capV, capT, points, normals, s);
    return true;
}

bool launch_fe_vertices_narrow(const void* vol, int dtype, const Grid& g, float iso, const FeBuffers& b,
                               const GenPlan& p, long long capV, long long capT, float* points, float* normals,
                               cudaStream_t s)
{
    if (!fe_writes_records(g, p)) return false;
    switch (dtype) {
        case ISO_INT8:
            launch_vertices_impl<false, 0, int8_t>(static_cast<const int8_t*>(vol), g, iso, b, p.kbeg, p.kend, p.nsm,
                                                   capV, capT, points, normals, s);
            break;
        case ISO_UINT8:
            launch_vertices_impl<false, 0, uint8_t>(static_cast<const uint8_t*>(vol), g, iso, b, p.kbeg, p.kend, p.nsm,
                                                    capV, capT, points, normals, s);
            break;
        case ISO_INT16:
            launch_vertices_impl<false, 0, int16_t>(static_cast<const int16_t*>(vol), g, iso, b, p.kbeg, p.kend, p.nsm,
                                                    capV, capT, points, normals, s);
            break;
        default:
            launch_vertices_impl<false, 0, uint16_t>(static_cast<const uint16_t*>(vol), g, iso, b, p.kbeg, p.kend,
                                                     p.nsm, capV, capT, points, normals, s);
            break;
    }
    return true;
}

template void launch_fe_gen_warps<uint32_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                            const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                            uint32_t*, int, cudaStream_t);
template void launch_fe_gen_warps<uint64_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                            const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                            uint64_t*, int, cudaStream_t);

}  // namespace iso

ISO_WAIT_STATS_ACCESSOR(iso_dbg_gen_waits)
