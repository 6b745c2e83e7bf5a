// Marching Cubes pass 4 (the kernels of gen_pairs.cuh for rows of up to 16
// words, else the warp-per-row kernels of gen_warps.cuh): vertex records
// in owner order with the Flying Edges -> MC index map, the vertices from the
// records (vertices.cuh), then the triangles with their corners mapped; and
// the duplicate-free order in one pass.
#include "../../include/miniiso.h"
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

bool launch_mc_vertices_narrow(const void* vol, int dtype, const Grid& g, float iso, const FeBuffers& b,
                               const GenPlan& p, long long capV, long long capT, float* points, float* normals,
                               cudaStream_t s)
{
    if (p.nsm <= 0) return false;
    switch (dtype) {
        case ISO_INT8:
            launch_vertices_impl<true, 2, int8_t>(static_cast<const int8_t*>(vol), g, iso, b, p.kemit, p.kend, p.nsm,
                                                  capV, capT, points, normals, s);
            break;
        case ISO_UINT8:
            launch_vertices_impl<true, 2, uint8_t>(static_cast<const uint8_t*>(vol), g, iso, b, p.kemit, p.kend, p.nsm,
                                                   capV, capT, points, normals, s);
            break;
        case ISO_INT16:
            launch_vertices_impl<true, 2, int16_t>(static_cast<const int16_t*>(vol), g, iso, b, p.kemit, p.kend, p.nsm,
                                                   capV, capT, points, normals, s);
            break;
        default:
            launch_vertices_impl<true, 2, uint16_t>(static_cast<const uint16_t*>(vol), g, iso, b, p.kemit, p.kend,
                                                    p.nsm, capV, capT, points, normals, s);
            break;
    }
    return true;
}

bool launch_dup_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                         long long capV, long long capT, float* points, float* normals, cudaStream_t s)
{
    if (p.nsm <= 0) return false;
    launch_vertices_impl<true, 0>(vol, g, iso, b, g.kr, g.ke, p.nsm, capV, capT, points, normals, s);
    return true;
}

// Marching Cubes over rows of up to 16 words in two passes instead of
// three: the owned vertices (records, FE -> MC map) and the triangles with
// the corners' Flying Edges ids in one generate pass, then k_mc_remap
// replaces every index by its MC id once the map is complete.
bool mc_fused(const Grid& g, const GenPlan& p) { return g.W <= 16 && p.nsm > 0 && p.kemit == g.kr; }

template <typename IndexT>
void launch_mc_gen_tris(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                        const GenPlan& p, long long capV, long long capT, float* points, IndexT* tris, int reverse,
                        cudaStream_t s)
{
    launch_gen_pairs_impl<IndexT, kGenMCT>(g, cases, b, cp, p, p.nsm, capV, capT, points, tris, reverse, s);
}

// tris[i] = fe2mc[tris[i]] for the 3 T indices (T from the totals); nothing
// when the mesh did not fit.  VEC (tris 16-byte aligned): groups of four
// indices (one 16-byte load and store each), kRemapUnroll groups per thread
// and step, all loaded before any gather so that 4 * kRemapUnroll gathers are
// in flight; the last n % 4 indices one by one.
constexpr int kRemapUnroll = 4;

template <typename IndexT>
__device__ __forceinline__ void load4(const IndexT* tris, unsigned long long q, IndexT (&v)[4])
{
    if (sizeof(IndexT) == 4) {
        const uint4 a = reinterpret_cast<const uint4*>(tris)[q];
        v[0] = (IndexT)a.x, v[1] = (IndexT)a.y, v[2] = (IndexT)a.z, v[3] = (IndexT)a.w;
    } else {
        const ulonglong2 a = reinterpret_cast<const ulonglong2*>(tris)[2 * q];
        const ulonglong2 b = reinterpret_cast<const ulonglong2*>(tris)[2 * q + 1];
        v[0] = (IndexT)a.x, v[1] = (IndexT)a.y, v[2] = (IndexT)b.x, v[3] = (IndexT)b.y;
    }
}

template <typename IndexT>
__device__ __forceinline__ void store4(IndexT* tris, unsigned long long q, const uint32_t (&m)[4])
{
    if (sizeof(IndexT) == 4) {
        reinterpret_cast<uint4*>(tris)[q] = make_uint4(m[0], m[1], m[2], m[3]);
    } else {
        reinterpret_cast<ulonglong2*>(tris)[2 * q] = make_ulonglong2(m[0], m[1]);
        reinterpret_cast<ulonglong2*>(tris)[2 * q + 1] = make_ulonglong2(m[2], m[3]);
    }
}

template <typename IndexT, bool VEC>
__global__ void k_mc_remap(IndexT* __restrict__ tris, const uint32_t* __restrict__ fe2mc,
                           const unsigned long long* __restrict__ totals, long long capV, long long capT)
{
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;
    const unsigned long long n = 3ull * totals[1];
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long t0 = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long done = 0;
    if (VEC) {
        const unsigned long long n4 = n / 4;
        for (unsigned long long q0 = t0; q0 < n4; q0 += kRemapUnroll * stride) {
            IndexT v[kRemapUnroll][4];
            uint32_t m[kRemapUnroll][4];
#pragma unroll
            for (int u = 0; u < kRemapUnroll; ++u)
                if (q0 + u * stride < n4) load4(tris, q0 + u * stride, v[u]);
#pragma unroll
            for (int u = 0; u < kRemapUnroll; ++u)
                if (q0 + u * stride < n4) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) m[u][c] = __ldg(fe2mc + (unsigned long long)v[u][c]);
                }
#pragma unroll
            for (int u = 0; u < kRemapUnroll; ++u)
                if (q0 + u * stride < n4) store4(tris, q0 + u * stride, m[u]);
        }
        done = 4 * n4;
    }
    for (unsigned long long i = done + t0; i < n; i += stride)
        tris[i] = (IndexT)__ldg(fe2mc + (unsigned long long)tris[i]);
}

template <typename IndexT>
void launch_mc_remap(const FeBuffers& b, const GenPlan& p, long long capV, long long capT, IndexT* tris,
                     cudaStream_t s)
{
    const long long wave = (long long)p.nsm * 4;  // one wave at 64 registers
    const long long need = (3 * capT / (4 * kRemapUnroll) + kThreads - 1) / kThreads;
    const unsigned blocks = (unsigned)std::max(1ll, std::min(wave, need));
    if ((reinterpret_cast<uintptr_t>(tris) & 15) == 0)
        k_mc_remap<IndexT, true><<<blocks, kThreads, 0, s>>>(tris, b.fe2mc, b.totals, capV, capT);
    else
        k_mc_remap<IndexT, false><<<blocks, kThreads, 0, s>>>(tris, b.fe2mc, b.totals, capV, capT);
}

template void launch_mc_gen_tris<uint32_t>(const Grid&, const CaseTables*, const FeBuffers&, const CountPlan&,
                                           const GenPlan&, long long, long long, float*, uint32_t*, int,
                                           cudaStream_t);
template void launch_mc_gen_tris<uint64_t>(const Grid&, const CaseTables*, const FeBuffers&, const CountPlan&,
                                           const GenPlan&, long long, long long, float*, uint64_t*, int,
                                           cudaStream_t);
template void launch_mc_remap<uint32_t>(const FeBuffers&, const GenPlan&, long long, long long, uint32_t*,
                                        cudaStream_t);
template void launch_mc_remap<uint64_t>(const FeBuffers&, const GenPlan&, long long, long long, uint64_t*,
                                        cudaStream_t);

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
