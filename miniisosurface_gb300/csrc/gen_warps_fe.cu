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

// The Flying Edges vertices of a list of requests (batch_kernels.cuh), one launch over the concatenation of
// their slots: slot v belongs to request list[q] for vfirst[q] <= v < vfirst[q + 1].  A CTA takes chunks of
// kVertexChunk consecutive slots (chunk c, c + gridDim.x, ...) and walks the requests a chunk overlaps -- one,
// nearly always -- with the request's parameters in shared memory (every thread sees the same requests, so
// the barriers are uniform); each thread loads its next slot's record before it works on the current one.
constexpr int kVertexChunk = 4 * kThreads;

__global__ void __launch_bounds__(kThreads, vertex_ctas_per_sm(false))
    k_vertices_batch(const BatchReq* __restrict__ reqs, const int* __restrict__ list,
                     const unsigned long long* __restrict__ vfirst, int m)
{
    __shared__ BatchReq s_d;
    constexpr int kReqWords = (int)(sizeof(BatchReq) / 4);
    const unsigned long long n = __ldg(&vfirst[m]);
    for (unsigned long long base = (unsigned long long)blockIdx.x * kVertexChunk; base < n;
         base += (unsigned long long)gridDim.x * kVertexChunk) {
        const unsigned long long end = min(base + kVertexChunk, n);
        int q = 0, hi = m - 1;  // the last q with vfirst[q] <= base
        while (q < hi) {
            const int mid = (q + hi + 1) >> 1;
            if (__ldg(&vfirst[mid]) <= base) q = mid;
            else hi = mid - 1;
        }
        for (; q < m; ++q) {
            const unsigned long long v0 = __ldg(&vfirst[q]);
            if (v0 >= end) break;
            const unsigned long long lo = max(v0, base), v1 = min(__ldg(&vfirst[q + 1]), end);
            if (v1 <= lo) continue;  // no slots of request q in the chunk
            __syncthreads();         // the previous request's reads of s_d are done
            if (threadIdx.x < kReqWords)
                reinterpret_cast<uint32_t*>(&s_d)[threadIdx.x] =
                    __ldg(reinterpret_cast<const uint32_t*>(reqs + __ldg(&list[q])) + threadIdx.x);
            __syncthreads();
            float* points = s_d.points;
            unsigned long long v = lo + threadIdx.x;
            uint2 next = v < v1 ? vertex_record(points, v - v0) : make_uint2(0u, 0u);
            for (; v < v1; v += kThreads) {
                const uint2 r = next;
                if (v + kThreads < v1) next = vertex_record(points, v + kThreads - v0);
                vertex_of_record<false, float>(s_d.vol, s_d.g, s_d.gs, s_d.iso, s_d.g.kr, s_d.g.ke, r, v - v0,
                                               points, s_d.normals);
            }
        }
    }
}

size_t gen_batch_ws_bytes(int W, int rpw) { return gen_pair_scratch_bytes(W, rpw, kGenFE); }

void launch_gen_batch(int rpw, int index_bytes, const BatchReq* reqs, const int* list, const unsigned* first, int m,
                      unsigned nitems, const CaseTables* cases, unsigned* work, int ws_bytes, int reverse, int nsm,
                      cudaStream_t s)
{
    long long blocks = ((long long)nitems + kGenRows - 1) / kGenRows;
    if (blocks > (long long)nsm * kGenPairCtasPerSm) blocks = (long long)nsm * kGenPairCtasPerSm;
    if (blocks < 1) return;
    const size_t smem = (size_t)kGenRows * ws_bytes;
#define ISO_GEN_BATCH(T, R)                                                                                    \
    {                                                                                                          \
        auto kern = k_gen_pairs_batch<T, R>;                                                                   \
        allow_smem(kern, smem);                                                                                \
        kern<<<(unsigned)blocks, kThreads, smem, s>>>(reqs, list, first, m, cases, work, ws_bytes, reverse);    \
    }
    if (index_bytes == 4) {
        if (rpw == 8) ISO_GEN_BATCH(uint32_t, 8)
        else if (rpw == 4) ISO_GEN_BATCH(uint32_t, 4)
        else ISO_GEN_BATCH(uint32_t, 2)
    } else {
        if (rpw == 8) ISO_GEN_BATCH(uint64_t, 8)
        else if (rpw == 4) ISO_GEN_BATCH(uint64_t, 4)
        else ISO_GEN_BATCH(uint64_t, 2)
    }
#undef ISO_GEN_BATCH
}

void launch_vertices_batch(const BatchReq* reqs, const int* list, const unsigned long long* vfirst, int m, int nsm,
                           cudaStream_t s)
{
    k_vertices_batch<<<(unsigned)(nsm * vertex_ctas_per_sm(false)), kThreads, 0, s>>>(reqs, list, vfirst, m);
}

template void launch_fe_gen_warps<uint32_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                            const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                            uint32_t*, int, cudaStream_t);
template void launch_fe_gen_warps<uint64_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                            const CountPlan&, const GenPlan&, long long, long long, float*, float*,
                                            uint64_t*, int, cudaStream_t);

}  // namespace iso

ISO_WAIT_STATS_ACCESSOR(iso_dbg_gen_waits)
