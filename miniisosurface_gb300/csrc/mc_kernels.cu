// Marching Cubes vertices on sm_103a (marchingCubes/serial/main.cpp:42-192).
//
// The serial reference walks cells in (k, j, i) order and creates a vertex
// the first time a triangle corner references an edge (std::unordered_map
// keyed by the global edge id, :139-177).  Because every cut edge of a case
// appears in its triangle list, that first reference always comes from the
// adjacent cell with the smallest linear index, so the numbering is:
//
//   cell rows in order -> cells by i -> the cell's owned cut edges in order
//   of first appearance in its triangle list,
//
// where an interior cell owns e5, e6 and e11, and cells on the i=0 / j=0 /
// k=0 faces own the extra edges returned by mc_owned_edges().  The count pass
// (k_count<.., true>) gives each cell row its number of owned vertices; this
// kernel writes them, computed with the owner cell's cube exactly as the
// reference does (getPosCube / getGradCube of that cell), and records the
// MC index of each vertex under its Flying Edges index.  The triangle pass of
// fe_kernels.cu then maps its Flying Edges corner ids through that table:
// the triangle sequence of both algorithms is the same.
#include "iso_kernels.h"
#include "iso_device.cuh"

namespace iso {

template <int G>
__global__ void __launch_bounds__(kThreads) k_mc_vertices(
    const float* __restrict__ vol, const uint32_t* __restrict__ bits, Grid g, float iso,
    const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, const uint4* __restrict__ rowpre,
    const unsigned long long* __restrict__ tiles, long long ntiles, const unsigned long long* __restrict__ totals,
    long long capV, long long capT, float* __restrict__ points, float* __restrict__ normals,
    uint32_t* __restrict__ fe2mc)
{
    __shared__ SharedCases s_cases;
    stage_cases(s_cases, cases, true);
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;

    const int lane = threadIdx.x & 31;
    const int lig = lane & (G - 1), grp = lane / G;
    constexpr int RPW = 32 / G;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nchunks = (g.W + G - 1) / G;
    const unsigned long long* tiles_v = tiles;
    const unsigned long long* tiles_m = tiles + 2 * ntiles;

    for (long long rb = gw * RPW; rb < g.R; rb += nw * RPW) {
        const long long r = rb + grp;
        const bool valid = r < g.R;
        const int j = valid ? (int)(r % g.ny) : 0;
        const int k = valid ? (int)(r / g.ny) : 0;
        const bool hasY = valid && j < g.ny - 1;
        const bool hasZ = valid && k < g.nz - 1;
        const bool cell = hasY && hasZ;
        CutBases base = {0, 0, 0, 0, 0, 0, 0, 0};
        unsigned long long mb = 0;
        if (cell) {
            const uint4 cA = __ldg(&rowcnt[r]);
            const long long rB = r + 1, rC = r + g.ny, rD = rC + 1;
            const uint4 cB = __ldg(&rowcnt[rB]);
            const uint4 cC = __ldg(&rowcnt[rC]);
            base.xA = row_base(tiles_v, rowpre, r, 0);
            base.yA = base.xA + cA.x;
            base.zA = base.yA + cA.y;
            base.xB = row_base(tiles_v, rowpre, rB, 0);
            base.zB = base.xB + cB.x + cB.y;
            base.xC = row_base(tiles_v, rowpre, rC, 0);
            base.yC = base.xC + cC.x;
            base.xD = row_base(tiles_v, rowpre, rD, 0);
            mb = row_base(tiles_m, rowpre, r, 2);
        }
        for (int ch = 0; ch < nchunks; ++ch) {
            const int w = ch * G + lig;
            const RowWords rw = load_row_words(bits, g, r, w, valid, hasY, hasZ);
            const uint32_t evalid = validmask(w, g.nx - 1);
            const uint32_t pvalid = validmask(w, g.nx);
            const CutMasks m = cut_masks(rw, evalid, pvalid, hasY, hasZ);
            const uint32_t act = cell ? active_cells(rw, evalid) : 0u;
            uint32_t nown = 0;
            for (uint32_t a = act; a; a &= a - 1) {
                const int bit = __ffs(a) - 1;
                const int c = cube_case(rw, bit);
                nown += __popc(mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cases.cut[c]);
            }
            const uint32_t p0 = __popc(m.xA) | (__popc(m.xB) << 16);
            const uint32_t p1 = __popc(m.xC) | (__popc(m.xD) << 16);
            const uint32_t p2 = __popc(m.yA) | (__popc(m.yC) << 16);
            const uint32_t p3 = __popc(m.zA) | (__popc(m.zB) << 16);
            const uint32_t i0 = group_incl_scan<G>(p0, lig, 0xffffffffu);
            const uint32_t i1 = group_incl_scan<G>(p1, lig, 0xffffffffu);
            const uint32_t i2 = group_incl_scan<G>(p2, lig, 0xffffffffu);
            const uint32_t i3 = group_incl_scan<G>(p3, lig, 0xffffffffu);
            const uint32_t i4 = group_incl_scan<G>(nown, lig, 0xffffffffu);
            const uint32_t e0 = i0 - p0, e1 = i1 - p1, e2 = i2 - p2, e3 = i3 - p3;
            CutBases b;
            b.xA = base.xA + (e0 & 0xffffu); b.xB = base.xB + (e0 >> 16);
            b.xC = base.xC + (e1 & 0xffffu); b.xD = base.xD + (e1 >> 16);
            b.yA = base.yA + (e2 & 0xffffu); b.yC = base.yC + (e2 >> 16);
            b.zA = base.zA + (e3 & 0xffffu); b.zB = base.zB + (e3 >> 16);
            unsigned long long id = mb + (i4 - nown);
            for (uint32_t a = act; a; a &= a - 1) {
                const int bit = __ffs(a) - 1, i = 32 * w + bit;
                const int c = cube_case(rw, bit);
                const uint32_t own = mc_owned_edges(i == 0, j == 0, k == 0) & s_cases.cut[c];
                if (!own) continue;
                const uint64_t ord = s_cases.order[c];
                const int ne = iso_case_ntris(ord);  // number of distinct edges (top nibble)
                for (int q = 0; q < ne; ++q) {
                    const int e = iso_case_edge(ord, q);
                    if (!((own >> e) & 1u)) continue;
                    int dx, dy, dz, axis;
                    cube_edge_geometry(e, dx, dy, dz, axis);
                    float3 p, n;
                    edge_vertex(vol, g, iso, axis, i + dx, j + dy, k + dz, i, j, k, p, n);
                    points[3 * id + 0] = p.x; points[3 * id + 1] = p.y; points[3 * id + 2] = p.z;
                    normals[3 * id + 0] = n.x; normals[3 * id + 1] = n.y; normals[3 * id + 2] = n.z;
                    fe2mc[fe_edge_id(m, b, e, bit)] = (uint32_t)id;
                    ++id;
                }
            }
            if (nchunks > 1) {
                const uint32_t t0 = group_bcast<G>(i0, G - 1, 0xffffffffu);
                const uint32_t t1 = group_bcast<G>(i1, G - 1, 0xffffffffu);
                const uint32_t t2 = group_bcast<G>(i2, G - 1, 0xffffffffu);
                const uint32_t t3 = group_bcast<G>(i3, G - 1, 0xffffffffu);
                const uint32_t t4 = group_bcast<G>(i4, G - 1, 0xffffffffu);
                base.xA += t0 & 0xffffu; base.xB += t0 >> 16;
                base.xC += t1 & 0xffffu; base.xD += t1 >> 16;
                base.yA += t2 & 0xffffu; base.yC += t2 >> 16;
                base.zA += t3 & 0xffffu; base.zB += t3 >> 16;
                mb += t4;
            }
        }
    }
}

#define ISO_DISPATCH_G(G, ...)                                  \
    switch (G) {                                                \
        case 1: { constexpr int kG = 1; __VA_ARGS__; } break;   \
        case 2: { constexpr int kG = 2; __VA_ARGS__; } break;   \
        case 4: { constexpr int kG = 4; __VA_ARGS__; } break;   \
        case 8: { constexpr int kG = 8; __VA_ARGS__; } break;   \
        case 16: { constexpr int kG = 16; __VA_ARGS__; } break; \
        default: { constexpr int kG = 32; __VA_ARGS__; } break; \
    }

void launch_mc_vertices(const float* vol, const uint32_t* bits, const Grid& g, float iso, const CaseTables* cases,
                        const FeBuffers& b, long long capV, long long capT, float* points, float* normals, int nsm,
                        cudaStream_t s)
{
    const int G = lanes_per_row(g.W);
    const int rpw = 32 / G;
    const long long warps_needed = (g.R + rpw - 1) / rpw;
    long long blocks = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
    const long long cap = (long long)nsm * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    const long long ntiles = (g.R + kTileRows - 1) / kTileRows;
    ISO_DISPATCH_G(G, (k_mc_vertices<kG><<<(unsigned)blocks, kThreads, 0, s>>>(
                          vol, bits, g, iso, cases, b.rowcnt, b.rowpre, b.tiles, ntiles, b.totals, capV, capT,
                          points, normals, b.fe2mc)));
}

}  // namespace iso
