// Pass 4, row-wise form: one group of G lanes per grid row, reading the bit
// mask written by the count pass and the volume through the read-only cache.
// Used for the Marching Cubes triangle pass (corner ids mapped from Flying
// Edges to MC numbering) and as the general path when a volume slab of the
// column kernels does not fit in shared memory (very wide rows).
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

template <int G, typename IndexT, bool EMIT_VERTS, bool MAPPED>
__global__ void __launch_bounds__(kThreads) k_gen_rows(
    const float* __restrict__ vol, const uint32_t* __restrict__ bits, Grid g, float iso,
    const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, RowStarts rs,
    const unsigned long long* __restrict__ totals,
    long long capV, long long capT, float* __restrict__ points, float* __restrict__ normals,
    IndexT* __restrict__ tris, const uint32_t* __restrict__ fe2mc)
{
    __shared__ SharedCases s_cases;
    stage_cases(s_cases, cases, false);
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;  // caller grows buffers

    const int lane = threadIdx.x & 31;
    const int lig = lane & (G - 1), grp = lane / G;
    constexpr int RPW = 32 / G;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nchunks = (g.W + G - 1) / G;

    for (long long rb = gw * RPW; rb < g.R; rb += nw * RPW) {
        const long long r = rb + grp;
        const bool valid = r < g.R;
        const int j = valid ? (int)(r % g.ny) : 0;
        const int k = valid ? (int)(r / g.ny) : 0;
        const bool hasY = valid && j < g.ny - 1;
        const bool hasZ = valid && k < g.nz - 1;
        const bool cell = hasY && hasZ;
        // row starts (gridEdge xstart/ystart/zstart of FlyingEdgesAlgorithm.h:52-72)
        CutBases base = {0, 0, 0, 0, 0, 0, 0, 0};
        unsigned long long tb = 0;
        if (valid) {
            const uint4 cA = __ldg(&rowcnt[r]);
            base.xA = rs.get(r, 0);
            base.yA = base.xA + cA.x;
            base.zA = base.yA + cA.y;
            if (cell) {
                const long long rB = r + 1, rC = r + g.ny, rD = rC + 1;
                const uint4 cB = __ldg(&rowcnt[rB]);
                const uint4 cC = __ldg(&rowcnt[rC]);
                base.xB = rs.get(rB, 0);
                base.zB = base.xB + cB.x + cB.y;
                base.xC = rs.get(rC, 0);
                base.yC = base.xC + cC.x;
                base.xD = rs.get(rD, 0);
                tb = rs.get(r, 1);
            }
        }
        const int cj = min(j, g.ny - 2), ck = min(k, g.nz - 2);
        for (int ch = 0; ch < nchunks; ++ch) {
            const int w = ch * G + lig;
            const RowWords rw = load_row_words(bits, g, r, w, valid, hasY, hasZ);
            const uint32_t evalid = validmask(w, g.nx - 1);
            const uint32_t pvalid = validmask(w, g.nx);
            const CutMasks m = cut_masks(rw, evalid, pvalid, hasY, hasZ);
            const uint32_t act = cell ? active_cells(rw, evalid) : 0u;
            uint32_t ntri = 0;
            for (uint32_t a = act; a; a &= a - 1) ntri += iso_case_ntris(s_cases.tris[cube_case(rw, __ffs(a) - 1)]);
            // per-lane exclusive prefixes inside the chunk (two 16-bit counts per scan)
            const uint32_t p0 = __popc(m.xA) | (__popc(m.xB) << 16);
            const uint32_t p1 = __popc(m.xC) | (__popc(m.xD) << 16);
            const uint32_t p2 = __popc(m.yA) | (__popc(m.yC) << 16);
            const uint32_t p3 = __popc(m.zA) | (__popc(m.zB) << 16);
            const uint32_t i0 = group_incl_scan<G>(p0, lig, 0xffffffffu);
            const uint32_t i1 = group_incl_scan<G>(p1, lig, 0xffffffffu);
            const uint32_t i2 = group_incl_scan<G>(p2, lig, 0xffffffffu);
            const uint32_t i3 = group_incl_scan<G>(p3, lig, 0xffffffffu);
            const uint32_t i4 = group_incl_scan<G>(ntri, lig, 0xffffffffu);
            const uint32_t e0 = i0 - p0, e1 = i1 - p1, e2 = i2 - p2, e3 = i3 - p3, e4 = i4 - ntri;
            CutBases b;
            b.xA = base.xA + (e0 & 0xffffu); b.xB = base.xB + (e0 >> 16);
            b.xC = base.xC + (e1 & 0xffffu); b.xD = base.xD + (e1 >> 16);
            b.yA = base.yA + (e2 & 0xffffu); b.yC = base.yC + (e2 >> 16);
            b.zA = base.zA + (e3 & 0xffffu); b.zB = base.zB + (e3 >> 16);

            if (EMIT_VERTS) {
                // vertices owned by grid row r (FlyingEdgesAlgorithm.cpp:340-484)
#pragma unroll 1
                for (int axis = 0; axis < 3; ++axis) {
                    const uint32_t mm = axis == 0 ? m.xA : (axis == 1 ? m.yA : m.zA);
                    const unsigned long long bb = axis == 0 ? b.xA : (axis == 1 ? b.yA : b.zA);
                    for (uint32_t a = mm; a; a &= a - 1) {
                        const int bit = __ffs(a) - 1, i = 32 * w + bit;
                        const unsigned long long id = bb + __popc(mm & lowmask(bit));
                        float3 p, n;
                        edge_vertex(vol, g, iso, axis, i, j, k, axis == 0 ? i : min(i, g.nx - 2),
                                    axis == 1 ? j : cj, axis == 2 ? k : ck, p, n);
                        points[3 * id + 0] = p.x; points[3 * id + 1] = p.y; points[3 * id + 2] = p.z;
                        normals[3 * id + 0] = n.x; normals[3 * id + 1] = n.y; normals[3 * id + 2] = n.z;
                    }
                }
            }

            // triangles of cell row (j,k)
            unsigned long long tcur = tb + e4;
            for (uint32_t a = act; a; a &= a - 1) {
                const int bit = __ffs(a) - 1;
                const uint64_t tl = s_cases.tris[cube_case(rw, bit)];
                const int nt = iso_case_ntris(tl);
                for (int q = 0; q < 3 * nt; ++q) {
                    const unsigned long long id = fe_edge_id(m, b, iso_case_edge(tl, q), bit);
                    tris[3 * tcur + q] = MAPPED ? (IndexT)__ldg(fe2mc + id) : (IndexT)id;
                }
                tcur += nt;
            }
            // carry the chunk totals to the next chunk (rows wider than 32*G points)
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
                tb += t4;
            }
        }
    }
}

template <int G>
__global__ void __launch_bounds__(kThreads) k_mc_vertices_rows(
    const float* __restrict__ vol, const uint32_t* __restrict__ bits, Grid g, float iso,
    const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, RowStarts rs,
    const unsigned long long* __restrict__ totals,
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
            base.xA = rs.get(r, 0);
            base.yA = base.xA + cA.x;
            base.zA = base.yA + cA.y;
            base.xB = rs.get(rB, 0);
            base.zB = base.xB + cB.x + cB.y;
            base.xC = rs.get(rC, 0);
            base.yC = base.xC + cC.x;
            base.xD = rs.get(rD, 0);
            mb = rs.get(r, 2);
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

static long long row_blocks(const Grid& g, int nsm)
{
    const int rpw = 32 / lanes_per_row(g.W);
    const long long warps_needed = (g.R + rpw - 1) / rpw;
    long long blocks = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
    const long long cap = (long long)nsm * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return blocks;
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

template <typename IndexT>
void launch_fe_gen_rows(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                        const CountPlan& cp, long long capV, long long capT, float* points, float* normals,
                        IndexT* tris, int nsm, cudaStream_t s)
{
    const unsigned blocks = (unsigned)row_blocks(g, nsm);
    const RowStarts rs = row_starts(g, cp, b);
    ISO_DISPATCH_G(lanes_per_row(g.W), (k_gen_rows<kG, IndexT, true, false><<<blocks, kThreads, 0, s>>>(
                                           vol, b.bits, g, iso, cases, b.rowcnt, rs, b.totals, capV, capT, points,
                                           normals, tris, nullptr)));
}

template <typename IndexT>
void launch_mc_triangles(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                         long long capV, long long capT, IndexT* tris, int nsm, cudaStream_t s)
{
    const unsigned blocks = (unsigned)row_blocks(g, nsm);
    const RowStarts rs = row_starts(g, cp, b);
    ISO_DISPATCH_G(lanes_per_row(g.W), (k_gen_rows<kG, IndexT, false, true><<<blocks, kThreads, 0, s>>>(
                                           nullptr, b.bits, g, 0.f, cases, b.rowcnt, rs, b.totals, capV, capT,
                                           nullptr, nullptr, tris, b.fe2mc)));
}

void launch_mc_vertices_rows(const float* vol, const Grid& g, float iso, const CaseTables* cases,
                             const FeBuffers& b, const CountPlan& cp, long long capV, long long capT, float* points,
                             float* normals, int nsm, cudaStream_t s)
{
    const unsigned blocks = (unsigned)row_blocks(g, nsm);
    const RowStarts rs = row_starts(g, cp, b);
    ISO_DISPATCH_G(lanes_per_row(g.W), (k_mc_vertices_rows<kG><<<blocks, kThreads, 0, s>>>(
                                           vol, b.bits, g, iso, cases, b.rowcnt, rs, b.totals, capV, capT, points,
                                           normals, b.fe2mc)));
}

#define ISO_INST(IndexT)                                                                                        \
    template void launch_fe_gen_rows<IndexT>(const float*, const Grid&, float, const CaseTables*,              \
                                             const FeBuffers&, const CountPlan&, long long, long long, float*, \
                                             float*, IndexT*, int, cudaStream_t);                              \
    template void launch_mc_triangles<IndexT>(const Grid&, const CaseTables*, const FeBuffers&,               \
                                              const CountPlan&, long long, long long, IndexT*, int, cudaStream_t);
ISO_INST(uint32_t)
ISO_INST(uint64_t)
#undef ISO_INST

}  // namespace iso
