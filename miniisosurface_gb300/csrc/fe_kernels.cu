// Flying Edges on sm_103a: the four passes of
// flyingEdges/serial/FlyingEdgesAlgorithm.cpp, re-designed around a 1-bit
// per point "value >= isovalue" mask instead of per-edge case bytes.
//
//   pass 1  k_classify       volume -> bit rows                     (FlyingEdgesAlgorithm.cpp:23-45)
//   pass 2  k_count          bit rows -> per-row x/y/z cuts, trims,
//                            triangle counts, in-tile prefix sums    (:47-65, :72-190)
//   pass 3  k_scan_tiles     tile totals -> tile offsets, totals     (:196-269)
//   pass 4  k_generate       points, normals, triangles              (:275-497)
//
// Vertex numbering follows the reference exactly: grid rows (j,k) in k-major
// order, and inside a row all cut x-edges by i, then the cut y-edges
// (i,j,k)->(i,j+1,k) by i, then the cut z-edges (i,j,k)->(i,j,k+1) by i.
// A vertex id is therefore row offset + popc of the cut mask below i.
// Triangles follow cell order (k, j, i) and the case table order.
//
// The same count / scan / triangle kernels serve Marching Cubes
// (marchingCubes/serial/main.cpp:42-192): the count pass adds the number of
// vertices each cell row owns under the MC numbering, mc_kernels.cu writes the
// MC-numbered vertices plus a map from Flying Edges index to MC index, and the
// triangle pass here translates its Flying Edges ids through that map.
#include "iso_kernels.h"
#include "iso_device.cuh"

namespace iso {

// ---------------------------------------------------------------------------
// pass 1: classification.  One warp per x-row; each lane turns 4 values into
// a nibble of the row's bit mask.  The float4 variant needs 16-byte aligned
// rows (nx % 4 == 0, aligned base); the scalar variant takes any layout.
// ---------------------------------------------------------------------------
template <int U>
__global__ void __launch_bounds__(kThreads) k_classify_vec4(const float4* __restrict__ vol4,
                                                            uint32_t* __restrict__ bits, int nx,
                                                            int W, long long R, float iso)
{
    const int lane = threadIdx.x & 31;
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nq = nx >> 2;
    for (long long row = warp0; row < R; row += nwarps) {
        const float4* src = vol4 + row * nq;
        uint32_t* dst = bits + row * W;
        for (int q0 = 0; q0 < nq; q0 += 32 * U) {
            float4 v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int q = q0 + u * 32 + lane;
                v[u] = q < nq ? __ldcs(src + q) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int q = q0 + u * 32 + lane;
                uint32_t nib = 0;
                if (q < nq) {
                    nib = (uint32_t)(v[u].x >= iso) | ((uint32_t)(v[u].y >= iso) << 1) |
                          ((uint32_t)(v[u].z >= iso) << 2) | ((uint32_t)(v[u].w >= iso) << 3);
                }
                uint32_t word = nib << (4 * (lane & 7));
                word |= __shfl_xor_sync(0xffffffffu, word, 1);
                word |= __shfl_xor_sync(0xffffffffu, word, 2);
                word |= __shfl_xor_sync(0xffffffffu, word, 4);
                if ((lane & 7) == 0 && q < nq) dst[q >> 3] = word;
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_classify_scalar(const float* __restrict__ vol,
                                                              uint32_t* __restrict__ bits, int nx,
                                                              int W, long long R, float iso)
{
    const int lane = threadIdx.x & 31;
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    constexpr int U = 4;
    for (long long row = warp0; row < R; row += nwarps) {
        const float* src = vol + row * nx;
        uint32_t* dst = bits + row * W;
        for (int w0 = 0; w0 < W; w0 += U) {
            float v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = 32 * (w0 + u) + lane;
                v[u] = i < nx ? __ldcs(src + i) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = 32 * (w0 + u) + lane;
                const uint32_t word = __ballot_sync(0xffffffffu, i < nx && v[u] >= iso);
                if (lane == 0 && w0 + u < W) dst[w0 + u] = word;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// pass 2: per grid row counts + trims + triangle counts (+ MC owned vertex
// counts), then an exclusive scan over the tile.  G lanes cooperate on one
// row (G = min(32, pow2 >= W)); a CTA covers kTileRows consecutive rows.
// ---------------------------------------------------------------------------
template <int G, bool MC>
__global__ void __launch_bounds__(kThreads) k_count(const uint32_t* __restrict__ bits, Grid g,
                                                    const CaseTables* __restrict__ cases,
                                                    uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                                    uint32_t* __restrict__ mccnt, uint4* __restrict__ rowpre,
                                                    unsigned long long* __restrict__ tiles, long long ntiles)
{
    __shared__ uint32_t s_cnt[3][kTileRows];
    __shared__ uint8_t s_ntris[256];
    __shared__ uint16_t s_cut[256];
    __shared__ uint32_t s_wsum[3][kThreads / 32];
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        s_ntris[c] = (uint8_t)iso_case_ntris(cases->tris[c]);
        s_cut[c] = cases->cut[c];
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lig = lane & (G - 1), grp = lane / G;
    constexpr int RPW = 32 / G;
    const long long r0 = (long long)blockIdx.x * kTileRows;
    const int nchunks = (g.W + G - 1) / G;

    for (int it = 0; it < 32 / RPW; ++it) {
        const int tr = warp * 32 + it * RPW + grp;
        const long long r = r0 + tr;
        const bool valid = r < g.R;
        const int j = valid ? (int)(r % g.ny) : 0;
        const int k = valid ? (int)(r / g.ny) : 0;
        const bool hasY = valid && j < g.ny - 1;
        const bool hasZ = valid && k < g.nz - 1;
        const bool cell = hasY && hasZ;
        uint32_t xc = 0, yc = 0, zc = 0, tc = 0, mc = 0, first = 0xffffffffu, last = 0;
        for (int ch = 0; ch < nchunks; ++ch) {
            const int w = ch * G + lig;
            const RowWords rw = load_row_words(bits, g, r, w, valid, hasY, hasZ);
            const uint32_t evalid = validmask(w, g.nx - 1);   // x-edges / cells: i <= nx-2
            const uint32_t pvalid = validmask(w, g.nx);       // points: i <= nx-1
            const uint32_t xm = (rw.a ^ rw.ash) & evalid;
            const uint32_t ym = hasY ? ((rw.a ^ rw.b) & pvalid) : 0u;
            const uint32_t zm = hasZ ? ((rw.a ^ rw.c) & pvalid) : 0u;
            xc += __popc(xm);
            yc += __popc(ym);
            zc += __popc(zm);
            // isCutEdge (FlyingEdgesAlgorithm.cpp:515-554): edge i is marked when
            // it is cut or the y/z edge at its left point is.
            const uint32_t marked = xm | ((ym | zm) & evalid);
            if (marked) {
                first = min(first, (uint32_t)(32 * w + __ffs(marked) - 1));
                last = max(last, (uint32_t)(32 * w + 32 - __clz(marked)));
            }
            if (cell) {
                uint32_t act = active_cells(rw, evalid);
                while (act) {
                    const int bit = __ffs(act) - 1;
                    act &= act - 1;
                    const int c = cube_case(rw, bit);
                    tc += s_ntris[c];
                    if (MC) mc += __popc(mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cut[c]);
                }
            }
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) {
            xc += __shfl_xor_sync(0xffffffffu, xc, d, G);
            yc += __shfl_xor_sync(0xffffffffu, yc, d, G);
            zc += __shfl_xor_sync(0xffffffffu, zc, d, G);
            tc += __shfl_xor_sync(0xffffffffu, tc, d, G);
            if (MC) mc += __shfl_xor_sync(0xffffffffu, mc, d, G);
        }
        first = group_min<G>(first, 0xffffffffu);
        last = group_max<G>(last, 0xffffffffu);
        if (lig == 0) {
            if (valid) {
                rowcnt[r] = make_uint4(xc, yc, zc, tc);
                trims[r] = make_uint2(first == 0xffffffffu ? (uint32_t)g.nx : first, last);
                if (MC) mccnt[r] = mc;
            }
            s_cnt[0][tr] = valid ? xc + yc + zc : 0u;
            s_cnt[1][tr] = valid ? tc : 0u;
            s_cnt[2][tr] = valid ? mc : 0u;
        }
    }
    __syncthreads();

    // exclusive scan of the tile's (vertex, triangle, mc vertex) counts
    const int t = threadIdx.x;
    uint32_t v[3], incl[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) { v[q] = s_cnt[q][t]; incl[q] = v[q]; }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const uint32_t a = __shfl_up_sync(0xffffffffu, incl[q], d);
            if (lane >= d) incl[q] += a;
        }
    }
    if (lane == 31) {
#pragma unroll
        for (int q = 0; q < 3; ++q) s_wsum[q][warp] = incl[q];
    }
    __syncthreads();
    uint32_t off[3] = {0, 0, 0}, tot[3] = {0, 0, 0};
    for (int w = 0; w < kThreads / 32; ++w) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (w < warp) off[q] += s_wsum[q][w];
            tot[q] += s_wsum[q][w];
        }
    }
    const long long r = r0 + t;
    if (r < g.R) rowpre[r] = make_uint4(off[0] + incl[0] - v[0], off[1] + incl[1] - v[1], off[2] + incl[2] - v[2], 0u);
    if (t == 0) {
        tiles[blockIdx.x] = tot[0];
        tiles[ntiles + blockIdx.x] = tot[1];
        tiles[2 * ntiles + blockIdx.x] = tot[2];
    }
}

// ---------------------------------------------------------------------------
// pass 3: exclusive scan of the tile totals (one CTA), plus the grand totals.
// tiles holds three arrays of ntiles (vertices, triangles, mc vertices).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_scan_tiles(unsigned long long* __restrict__ tiles, long long ntiles,
                                                     unsigned long long* __restrict__ totals)
{
    __shared__ unsigned long long s_w[3][32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long long per = (ntiles + blockDim.x - 1) / blockDim.x;
    const long long b = t * per, e = min(ntiles, b + per);
    unsigned long long s[3] = {0, 0, 0}, incl[3];
    for (long long q = b; q < e; ++q) {
#pragma unroll
        for (int a = 0; a < 3; ++a) s[a] += tiles[a * ntiles + q];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) incl[a] = s[a];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const unsigned long long x = __shfl_up_sync(0xffffffffu, incl[a], d);
            if (lane >= d) incl[a] += x;
        }
    }
    if (lane == 31) {
#pragma unroll
        for (int a = 0; a < 3; ++a) s_w[a][warp] = incl[a];
    }
    __syncthreads();
    unsigned long long run[3] = {0, 0, 0}, tot[3] = {0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (w < warp) run[a] += s_w[a][w];
            tot[a] += s_w[a][w];
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) run[a] += incl[a] - s[a];
    for (long long q = b; q < e; ++q) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const unsigned long long x = tiles[a * ntiles + q];
            tiles[a * ntiles + q] = run[a];
            run[a] += x;
        }
    }
    if (t == 0) {
        totals[0] = tot[0];
        totals[1] = tot[1];
        totals[2] = tot[2];
    }
}

// ---------------------------------------------------------------------------
// pass 4: points, normals and triangles.  One group of G lanes per grid row
// r = (j,k): it writes the vertices owned by grid row r (EMIT_VERTS) and the
// triangles of cell row (j,k).  With a map (Marching Cubes) the triangle
// corners are translated from Flying Edges to MC vertex numbering.
// ---------------------------------------------------------------------------
template <int G, typename IndexT, bool EMIT_VERTS, bool MAPPED>
__global__ void __launch_bounds__(kThreads) k_generate(
    const float* __restrict__ vol, const uint32_t* __restrict__ bits, Grid g, float iso,
    const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, const uint4* __restrict__ rowpre,
    const unsigned long long* __restrict__ tiles, long long ntiles, const unsigned long long* __restrict__ totals,
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
    const unsigned long long* tiles_v = tiles;
    const unsigned long long* tiles_t = tiles + ntiles;

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
            base.xA = row_base(tiles_v, rowpre, r, 0);
            base.yA = base.xA + cA.x;
            base.zA = base.yA + cA.y;
            if (cell) {
                const long long rB = r + 1, rC = r + g.ny, rD = rC + 1;
                const uint4 cB = __ldg(&rowcnt[rB]);
                const uint4 cC = __ldg(&rowcnt[rC]);
                base.xB = row_base(tiles_v, rowpre, rB, 0);
                base.zB = base.xB + cB.x + cB.y;
                base.xC = row_base(tiles_v, rowpre, rC, 0);
                base.yC = base.xC + cC.x;
                base.xD = row_base(tiles_v, rowpre, rD, 0);
                tb = row_base(tiles_t, rowpre, r, 1);
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

// ---------------------------------------------------------------------------
// Gather the reference's gridEdge records {xl, xr, xstart, ystart, zstart}
// and triCounter (counts after pass 2, offsets after pass 3), for
// pass-by-pass inspection.
// ---------------------------------------------------------------------------
__global__ void k_fe_grid_edges(Grid g, const uint4* __restrict__ rowcnt, const uint2* __restrict__ trims,
                                const uint4* __restrict__ rowpre, const unsigned long long* __restrict__ tiles,
                                long long ntiles, int scanned, unsigned long long* __restrict__ ge,
                                unsigned long long* __restrict__ tri_counter)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.R) return;
    const uint4 c = rowcnt[r];
    const uint2 tr = trims[r];
    unsigned long long* o = ge + 5 * r;
    o[0] = tr.x;
    o[1] = tr.y;
    if (scanned) {
        const unsigned long long b = tiles[r / kTileRows] + rowpre[r].x;
        o[2] = b; o[3] = b + c.x; o[4] = b + c.x + c.y;
    } else {
        o[2] = c.x; o[3] = c.y; o[4] = c.z;
    }
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    if (j < g.ny - 1 && k < g.nz - 1) {
        const long long cr = (long long)k * (g.ny - 1) + j;
        tri_counter[cr] = scanned ? tiles[ntiles + r / kTileRows] + rowpre[r].y : c.w;
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
int lanes_per_row(int W)
{
    int G = 1;
    while (G < W && G < 32) G <<= 1;
    return G;
}

long long num_tiles(const Grid& g) { return (g.R + kTileRows - 1) / kTileRows; }

void launch_classify(const float* vol, uint32_t* bits, const Grid& g, float iso, int nsm, cudaStream_t s)
{
    long long blocks = (g.R + (kThreads / 32) - 1) / (kThreads / 32);
    const long long cap = (long long)nsm * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    const bool aligned = (g.nx % 4 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
    if (aligned) {
        k_classify_vec4<4><<<(unsigned)blocks, kThreads, 0, s>>>(reinterpret_cast<const float4*>(vol), bits,
                                                                 g.nx, g.W, g.R, iso);
    } else {
        k_classify_scalar<<<(unsigned)blocks, kThreads, 0, s>>>(vol, bits, g.nx, g.W, g.R, iso);
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

void launch_count(const uint32_t* bits, const Grid& g, const CaseTables* cases, bool mc, FeBuffers& b,
                  cudaStream_t s)
{
    const long long ntiles = num_tiles(g);
    const int G = lanes_per_row(g.W);
    if (mc) {
        ISO_DISPATCH_G(G, (k_count<kG, true><<<(unsigned)ntiles, kThreads, 0, s>>>(
                              bits, g, cases, b.rowcnt, b.trims, b.mccnt, b.rowpre, b.tiles, ntiles)));
    } else {
        ISO_DISPATCH_G(G, (k_count<kG, false><<<(unsigned)ntiles, kThreads, 0, s>>>(
                              bits, g, cases, b.rowcnt, b.trims, b.mccnt, b.rowpre, b.tiles, ntiles)));
    }
}

void launch_scan_tiles(const Grid& g, FeBuffers& b, cudaStream_t s)
{
    k_scan_tiles<<<1, 1024, 0, s>>>(b.tiles, num_tiles(g), b.totals);
}

static long long generate_blocks(const Grid& g, int nsm)
{
    const int rpw = 32 / lanes_per_row(g.W);
    const long long warps_needed = (g.R + rpw - 1) / rpw;
    long long blocks = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
    const long long cap = (long long)nsm * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return blocks;
}

template <typename IndexT>
void launch_fe_generate(const float* vol, const uint32_t* bits, const Grid& g, float iso, const CaseTables* cases,
                        const FeBuffers& b, long long capV, long long capT, float* points, float* normals,
                        IndexT* tris, int nsm, cudaStream_t s)
{
    const int G = lanes_per_row(g.W);
    const long long blocks = generate_blocks(g, nsm);
    ISO_DISPATCH_G(G, (k_generate<kG, IndexT, true, false><<<(unsigned)blocks, kThreads, 0, s>>>(
                          vol, bits, g, iso, cases, b.rowcnt, b.rowpre, b.tiles, num_tiles(g), b.totals, capV, capT,
                          points, normals, tris, nullptr)));
}

template <typename IndexT>
void launch_mc_triangles(const uint32_t* bits, const Grid& g, const CaseTables* cases, const FeBuffers& b,
                         long long capV, long long capT, IndexT* tris, int nsm, cudaStream_t s)
{
    const int G = lanes_per_row(g.W);
    const long long blocks = generate_blocks(g, nsm);
    ISO_DISPATCH_G(G, (k_generate<kG, IndexT, false, true><<<(unsigned)blocks, kThreads, 0, s>>>(
                          nullptr, bits, g, 0.f, cases, b.rowcnt, b.rowpre, b.tiles, num_tiles(g), b.totals, capV,
                          capT, nullptr, nullptr, tris, b.fe2mc)));
}

#define ISO_INST(IndexT)                                                                                        \
    template void launch_fe_generate<IndexT>(const float*, const uint32_t*, const Grid&, float,                \
                                             const CaseTables*, const FeBuffers&, long long, long long, float*, \
                                             float*, IndexT*, int, cudaStream_t);                              \
    template void launch_mc_triangles<IndexT>(const uint32_t*, const Grid&, const CaseTables*,                 \
                                              const FeBuffers&, long long, long long, IndexT*, int, cudaStream_t);
ISO_INST(uint32_t)
ISO_INST(uint64_t)
#undef ISO_INST

void launch_fe_grid_edges(const Grid& g, const FeBuffers& b, int scanned, unsigned long long* ge,
                          unsigned long long* tri_counter, cudaStream_t s)
{
    const long long blocks = (g.R + 255) / 256;
    k_fe_grid_edges<<<(unsigned)blocks, 256, 0, s>>>(g, b.rowcnt, b.trims, b.rowpre, b.tiles, num_tiles(g), scanned,
                                                     ge, tri_counter);
}

}  // namespace iso
