// Flying Edges pass 4 (FlyingEdgesAlgorithm.cpp:271-500) for rows of up to
// 16 words (nx <= 512), several grid rows per warp (included by
// gen_warps_fe.cu and gen_warps_mc.cu): two for rows of 9-16 words, four for
// rows of 5-8, eight for rows of up to 4, so that no lane idles on words past
// a short row.
//
// Lanes LPR*h .. LPR*h + LPR-1 (LPR = 32 / rows per warp) hold the words of
// grid row j = jw + h.  Rows (jw, k), (jw+1, k), ... are neighbours in the
// output order (rows in (k, j) order, the reference's), so the step's vertices
// are one list -- those of row jw, then jw+1, ..., numbered from the first
// vertex of row jw -- and so are its triangles -- cell row jw, then jw+1, ...,
// from the first triangle of cell row jw.  Each step runs the phases of
// k_gen_warps once for all the warp's rows: the cut masks, their per-row
// prefix scans and the edge-id tables (one per row), then the active cells of
// the rows 32 at a time and their triangles 32 at a time, so that the fixed
// work of a step is shared and the batches fill from all rows.  Each cell lane
// finds its cell by a shuffle binary search over the lanes' running counts:
// no per-lane loop, which diverges where the active cells cluster along the
// surface.
//
// The vertices are not computed here: each lane writes, for every cut edge its
// word owns, a record (i, axis, j, k) into the first 8 bytes of the vertex's
// own 12-byte slot of the points buffer, and k_vertices -- one thread per
// vertex, many warps per SM to cover the latency of the volume gathers --
// turns each record into the vertex's position and normal in place.
#pragma once
#include "batch_kernels.cuh"
#include "gen_warps.cuh"
#include "vertices.cuh"

namespace iso {

constexpr int kGenPairCtasPerSm = 4;        // resident CTAs per SM the kernel is built for

// Per-warp scratch: mb[RPW][8][W] uint2, rwt[RPW][W][8], cell[32], the
// batch's list (gen_list_bytes: triangles, or Marching Cubes owned vertices).
__host__ __device__ inline size_t gen_pair_scratch_bytes(int W, int RPW, int mode)
{
    return ((size_t)RPW * 8 * W * 8 + (size_t)RPW * 8 * W * 4 + kGenCells * 4 + gen_list_bytes(mode) + 15) &
           ~(size_t)15;
}

// One wave of CTAs; every warp takes work items -- a group of RPW rows and a
// run of KC planes -- from the counter `work` until none is left, so no warp
// waits for another and no CTA stays resident for its slowest warp.  Item q is
// row group q % ngroups of plane run q / ngroups (runs walked backwards when
// `reverse`).  RPW = 2 for rows of up to 16 words, 4 for up to 8, 8 for up to 4: lanes
// LPR*h .. LPR*h + LPR-1 hold the words of row jw + h.
// MODE kGenFE: Flying Edges vertex records and triangles.  kGenMC: the
// Marching Cubes vertices the cells own (marchingCubes/serial/main.cpp:
// 139-177: cell order, then first appearance in the cell's triangle list)
// get their ids, records for the rows from kemit on, and the FE -> MC map
// entry of their edge.  kGenTri: the triangles, corners mapped through it.
// The kernel's per-case tables in shared memory.  s_tri: per case, each triangle corner as the nibble (edge-id
// table row | point offset << 3) of fe_edge_rel, the triangle count in bits 60..63 (the packed triangle list
// with edges replaced); s_order: the first-appearance order of the cut edges; s_cut: the cut edges.
template <int MODE>
struct GenPairTables {
    static constexpr bool OWNS = MODE == kGenMC || MODE == kGenMCT;  // numbers the MC vertices its cells own
    uint64_t tri[MODE == kGenMC ? 1 : 256];
    uint64_t order[OWNS ? 256 : 1];
    uint16_t cut[OWNS ? 256 : 1];
};

template <int MODE>
__device__ __forceinline__ void gen_pair_tables(const CaseTables* __restrict__ cases, GenPairTables<MODE>& t)
{
    for (int c = threadIdx.x; c < 256; c += kThreads) {
        if (GenPairTables<MODE>::OWNS) {
            t.order[c] = cases->order[c];
            t.cut[c] = cases->cut[c];
            if (MODE == kGenMC) continue;
        }
        const uint64_t w = cases->tris[c];
        uint64_t x = w & (0xfull << 60);
        for (int q = 0; q < 15; ++q) {
            const int e = (int)((w >> (4 * q)) & 15u);
            const uint64_t nib = e < 12 ? (((0x776653524140ull >> (4 * e)) & 7u) | (((0xA22u >> e) & 1u) << 3)) : 0u;
            x |= nib << (4 * q);
        }
        t.tri[c] = x;
    }
}

// Work item `item` of an extraction, run by one warp with its ws_bytes of shared memory at ws.
template <typename IndexT, int RPW, int MODE>
__device__ __forceinline__ void gen_pairs_item(
    uint32_t item, unsigned char* ws, const GenPairTables<MODE>& tabs, const uint32_t* __restrict__ bits,
    const Grid& g, int KC, int ngroups, int nkc, int kbeg, int kend, int kemit, unsigned long long vbase,
    unsigned long long tbase, const uint4* __restrict__ rowcnt, const RowStarts& rs, float* __restrict__ points,
    IndexT* __restrict__ tris, uint32_t* __restrict__ fe2mc, int reverse)
{
    constexpr bool OWNS = GenPairTables<MODE>::OWNS;
    constexpr int LPR = 32 / RPW;  // lanes per row
    const uint64_t* s_tri = tabs.tri;
    const uint64_t* s_order = tabs.order;
    const uint16_t* s_cut = tabs.cut;
    const int lane = threadIdx.x & 31, h = lane / LPR, lw = lane % LPR;
    const int W = g.W;
    uint2* mb = reinterpret_cast<uint2*>(ws);                                    // [RPW][8][W]
    uint32_t* rwt = reinterpret_cast<uint32_t*>(ws + (size_t)RPW * 8 * W * 8);  // [RPW][W][8]
    uint32_t* cell = rwt + RPW * 8 * W;
    unsigned char* list = reinterpret_cast<unsigned char*>(cell + kGenCells);
    const bool in1 = lw + 1 < W;
    const uint32_t evalid = validmask(lw, g.nx - 1);  // x-edges / cells: i <= nx-2
    const uint32_t pvalid = validmask(lw, g.nx);      // points: i <= nx-1
    uint2* mbh = mb + h * 8 * W;
    uint32_t* rwth = rwt + h * 8 * W;
    {
        const int col = (int)(item / (uint32_t)ngroups);
        const int kc = reverse ? nkc - 1 - col : col;
        const int jw = RPW * (int)(item % (uint32_t)ngroups);
        const int kb = kbeg + kc * KC, ke = min(kb + KC, kend);
        const int j = jw + h;
        const bool row_ok = j < g.ny;
        const bool hasY = row_ok && j < g.ny - 1;
        const bool in = row_ok && lw < W;

        // Bit words of rows (j, p) and (j+1, p).
        auto load_words = [&](int p, uint32_t& wa, uint32_t& wb) {
            const bool okp = p < g.ke;  // rows of the window
            const long long r = (long long)(p - g.kr) * g.ny + j;
            wa = (in && okp) ? __ldg(&bits[r * W + lw]) : 0u;
            wb = (in && okp && hasY) ? __ldg(&bits[(r + 1) * W + lw]) : 0u;
        };
        // Row starts of step p, in lanes 0..3 of each row's lanes: s1 = the
        // first vertex of rows A = (j,p), B = (j+1,p), C = (j,p+1), D = (j+1,p+1);
        // s2 = the first triangle (kGenMC: owned MC vertex) of cell row A (lane 0)
        // and the x + y cuts of row B (lane 1).
        auto load_starts = [&](int p, unsigned long long& s1, unsigned long long& s2) {
            const int dk = (lw >> 1) & 1, dj = lw & 1;
            const bool hasZp = p + 1 < g.ke;
            const long long rA = (long long)(p - g.kr) * g.ny + j;
            s1 = s2 = 0ull;
            if (row_ok && lw < 4 && (dj == 0 || hasY) && (dk == 0 || hasZp))
                s1 = rs.get(rA + (long long)dk * g.ny + dj, 0);
            if (row_ok && lw == 0) s2 = rs.get(rA, OWNS ? 2 : 1);
            if (MODE == kGenMCT && row_ok && lw == 2) s2 = rs.get(rA, 1);  // first triangle of cell row A
            if (row_ok && lw == 1 && hasY) {
                const uint2 c = __ldg(reinterpret_cast<const uint2*>(&rowcnt[rA + 1]));
                s2 = (unsigned long long)c.x + c.y;
            }
        };

        uint32_t wA = 0, wB = 0, wC = 0, wD = 0;
        load_words(kb, wA, wB);
        load_words(kb + 1, wC, wD);
        unsigned long long st, st2;
        load_starts(kb, st, st2);

        for (int k = kb; k < ke; ++k) {
            const bool hasZ = k + 1 < g.nz;
            // the next step's words and starts, in flight while this step runs
            uint32_t nC = 0, nD = 0;
            unsigned long long nst = 0, nst2 = 0;
            if (k + 1 < ke) {
                load_words(k + 2, nC, nD);
                load_starts(k + 1, nst, nst2);
            }
            const bool cellrow = hasY && hasZ;
            RowWords rw;
            rw.a = wA;
            rw.b = wB;
            rw.c = hasZ ? wC : 0u;
            rw.d = cellrow ? wD : 0u;
            const uint32_t an = __shfl_down_sync(0xffffffffu, rw.a, 1, LPR);
            const uint32_t bn = __shfl_down_sync(0xffffffffu, rw.b, 1, LPR);
            const uint32_t cn = __shfl_down_sync(0xffffffffu, rw.c, 1, LPR);
            const uint32_t dn = __shfl_down_sync(0xffffffffu, rw.d, 1, LPR);
            rw.ash = (rw.a >> 1) | ((in1 ? an : 0u) << 31);
            rw.bsh = (rw.b >> 1) | ((in1 ? bn : 0u) << 31);
            rw.csh = (rw.c >> 1) | ((in1 ? cn : 0u) << 31);
            rw.dsh = (rw.d >> 1) | ((in1 ? dn : 0u) << 31);
            const CutMasks m = cut_masks(rw, evalid, pvalid, hasY, hasZ);
            // popc prefixes within each row's lanes, two 16-bit counts per scan
            const uint32_t p0 = __popc(m.xA) | (__popc(m.xB) << 16);
            const uint32_t p1 = __popc(m.xC) | (__popc(m.xD) << 16);
            const uint32_t p2 = __popc(m.yA) | (__popc(m.yC) << 16);
            const uint32_t p3 = __popc(m.zA) | (__popc(m.zB) << 16);
            const uint32_t i0 = group_incl_scan<LPR>(p0, lw, 0xffffffffu);
            const uint32_t i1 = group_incl_scan<LPR>(p1, lw, 0xffffffffu);
            const uint32_t i2 = group_incl_scan<LPR>(p2, lw, 0xffffffffu);
            const uint32_t i3 = group_incl_scan<LPR>(p3, lw, 0xffffffffu);
            const uint32_t e0 = i0 - p0, e1 = i1 - p1, e2 = i2 - p2, e3 = i3 - p3;
            const uint32_t t0 = __shfl_sync(0xffffffffu, i0, LPR - 1, LPR);
            const uint32_t t1 = __shfl_sync(0xffffffffu, i1, LPR - 1, LPR);
            const uint32_t t2 = __shfl_sync(0xffffffffu, i2, LPR - 1, LPR);
            const uint32_t t3 = __shfl_sync(0xffffffffu, i3, LPR - 1, LPR);
            const unsigned long long xsA = __shfl_sync(0xffffffffu, st, 0, LPR);  // this lane's row
            const unsigned long long xs0 = __shfl_sync(0xffffffffu, st, 0);      // row jw: the step's numbering
            const uint32_t dB = (uint32_t)(__shfl_sync(0xffffffffu, st, 1, LPR) - xsA);
            const uint32_t dC = (uint32_t)(__shfl_sync(0xffffffffu, st, 2, LPR) - xsA);
            const uint32_t dD = (uint32_t)(__shfl_sync(0xffffffffu, st, 3, LPR) - xsA);
            const uint32_t cntB = (uint32_t)__shfl_sync(0xffffffffu, st2, 1, LPR);
            // first triangle (kGenMC: first owned MC vertex) of cell row jw
            const unsigned long long ts0 = __shfl_sync(0xffffffffu, st2, 0);
            // kGenMCT: first triangle of cell row jw (ts0 numbers the owned MC vertices)
            const unsigned long long tt0 = MODE == kGenMCT ? __shfl_sync(0xffffffffu, st2, 2) : 0ull;
            const uint32_t nxA = t0 & 0xffffu, nyA = t2 & 0xffffu, nxC = t1 & 0xffffu;
            const uint32_t off = (uint32_t)(xsA - xs0);  // the vertices of rows jw .. j-1
            if (in) {  // first ids of the word's cut edges, relative to xs0
                mbh[0 * W + lw] = make_uint2(m.xA, off + (e0 & 0xffffu));
                mbh[1 * W + lw] = make_uint2(m.xB, off + dB + (e0 >> 16));
                mbh[2 * W + lw] = make_uint2(m.xC, off + dC + (e1 & 0xffffu));
                mbh[3 * W + lw] = make_uint2(m.xD, off + dD + (e1 >> 16));
                mbh[4 * W + lw] = make_uint2(m.yA, off + nxA + (e2 & 0xffffu));
                mbh[5 * W + lw] = make_uint2(m.yC, off + dC + nxC + (e2 >> 16));
                mbh[6 * W + lw] = make_uint2(m.zA, off + nxA + nyA + (e3 & 0xffffu));
                mbh[7 * W + lw] = make_uint2(m.zB, off + dB + cntB + (e3 >> 16));
                if (cellrow) {  // corner order of the cube case: bit v = corner v
                    uint4* t = reinterpret_cast<uint4*>(rwth + 8 * lw);
                    t[0] = make_uint4(rw.a, rw.ash, rw.bsh, rw.b);
                    t[1] = make_uint4(rw.c, rw.csh, rw.dsh, rw.d);
                }
            }
            __syncwarp();

            // ---- vertex records of grid row (j, k): the x, y, z cuts its word owns
            if (MODE == kGenFE && in) {
                auto records = [&](uint32_t mk, uint32_t first, uint32_t axis) {
                    unsigned long long idx = xs0 + first - vbase;
                    while (mk != 0u) {
                        put_vertex_record(points, idx, (uint32_t)(32 * lw + __ffs(mk) - 1), axis, (uint32_t)j,
                                          (uint32_t)k);
                        mk &= mk - 1u;
                        ++idx;
                    }
                };
                records(m.xA, off + (e0 & 0xffffu), 0u);
                records(m.yA, off + nxA + (e2 & 0xffffu), 1u);
                records(m.zA, off + nxA + nyA + (e3 & 0xffffu), 2u);
            }

            // ---- active cells of cell rows (jw, k) .. (jw+RPW-1, k), 32 at a time
            const uint32_t act = (in && cellrow) ? active_cells(rw, evalid) : 0u;
            const uint32_t na = __popc(act);
            const uint32_t ia = warp_incl_scan(na, lane);  // the cells of row jw come first
            const uint32_t tot = __shfl_sync(0xffffffffu, ia, 31);
            unsigned long long tcur = ts0;
            unsigned long long ttri = tt0;
            for (uint32_t c0 = 0; c0 < tot; c0 += kGenCells) {
                // lane L takes active cell c0 + L: the first lane whose inclusive count passes it
                // (a shuffle binary search over the lanes), then the bit by __fns
                const uint32_t target = c0 + (uint32_t)lane;
                int src = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const uint32_t before = __shfl_sync(0xffffffffu, ia, (src + step - 1) & 31);
                    if (before <= target) src += step;
                }
                const uint32_t srcact = __shfl_sync(0xffffffffu, act, src);
                const uint32_t srcexc = __shfl_sync(0xffffffffu, ia - na, src);
                const uint32_t nc = min(tot - c0, (uint32_t)kGenCells);
                const bool live = (uint32_t)lane < nc;
                uint32_t rec = 0u;
                if (live) {  // the cell's cube case from its word's row words
                    const uint32_t ch =
                        (uint32_t)(32 * (src % LPR) + (int)__fns(srcact, 0, (int)(target - srcexc) + 1)) |
                        ((uint32_t)(src / LPR) << 9);  // i | row << 9
                    const uint32_t ci = ch & 511u;
                    const uint4* t = reinterpret_cast<const uint4*>(rwt + (ch >> 9) * 8 * W + 8 * (ci >> 5));
                    const uint4 lo4 = t[0], hi4 = t[1];
                    const int b = (int)(ci & 31u);
                    const uint32_t cs = ((lo4.x >> b) & 1u) | (((lo4.y >> b) & 1u) << 1) | (((lo4.z >> b) & 1u) << 2) |
                                        (((lo4.w >> b) & 1u) << 3) | (((hi4.x >> b) & 1u) << 4) |
                                        (((hi4.y >> b) & 1u) << 5) | (((hi4.z >> b) & 1u) << 6) |
                                        (((hi4.w >> b) & 1u) << 7);
                    rec = ch | (cs << 16);
                    cell[lane] = rec;
                }
                const int cs = (int)(rec >> 16);
                // triangles: kGenFE / kGenMCT with the corners' FE ids, kGenTri mapped to MC ids; kGenMCT
                // only for the cell rows it emits (the rows below kemit belong to the slab below)
                if (MODE == kGenFE || MODE == kGenTri || (MODE == kGenMCT && k >= kemit)) {
                    unsigned long long& tc = MODE == kGenMCT ? ttri : tcur;
                    const uint32_t nt = live ? (uint32_t)iso_case_ntris(s_tri[cs]) : 0u;
                    const uint32_t it = warp_incl_scan(nt, lane);
                    const uint32_t ntb = __shfl_sync(0xffffffffu, it, 31);
                    for (uint32_t q = 0; q < nt; ++q) list[it - nt + q] = (unsigned char)(lane | (q << 5));
                    __syncwarp();
                    for (uint32_t tb = 0; tb < ntb; tb += 32) {
                        const uint32_t t = tb + lane;
                        if (t < ntb) {
                            const uint32_t tr = list[t];
                            const uint32_t cr = cell[tr & 31u];
                            const int q = (int)(tr >> 5);
                            const int ci = (int)(cr & 511u);
                            const uint2* mbc = mb + ((cr >> 9) & 7u) * 8 * W + (ci >> 5);
                            const uint32_t corners = (uint32_t)(s_tri[cr >> 16] >> (12 * q)) & 0xfffu;
                            const int bit = ci & 31;
                            IndexT* o = tris + 3 * (tc + t - tbase);
#pragma unroll
                            for (int c = 0; c < 3; ++c) {  // fe_edge_rel with its table row and offset precomputed
                                const uint32_t nib = (corners >> (4 * c)) & 15u;
                                const uint2 pm = mbc[(nib & 7u) * W];
                                // popc of the mask's bits below bit + offset (the funnel shift clamps at 32)
                                const int pos = bit + (int)(nib >> 3);
                                const uint32_t rel = pm.y + __popc(__funnelshift_lc(0u, pm.x, 32 - pos));
                                if (MODE == kGenTri)  // the corner's MC id through the FE -> MC map
                                    o[c] = (IndexT)__ldg(fe2mc + (xs0 + rel));
                                else if constexpr (sizeof(IndexT) == 4)
                                    o[c] = (IndexT)((uint32_t)xs0 + rel);  // 32-bit ids: V < 2^32
                                else
                                    o[c] = (IndexT)(xs0 + rel);
                            }
                        }
                    }
                    tc += ntb;
                }
                if (OWNS) {
                    if (MODE == kGenMCT) __syncwarp();  // the triangle list is read before the vertex list reuses it
                    // ---- the MC vertices the batch's cells own: cell order, then order of first appearance in
                    // the cell's triangle list (marchingCubes/serial/main.cpp:139-177)
                    const int cci = (int)(rec & 511u), cj = jw + (int)((rec >> 9) & 7u);
                    const uint32_t own = live ? (mc_owned_edges(cci == 0, cj == 0, k == 0) & s_cut[cs]) : 0u;
                    const uint32_t no = __popc(own);
                    const uint32_t io = warp_incl_scan(no, lane);
                    const uint32_t nob = __shfl_sync(0xffffffffu, io, 31);
                    uint16_t* vl = reinterpret_cast<uint16_t*>(list);
                    if (own) {
                        const uint64_t ord = s_order[cs];
                        uint32_t o = io - no;
                        for (int q = 0; q < iso_case_ntris(ord); ++q) {
                            const int ed = iso_case_edge(ord, q);
                            if ((own >> ed) & 1u) vl[o++] = (uint16_t)(lane | (ed << 5));
                        }
                    }
                    __syncwarp();
                    for (uint32_t vb = 0; vb < nob; vb += 32) {
                        const uint32_t v = vb + lane;
                        if (v < nob) {
                            const uint32_t vr = vl[v];
                            const uint32_t cr = cell[vr & 31u];
                            const int e12 = (int)(vr >> 5);
                            const int i = (int)(cr & 511u), jc = jw + (int)((cr >> 9) & 7u);
                            const unsigned long long id = tcur + v;
                            if (k >= kemit) {  // cell rows below kemit belong to the slab below: map only
                                int dx, dy, dz, axis;
                                cube_edge_geometry(e12, dx, dy, dz, axis);
                                put_mc_record(points, id - vbase, (uint32_t)(i + dx), (uint32_t)axis,
                                              (uint32_t)(dx | (dy << 1) | (dz << 2)), (uint32_t)(jc + dy),
                                              (uint32_t)(k + dz));
                            }
                            const uint2* mbc = mb + ((cr >> 9) & 7u) * 8 * W;
                            fe2mc[xs0 + fe_edge_rel(mbc, W, e12, i >> 5, i & 31)] = (uint32_t)id;
                        }
                    }
                    tcur += nob;
                }
                __syncwarp();  // the next batch overwrites the lists
            }
            __syncwarp();  // the next step overwrites mb
            wA = wC;
            wB = wD;
            wC = nC;
            wD = nD;
            st = nst;
            st2 = nst2;
        }
    }
}

// One wave of CTAs; every warp takes work items from the counter `work` until none is left.
template <typename IndexT, int RPW, int MODE>
__global__ void __launch_bounds__(kThreads, kGenPairCtasPerSm) k_gen_pairs(
    const uint32_t* __restrict__ bits, Grid g, int KC, int ngroups, int nkc, int kbeg, int kend,
    int kemit, unsigned long long vbase, unsigned long long tbase, int ws_bytes,
    const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, RowStarts rs,
    const unsigned long long* __restrict__ totals, unsigned int* __restrict__ work, long long capV, long long capT,
    float* __restrict__ points, IndexT* __restrict__ tris, uint32_t* __restrict__ fe2mc, int reverse)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ GenPairTables<MODE> tabs;
    gen_pair_tables<MODE>(cases, tabs);
    __syncthreads();  // the only CTA barrier: from here on every warp runs alone
    // Caller grows buffers.  Past this check every record slot and triangle index written below lies
    // under the totals, because the count pass derives the counts and starts from the same bit words
    // with the same masks (cut_masks, tris_of_word); the writes are not checked one by one.
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;
    unsigned char* ws = s_raw + (size_t)(threadIdx.x >> 5) * ws_bytes;
    const uint32_t nitems = (uint32_t)ngroups * (uint32_t)nkc;
    for (;;) {
        uint32_t item = 0u;
        if ((threadIdx.x & 31) == 0) item = atomicAdd(work, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitems) break;
        gen_pairs_item<IndexT, RPW, MODE>(item, ws, tabs, bits, g, KC, ngroups, nkc, kbeg, kend, kemit, vbase, tbase,
                                          rowcnt, rs, points, tris, fe2mc, reverse);
    }
}

// The Flying Edges generate items of a list of requests (batch_kernels.cuh), one launch: item x is item
// x - first[q] of request list[q]; the items of a request whose mesh cannot hold its counts are skipped.
template <typename IndexT, int RPW>
__global__ void __launch_bounds__(kThreads, kGenPairCtasPerSm) k_gen_pairs_batch(
    const BatchReq* __restrict__ reqs, const int* __restrict__ list, const unsigned* __restrict__ first, int m,
    const CaseTables* __restrict__ cases, unsigned int* __restrict__ work, int ws_bytes, int reverse)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ GenPairTables<kGenFE> tabs;
    gen_pair_tables<kGenFE>(cases, tabs);
    __syncthreads();
    unsigned char* ws = s_raw + (size_t)(threadIdx.x >> 5) * ws_bytes;
    const uint32_t nitems = __ldg(&first[m]);
    for (;;) {
        uint32_t item = 0u;
        if ((threadIdx.x & 31) == 0) item = atomicAdd(work, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitems) break;
        const int q = batch_find(first, m, item);
        const BatchReq* d = reqs + __ldg(&list[q]);
        if ((long long)d->totals[0] > d->capV || (long long)d->totals[1] > d->capT) continue;
        if (item - __ldg(&first[q]) >= (uint32_t)d->gen_ngroups * (uint32_t)d->gen_nkc) continue;  // past its items
        const Grid g = d->g;
        RowStarts rs;
        rs.starts = d->starts;
        rs.R = g.R;
        rs.ny = g.ny;
        rs.kr = g.kr;
        rs.add[0] = rs.add[1] = rs.add[2] = rs.add[3] = 0;
        gen_pairs_item<IndexT, RPW, kGenFE>(item - __ldg(&first[q]), ws, tabs, d->bits, g, d->gen_KC, d->gen_ngroups,
                                            d->gen_nkc, g.kr, g.ke, g.kr, 0ull, 0ull, d->rowcnt, rs, d->points,
                                            static_cast<IndexT*>(d->tris), nullptr, reverse);
    }
}

// Rows of up to 16 words (gen_plan's fits, and W <= 16) in MODE over the
// plan's planes [kbeg, kend).
template <typename IndexT, int MODE>
void launch_gen_pairs_impl(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                           const GenPlan& p, int nsm, long long capV, long long capT, float* points, IndexT* tris,
                           int reverse, cudaStream_t s)
{
    const int nzw = p.kend - p.kbeg;
    if (nzw <= 0) return;
    // items of KC planes: about sixteen per warp of one wave, at least 2 planes (the last items are short, so
    // the warps finish together: 512^3 FE 181 -> 169 us against four per warp and 4 planes)
    const int rpw = g.W <= 4 ? 8 : (g.W <= 8 ? 4 : 2);
    const long long npairs = (g.ny + rpw - 1) / rpw;  // row groups
    const long long warps = (long long)nsm * kGenPairCtasPerSm * kGenRows;
    long long KC = (npairs * nzw + 16 * warps - 1) / (16 * warps);
    if (KC < 2) KC = 2;
    while (npairs * ((nzw + KC - 1) / KC) >= (1ll << 31)) KC *= 2;  // item numbers stay below 2^31
    if (KC > nzw) KC = nzw;
    const int nkc = (int)((nzw + KC - 1) / KC);
    const long long nitems = npairs * nkc;
    long long blocks = (nitems + kGenRows - 1) / kGenRows;
    if (blocks > (long long)nsm * kGenPairCtasPerSm) blocks = (long long)nsm * kGenPairCtasPerSm;
    RowStarts rs = row_starts(g, cp, b);
    for (int a = 0; a < 3; ++a) rs.add[a] = p.add[a];
    unsigned int* work = reinterpret_cast<unsigned int*>(b.totals + 7);
    cudaMemsetAsync(work, 0, sizeof(unsigned int), s);
    const int ws_bytes = (int)gen_pair_scratch_bytes(g.W, rpw, MODE);
    const size_t smem = (size_t)kGenRows * ws_bytes;
    auto kern = rpw == 8 ? k_gen_pairs<IndexT, 8, MODE>
                         : (rpw == 4 ? k_gen_pairs<IndexT, 4, MODE> : k_gen_pairs<IndexT, 2, MODE>);
    allow_smem(kern, smem);
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(b.bits, g, (int)KC, (int)npairs, nkc, p.kbeg, p.kend, p.kemit,
                                                  p.vbase, p.tbase, ws_bytes, cases, b.rowcnt, rs, b.totals, work,
                                                  capV, capT, points, tris, b.fe2mc, reverse);
}

}  // namespace iso
