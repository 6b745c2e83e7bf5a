// Pass 4 on sm_103a, one grid row per warp (included by gen_warps_fe.cu,
// gen_pairs.cuh and gen_warps_mc.cu): rows of 17-32 words, and the
// duplicate-free Marching Cubes order; rows of up to 16 words run on the
// multi-row kernel of gen_pairs.cuh, which reuses the helpers here.
//
// One wave of CTAs of 8 warps; every warp takes (grid row j, run of KC planes)
// work items from a counter and marches along z on its own (the only CTA
// barrier stages the case tables).  The count pass's bit rows say where the
// surface is.
//
// Per step a warp handles grid row (j, k) with one 32-bit word of the bit
// mask per lane (the bit words and row starts of the next step load while
// this one runs):
//   the 8 cut masks of the cell row and their popc prefixes (warp scans)
//   give, per word, the id of each mask's first cut edge relative to the
//   row's first vertex; the warp keeps them in shared memory (mb), with the
//   row words (rwt), so that any lane numbers any edge of any cell with one
//   8-byte load and a popc;
//   FE  : the row's vertices, one per lane: a shuffle binary search maps the
//         lane's vertex rank to a word and __fns to a bit; the vertex goes to
//         its axis' queue (shared memory), and every full batch of 32 is
//         computed by the axis' own code from the volume (no divergence by
//         axis, full lanes);
//   the active cells of the cell row, 32 at a time: each cell lane finds its
//   cell by a shuffle binary search over the lanes' counts and computes its
//   cube case, then
//   FE, TRI: the cells' triangles are listed as (cell, triangle) pairs and
//         written one triangle per lane, consecutive lanes storing consecutive
//         triangles (TRI, without volume, maps the corners through the
//         Flying Edges -> MC index map);
//   MC, Dup: the vertices the cells own, in owner-cell / first-appearance
//         order (marchingCubes/serial/main.cpp:139-177), one per lane: their
//         ids (owner order, or the global-edge-index order for Dup) and a
//         record each for k_vertices (vertices.cuh); MC also the map.
#pragma once
#include <cmath>
#include <type_traits>

#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

constexpr int kGenRows = 8;       // grid rows per CTA, one per warp
constexpr int kGenCtasPerSm = 3;  // resident CTAs per SM the kernel is built for
constexpr int kGenCells = 32;  // cells per batch
constexpr int kGenTris = 5 * kGenCells;    // triangles of a batch, at most
constexpr int kGenOwned = 12 * kGenCells;  // MC vertices owned by a batch, at most
constexpr int kGenVq = 64;                 // FE vertex queue per axis and warp (a ring of two batches)
enum GenMode { kGenFE = 0, kGenMC = 1, kGenTri = 2, kGenDup = 3, kGenMCT = 4 };

// Per-warp scratch in shared memory:
//   mb[8][W]   {cut mask, id of its first cut edge - the row's first vertex}
//              per mask (xA xB xC xD yA yC zA zB) and word
//   rwt[W][8]  the word's row words (a ash bsh b c csh dsh d: corners 0..7)
//   cell[32]   the batch's active cells: i | cube case << 16
//   list[...]  FE / TRI: the batch's triangles, cell | triangle << 5 (u8);
//              MC: the batch's owned vertices, cell | cube edge << 5 (u16)
//   FE: vertex queues per axis (rings of kGenVq): ids (u64), then i | k << 10
__host__ __device__ inline size_t gen_list_bytes(int mode)
{
    return mode == kGenMC || mode == kGenDup || mode == kGenMCT ? (size_t)kGenOwned * 2 : (size_t)kGenTris;
}
//   Dup: db[8][W] the global-edge-index order id of each mask's first cut
//        edge, after the list
__host__ __device__ inline size_t gen_warp_scratch_bytes(int W, int mode)
{
    const size_t vq = mode == kGenFE ? (size_t)3 * kGenVq * 12 : 0;
    const size_t db = mode == kGenDup ? (size_t)8 * W * 8 : 0;
    return ((size_t)8 * W * 8 + (size_t)8 * W * 4 + kGenCells * 4 + gen_list_bytes(mode) + vq + db + 15) &
           ~(size_t)15;
}

// Divisors of the gradient: the reference divides by the spacing (one-sided
// differences at the faces) or by twice the spacing.  When every spacing is
// a power of two, dividing equals multiplying by the exact reciprocal: both
// round the same real number.
struct GradScale {
    float sp[3], inv1[3], inv2[3];
    int exact;
};

inline GradScale make_grad_scale(const Grid& g)
{
    GradScale s;
    s.exact = 1;
    for (int a = 0; a < 3; ++a) {
        const float sp = g.sp[a];
        int e = 0;
        const float m = std::frexp(sp, &e);  // sp = m * 2^e, m in [0.5, 1)
        const bool pow2 = sp > 0.f && m == 0.5f && e >= -124 && e <= 126;
        if (!pow2) s.exact = 0;
        s.sp[a] = sp;
        s.inv1[a] = pow2 ? std::ldexp(1.0f, 1 - e) : 0.f;  // 1 / sp
        s.inv2[a] = pow2 ? std::ldexp(1.0f, -e) : 0.f;     // 1 / (2 sp)
    }
    return s;
}

// grad_component() of iso_device.cuh along axis a (negated central
// difference, one-sided at the faces).
__device__ __forceinline__ float grad_axis(float prev, float here, float next, int p, int n, int a,
                                           const GradScale& gs)
{
    const bool lo = p == 0, hi = p == n - 1;
    const float num = lo ? fsub(here, next) : (hi ? fsub(prev, here) : fsub(prev, next));
    const bool one = lo || hi;
    if (gs.exact) {
        const float r1 = a == 0 ? gs.inv1[0] : (a == 1 ? gs.inv1[1] : gs.inv1[2]);
        const float r2 = a == 0 ? gs.inv2[0] : (a == 1 ? gs.inv2[1] : gs.inv2[2]);
        return fmul(num, one ? r1 : r2);
    }
    const float sp = a == 0 ? gs.sp[0] : (a == 1 ? gs.sp[1] : gs.sp[2]);
    return fdiv(num, one ? sp : fmul(2.0f, sp));
}

// Gradient components at one point from its six neighbours (grad_component
// of iso_device.cuh per axis).
__device__ __forceinline__ float3 grad3(float xm, float xp, float ym, float yp, float zm, float zp, float here, int i,
                                        int j, int kk, const Grid& g, const GradScale& gs)
{
    return make_float3(grad_axis(xm, here, xp, i, g.nx, 0, gs), grad_axis(ym, here, yp, j, g.ny, 1, gs),
                       grad_axis(zm, here, zp, kk, g.nz, 2, gs));
}

// edge_vertex() of iso_device.cuh for a Flying Edges edge along the fixed
// axis A from P0 = (i, j, kk), values read from the volume: planes kk-1 ..
// kk+2 as lo, at, hi, hi2, each addressed from row jlo (planes outside the
// grid alias a valid one and are not read).  The cube base is the edge's own
// index along A and the clamped one (n-2) across, the cube that owns the
// edge in Image3D::getPosCube terms.
template <int A>
__device__ __forceinline__ void vertex_axis(const float* lo, const float* at, const float* hi, const float* hi2,
                                            int jlo, const Grid& g, const GradScale& gs, float iso, int i, int j,
                                            int kk, float3& pos, float3& nrm)
{
    const int nx = g.nx;
    const int o = (j - jlo) * nx + i;
    const bool xl = i > 0, yl = j > 0, zl = kk > 0;
    const bool xh = i < g.nx - 1, yh = j < g.ny - 1, zh = kk < g.nz - 1;
    const float v0 = __ldg(at + o);
    float v1;
    float3 g0, g1;
    if constexpr (A == 0) {
        const int o1 = o + 1;
        v1 = __ldg(at + o1);
        g0 = grad3(xl ? __ldg(at + o - 1) : 0.f, v1, yl ? __ldg(at + o - nx) : 0.f, yh ? __ldg(at + o + nx) : 0.f,
                   zl ? __ldg(lo + o) : 0.f, zh ? __ldg(hi + o) : 0.f, v0, i, j, kk, g, gs);
        g1 = grad3(v0, i + 1 < g.nx - 1 ? __ldg(at + o1 + 1) : 0.f, yl ? __ldg(at + o1 - nx) : 0.f,
                   yh ? __ldg(at + o1 + nx) : 0.f, zl ? __ldg(lo + o1) : 0.f, zh ? __ldg(hi + o1) : 0.f, v1, i + 1,
                   j, kk, g, gs);
    } else if constexpr (A == 1) {
        const int o1 = o + nx;
        v1 = __ldg(at + o1);
        g0 = grad3(xl ? __ldg(at + o - 1) : 0.f, xh ? __ldg(at + o + 1) : 0.f, yl ? __ldg(at + o - nx) : 0.f, v1,
                   zl ? __ldg(lo + o) : 0.f, zh ? __ldg(hi + o) : 0.f, v0, i, j, kk, g, gs);
        g1 = grad3(xl ? __ldg(at + o1 - 1) : 0.f, xh ? __ldg(at + o1 + 1) : 0.f, v0,
                   j + 1 < g.ny - 1 ? __ldg(at + o1 + nx) : 0.f, zl ? __ldg(lo + o1) : 0.f,
                   zh ? __ldg(hi + o1) : 0.f, v1, i, j + 1, kk, g, gs);
    } else {
        v1 = __ldg(hi + o);
        g0 = grad3(xl ? __ldg(at + o - 1) : 0.f, xh ? __ldg(at + o + 1) : 0.f, yl ? __ldg(at + o - nx) : 0.f,
                   yh ? __ldg(at + o + nx) : 0.f, zl ? __ldg(lo + o) : 0.f, v1, v0, i, j, kk, g, gs);
        g1 = grad3(xl ? __ldg(hi + o - 1) : 0.f, xh ? __ldg(hi + o + 1) : 0.f, yl ? __ldg(hi + o - nx) : 0.f,
                   yh ? __ldg(hi + o + nx) : 0.f, v0, kk + 1 < g.nz - 1 ? __ldg(hi2 + o) : 0.f, v1, i, j, kk + 1, g,
                   gs);
    }
    const float w = fdiv(fsub(iso, v0), fsub(v1, v0));
    const int ci = A == 0 ? i : min(i, g.nx - 2), cj = A == 1 ? j : min(j, g.ny - 2);
    const int ck = A == 2 ? kk : min(kk, g.nz - 2);
    const int i1 = i + (A == 0), j1 = j + (A == 1), k1 = kk + (A == 2);
    pos.x = lerp_ref(cube_coord(ci, i - ci, g.zp[0], g.sp[0]), cube_coord(ci, i1 - ci, g.zp[0], g.sp[0]), w);
    pos.y = lerp_ref(cube_coord(cj, j - cj, g.zp[1], g.sp[1]), cube_coord(cj, j1 - cj, g.zp[1], g.sp[1]), w);
    pos.z = lerp_ref(cube_coord(ck, kk - ck, g.zp[2], g.sp[2]), cube_coord(ck, k1 - ck, g.zp[2], g.sp[2]), w);
    nrm.x = lerp_ref(g0.x, g1.x, w);
    nrm.y = lerp_ref(g0.y, g1.y, w);
    nrm.z = lerp_ref(g0.z, g1.z, w);
}

__device__ __forceinline__ void store_vertex(float* __restrict__ points, float* __restrict__ normals,
                                             unsigned long long id, const float3& p, const float3& n)
{
    points[3 * id + 0] = p.x;
    points[3 * id + 1] = p.y;
    points[3 * id + 2] = p.z;
    normals[3 * id + 0] = n.x;
    normals[3 * id + 1] = n.y;
    normals[3 * id + 2] = n.z;
}

// Marching Cubes vertex record in the first 8 bytes of the vertex's points
// slot: the edge's lower point (i, j, k), its axis and the offset d (bit 0 x,
// 1 y, 2 z) of that point from the owner cell, whose cube places the vertex:
// word 0 = i | axis << 10 | d << 12 | (j & 0x1ffff) << 15, word 1 = j >> 17 |
// k << 10 (i < 1024, j < 2^27, k < 2^22).
__device__ __forceinline__ void put_mc_record(float* points, unsigned long long idx, uint32_t i, uint32_t axis,
                                              uint32_t d, uint32_t j, uint32_t k)
{
    uint32_t* r = reinterpret_cast<uint32_t*>(points) + 3 * idx;
    r[0] = i | (axis << 10) | (d << 12) | ((j & 0x1ffffu) << 15);
    r[1] = (j >> 17) | (k << 10);
}

// Inclusive warp scan.
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

// Flying Edges id of cube edge e of the cell at bit `bit` of word w, relative
// to the row's first vertex, from the warp's mask table:
//   e : 0  1  2  3  4  5  6  7  8  9  10 11
//   mask xA yA xB yA xC yC xD yC zA zA zB zB    (index 0..7 below)
//   +1  .  1  .  .  .  1  .  .  .  1  .  1      (edge at point i+1)
__device__ __forceinline__ uint32_t fe_edge_rel(const uint2* mb, int W, int e, int w, int bit)
{
    const int sel = (int)((0x776653524140ull >> (4 * e)) & 7u);
    const int off = (0xA22 >> e) & 1;
    const uint2 p = mb[sel * W + w];
    return p.y + __popc(p.x & lowmask(bit + off));
}

// Id in the global-edge-index order (x block, y block, z block) of cube edge
// e of the cell at bit `bit` of word w: util::duplicateRemover's order
// (marchingCubes/util/DuplicateRemover.h:38-103).
__device__ __forceinline__ unsigned long long dup_edge_id(const uint2* mb, const unsigned long long* db, int W, int e,
                                                          int w, int bit)
{
    const int sel = (int)((0x776653524140ull >> (4 * e)) & 7u);
    const int off = (0xA22 >> e) & 1;
    return db[sel * W + w] + __popc(mb[sel * W + w].x & lowmask(bit + off));
}

template <int MODE, typename IndexT>
__global__ void __launch_bounds__(kThreads, kGenCtasPerSm) k_gen_warps(
    const float* __restrict__ vol, const uint32_t* __restrict__ bits, Grid g, GradScale gs, float iso, int KC,
    int nkc, int kbeg, int kend, int kemit, unsigned long long vbase, unsigned long long tbase, int ws_bytes,
    const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, RowStarts rs,
    unsigned long long* __restrict__ totals, unsigned int* __restrict__ work, long long capV, long long capT,
    float* __restrict__ points,
    float* __restrict__ normals, IndexT* __restrict__ tris, uint32_t* __restrict__ fe2mc, int reverse)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr bool OWNED = MODE == kGenMC || MODE == kGenDup;  // vertices computed by their owner cell
    __shared__ uint64_t s_tris[MODE == kGenMC ? 1 : 256];
    __shared__ uint64_t s_order[OWNED ? 256 : 1];
    __shared__ uint16_t s_cut[OWNED ? 256 : 1];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = g.W;
    unsigned char* ws = s_raw + (size_t)warp * ws_bytes;
    uint2* mb = reinterpret_cast<uint2*>(ws);
    uint32_t* rwt = reinterpret_cast<uint32_t*>(ws + (size_t)8 * W * 8);
    uint32_t* cell = rwt + 8 * W;
    unsigned char* list = reinterpret_cast<unsigned char*>(cell + kGenCells);
    unsigned long long* vq_id = reinterpret_cast<unsigned long long*>(list + gen_list_bytes(MODE));
    uint32_t* vq_pos = reinterpret_cast<uint32_t*>(vq_id + 3 * kGenVq);
    unsigned long long* db = reinterpret_cast<unsigned long long*>(list + gen_list_bytes(MODE));  // Dup
    for (int c = tid; c < 256; c += kThreads) {
        if (OWNED) {
            s_order[c] = cases->order[c];
            s_cut[c] = cases->cut[c];
        }
        if (MODE != kGenMC) s_tris[c] = cases->tris[c];
    }
    __syncthreads();  // the only CTA barrier: from here on every warp runs alone
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;  // caller grows buffers

    // work items: grid row j and a run of KC planes, taken from the counter `work`
    // (one wave of CTAs; no warp waits for another, no CTA stays for its slowest warp)
    const uint32_t nitems = (uint32_t)g.ny * (uint32_t)nkc;
    for (;;) {
        uint32_t item = 0u;
        if (lane == 0) item = atomicAdd(work, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitems) break;
        const int col = (int)(item / (uint32_t)g.ny);
        const int kc = reverse ? nkc - 1 - col : col;
        const int kb = kbeg + kc * KC, ke = min(kb + KC, kend);
        const int j = (int)(item % (uint32_t)g.ny);
        const int jlo = j > 0 ? j - 1 : 0;  // planes are addressed from this row
        const long long plane = (long long)g.ny * g.nx;
        auto plane_ptr = [&](int p) { return vol + (long long)(p - g.kd) * plane + (long long)jlo * g.nx; };

        const bool hasY = j < g.ny - 1;

        const bool in = lane < W, in1 = lane + 1 < W;
        const uint32_t evalid = validmask(lane, g.nx - 1);  // x-edges / cells: i <= nx-2
        const uint32_t pvalid = validmask(lane, g.nx);      // points: i <= nx-1

        // Bit words of rows (j, p) and (j+1, p).
        auto load_words = [&](int p, uint32_t& wa, uint32_t& wb) {
            const bool okp = p < g.ke;  // rows of the window
            const long long r = (long long)(p - g.kr) * g.ny + j;
            wa = (in && okp) ? __ldg(&bits[r * W + lane]) : 0u;
            wb = (in && okp && hasY) ? __ldg(&bits[(r + 1) * W + lane]) : 0u;
        };
        // Row starts of step p, one per lane: lanes 0..3 the first vertex of rows
        // A = (j,p), B = (j+1,p), C = (j,p+1), D = (j+1,p+1); lane 4 the first
        // triangle (FE, TRI) or MC vertex (MC) of cell row A; lane 5 the x + y
        // cuts of row B.
        // Dup instead: lanes 0..3 the first x cut of rows A..D, lane 4 the first
        // triangle of cell row A, lanes 5, 6 the first y cut of rows A, C, lanes
        // 7, 8 the first z cut of rows A, B (each block's own numbering).
        auto load_starts_dup = [&](int p) -> unsigned long long {
            const long long rA = (long long)(p - g.kr) * g.ny + j;
            const bool hasZp = p + 1 < g.ke;
            // (row offset dk * ny + dj, component, exists)
            int dk = 0, dj = 0, comp = 0;
            bool ok = true;
            if (lane < 4) {
                dk = (lane >> 1) & 1;
                dj = lane & 1;
                ok = (dj == 0 || hasY) && (dk == 0 || hasZp);
            } else if (lane == 4) {
                comp = 1;
            } else if (lane <= 6) {
                comp = 2;
                dk = lane - 5;
                ok = dk == 0 || hasZp;
            } else if (lane <= 8) {
                comp = 3;
                dj = lane - 7;
                ok = dj == 0 || hasY;
            } else {
                ok = false;
            }
            return ok ? rs.get(rA + (long long)dk * g.ny + dj, comp) : 0ull;
        };
        auto load_starts = [&](int p) -> unsigned long long {
            if (MODE == kGenDup) return load_starts_dup(p);
            const int dk = (lane >> 1) & 1, dj = lane & 1;
            const bool hasZp = p + 1 < g.ke;
            bool ok = lane < 6;
            if (lane < 4) ok = ok && (dj == 0 || hasY) && (dk == 0 || hasZp);
            if (lane == 5) ok = ok && hasY;
            if (!ok) return 0ull;
            const long long rA = (long long)(p - g.kr) * g.ny + j;
            if (lane == 5) {
                const uint2 c = __ldg(reinterpret_cast<const uint2*>(&rowcnt[rA + 1]));
                return (unsigned long long)c.x + c.y;
            }
            const long long r = lane < 4 ? rA + (long long)dk * g.ny + dj : rA;
            return rs.get(r, lane < 4 ? 0 : (MODE == kGenMC ? 2 : 1));
        };

        const unsigned long long dupY = MODE == kGenDup ? totals[4] : 0ull;  // all x cuts
        const unsigned long long dupZ = MODE == kGenDup ? totals[4] + totals[5] : 0ull;  // all x and y cuts
        uint32_t wA = 0, wB = 0, wC = 0, wD = 0;
        load_words(kb, wA, wB);
        load_words(kb + 1, wC, wD);
        unsigned long long st = load_starts(kb);

        // FE vertex queues: ring heads and fill per axis (warp-uniform)
        uint32_t vh0 = 0, vh1 = 0, vh2 = 0, vn0 = 0, vn1 = 0, vn2 = 0;
        // (copied in and out by value: a reference would put them in local memory)
        auto vq_get = [&](auto axis_tag, uint32_t& head, uint32_t& cnt) {
            constexpr int A = decltype(axis_tag)::value;
            if constexpr (A == 0) {
                head = vh0;
                cnt = vn0;
            } else if constexpr (A == 1) {
                head = vh1;
                cnt = vn1;
            } else {
                head = vh2;
                cnt = vn2;
            }
        };
        auto vq_set = [&](auto axis_tag, uint32_t head, uint32_t cnt) {
            constexpr int A = decltype(axis_tag)::value;
            if constexpr (A == 0) {
                vh0 = head;
                vn0 = cnt;
            } else if constexpr (A == 1) {
                vh1 = head;
                vn1 = cnt;
            } else {
                vh2 = head;
                vn2 = cnt;
            }
        };
        // Vertex batches of axis A from the queue: full ones, or all that is left
        // at the end.  Each lane computes one vertex with the axis-A code.
        auto drain = [&](auto axis_tag, bool all) {
            constexpr int A = decltype(axis_tag)::value;
            uint32_t head, cnt;
            vq_get(axis_tag, head, cnt);
            while (cnt >= 32u || (all && cnt > 0u)) {
                const uint32_t nb = min(cnt, 32u);
                if ((uint32_t)lane < nb) {
                    const uint32_t slot = A * kGenVq + ((head + lane) & (kGenVq - 1));
                    const uint32_t pos = vq_pos[slot];
                    const int i = (int)(pos & 1023u), kk = (int)(pos >> 10);
                    const float* at = plane_ptr(kk);
                    const float* lo = kk > 0 ? plane_ptr(kk - 1) : at;
                    const float* hi = kk + 1 < g.nz ? plane_ptr(kk + 1) : at;
                    const float* hi2 = kk + 2 < g.nz ? plane_ptr(kk + 2) : hi;
                    float3 p, n;
                    vertex_axis<A>(lo, at, hi, hi2, jlo, g, gs, iso, i, j, kk, p, n);
                    store_vertex(points, normals, vq_id[slot] - vbase, p, n);
                }
                head = (head + nb) & (kGenVq - 1);
                cnt -= nb;
            }
            vq_set(axis_tag, head, cnt);
        };

        // One step past the column (fin): no row, the queued vertices are drained
        // (one drain site per axis keeps the kernel's code small).
        for (int k = kb; k <= ke; ++k) {
            const bool fin = k == ke;
            const bool hasZ = k + 1 < g.nz;
            // the next step's words and starts, in flight while this step runs
            uint32_t nC = 0, nD = 0;
            unsigned long long nst = 0;
            if (k + 1 < ke) {
                load_words(k + 2, nC, nD);
                nst = load_starts(k + 1);
            }
            const bool cellrow = hasY && hasZ;
            RowWords rw;
            rw.a = fin ? 0u : wA;
            rw.b = fin ? 0u : wB;
            rw.c = hasZ && !fin ? wC : 0u;
            rw.d = cellrow && !fin ? wD : 0u;
            const uint32_t an = __shfl_down_sync(0xffffffffu, rw.a, 1);
            const uint32_t bn = __shfl_down_sync(0xffffffffu, rw.b, 1);
            const uint32_t cn = __shfl_down_sync(0xffffffffu, rw.c, 1);
            const uint32_t dn = __shfl_down_sync(0xffffffffu, rw.d, 1);
            rw.ash = (rw.a >> 1) | ((in1 ? an : 0u) << 31);
            rw.bsh = (rw.b >> 1) | ((in1 ? bn : 0u) << 31);
            rw.csh = (rw.c >> 1) | ((in1 ? cn : 0u) << 31);
            rw.dsh = (rw.d >> 1) | ((in1 ? dn : 0u) << 31);
            const CutMasks m = cut_masks(rw, evalid, pvalid, hasY, hasZ);
            // popc prefixes, two 16-bit counts per scan
            const uint32_t p0 = __popc(m.xA) | (__popc(m.xB) << 16);
            const uint32_t p1 = __popc(m.xC) | (__popc(m.xD) << 16);
            const uint32_t p2 = __popc(m.yA) | (__popc(m.yC) << 16);
            const uint32_t p3 = __popc(m.zA) | (__popc(m.zB) << 16);
            const uint32_t i0 = warp_incl_scan(p0, lane), i1 = warp_incl_scan(p1, lane);
            const uint32_t i2 = warp_incl_scan(p2, lane), i3 = warp_incl_scan(p3, lane);
            const uint32_t e0 = i0 - p0, e1 = i1 - p1, e2 = i2 - p2, e3 = i3 - p3;
            const uint32_t t0 = __shfl_sync(0xffffffffu, i0, 31), t2 = __shfl_sync(0xffffffffu, i2, 31);
            const uint32_t t1 = __shfl_sync(0xffffffffu, i1, 31), t3 = __shfl_sync(0xffffffffu, i3, 31);
            const unsigned long long xsA = __shfl_sync(0xffffffffu, st, 0);
            const uint32_t dB = (uint32_t)(__shfl_sync(0xffffffffu, st, 1) - xsA);
            const uint32_t dC = (uint32_t)(__shfl_sync(0xffffffffu, st, 2) - xsA);
            const uint32_t dD = (uint32_t)(__shfl_sync(0xffffffffu, st, 3) - xsA);
            const unsigned long long ts = __shfl_sync(0xffffffffu, st, 4);
            const uint32_t cntB = (uint32_t)__shfl_sync(0xffffffffu, st, 5);
            const uint32_t nxA = t0 & 0xffffu, nyA = t2 & 0xffffu, nzA = t3 & 0xffffu, nxC = t1 & 0xffffu;
            unsigned long long dxB[8];  // Dup: block starts of the 8 masks' rows (x A B C D, y A C, z A B)
            if (MODE == kGenDup) {
#pragma unroll
                for (int q = 0; q < 8; ++q) dxB[q] = __shfl_sync(0xffffffffu, st, q < 4 ? q : q + 1);
            }
            if (in) {  // first ids of the word's cut edges, relative to xsA
                mb[0 * W + lane] = make_uint2(m.xA, e0 & 0xffffu);
                mb[1 * W + lane] = make_uint2(m.xB, dB + (e0 >> 16));
                mb[2 * W + lane] = make_uint2(m.xC, dC + (e1 & 0xffffu));
                mb[3 * W + lane] = make_uint2(m.xD, dD + (e1 >> 16));
                mb[4 * W + lane] = make_uint2(m.yA, nxA + (e2 & 0xffffu));
                mb[5 * W + lane] = make_uint2(m.yC, dC + nxC + (e2 >> 16));
                mb[6 * W + lane] = make_uint2(m.zA, nxA + nyA + (e3 & 0xffffu));
                mb[7 * W + lane] = make_uint2(m.zB, dB + cntB + (e3 >> 16));
                if (MODE == kGenDup) {  // ids in the global-edge-index order: x block, y block, z block
                    db[0 * W + lane] = dxB[0] + (e0 & 0xffffu);
                    db[1 * W + lane] = dxB[1] + (e0 >> 16);
                    db[2 * W + lane] = dxB[2] + (e1 & 0xffffu);
                    db[3 * W + lane] = dxB[3] + (e1 >> 16);
                    db[4 * W + lane] = dupY + dxB[4] + (e2 & 0xffffu);
                    db[5 * W + lane] = dupY + dxB[5] + (e2 >> 16);
                    db[6 * W + lane] = dupZ + dxB[6] + (e3 & 0xffffu);
                    db[7 * W + lane] = dupZ + dxB[7] + (e3 >> 16);
                }
                if (cellrow) {  // corner order of the cube case: bit v = corner v
                    uint4* t = reinterpret_cast<uint4*>(rwt + 8 * lane);
                    t[0] = make_uint4(rw.a, rw.ash, rw.bsh, rw.b);
                    t[1] = make_uint4(rw.c, rw.csh, rw.dsh, rw.d);
                }
            }
            __syncwarp();
            if (MODE == kGenFE) {
                // ---- vertices of grid row (j, k): x, y then z sections
                const uint32_t nv = nxA + nyA + nzA;
                // word prefixes of the x, y and z sections in one word: 10 + 11 + 11 bits
                const uint32_t P = (e0 & 0x3ffu) | ((e2 & 0x7ffu) << 10) | ((e3 & 0x7ffu) << 21);
                for (uint32_t v0 = 0; v0 < nv || (fin && v0 == 0); v0 += 32) {
                    const uint32_t v = v0 + lane;
                    const int axis = v < nxA ? 0 : (v < nxA + nyA ? 1 : 2);
                    const uint32_t r = v - (axis == 0 ? 0u : (axis == 1 ? nxA : nxA + nyA));
                    const int sh = axis == 0 ? 0 : (axis == 1 ? 10 : 21);
                    const uint32_t fm = axis == 0 ? 0x3ffu : 0x7ffu;
                    int lo = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int mid = lo + step;
                        const uint32_t pv = (__shfl_sync(0xffffffffu, P, mid & 31) >> sh) & fm;
                        if (mid < W && pv <= r) lo = mid;
                    }
                    int i = 0;
                    if (v < nv) {
                        const uint2 e = mb[(axis == 0 ? 0 : (axis == 1 ? 4 : 6)) * W + lo];
                        i = 32 * lo + (int)__fns(e.x, 0, (int)(v - e.y) + 1);
                    }
                    // append to the axis queues (each had < 32 entries: room for 32 more)
                    auto append = [&](auto axis_tag) {
                        constexpr int a = decltype(axis_tag)::value;
                        const bool mine = v < nv && axis == a;
                        const uint32_t ball = __ballot_sync(0xffffffffu, mine);
                        uint32_t head, cnt;
                        vq_get(axis_tag, head, cnt);
                        if (mine) {
                            const uint32_t slot =
                                a * kGenVq + ((head + cnt + __popc(ball & ((1u << lane) - 1u))) & (kGenVq - 1));
                            vq_id[slot] = xsA + v;
                            vq_pos[slot] = (uint32_t)i | ((uint32_t)k << 10);
                        }
                        vq_set(axis_tag, head, cnt + __popc(ball));
                    };
                    append(std::integral_constant<int, 0>());
                    append(std::integral_constant<int, 1>());
                    append(std::integral_constant<int, 2>());
                    __syncwarp();
                    drain(std::integral_constant<int, 0>(), fin);
                    drain(std::integral_constant<int, 1>(), fin);
                    drain(std::integral_constant<int, 2>(), fin);
                    __syncwarp();
                }
            }
            if (cellrow) {
                // ---- active cells of cell row (j, k), 32 at a time
                const uint32_t act = in ? active_cells(rw, evalid) : 0u;
                const uint32_t na = __popc(act);
                const uint32_t ia = warp_incl_scan(na, lane);
                const uint32_t tot = __shfl_sync(0xffffffffu, ia, 31);
                unsigned long long tcur = ts;  // FE / TRI / Dup: next triangle
                unsigned long long mcur = ts;  // MC: next vertex
                for (uint32_t c0 = 0; c0 < tot; c0 += kGenCells) {
                    // lane L takes active cell c0 + L: the first lane whose inclusive count passes it (a
                    // shuffle binary search over the lanes), then the bit by __fns -- no per-lane loop,
                    // which diverges where the active cells cluster along the surface
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
                        const uint32_t ci = (uint32_t)(32 * src + (int)__fns(srcact, 0, (int)(target - srcexc) + 1));
                        const uint4* t = reinterpret_cast<const uint4*>(rwt + 8 * (ci >> 5));
                        const uint4 lo4 = t[0], hi4 = t[1];
                        const int b = (int)(ci & 31u);
                        const uint32_t cs = ((lo4.x >> b) & 1u) | (((lo4.y >> b) & 1u) << 1) |
                                            (((lo4.z >> b) & 1u) << 2) | (((lo4.w >> b) & 1u) << 3) |
                                            (((hi4.x >> b) & 1u) << 4) |
                                            (((hi4.y >> b) & 1u) << 5) | (((hi4.z >> b) & 1u) << 6) |
                                            (((hi4.w >> b) & 1u) << 7);
                        rec = ci | (cs << 16);
                        cell[lane] = rec;
                    }
                    const int cs = (int)(rec >> 16);
                    if (MODE != kGenMC) {
                        const uint32_t nt = live ? (uint32_t)iso_case_ntris(s_tris[cs]) : 0u;
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
                                const int ci = (int)(cr & 0xffffu);
                                const uint64_t tl = s_tris[cr >> 16];
                                const int w = ci >> 5, bit = ci & 31;
                                IndexT* o = tris + 3 * (tcur + t - tbase);
#pragma unroll
                                for (int c = 0; c < 3; ++c) {
                                    const int e = iso_case_edge(tl, 3 * q + c);
                                    if (MODE == kGenDup) {
                                        o[c] = (IndexT)dup_edge_id(mb, db, W, e, w, bit);
                                    } else {
                                        const unsigned long long id = xsA + fe_edge_rel(mb, W, e, w, bit);
                                        o[c] = MODE == kGenTri ? (IndexT)__ldg(fe2mc + id) : (IndexT)id;
                                    }
                                }
                            }
                        }
                        tcur += ntb;
                    }
                    if (MODE == kGenDup) __syncwarp();  // the vertex list below reuses the triangle list
                    if (OWNED) {
                        // ---- MC vertices owned by the batch's cells: cell order, then order of
                        // first appearance in the cell's triangle list
                        const int ci = (int)(rec & 0xffffu);
                        const uint32_t own = live ? (mc_owned_edges(ci == 0, j == 0, k == 0) & s_cut[cs]) : 0u;
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
                                const int i = (int)(cr & 0xffffu);
                                // MC: owner order; Dup: the edge's place in the global-edge-index order
                                const unsigned long long id =
                                    MODE == kGenDup ? dup_edge_id(mb, db, W, e12, i >> 5, i & 31) : mcur + v;
                                if (k >= kemit) {  // cell rows below kemit belong to the slab below: map only
                                    int dx, dy, dz, axis;
                                    cube_edge_geometry(e12, dx, dy, dz, axis);
                                    // the record kernel (k_vertices) computes the vertex from its record
                                    put_mc_record(points, id - vbase, (uint32_t)(i + dx), (uint32_t)axis,
                                                  (uint32_t)(dx | (dy << 1) | (dz << 2)), (uint32_t)(j + dy),
                                                  (uint32_t)(k + dz));
                                }
                                if (MODE == kGenMC) fe2mc[xsA + fe_edge_rel(mb, W, e12, i >> 5, i & 31)] = (uint32_t)id;
                            }
                        }
                        mcur += nob;
                    }
                    __syncwarp();  // the next batch overwrites the lists
                }
            }
            __syncwarp();  // the next step overwrites mb
            wA = wC;
            wB = wD;
            wC = nC;
            wD = nD;
            st = nst;
        }
    }  // work items
}

template <int MODE, typename IndexT>
void launch_gen_warps_impl(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                           const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                           float* normals, IndexT* tris, int reverse, cudaStream_t s)
{
    const int nzw = p.kend - p.kbeg;
    if (nzw <= 0) return;
    // items of KC planes: about eight per warp of one wave, at least 2 planes (667 x 228 x 724: FE 635 -> 631,
    // MC 687 -> 676 us against four per warp and 4 planes; sixteen per warp: 644 / 680)
    const long long warps = (long long)p.nsm * kGenCtasPerSm * kGenRows;
    long long KC = ((long long)g.ny * nzw + 8 * warps - 1) / (8 * warps);
    if (KC < 2) KC = 2;
    while ((long long)g.ny * ((nzw + KC - 1) / KC) >= (1ll << 31)) KC *= 2;  // item numbers stay below 2^31
    if (KC > nzw) KC = nzw;
    const int nkc = (int)((nzw + KC - 1) / KC);
    const long long nitems = (long long)g.ny * nkc;
    long long blocks = (nitems + kGenRows - 1) / kGenRows;
    if (blocks > (long long)p.nsm * kGenCtasPerSm) blocks = (long long)p.nsm * kGenCtasPerSm;
    RowStarts rs = row_starts(g, cp, b);
    for (int a = 0; a < 3; ++a) rs.add[a] = p.add[a];
    unsigned int* work = reinterpret_cast<unsigned int*>(b.totals + 7);
    cudaMemsetAsync(work, 0, sizeof(unsigned int), s);
    const int ws_bytes = (int)gen_warp_scratch_bytes(g.W, MODE);
    const size_t smem = (size_t)kGenRows * ws_bytes;
    auto kern = k_gen_warps<MODE, IndexT>;
    allow_smem(kern, smem);
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(vol, b.bits, g, make_grad_scale(g), iso, (int)KC, nkc, p.kbeg,
                                                  p.kend, p.kemit, p.vbase, p.tbase, ws_bytes, cases, b.rowcnt, rs,
                                                  b.totals, work, capV, capT, points, normals, tris, b.fe2mc,
                                                  reverse);
}

}  // namespace iso
