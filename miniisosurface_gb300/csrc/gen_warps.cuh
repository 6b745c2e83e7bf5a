// Pass 4 on sm_103a (included by gen_warps_fe.cu and gen_warps_mc.cu).
//
// A CTA owns a block of J = 8 grid rows (j0 .. j0+7, one warp per row) and a
// run of KC planes, and marches along z.  The warps never wait for one
// another except through a ring of kGenSlots plane slabs in shared memory:
//
//   full[s]   the slab in slot s has landed (TMA bulk copy, or cp.async when
//             rows are not 16-byte aligned), issued by warp 0 lane 0
//   empty[s]  all 8 warps are done with the plane in slot s
//
// A slab holds rows j0-1 .. j0+J+1 of a plane (contiguous in memory), so a
// warp finds every value it interpolates at planes k and k+1 in shared
// memory; the gradient neighbours at planes k-1 and k+2 come from L2.
//
// Per step a warp handles grid row (j, k) with one 32-bit word of the bit
// mask written by the count pass per lane:
//   masks + popc prefixes (warp scans) of the 8 cut masks of the cell row;
//   FE  : the row's vertices, one per lane (a shuffle binary search maps the
//         lane's vertex rank to a word and __fns to a bit), written to
//         consecutive ids; then the row's active cells, one per lane, each
//         writing its triangles (corner ids = popc ranks)
//   MC  : the vertices owned by cell row (j, k) in owner-cell /
//         first-appearance order (marchingCubes/serial/main.cpp:139-177),
//         one per lane, and the Flying Edges -> MC index map
//   TRI : (no volume) triangles with corners mapped through that map.
#pragma once
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

constexpr int kGenRows = 8;    // grid rows per CTA, one per warp
constexpr int kGenSlots = 4;   // planes k, k+1 resident; k+2, k+3 in flight
enum GenMode { kGenFE = 0, kGenMC = 1, kGenTri = 2 };

struct GenSlab {
    int jlo, nrows;  // first row and number of rows of a slab
};

__host__ __device__ inline GenSlab gen_slab_rows(int j0, int ny)
{
    GenSlab s;
    s.jlo = j0 > 0 ? j0 - 1 : 0;
    const int jhi = min(j0 + kGenRows + 2, ny);
    s.nrows = jhi - s.jlo;
    return s;
}

// Values of the volume around the row while planes k and k+1 are staged.
struct WarpSlab {
    const float* vol;
    const float* sk;   // slab of plane k, indexed by (j - jlo) * nx + i
    const float* sk1;  // slab of plane k+1
    int k, jlo, nx, ny;
    __device__ __forceinline__ float operator()(int i, int j, int p) const
    {
        if (p == k) return sk[(j - jlo) * nx + i];
        if (p == k + 1) return sk1[(j - jlo) * nx + i];
        return __ldg(vol + ((long long)p * ny + j) * nx + i);
    }
};

template <typename Acc>
__device__ __forceinline__ float3 gradient_acc(const Acc& acc, const Grid& g, int i, int j, int k)
{
    const float here = acc(i, j, k);
    const float xm = i > 0 ? acc(i - 1, j, k) : 0.f, xp = i < g.nx - 1 ? acc(i + 1, j, k) : 0.f;
    const float ym = j > 0 ? acc(i, j - 1, k) : 0.f, yp = j < g.ny - 1 ? acc(i, j + 1, k) : 0.f;
    const float zm = k > 0 ? acc(i, j, k - 1) : 0.f, zp = k < g.nz - 1 ? acc(i, j, k + 1) : 0.f;
    float3 r;
    r.x = grad_component(xm, here, xp, i, g.nx, g.sp[0]);
    r.y = grad_component(ym, here, yp, j, g.ny, g.sp[1]);
    r.z = grad_component(zm, here, zp, k, g.nz, g.sp[2]);
    return r;
}

// edge_vertex() of iso_device.cuh with values from an accessor.
template <typename Acc>
__device__ __forceinline__ void edge_vertex_acc(const Acc& acc, const Grid& g, float iso, int axis, int i, int j,
                                                int k, int ci, int cj, int ck, float3& pos, float3& nrm)
{
    const int i1 = i + (axis == 0), j1 = j + (axis == 1), k1 = k + (axis == 2);
    const float v0 = acc(i, j, k);
    const float v1 = acc(i1, j1, k1);
    const float w = fdiv(fsub(iso, v0), fsub(v1, v0));
    pos.x = lerp_ref(cube_coord(ci, i - ci, g.zp[0], g.sp[0]), cube_coord(ci, i1 - ci, g.zp[0], g.sp[0]), w);
    pos.y = lerp_ref(cube_coord(cj, j - cj, g.zp[1], g.sp[1]), cube_coord(cj, j1 - cj, g.zp[1], g.sp[1]), w);
    pos.z = lerp_ref(cube_coord(ck, k - ck, g.zp[2], g.sp[2]), cube_coord(ck, k1 - ck, g.zp[2], g.sp[2]), w);
    const float3 g0 = gradient_acc(acc, g, i, j, k);
    const float3 g1 = gradient_acc(acc, g, i1, j1, k1);
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

// Largest lane w < W with pre(w) <= r, where pre is a per-lane non-decreasing
// prefix with pre(0) == 0 (all 32 lanes must call).
__device__ __forceinline__ int lane_search(uint32_t pre, uint32_t r, int W)
{
    int lo = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const int mid = lo + step;
        const uint32_t v = __shfl_sync(0xffffffffu, pre, mid & 31);
        if (mid < W && v <= r) lo = mid;
    }
    return lo;
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

// The four bit words of the lane (rows A, B, C, D of the cell row) and their
// i+1 neighbours, fetched from lane `src`.
__device__ __forceinline__ RowWords words_from(const RowWords& mine, int src)
{
    RowWords r;
    r.a = __shfl_sync(0xffffffffu, mine.a, src);
    r.b = __shfl_sync(0xffffffffu, mine.b, src);
    r.c = __shfl_sync(0xffffffffu, mine.c, src);
    r.d = __shfl_sync(0xffffffffu, mine.d, src);
    r.ash = __shfl_sync(0xffffffffu, mine.ash, src);
    r.bsh = __shfl_sync(0xffffffffu, mine.bsh, src);
    r.csh = __shfl_sync(0xffffffffu, mine.csh, src);
    r.dsh = __shfl_sync(0xffffffffu, mine.dsh, src);
    return r;
}

__device__ __forceinline__ CutMasks masks_from(const CutMasks& mine, int src)
{
    CutMasks m;
    m.xA = __shfl_sync(0xffffffffu, mine.xA, src);
    m.xB = __shfl_sync(0xffffffffu, mine.xB, src);
    m.xC = __shfl_sync(0xffffffffu, mine.xC, src);
    m.xD = __shfl_sync(0xffffffffu, mine.xD, src);
    m.yA = __shfl_sync(0xffffffffu, mine.yA, src);
    m.yC = __shfl_sync(0xffffffffu, mine.yC, src);
    m.zA = __shfl_sync(0xffffffffu, mine.zA, src);
    m.zB = __shfl_sync(0xffffffffu, mine.zB, src);
    return m;
}

template <int MODE, typename IndexT, bool BULK>
__global__ void __launch_bounds__(kThreads) k_gen_warps(
    const float* __restrict__ vol, const uint32_t* __restrict__ bits, Grid g, float iso, int KC, int nyb,
    int slab_floats, const CaseTables* __restrict__ cases, const uint4* __restrict__ rowcnt, RowStarts rs,
    unsigned long long* __restrict__ totals, long long capV, long long capT, float* __restrict__ points,
    float* __restrict__ normals, IndexT* __restrict__ tris, uint32_t* __restrict__ fe2mc, int reverse)
{
    constexpr bool VOL = MODE != kGenTri;
    constexpr int NS = kGenSlots;
    extern __shared__ __align__(128) unsigned char s_raw[];
    __shared__ SharedCases s_cases;
    float* slots = reinterpret_cast<float*>(s_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(s_raw + (size_t)NS * slab_floats * 4);
    uint64_t* empty = full + NS;
    stage_cases(s_cases, cases, MODE == kGenMC);  // includes __syncthreads
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;  // caller grows buffers

    const int nkc = gridDim.x / nyb;
    const int jb = blockIdx.x % nyb;
    const int kc = reverse ? nkc - 1 - (int)(blockIdx.x / nyb) : (int)(blockIdx.x / nyb);
    const int j0 = jb * kGenRows;
    const int kb = kc * KC, ke = min(kb + KC, g.nz);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = g.W;
    const int j = j0 + warp;
    const bool row_ok = j < g.ny;
    const GenSlab sl = gen_slab_rows(j0, g.ny);
    const int nfl = sl.nrows * g.nx;

    if (VOL && tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], BULK ? 1u : 32u);
            mbar_init(&empty[s], (unsigned)kGenRows);
        }
        fence_mbar_init();
    }
    __syncthreads();

    // ---- slab ring.  Plane p lives in slot p % NS; its use index in the slot
    // is (p - kb) / NS, which gives the phase parity of both barriers.
    bool alive = true;
    uint32_t issued = 0;  // producer: planes issued so far, as kb + issued
    auto issue_upto = [&](int plast) -> bool {  // warp 0 only: issue planes <= plast
        bool ok = true;
        const int pmax = min(plast, min(ke, g.nz - 1));
        while (ok && kb + (int)issued <= pmax) {
            const int p = kb + (int)issued;
            const int s = p % NS;
            if (p - kb >= NS) ok = mbar_wait(&empty[s], (((p - kb) / NS) - 1) & 1);  // previous plane released
            if (ok) {
                slab_copy<BULK>(slots + (size_t)s * slab_floats, vol + ((long long)p * g.ny + sl.jlo) * g.nx, nfl,
                                &full[s], lane, 32);
            }
            ++issued;
        }
        return ok;
    };
    auto wait_plane = [&](int p) -> bool { return mbar_wait(&full[p % NS], ((p - kb) / NS) & 1); };

    if (VOL && warp == 0) alive = issue_upto(kb + NS - 2);
    alive = __syncthreads_and(alive);

    const bool in = lane < W, in1 = lane + 1 < W;
    const uint32_t evalid = validmask(lane, g.nx - 1);  // x-edges / cells: i <= nx-2
    const uint32_t pvalid = validmask(lane, g.nx);      // points: i <= nx-1

    for (int k = kb; k < ke && alive; ++k) {
        if (VOL && warp == 0) alive = issue_upto(k + NS - 1) && alive;
        const bool hasZ = k + 1 < g.nz;
        if (VOL) {
            bool ok = wait_plane(k);
            if (hasZ) ok = ok && wait_plane(k + 1);
            alive = alive && ok;
        }
        if (!__all_sync(0xffffffffu, alive)) {
            alive = false;
            break;
        }
        if (row_ok) {
            const bool hasY = j < g.ny - 1, cell = hasY && hasZ;
            // ---- bit words of rows A = (j,k), B = (j+1,k), C = (j,k+1), D = (j+1,k+1)
            const long long rA = (long long)k * g.ny + j;
            RowWords rw;
            rw.a = in ? __ldg(&bits[rA * W + lane]) : 0u;
            rw.b = (in && hasY) ? __ldg(&bits[(rA + 1) * W + lane]) : 0u;
            rw.c = (in && hasZ) ? __ldg(&bits[(rA + g.ny) * W + lane]) : 0u;
            rw.d = (in && cell) ? __ldg(&bits[(rA + g.ny + 1) * W + lane]) : 0u;
            // row starts: lanes 0..5 fetch, then broadcast
            unsigned long long st = 0;
            if (lane == 0) st = rs.get(k, j, 0);
            else if (lane == 1 && hasY) st = rs.get(k, j + 1, 0);
            else if (lane == 2 && hasZ) st = rs.get(k + 1, j, 0);
            else if (lane == 3 && cell) st = rs.get(k + 1, j + 1, 0);
            else if (lane == 4) st = rs.get(k, j, MODE == kGenMC ? 2 : 1);
            else if (lane == 5 && hasY) {
                const uint4 cb = __ldg(&rowcnt[rA + 1]);
                st = (unsigned long long)cb.x + cb.y;
            }
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
            const unsigned long long xsB = __shfl_sync(0xffffffffu, st, 1);
            const unsigned long long xsC = __shfl_sync(0xffffffffu, st, 2);
            const unsigned long long xsD = __shfl_sync(0xffffffffu, st, 3);
            const unsigned long long ts = __shfl_sync(0xffffffffu, st, 4);
            const unsigned long long cntB = __shfl_sync(0xffffffffu, st, 5);
            const uint32_t nxA = t0 & 0xffffu, nyA = t2 & 0xffffu, nzA = t3 & 0xffffu, nxC = t1 & 0xffffu;
            CutBases base;  // this lane's word
            base.xA = xsA + (e0 & 0xffffu);
            base.xB = xsB + (e0 >> 16);
            base.xC = xsC + (e1 & 0xffffu);
            base.xD = xsD + (e1 >> 16);
            base.yA = xsA + nxA + (e2 & 0xffffu);
            base.yC = xsC + nxC + (e2 >> 16);
            base.zA = xsA + nxA + nyA + (e3 & 0xffffu);
            base.zB = xsB + cntB + (e3 >> 16);

            if (MODE == kGenFE || MODE == kGenMC) {
                const float* sk = slots + (size_t)(k % NS) * slab_floats;
                const float* sk1 = slots + (size_t)((k + 1) % NS) * slab_floats;
                const WarpSlab acc{vol, sk, sk1, k, sl.jlo, g.nx, g.ny};
                if (MODE == kGenFE) {
                    // ---- vertices of grid row (j, k): x, y then z sections
                    const uint32_t nv = nxA + nyA + nzA;
                    const int ck = min(k, g.nz - 2), cj = min(j, g.ny - 2);
                    for (uint32_t v0 = 0; v0 < nv; v0 += 32) {
                        const uint32_t v = v0 + lane;
                        const int axis = v < nxA ? 0 : (v < nxA + nyA ? 1 : 2);
                        const uint32_t r = v - (axis == 0 ? 0u : (axis == 1 ? nxA : nxA + nyA));
                        const uint32_t ex = e0 & 0xffffu, ey = e2 & 0xffffu, ez = e3 & 0xffffu;
                        // word holding rank r of the axis' cut mask
                        int lo = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1) {
                            const int mid = lo + step;
                            const uint32_t px = __shfl_sync(0xffffffffu, ex, mid & 31);
                            const uint32_t py = __shfl_sync(0xffffffffu, ey, mid & 31);
                            const uint32_t pz = __shfl_sync(0xffffffffu, ez, mid & 31);
                            const uint32_t pv = axis == 0 ? px : (axis == 1 ? py : pz);
                            if (mid < W && pv <= r) lo = mid;
                        }
                        const uint32_t mxw = __shfl_sync(0xffffffffu, m.xA, lo);
                        const uint32_t myw = __shfl_sync(0xffffffffu, m.yA, lo);
                        const uint32_t mzw = __shfl_sync(0xffffffffu, m.zA, lo);
                        const uint32_t pxw = __shfl_sync(0xffffffffu, ex, lo);
                        const uint32_t pyw = __shfl_sync(0xffffffffu, ey, lo);
                        const uint32_t pzw = __shfl_sync(0xffffffffu, ez, lo);
                        if (v < nv) {
                            const uint32_t mw = axis == 0 ? mxw : (axis == 1 ? myw : mzw);
                            const uint32_t pw = axis == 0 ? pxw : (axis == 1 ? pyw : pzw);
                            const int bit = (int)__fns(mw, 0, (int)(r - pw) + 1);
                            const int i = 32 * lo + bit;
                            float3 p, n;
                            edge_vertex_acc(acc, g, iso, axis, i, j, k, axis == 0 ? i : min(i, g.nx - 2),
                                            axis == 1 ? j : cj, axis == 2 ? k : ck, p, n);
                            store_vertex(points, normals, xsA + v, p, n);
                        }
                    }
                }
            }
            if (cell && (MODE == kGenFE || MODE == kGenTri)) {
                // ---- triangles of cell row (j, k): one active cell per lane
                const uint32_t act = in ? active_cells(rw, evalid) : 0u;
                const uint32_t na = __popc(act);
                const uint32_t ia = warp_incl_scan(na, lane);
                const uint32_t ea = ia - na, tot = __shfl_sync(0xffffffffu, ia, 31);
                unsigned long long tcur = ts;
                for (uint32_t c0 = 0; c0 < tot; c0 += 32) {
                    const uint32_t cidx = c0 + lane;
                    const int w = lane_search(ea, cidx, W);
                    const RowWords ww = words_from(rw, w);
                    const uint32_t aw = __shfl_sync(0xffffffffu, act, w);
                    const uint32_t eaw = __shfl_sync(0xffffffffu, ea, w);
                    const CutMasks mw = masks_from(m, w);
                    CutBases bw;
                    bw.xA = __shfl_sync(0xffffffffu, base.xA, w);
                    bw.xB = __shfl_sync(0xffffffffu, base.xB, w);
                    bw.xC = __shfl_sync(0xffffffffu, base.xC, w);
                    bw.xD = __shfl_sync(0xffffffffu, base.xD, w);
                    bw.yA = __shfl_sync(0xffffffffu, base.yA, w);
                    bw.yC = __shfl_sync(0xffffffffu, base.yC, w);
                    bw.zA = __shfl_sync(0xffffffffu, base.zA, w);
                    bw.zB = __shfl_sync(0xffffffffu, base.zB, w);
                    const bool live = cidx < tot;
                    const int bit = live ? (int)__fns(aw, 0, (int)(cidx - eaw) + 1) : 0;
                    const uint64_t tl = s_cases.tris[live ? cube_case(ww, bit) : 0];
                    const uint32_t nt = live ? (uint32_t)iso_case_ntris(tl) : 0u;
                    const uint32_t it = warp_incl_scan(nt, lane);
                    const unsigned long long t = tcur + (it - nt);
                    for (int q = 0; q < 3 * (int)nt; ++q) {
                        const unsigned long long id = fe_edge_id(mw, bw, iso_case_edge(tl, q), bit);
                        tris[3 * t + q] = MODE == kGenTri ? (IndexT)__ldg(fe2mc + id) : (IndexT)id;
                    }
                    tcur += __shfl_sync(0xffffffffu, it, 31);
                }
            }
            if (MODE == kGenMC && cell) {
                // ---- MC vertices owned by cell row (j, k), owner order
                const float* sk = slots + (size_t)(k % NS) * slab_floats;
                const float* sk1 = slots + (size_t)((k + 1) % NS) * slab_floats;
                const WarpSlab acc{vol, sk, sk1, k, sl.jlo, g.nx, g.ny};
                const uint32_t act = in ? active_cells(rw, evalid) : 0u;
                uint32_t no = 0;
                for (uint32_t a = act; a; a &= a - 1) {
                    const int bit = __ffs(a) - 1;
                    no += __popc(mc_owned_edges(32 * lane + bit == 0, j == 0, k == 0) & s_cases.cut[cube_case(rw, bit)]);
                }
                const uint32_t io = warp_incl_scan(no, lane);
                const uint32_t eo = io - no, tot = __shfl_sync(0xffffffffu, io, 31);
                for (uint32_t v0 = 0; v0 < tot; v0 += 32) {
                    const uint32_t v = v0 + lane;
                    const int w = lane_search(eo, v, W);
                    const RowWords ww = words_from(rw, w);
                    const uint32_t aw = __shfl_sync(0xffffffffu, act, w);
                    const uint32_t eow = __shfl_sync(0xffffffffu, eo, w);
                    const CutMasks mw = masks_from(m, w);
                    CutBases bw;
                    bw.xA = __shfl_sync(0xffffffffu, base.xA, w);
                    bw.xB = __shfl_sync(0xffffffffu, base.xB, w);
                    bw.xC = __shfl_sync(0xffffffffu, base.xC, w);
                    bw.xD = __shfl_sync(0xffffffffu, base.xD, w);
                    bw.yA = __shfl_sync(0xffffffffu, base.yA, w);
                    bw.yC = __shfl_sync(0xffffffffu, base.yC, w);
                    bw.zA = __shfl_sync(0xffffffffu, base.zA, w);
                    bw.zB = __shfl_sync(0xffffffffu, base.zB, w);
                    if (v < tot) {
                        uint32_t rank = v - eow;
                        int bit = 0, c = 0;
                        uint32_t own = 0;
                        for (uint32_t a = aw; a; a &= a - 1) {  // the cell holding this vertex
                            bit = __ffs(a) - 1;
                            c = cube_case(ww, bit);
                            own = mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cases.cut[c];
                            const uint32_t n = __popc(own);
                            if (rank < n) break;
                            rank -= n;
                        }
                        const uint64_t ord = s_cases.order[c];
                        int e12 = 0;
                        for (int q = 0; q < iso_case_ntris(ord); ++q) {  // rank-th owned edge
                            const int ed = iso_case_edge(ord, q);
                            if ((own >> ed) & 1u) {
                                if (rank == 0) {
                                    e12 = ed;
                                    break;
                                }
                                --rank;
                            }
                        }
                        int dx, dy, dz, axis;
                        cube_edge_geometry(e12, dx, dy, dz, axis);
                        const int i = 32 * w + bit;
                        float3 p, n;
                        edge_vertex_acc(acc, g, iso, axis, i + dx, j + dy, k + dz, i, j, k, p, n);
                        const unsigned long long id = ts + v;
                        store_vertex(points, normals, id, p, n);
                        fe2mc[fe_edge_id(mw, bw, e12, bit)] = (uint32_t)id;
                    }
                }
            }
        }
        __syncwarp();
        if (VOL && lane == 0) mbar_arrive(&empty[k % NS]);  // this warp is done with plane k
    }
    if (!alive && tid == 0) atomicOr(&totals[3], kStatusTimeout);
    if (VOL && warp == 0) {  // copies still in flight must land before the CTA exits
        for (int p = kb; p < kb + (int)issued; ++p) {
            if (p >= ke || !alive) mbar_wait(&full[p % NS], ((p - kb) / NS) & 1);
        }
    }
}

template <int MODE, typename IndexT>
void launch_gen_warps_impl(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                           const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                           float* normals, IndexT* tris, int reverse, cudaStream_t s)
{
    const RowStarts rs = row_starts(g, cp, b);
    const bool bulk = (g.nx % 4 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
    const unsigned blocks = (unsigned)(p.nyb * p.nkc);
    auto kern = bulk ? k_gen_warps<MODE, IndexT, true> : k_gen_warps<MODE, IndexT, false>;
    allow_smem(kern, p.smem);
    kern<<<blocks, kThreads, p.smem, s>>>(vol, b.bits, g, iso, p.KC, p.nyb, p.slab_floats, cases, b.rowcnt, rs,
                                          b.totals, capV, capT, points, normals, tris, b.fe2mc, reverse);
}

}  // namespace iso
