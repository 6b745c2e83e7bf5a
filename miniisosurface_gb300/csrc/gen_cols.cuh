// Pass 4 on sm_103a, column-marching form (included by gen_cols_fe.cu and
// gen_cols_mc.cu).
//
// A CTA owns a block of J grid rows (j0 .. j0+J-1) and a run of KC planes and
// marches along z.  The volume slab of a plane (rows j0 .. j0+J, contiguous in
// memory) is staged in shared memory by the TMA bulk-copy engine
// (cp.async.bulk, one instruction per slab, completion on an mbarrier) -- or by
// cp.async when rows are not 16-byte aligned -- NSLOT slots deep, so the
// copies of planes k+2 and k+3 are in flight while plane k is processed.
//
// Step k (planes k and k+1 resident):
//   prepare(k+1)  bit mask of plane k+1 from its slab; cut masks of the rows
//                 and their in-row popc prefixes; the z cut masks of plane k;
//                 the rows' first vertex ids (from the scan).
//   FE:  vertices of grid rows (j,k): one thread per vertex, found by a binary
//        search over per-(row, axis, word) prefix counts -- every thread does
//        the same amount of work and consecutive threads write consecutive
//        vertices; then triangles of cell rows (j,k), one thread per 32 cells.
//   MC:  vertices owned by cell rows (j,k) in owner-cell / first-appearance
//        order (marchingCubes/serial/main.cpp:139-177), one thread per vertex,
//        plus the Flying Edges index -> MC index map for the triangle pass.
//
// Values outside the staged planes / rows (gradient neighbours in planes k-1
// and k+2 and rows j0-1, j0+J+1) are read from global memory (L2).
#pragma once
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

constexpr int kSlots = 4;

// Shared-memory layout of k_gen_cols, shared by the kernel and its launcher.
struct GenLayout {
    int J, W, nx;
    size_t slab_floats, off_mbar, off_u32, rw, off_u64, nf, off_f, total;
    __host__ __device__ GenLayout(int J_, int W_, int nx_) : J(J_), W(W_), nx(nx_)
    {
        slab_floats = (((size_t)(J + 1) * nx) + 31) & ~(size_t)31;
        off_mbar = kSlots * slab_floats * 4;
        off_u32 = off_mbar + kSlots * 8;
        rw = (size_t)(J + 1) * W;
        off_u64 = off_u32 + 12 * rw * 4;
        off_u64 = (off_u64 + 7) & ~(size_t)7;
        nf = (size_t)J * 3 * W;
        off_f = off_u64 + 12 * (size_t)(J + 1) * 8;
        total = off_f + nf * 4;
    }
};

// Shared-memory arrays of k_gen_cols.  Double-buffered arrays (one buffer per
// plane parity b) are addressed as base + b * stride, so that no array of
// pointers is indexed at run time.
struct GenShared {
    float* slots;
    uint64_t* mbar;
    uint32_t* u;               // 12 arrays of rw words: bits0 bits1 mx0 mx1 my0 my1 px0 px1 py0 py1 mz pz
    unsigned long long* q;     // 12 arrays of J+1:     xs0 xs1 ys0 ys1 zs0 zs1 ze0 ze1 ts0 ts1 ms0 ms1
    uint32_t* F;
    int rw, n1;
    __device__ __forceinline__ uint32_t* bits(int b) const { return u + b * rw; }
    __device__ __forceinline__ uint32_t* mx(int b) const { return u + (2 + b) * rw; }
    __device__ __forceinline__ uint32_t* my(int b) const { return u + (4 + b) * rw; }
    __device__ __forceinline__ uint32_t* px(int b) const { return u + (6 + b) * rw; }
    __device__ __forceinline__ uint32_t* py(int b) const { return u + (8 + b) * rw; }
    __device__ __forceinline__ uint32_t* mz() const { return u + 10 * rw; }
    __device__ __forceinline__ uint32_t* pz() const { return u + 11 * rw; }
    __device__ __forceinline__ unsigned long long* xs(int b) const { return q + b * n1; }
    __device__ __forceinline__ unsigned long long* ys(int b) const { return q + (2 + b) * n1; }
    __device__ __forceinline__ unsigned long long* zs(int b) const { return q + (4 + b) * n1; }
    __device__ __forceinline__ unsigned long long* ze(int b) const { return q + (6 + b) * n1; }
    __device__ __forceinline__ unsigned long long* ts(int b) const { return q + (8 + b) * n1; }
    __device__ __forceinline__ unsigned long long* ms(int b) const { return q + (10 + b) * n1; }
};

// Value of the volume at (i, j, p) while planes k and k+1 are staged.
struct SlabAccess {
    const float* vol;
    const float* slab_k;
    const float* slab_k1;
    int k, j0, nbr, nx, ny;
    __device__ __forceinline__ float operator()(int i, int j, int p) const
    {
        const int jj = j - j0;
        if (jj >= 0 && jj < nbr) {
            if (p == k) return slab_k[jj * nx + i];
            if (p == k + 1) return slab_k1[jj * nx + i];
        }
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

// Largest idx in [0, n) with F[idx] <= e (F non-decreasing, F[0] == 0).
__device__ __forceinline__ int search_le(const uint32_t* __restrict__ F, int n, uint32_t e)
{
    int lo = 0, hi = n;  // F[lo] <= e, answer in [lo, hi)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (F[mid] <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int G, bool MC, typename IndexT, bool BULK>
__global__ void __launch_bounds__(kThreads) k_gen_cols(
    const float* __restrict__ vol, Grid g, float iso, int KC, int nyb, const CaseTables* __restrict__ cases,
    const uint4* __restrict__ rowcnt, const uint32_t* __restrict__ mccnt, RowStarts rs,
    unsigned long long* __restrict__ totals, long long capV, long long capT, float* __restrict__ points,
    float* __restrict__ normals, IndexT* __restrict__ tris, uint32_t* __restrict__ fe2mc, int reverse)
{
    constexpr int J = kThreads / G;
    extern __shared__ __align__(128) unsigned char s_raw[];
    __shared__ SharedCases s_cases;
    const GenLayout L(J, g.W, g.nx);
    const int W = g.W, RW = (int)L.rw;
    GenShared S;
    S.slots = reinterpret_cast<float*>(s_raw);
    S.mbar = reinterpret_cast<uint64_t*>(s_raw + L.off_mbar);
    S.u = reinterpret_cast<uint32_t*>(s_raw + L.off_u32);
    S.q = reinterpret_cast<unsigned long long*>(s_raw + L.off_u64);
    S.F = reinterpret_cast<uint32_t*>(s_raw + L.off_f);
    S.rw = RW;
    S.n1 = J + 1;
    stage_cases(s_cases, cases, MC);  // includes __syncthreads
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;  // caller grows buffers

    const int nkc = gridDim.x / nyb;
    const int jb = blockIdx.x % nyb;
    const int kc = reverse ? nkc - 1 - (int)(blockIdx.x / nyb) : (int)(blockIdx.x / nyb);
    const int j0 = jb * J, JB = min(J, g.ny - j0), nbr = min(J + 1, g.ny - j0);
    const int kb = kc * KC, ke = min(kb + KC, g.nz);
    const int tid = threadIdx.x, lane = tid & 31, lig = lane & (G - 1);
    const int nchunks = (W + G - 1) / G;
    const int nfl = nbr * g.nx;
    const float invW = 1.0f / (float)W, inv3W = 1.0f / (float)(3 * W);

    if (tid == 0) {
        for (int s = 0; s < kSlots; ++s) mbar_init(&S.mbar[s], BULK ? 1u : (unsigned)kThreads);
        fence_mbar_init();
    }
    __syncthreads();

    // per slot: bit s of `pending` = a copy was issued and not yet waited
    // for; bit s of `parity` = mbarrier phase parity of the next wait
    uint32_t pending = 0, parity = 0;
    bool alive = true;

    auto issue = [&](int p) {
        if (p >= ke + 1 || p >= g.nz) return;  // planes kb .. ke are ever needed
        const int s = p % kSlots;
        float* dst = S.slots + (size_t)s * L.slab_floats;
        const float* src = vol + ((long long)p * g.ny + j0) * g.nx;
        if (BULK) {
            if (tid == 0) {
                fence_proxy_async();
                mbar_arrive_expect_tx(&S.mbar[s], (unsigned)nfl * 4u);
                bulk_copy_g2s(dst, src, (unsigned)nfl * 4u, &S.mbar[s]);
            }
        } else {
            for (int q = tid; q < nfl; q += kThreads) cp_async4(dst + q, src + q);
            cp_async_arrive(&S.mbar[s]);
        }
        pending |= 1u << s;
    };
    auto wait = [&](int p) -> bool {
        const int s = p % kSlots;
        const bool ok = mbar_wait(&S.mbar[s], (parity >> s) & 1u);
        parity ^= 1u << s;
        pending &= ~(1u << s);
        return ok;
    };
    auto drain = [&]() {  // after a timeout: let in-flight copies land (bounded)
        for (int s = 0; s < kSlots; ++s) {
            if ((pending >> s) & 1u) {
                mbar_wait(&S.mbar[s], (parity >> s) & 1u);
                parity ^= 1u << s;
                pending &= ~(1u << s);
            }
        }
    };

    // prepare(p): bits, starts and cut masks of plane p; z masks of plane p-1
    // when with_z.  Ends with __syncthreads.
    auto prepare = [&](int p, bool with_z) {
        const int b = p & 1;
        const float* slab = S.slots + (size_t)(p % kSlots) * L.slab_floats;
        uint32_t* bits = S.bits(b);
        // (a) bit mask from the slab
        if ((g.nx & 3) == 0) classify_block<true, true>(slab, g.nx, W, nbr, iso, bits);
        else classify_block<false, true>(slab, g.nx, W, nbr, iso, bits);
        // (b) first vertex ids of the rows (gridEdge xstart/ystart/zstart)
        if (tid < nbr) {
            const long long r = (long long)p * g.ny + j0 + tid;
            const uint4 c = __ldg(&rowcnt[r]);
            const unsigned long long x0 = rs.get(p, j0 + tid, 0);
            S.xs(b)[tid] = x0;
            S.ys(b)[tid] = x0 + c.x;
            S.zs(b)[tid] = x0 + c.x + c.y;
            S.ze(b)[tid] = x0 + c.x + c.y + c.z;
            if (tid < JB) {
                S.ts(b)[tid] = rs.get(p, j0 + tid, 1);
                if (MC) S.ms(b)[tid] = rs.get(p, j0 + tid, 2);
            }
        }
        __syncthreads();
        // (c) cut masks and their in-row prefixes; G lanes per row
        const uint32_t* prev = S.bits(b ^ 1);
        for (int it = 0; it < 2; ++it) {
            const int jr = tid / G + it * J;
            const bool rv = jr < nbr;
            const bool hasY = rv && jr + 1 < nbr && j0 + jr < g.ny - 1;
            uint32_t cx = 0, cy = 0, cz = 0;
            for (int ch = 0; ch < nchunks; ++ch) {
                const int w = ch * G + lig;
                const bool in = rv && w < W;
                const uint32_t a = in ? bits[jr * W + w] : 0u;
                const uint32_t an = (in && w + 1 < W) ? bits[jr * W + w + 1] : 0u;
                const uint32_t xm = (a ^ ((a >> 1) | (an << 31))) & validmask(w, g.nx - 1);
                const uint32_t ym = (in && hasY) ? ((a ^ bits[(jr + 1) * W + w]) & validmask(w, g.nx)) : 0u;
                const uint32_t zm = (in && with_z) ? ((prev[jr * W + w] ^ a) & validmask(w, g.nx)) : 0u;
                const uint32_t pxm = __popc(xm), pym = __popc(ym), pzm = __popc(zm);
                const uint32_t ix = group_incl_scan<G>(pxm, lig, 0xffffffffu);
                const uint32_t iy = group_incl_scan<G>(pym, lig, 0xffffffffu);
                const uint32_t iz = group_incl_scan<G>(pzm, lig, 0xffffffffu);
                if (in) {
                    S.mx(b)[jr * W + w] = xm;
                    S.px(b)[jr * W + w] = cx + ix - pxm;
                    S.my(b)[jr * W + w] = ym;
                    S.py(b)[jr * W + w] = cy + iy - pym;
                    if (with_z) {
                        S.mz()[jr * W + w] = zm;
                        S.pz()[jr * W + w] = cz + iz - pzm;
                    }
                }
                cx += group_bcast<G>(ix, G - 1, 0xffffffffu);
                cy += group_bcast<G>(iy, G - 1, 0xffffffffu);
                cz += group_bcast<G>(iz, G - 1, 0xffffffffu);
            }
        }
        __syncthreads();
    };

    // ---- prologue
    issue(kb);
    issue(kb + 1);
    issue(kb + 2);
    alive = __syncthreads_and(wait(kb));
    if (!alive) {
        if (tid == 0) totals[3] = kStatusTimeout;
        drain();
        return;
    }
    prepare(kb, false);

    for (int k = kb; k < ke; ++k) {
        const int b0 = k & 1, b1 = b0 ^ 1;
        issue(k + 3);
        const bool has_next = k + 1 < g.nz;
        if (has_next) {
            alive = __syncthreads_and(wait(k + 1));
            if (!alive) break;
            prepare(k + 1, true);
        } else {
            for (int q = tid; q < RW; q += kThreads) { S.mz()[q] = 0u; S.pz()[q] = 0u; }
            __syncthreads();
        }
        const SlabAccess acc{vol, S.slots + (size_t)(k % kSlots) * L.slab_floats,
                             S.slots + (size_t)((k + 1) % kSlots) * L.slab_floats, k, j0, nbr, g.nx, g.ny};
        const bool cells = has_next;  // cell rows exist at plane k

        if (!MC) {
            // ---- vertices of grid rows (j0 .. j0+JB-1, k), one per thread
            const int nF = JB * 3 * W;
            const unsigned long long vbase = S.xs(b0)[0];
            for (int q = tid; q < nF; q += kThreads) {
                const int jj = fastdiv(q, 3 * W, inv3W), rem = q - jj * 3 * W, axis = fastdiv(rem, W, invW),
                          w = rem - axis * W;
                const unsigned long long st = axis == 0 ? S.xs(b0)[jj] : (axis == 1 ? S.ys(b0)[jj] : S.zs(b0)[jj]);
                const uint32_t pre = axis == 0 ? S.px(b0)[jj * W + w] : (axis == 1 ? S.py(b0)[jj * W + w] : S.pz()[jj * W + w]);
                S.F[q] = (uint32_t)(st - vbase) + pre;
            }
            __syncthreads();
            const uint32_t nv = (uint32_t)(S.ze(b0)[JB - 1] - vbase);
            for (uint32_t e = tid; e < nv; e += kThreads) {
                const int idx = search_le(S.F, nF, e);
                const int jj = fastdiv(idx, 3 * W, inv3W), rem = idx - jj * 3 * W, axis = fastdiv(rem, W, invW),
                          w = rem - axis * W;
                const uint32_t m = axis == 0 ? S.mx(b0)[jj * W + w] : (axis == 1 ? S.my(b0)[jj * W + w] : S.mz()[jj * W + w]);
                const int bit = (int)__fns(m, 0, (int)(e - S.F[idx]) + 1);
                const int i = 32 * w + bit, j = j0 + jj;
                float3 p, n;
                edge_vertex_acc(acc, g, iso, axis, i, j, k, axis == 0 ? i : min(i, g.nx - 2),
                                axis == 1 ? j : min(j, g.ny - 2), axis == 2 ? k : min(k, g.nz - 2), p, n);
                store_vertex(points, normals, vbase + e, p, n);
            }
            // ---- triangles of cell rows (j, k), G lanes per row
            if (cells) {
                const int jj = tid / G, j = j0 + jj;
                const bool crow = jj < JB && j < g.ny - 1;
                unsigned long long tcur = crow ? S.ts(b0)[jj] : 0ull;
                for (int ch = 0; ch < nchunks; ++ch) {
                    const int w = ch * G + lig;
                    const bool in = crow && w < W, in1 = crow && w + 1 < W;
                    RowWords rw;
                    const uint32_t* A = S.bits(b0) + jj * W;
                    const uint32_t* Cc = S.bits(b1) + jj * W;
                    rw.a = in ? A[w] : 0u;
                    rw.b = in ? A[W + w] : 0u;
                    rw.c = in ? Cc[w] : 0u;
                    rw.d = in ? Cc[W + w] : 0u;
                    rw.ash = (rw.a >> 1) | ((in1 ? A[w + 1] : 0u) << 31);
                    rw.bsh = (rw.b >> 1) | ((in1 ? A[W + w + 1] : 0u) << 31);
                    rw.csh = (rw.c >> 1) | ((in1 ? Cc[w + 1] : 0u) << 31);
                    rw.dsh = (rw.d >> 1) | ((in1 ? Cc[W + w + 1] : 0u) << 31);
                    const uint32_t act = in ? active_cells(rw, validmask(w, g.nx - 1)) : 0u;
                    uint32_t nt = 0;
                    for (uint32_t a = act; a; a &= a - 1) nt += iso_case_ntris(s_cases.tris[cube_case(rw, __ffs(a) - 1)]);
                    const uint32_t inc = group_incl_scan<G>(nt, lig, 0xffffffffu);
                    if (act) {
                        const int o = jj * W + w;
                        CutMasks m;
                        m.xA = S.mx(b0)[o]; m.xB = S.mx(b0)[o + W]; m.xC = S.mx(b1)[o]; m.xD = S.mx(b1)[o + W];
                        m.yA = S.my(b0)[o]; m.yC = S.my(b1)[o]; m.zA = S.mz()[o]; m.zB = S.mz()[o + W];
                        CutBases cb;
                        cb.xA = S.xs(b0)[jj] + S.px(b0)[o];
                        cb.xB = S.xs(b0)[jj + 1] + S.px(b0)[o + W];
                        cb.xC = S.xs(b1)[jj] + S.px(b1)[o];
                        cb.xD = S.xs(b1)[jj + 1] + S.px(b1)[o + W];
                        cb.yA = S.ys(b0)[jj] + S.py(b0)[o];
                        cb.yC = S.ys(b1)[jj] + S.py(b1)[o];
                        cb.zA = S.zs(b0)[jj] + S.pz()[o];
                        cb.zB = S.zs(b0)[jj + 1] + S.pz()[o + W];
                        unsigned long long t = tcur + (inc - nt);
                        for (uint32_t a = act; a; a &= a - 1) {
                            const int bit = __ffs(a) - 1;
                            const uint64_t tl = s_cases.tris[cube_case(rw, bit)];
                            const int ntc = iso_case_ntris(tl);
                            for (int q = 0; q < 3 * ntc; ++q)
                                tris[3 * t + q] = (IndexT)fe_edge_id(m, cb, iso_case_edge(tl, q), bit);
                            t += ntc;
                        }
                    }
                    tcur += group_bcast<G>(inc, G - 1, 0xffffffffu);
                }
            }
        } else if (cells) {
            // ---- MC vertices owned by cell rows (j, k), in owner order
            const int jj = tid / G, j = j0 + jj;
            const bool crow = jj < JB && j < g.ny - 1;
            uint32_t cm = 0;
            for (int ch = 0; ch < nchunks; ++ch) {  // owned counts per word -> F
                const int w = ch * G + lig;
                const bool in = crow && w < W, in1 = crow && w + 1 < W;
                const uint32_t* A = S.bits(b0) + jj * W;
                const uint32_t* Cc = S.bits(b1) + jj * W;
                RowWords rw;
                rw.a = in ? A[w] : 0u; rw.b = in ? A[W + w] : 0u; rw.c = in ? Cc[w] : 0u; rw.d = in ? Cc[W + w] : 0u;
                rw.ash = (rw.a >> 1) | ((in1 ? A[w + 1] : 0u) << 31);
                rw.bsh = (rw.b >> 1) | ((in1 ? A[W + w + 1] : 0u) << 31);
                rw.csh = (rw.c >> 1) | ((in1 ? Cc[w + 1] : 0u) << 31);
                rw.dsh = (rw.d >> 1) | ((in1 ? Cc[W + w + 1] : 0u) << 31);
                const uint32_t act = in ? active_cells(rw, validmask(w, g.nx - 1)) : 0u;
                uint32_t no = 0;
                for (uint32_t a = act; a; a &= a - 1) {
                    const int bit = __ffs(a) - 1;
                    no += __popc(mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cases.cut[cube_case(rw, bit)]);
                }
                const uint32_t inc = group_incl_scan<G>(no, lig, 0xffffffffu);
                if (in) S.F[jj * W + w] = (crow ? (uint32_t)(S.ms(b0)[jj] - S.ms(b0)[0]) : 0u) + cm + inc - no;
                cm += group_bcast<G>(inc, G - 1, 0xffffffffu);
            }
            // rows past the last cell row: pad F so the search never lands there
            const int ncr = min(JB, g.ny - 1 - j0);  // cell rows in the block
            __syncthreads();
            const unsigned long long mbase = S.ms(b0)[0];
            const uint32_t nv = ncr > 0 ? (uint32_t)(rs.get(k, j0 + ncr - 1, 2) +
                                                     __ldg(&mccnt[(long long)k * g.ny + j0 + ncr - 1]) - mbase)
                                        : 0u;
            const int nF = ncr * W;
            for (uint32_t e = tid; e < nv; e += kThreads) {
                const int idx = search_le(S.F, nF, e);
                const int jr = fastdiv(idx, W, invW), w = idx - jr * W, jrow = j0 + jr;
                uint32_t rank = e - S.F[idx];
                const uint32_t* A = S.bits(b0) + jr * W;
                const uint32_t* Cc = S.bits(b1) + jr * W;
                const bool in1 = w + 1 < W;
                RowWords rw;
                rw.a = A[w]; rw.b = A[W + w]; rw.c = Cc[w]; rw.d = Cc[W + w];
                rw.ash = (rw.a >> 1) | ((in1 ? A[w + 1] : 0u) << 31);
                rw.bsh = (rw.b >> 1) | ((in1 ? A[W + w + 1] : 0u) << 31);
                rw.csh = (rw.c >> 1) | ((in1 ? Cc[w + 1] : 0u) << 31);
                rw.dsh = (rw.d >> 1) | ((in1 ? Cc[W + w + 1] : 0u) << 31);
                uint32_t act = active_cells(rw, validmask(w, g.nx - 1));
                int bit = 0, c = 0;
                uint32_t own = 0;
                while (act) {  // the cell holding this vertex
                    bit = __ffs(act) - 1;
                    act &= act - 1;
                    c = cube_case(rw, bit);
                    own = mc_owned_edges(32 * w + bit == 0, jrow == 0, k == 0) & s_cases.cut[c];
                    const uint32_t n = __popc(own);
                    if (rank < n) break;
                    rank -= n;
                }
                const uint64_t ord = s_cases.order[c];
                int e12 = 0;
                for (int q = 0; q < iso_case_ntris(ord); ++q) {  // rank-th owned edge, first-appearance order
                    const int ed = iso_case_edge(ord, q);
                    if ((own >> ed) & 1u) {
                        if (rank == 0) { e12 = ed; break; }
                        --rank;
                    }
                }
                int dx, dy, dz, axis;
                cube_edge_geometry(e12, dx, dy, dz, axis);
                const int i = 32 * w + bit;
                float3 p, n;
                edge_vertex_acc(acc, g, iso, axis, i + dx, jrow + dy, k + dz, i, jrow, k, p, n);
                const unsigned long long id = mbase + e;
                store_vertex(points, normals, id, p, n);
                const int o = jr * W + w;
                CutMasks m;
                m.xA = S.mx(b0)[o]; m.xB = S.mx(b0)[o + W]; m.xC = S.mx(b1)[o]; m.xD = S.mx(b1)[o + W];
                m.yA = S.my(b0)[o]; m.yC = S.my(b1)[o]; m.zA = S.mz()[o]; m.zB = S.mz()[o + W];
                CutBases cb;
                cb.xA = S.xs(b0)[jr] + S.px(b0)[o];
                cb.xB = S.xs(b0)[jr + 1] + S.px(b0)[o + W];
                cb.xC = S.xs(b1)[jr] + S.px(b1)[o];
                cb.xD = S.xs(b1)[jr + 1] + S.px(b1)[o + W];
                cb.yA = S.ys(b0)[jr] + S.py(b0)[o];
                cb.yC = S.ys(b1)[jr] + S.py(b1)[o];
                cb.zA = S.zs(b0)[jr] + S.pz()[o];
                cb.zB = S.zs(b0)[jr + 1] + S.pz()[o + W];
                fe2mc[fe_edge_id(m, cb, e12, bit)] = (uint32_t)id;
            }
        }
        __syncthreads();  // planes k's slot and the b0 buffers are reused next step
    }
    if (!alive) {
        if (tid == 0) totals[3] = kStatusTimeout;
    }
    drain();
}

template <bool MC, typename IndexT>
void launch_gen_cols_impl(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                          const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                          float* normals, IndexT* tris, int reverse, cudaStream_t s)
{
    const RowStarts rs = row_starts(g, cp, b);
    const bool bulk = (g.nx % 4 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
    const unsigned blocks = (unsigned)(p.nyb * p.nkc);
#define ISO_GEN_LAUNCH(GG)                                                                                       \
    {                                                                                                            \
        auto kern = bulk ? k_gen_cols<GG, MC, IndexT, true> : k_gen_cols<GG, MC, IndexT, false>;                \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);                   \
        kern<<<blocks, kThreads, p.smem, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt, b.mccnt, rs, b.totals,   \
                                              capV, capT, points, normals, tris, b.fe2mc, reverse);              \
    }
    switch (p.G) {
        case 4: ISO_GEN_LAUNCH(4) break;
        case 8: ISO_GEN_LAUNCH(8) break;
        case 16: ISO_GEN_LAUNCH(16) break;
        default: ISO_GEN_LAUNCH(32) break;
    }
#undef ISO_GEN_LAUNCH
}

}  // namespace iso
