// Passes 1-3 of Flying Edges (flyingEdges/serial/FlyingEdgesAlgorithm.cpp:23-269)
// on sm_103a, with pass 1 (x-edge classification, trims) fused into pass 2
// (cube cases, per-row counts):
//
//   k_count_tma    (rows up to 1024 points, 16-byte aligned) a CTA owns a block
//   k_count_warps  (up to 2048) of 16 or 32 grid rows (k_count_tma: a half- or
//                  quarter-warp per row) / 8 rows (k_count_warps: a warp per row) and a run of
//                  KC planes and marches along z.  Each row's words of plane
//                  k+1 are classified straight from the volume (plane k+2
//                  already in flight: a TMA bulk copy into the warp's shared
//                  buffer, or float4 loads into registers) into bit-per-point
//                  words held one per lane -- the reference's edgeCases bytes
//                  are never materialised -- and counted for grid row (j,k): its cut
//                  x, y and z edges (the vertices it owns), the trims xl/xr,
//                  the triangles of cell row (j,k) and, for Marching Cubes,
//                  the vertices cell row (j,k) owns, all 32 cells of a word at
//                  once (tris_of_word, mc_verts_of_word).  Writes the bit
//                  words for pass 4.  No warp waits for another.
//   k_count_wide   rows longer than 2048 points, walked in chunks.
//   k_scan_*       exclusive scans of the per-row counts in (k, j) order, the
//                  reference's row order: the first vertex / triangle / MC
//                  vertex of every row (gridEdge xstart and triCounter after
//                  pass 3) and the totals.
#include "batch_kernels.cuh"
#include "count_words.cuh"
#include "iso_kernels.h"

namespace iso {


// Raw values of one row held by a warp: lane l holds float4 l + 32u.
template <int U>
struct RowVals {
    float4 v[U];
};

template <int U>
__device__ __forceinline__ void load_row_vec4(const float* __restrict__ row, int nq, int lane, bool ok, RowVals<U>& r)
{
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int q = lane + 32 * u;
        r.v[u] = (ok && q < nq) ? __ldg(reinterpret_cast<const float4*>(row) + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Bit words "value >= iso" of a row: word w ends up in lane w % 32, slot w / 32.
template <int U, int NW>
__device__ __forceinline__ void words_vec4(const RowVals<U>& r, int nq, int lane, float iso, uint32_t (&out)[NW])
{
#pragma unroll
    for (int q = 0; q < NW; ++q) out[q] = 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int f = lane + 32 * u;
        const float4 v = r.v[u];
        const uint32_t nib = f < nq ? ((uint32_t)(v.x >= iso) | ((uint32_t)(v.y >= iso) << 1) |
                                       ((uint32_t)(v.z >= iso) << 2) | ((uint32_t)(v.w >= iso) << 3))
                                    : 0u;
        uint32_t word = nib << (4 * (lane & 7));
        word |= __shfl_xor_sync(0xffffffffu, word, 1);
        word |= __shfl_xor_sync(0xffffffffu, word, 2);
        word |= __shfl_xor_sync(0xffffffffu, word, 4);
        // lanes 8g..8g+7 now hold word 4u+g; lane L wants word L + 32q
        const uint32_t x = __shfl_sync(0xffffffffu, word, 8 * (lane & 3));
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            if (u == (lane >> 2) + 8 * q) out[q] = x;
        }
    }
}

template <int NW>
__device__ __forceinline__ void words_scalar(const float* __restrict__ row, int nx, int W, bool ok, int lane, float iso,
                                             uint32_t (&out)[NW])
{
#pragma unroll
    for (int q = 0; q < NW; ++q) out[q] = 0u;
    for (int w = 0; w < W; ++w) {
        const int i = 32 * w + lane;
        const float v = (ok && i < nx) ? __ldg(row + i) : 0.f;
        const uint32_t m = __ballot_sync(0xffffffffu, ok && i < nx && v >= iso);
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            if (w == lane + 32 * q) out[q] = m;
        }
    }
}

// Next word (the source of bit i+1) of the lane's slot q.
template <int NW>
__device__ __forceinline__ uint32_t next_word(const uint32_t (&w)[NW], int q, int lane)
{
    const uint32_t dn = __shfl_down_sync(0xffffffffu, w[q], 1);
    const uint32_t wrap = __shfl_sync(0xffffffffu, w[q + 1 < NW ? q + 1 : q], 0);
    if (lane < 31) return dn;
    return q + 1 < NW ? wrap : 0u;
}

// Warp totals of row r; lane 0 stores them.
template <bool MC>
__device__ __forceinline__ void finish_row(RowCounts& rc, int lane, long long r, const Grid& g,
                                           uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                           uint32_t* __restrict__ mccnt)
{
    rc.xc = __reduce_add_sync(0xffffffffu, rc.xc);
    rc.yc = __reduce_add_sync(0xffffffffu, rc.yc);
    rc.zc = __reduce_add_sync(0xffffffffu, rc.zc);
    rc.tc = __reduce_add_sync(0xffffffffu, rc.tc);
    if (MC) rc.mc = __reduce_add_sync(0xffffffffu, rc.mc);
    if (trims) {
        rc.first = __reduce_min_sync(0xffffffffu, rc.first);
        rc.last = __reduce_max_sync(0xffffffffu, rc.last);
    }
    if (lane == 0) {
        rowcnt[r] = make_uint4(rc.xc, rc.yc, rc.zc, rc.tc);
        if (trims) trims[r] = make_uint2(rc.first == 0xffffffffu ? (uint32_t)g.nx : rc.first, rc.last);
        if (MC) mccnt[r] = rc.mc;
    }
}

template <bool MC, bool VEC4, int U, int NW>
__global__ void __launch_bounds__(kThreads) k_count_warps(const float* __restrict__ vol, Grid g, float iso, int KC,
                                                          int nyb, const CaseTables* __restrict__ cases,
                                                          uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                                          uint32_t* __restrict__ mccnt, uint32_t* __restrict__ bits_out)
{
    (void)cases;  // the counts need no case table (tris_of_word, mc_verts_of_word)
    const int jb = blockIdx.x % nyb, kc = blockIdx.x / nyb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = jb * kCountRows + warp;
    if (j >= g.ny) return;
    const int kb = g.kr + kc * KC, ke = min(kb + KC, g.ke);
    const bool hasY = j < g.ny - 1;
    const int jy = hasY ? j + 1 : j;  // row B (a valid address even when B does not exist)
    const int nq = g.nx >> 2;
    auto rowptr = [&](int k, int jj) { return vol + ((long long)(k - g.kd) * g.ny + jj) * g.nx; };

    // words of rows A = (j,k), B = (j+1,k); Cw, Dw = the same rows at plane k+1
    uint32_t A[NW], B[NW], Cw[NW], Dw[NW];
    RowVals<U> pc, pd;  // raw values of plane k+1 (VEC4), loaded one step ahead
    if (VEC4) {
        RowVals<U> ra, rbv;
        load_row_vec4<U>(rowptr(kb, j), nq, lane, true, ra);
        load_row_vec4<U>(rowptr(kb, jy), nq, lane, hasY, rbv);
        if (kb + 1 < g.nz) {
            load_row_vec4<U>(rowptr(kb + 1, j), nq, lane, true, pc);
            load_row_vec4<U>(rowptr(kb + 1, jy), nq, lane, hasY, pd);
        }
        words_vec4<U, NW>(ra, nq, lane, iso, A);
        words_vec4<U, NW>(rbv, nq, lane, iso, B);
    } else {
        words_scalar<NW>(rowptr(kb, j), g.nx, g.W, true, lane, iso, A);
        words_scalar<NW>(rowptr(kb, jy), g.nx, g.W, hasY, lane, iso, B);
    }
    for (int k = kb; k < ke; ++k) {
        const bool hasZ = k + 1 < g.nz;
        if (VEC4) {
            words_vec4<U, NW>(pc, nq, lane, iso, Cw);
            words_vec4<U, NW>(pd, nq, lane, iso, Dw);
            if (k + 2 < g.nz && k + 1 < ke) {  // plane k+2 for the next step
                load_row_vec4<U>(rowptr(k + 2, j), nq, lane, true, pc);
                load_row_vec4<U>(rowptr(k + 2, jy), nq, lane, hasY, pd);
            }
        } else if (hasZ) {
            words_scalar<NW>(rowptr(k + 1, j), g.nx, g.W, true, lane, iso, Cw);
            words_scalar<NW>(rowptr(k + 1, jy), g.nx, g.W, hasY, lane, iso, Dw);
        }
        if (!hasZ) {
#pragma unroll
            for (int q = 0; q < NW; ++q) Cw[q] = Dw[q] = 0u;
        }
        RowCounts rc;
        const long long r = (long long)(k - g.kr) * g.ny + j;
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const int w = lane + 32 * q;
            RowWords rw;
            rw.a = A[q];
            rw.b = B[q];
            rw.c = Cw[q];
            rw.d = Dw[q];
            rw.ash = (rw.a >> 1) | (next_word<NW>(A, q, lane) << 31);
            rw.bsh = (rw.b >> 1) | (next_word<NW>(B, q, lane) << 31);
            rw.csh = (rw.c >> 1) | (next_word<NW>(Cw, q, lane) << 31);
            rw.dsh = (rw.d >> 1) | (next_word<NW>(Dw, q, lane) << 31);
            count_word<MC>(rw, w, g, j, k, hasY, hasZ, trims != nullptr, rc);
            if (w < g.W) bits_out[r * g.W + w] = rw.a;
        }
        finish_row<MC>(rc, lane, r, g, rowcnt, trims, mccnt);
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            A[q] = Cw[q];
            B[q] = Dw[q];
        }
    }
}

// Word wd of a row that starts o floats into a 16-byte aligned buffer and is
// npts points long, for rows at any offset: the 8 float4 from the one that
// holds the word's first point (rotated over the lanes as in row_word), the 4
// points after them from the next lane's word of the same row (lane wd + 1
// builds its own first float4 from them) or, for the last lane of the row's
// group (last), by one more load; the 36 bits shifted down by o & 3.  Every
// lane of the warp calls it (the shuffle); only float4 that hold points of the
// row are read.
__device__ __forceinline__ uint32_t row_word_shift(const float* buf, int o, int npts, int wd, int rot, bool last,
                                                   float iso)
{
    const int base = o + 32 * wd, b4 = base >> 2, sh = base & 3;
    const int nvq = ((o + npts + 3) >> 2) - b4;  // float4 from b4 on that hold points of the row
    const float4* r4 = reinterpret_cast<const float4*>(buf) + b4;
    uint32_t w = 0u;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int q = (u + rot) & 7;
        if (q < nvq) {
            const float4 v = r4[q];
            w |= ge_mask(v.x, iso) & (1u << (4 * u));
            w |= ge_mask(v.y, iso) & (2u << (4 * u));
            w |= ge_mask(v.z, iso) & (4u << (4 * u));
            w |= ge_mask(v.w, iso) & (8u << (4 * u));
        }
    }
    w = __funnelshift_l(w, w, 4 * rot);
    uint32_t hi = __shfl_down_sync(0xffffffffu, w, 1);
    if (last) {
        hi = 0u;
        if (nvq > 8) {
            const float4 v = r4[8];
            hi = (ge_mask(v.x, iso) & 1u) | (ge_mask(v.y, iso) & 2u) | (ge_mask(v.z, iso) & 4u) |
                 (ge_mask(v.w, iso) & 8u);
        }
    }
    const uint32_t r = __funnelshift_r(w, hi, sh);
    const int nv = npts - 32 * wd;  // points of the word inside the row
    return nv >= 32 ? r : (nv > 0 ? r & ((1u << nv) - 1u) : 0u);
}

// Floats of a warp's buffer in k_count_tma: RPW + 1 rows (plus up to 3 points
// of lead-in and padding to 16 bytes when the rows are not 16-byte aligned).
__host__ __device__ inline int count_buffer_floats(int nx, int rpw, bool aligned)
{
    return aligned ? (rpw + 1) * nx : (((rpw + 1) * nx + 3) + 3) & ~3;
}

// Rows of up to 32 words (nx <= 1024), several per warp up to 16 words so
// that no lane idles on words past a short row: the counts of k_count_warps,
// with the volume brought in by the TMA bulk engine.  A warp's grid rows
// jw .. jw+RPW-1 read rows jw .. jw+RPW of every plane (A and B of each
// row's lanes), which lie next to each other in memory: one cp.async.bulk per
// plane fills the warp's buffer and completes on the warp's mbarrier.  The
// words of plane k+1 are taken from the buffer before the copy of plane k+2
// is issued into it, so the copy runs while step k is counted; no register
// holds raw values across a step.  Rows whose length is not a multiple of 4
// points (ALIGNED false; the volume itself 16-byte aligned): the copy runs
// from the rows' first point rounded down to 16 bytes to their last rounded
// down, the last few points come by plain loads, and row_word_shift builds
// the words at the rows' offsets in the buffer.
// RPW grid rows per warp (1: rows of 17-32 words, 2: up to 16, 4: up to 8, 8: up to 4), LPR =
// 32 / RPW lanes per row; a warp's rows jw .. jw+RPW-1 read rows jw .. jw+RPW
// of every plane, RPW + 1 rows of its buffer.  FULL: every lane's word is
// inside the row (nx = 32 * LPR).

// Block blk of the grid: row block blk % nyb, plane column blk / nyb.
template <bool MC, bool FULL, int RPW, bool ALIGNED>
__device__ __forceinline__ void count_tma_block(const float* __restrict__ vol, const Grid& g, float iso, int KC,
                                                int nyb, int blk, uint4* __restrict__ rowcnt,
                                                uint2* __restrict__ trims, uint32_t* __restrict__ mccnt,
                                                uint32_t* __restrict__ bits_out,
                                                unsigned long long* __restrict__ status)
{
    constexpr int LPR = 32 / RPW, NBUF = RPW + 1;
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ uint64_t s_bar[kCountRows];
    const int jb = blk % nyb, kc = blk / nyb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, h = lane / LPR, lw = lane % LPR;
    const int jw = jb * kCountRows * RPW + RPW * warp;
    if (jw >= g.ny) return;  // all the warp's rows past the grid
    float* buf = reinterpret_cast<float*>(s_raw) + (size_t)warp * count_buffer_floats(g.nx, RPW, ALIGNED);
    uint64_t* bar = &s_bar[warp];
    if (lane == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncwarp();
    const int j = jw + h;
    const bool row_ok = j < g.ny;
    const int kb = g.kr + kc * KC, ke = min(kb + KC, g.ke);
    if (kb >= ke) {  // a block past the grid's last plane column: nothing to copy (no launch makes one today)
        return;
    }
    const bool hasY = row_ok && j < g.ny - 1;
    const int nq = g.nx >> 2;
    const int nrows = min(NBUF, g.ny - jw);
    const unsigned bytes = (unsigned)(nrows * g.nx * 4);
    int lead = 0;      // points of the buffer before the warp's first row (ALIGNED false)
    int tail_at = -1;  // this lane's place in the buffer for one of the rows' last points, or -1
    float tail_v = 0.f;

    // plane p -> buffer (lane 0 issues the copy); earlier reads of the buffer
    // are ordered before the engine's writes by the caller's __syncwarp and
    // the fence
    auto issue = [&](int p) {
        const long long s0 = ((long long)(p - g.kd) * g.ny + jw) * g.nx;
        if (ALIGNED) {
            if (lane == 0) {
                fence_proxy_async();
                mbar_arrive_expect_tx(bar, bytes);
                bulk_copy_g2s(buf, vol + s0, bytes, bar);
            }
        } else {  // [a0, e0) by the engine, [max(e0, s0), e) by plain loads; all inside the volume
            const long long a0 = s0 & ~3ll, e = s0 + (long long)nrows * g.nx, e0 = e & ~3ll;
            const unsigned nb = e0 > a0 ? (unsigned)((e0 - a0) * 4) : 0u;
            lead = (int)(s0 - a0);
            if (lane == 0) {
                fence_proxy_async();
                mbar_arrive_expect_tx(bar, nb);
                if (nb) bulk_copy_g2s(buf, vol + a0, nb, bar);
            }
            // loaded now, stored by take(): the warp does not wait here for the load
            const long long lo = e0 > s0 ? e0 : s0;
            tail_at = lane < (int)(e - lo) ? (int)(lo - a0) + lane : -1;
            if (tail_at >= 0) tail_v = __ldg(vol + lo + lane);
        }
    };
    unsigned phase = 0;
    // words of rows A = buffer row h and B = buffer row h+1 of the plane in the buffer
    auto take = [&](uint32_t& wa, uint32_t& wb) -> bool {
        if (!ALIGNED && tail_at >= 0) buf[tail_at] = tail_v;
        __syncwarp();  // the plain loads of the buffer's last points are visible
        const bool done = mbar_wait(bar, phase);
        if (!__all_sync(0xffffffffu, done)) return false;
        phase ^= 1u;
        if (ALIGNED) {
            wa = row_ok ? row_word<FULL>(buf + h * g.nx, nq, lw, lane & 7, iso) : 0u;
            wb = hasY ? row_word<FULL>(buf + (h + 1) * g.nx, nq, lw, lane & 7, iso) : 0u;
        } else {
            // every lane builds both words (the shuffles); rows past the grid read stale buffer rows
            wa = row_word_shift(buf, lead + h * g.nx, g.nx, lw, lane & 7, lw == LPR - 1, iso);
            wb = row_word_shift(buf, lead + (h + 1) * g.nx, g.nx, lw, lane & 7, lw == LPR - 1, iso);
            wa = row_ok ? wa : 0u;
            wb = hasY ? wb : 0u;
            // the plain stores of the last points (lanes 0-2) may lie where the next copies write:
            // each writer orders them before the async proxy, not only the lane that issues the copy
            fence_proxy_async();
        }
        __syncwarp();  // every lane has read the buffer before it is refilled
        return true;
    };
    // per-row totals: rows 2p, 2p+1 of the warp in the two 16-bit halves of reduction p (one row per warp:
    // the warp's sum)
    auto row_sum = [&](uint32_t v) -> uint32_t {
        if (RPW == 1) return __reduce_add_sync(0xffffffffu, v);
        const int sh = 16 * (h & 1);
        uint32_t mine = 0u;
#pragma unroll
        for (int p = 0; p < RPW / 2; ++p) {
            const uint32_t s = __reduce_add_sync(0xffffffffu, (h >> 1) == p ? v << sh : 0u);
            if ((h >> 1) == p) mine = s;
        }
        return (mine >> sh) & 0xffffu;
    };

    uint32_t A = 0, B = 0, Cw = 0, Dw = 0;
    bool ok = true;
    issue(kb);
    ok = take(A, B);
    if (ok && kb + 1 < g.nz) issue(kb + 1);
    for (int k = kb; ok && k < ke; ++k) {
        const bool hasZ = k + 1 < g.nz;
        Cw = Dw = 0u;
        if (hasZ) {  // plane k+1 was issued one step earlier
            if (!(ok = take(Cw, Dw))) break;
            if (k + 2 < g.nz && k + 1 < ke) issue(k + 2);
        }
        RowCounts rc;
        RowWords rw;
        rw.a = A;
        rw.b = B;
        rw.c = Cw;
        rw.d = Dw;
        const uint32_t an = __shfl_down_sync(0xffffffffu, rw.a, 1, LPR);
        const uint32_t bn = __shfl_down_sync(0xffffffffu, rw.b, 1, LPR);
        const uint32_t cn = __shfl_down_sync(0xffffffffu, rw.c, 1, LPR);
        const uint32_t dn = __shfl_down_sync(0xffffffffu, rw.d, 1, LPR);
        const bool nxt = lw < LPR - 1;
        rw.ash = (rw.a >> 1) | ((nxt ? an : 0u) << 31);
        rw.bsh = (rw.b >> 1) | ((nxt ? bn : 0u) << 31);
        rw.csh = (rw.c >> 1) | ((nxt ? cn : 0u) << 31);
        rw.dsh = (rw.d >> 1) | ((nxt ? dn : 0u) << 31);
        if (row_ok) count_word<MC>(rw, lw, g, j, k, hasY, hasZ, trims != nullptr, rc);
        const long long r = (long long)(k - g.kr) * g.ny + j;
        if (row_ok && lw < g.W) bits_out[r * g.W + lw] = rw.a;
        const uint32_t sx = row_sum(rc.xc), sy = row_sum(rc.yc), sz = row_sum(rc.zc), st = row_sum(rc.tc);
        const uint32_t sm = MC ? row_sum(rc.mc) : 0u;
        uint32_t first = 0u, last = 0u;
        if (trims) {  // each row's own minimum and maximum, the other rows contributing the identity
#pragma unroll
            for (int q = 0; q < RPW; ++q) {
                const uint32_t f = __reduce_min_sync(0xffffffffu, h == q ? rc.first : 0xffffffffu);
                const uint32_t x = __reduce_max_sync(0xffffffffu, h == q ? rc.last : 0u);
                if (h == q) {
                    first = f;
                    last = x;
                }
            }
        }
        if (row_ok && lw == 0) {
            rowcnt[r] = make_uint4(sx, sy, sz, st);
            if (trims) trims[r] = make_uint2(first == 0xffffffffu ? (uint32_t)g.nx : first, last);
            if (MC) mccnt[r] = sm;
        }
        A = Cw;
        B = Dw;
    }
    if (!ok) {  // a copy did not complete in time: report it, and let the copy land before the CTA ends
        if (lane == 0) atomicOr(status, kStatusTimeout);
        mbar_wait(bar, phase);
    }
}

template <bool MC, bool FULL, int RPW, bool ALIGNED>
__global__ void __launch_bounds__(kThreads, 4) k_count_tma(const float* __restrict__ vol, Grid g, float iso, int KC,
                                                        int nyb, uint4* __restrict__ rowcnt,
                                                        uint2* __restrict__ trims, uint32_t* __restrict__ mccnt,
                                                        uint32_t* __restrict__ bits_out,
                                                        unsigned long long* __restrict__ status)
{
    count_tma_block<MC, FULL, RPW, ALIGNED>(vol, g, iso, KC, nyb, (int)blockIdx.x, rowcnt, trims, mccnt, bits_out,
                                            status);
}

// The Flying Edges count blocks of a list of requests (batch_kernels.cuh), one launch.
template <bool FULL, int RPW, bool ALIGNED>
__global__ void __launch_bounds__(kThreads, 4) k_count_tma_batch(const BatchReq* __restrict__ reqs,
                                                              const int* __restrict__ list,
                                                              const unsigned* __restrict__ first, int m)
{
    const int q = batch_find(first, m, blockIdx.x);
    const BatchReq* d = reqs + __ldg(&list[q]);
    const Grid g = d->g;
    count_tma_block<false, FULL, RPW, ALIGNED>(d->vol, g, d->iso, d->count_KC, d->count_nyb,
                                               (int)(blockIdx.x - __ldg(&first[q])), d->rowcnt, nullptr, nullptr,
                                               d->bits, d->totals + 3);
}

// Word c*32 + lane of a row and, uniform over the warp, word c*32 + 32 (the
// source of lane 31's bit 32): 33 coalesced 128-byte loads.
__device__ __forceinline__ void chunk_words(const float* __restrict__ row, bool ok, int c, int nx, int lane, float iso,
                                            uint32_t& word, uint32_t& next)
{
    word = 0u;
    for (int t = 0; t <= 32; ++t) {
        const long long i = 32ll * (32 * c + t) + lane;
        const bool in = ok && i < nx;
        const uint32_t m = __ballot_sync(0xffffffffu, in && __ldg(row + i) >= iso);
        if (t == lane) word = m;
        next = m;
    }
}

// Rows longer than 64 words (nx > 2048): the same counts as k_count_warps,
// the row walked in chunks of 32 words, the four rows of a step re-read from
// the volume for every plane (twice the reads of the narrow kernel).
template <bool MC>
__global__ void __launch_bounds__(kThreads) k_count_wide(const float* __restrict__ vol, Grid g, float iso, int KC,
                                                         int nyb, const CaseTables* __restrict__ cases,
                                                         uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                                         uint32_t* __restrict__ mccnt, uint32_t* __restrict__ bits_out)
{
    (void)cases;  // the counts need no case table (tris_of_word, mc_verts_of_word)
    const int jb = blockIdx.x % nyb, kc = blockIdx.x / nyb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = jb * kCountRows + warp;
    if (j >= g.ny) return;
    const int kb = g.kr + kc * KC, ke = min(kb + KC, g.ke);
    const bool hasY = j < g.ny - 1;
    const int jy = hasY ? j + 1 : j;
    const int nchunks = (g.W + 31) / 32;
    auto rowptr = [&](int k, int jj) { return vol + ((long long)(k - g.kd) * g.ny + jj) * g.nx; };
    for (int k = kb; k < ke; ++k) {
        const bool hasZ = k + 1 < g.nz;
        const int kz = hasZ ? k + 1 : k;
        RowCounts rc;
        const long long r = (long long)(k - g.kr) * g.ny + j;
        for (int c = 0; c < nchunks; ++c) {
            RowWords rw;
            uint32_t na, nb, nc, nd;
            chunk_words(rowptr(k, j), true, c, g.nx, lane, iso, rw.a, na);
            chunk_words(rowptr(k, jy), hasY, c, g.nx, lane, iso, rw.b, nb);
            chunk_words(rowptr(kz, j), hasZ, c, g.nx, lane, iso, rw.c, nc);
            chunk_words(rowptr(kz, jy), hasY && hasZ, c, g.nx, lane, iso, rw.d, nd);
            const uint32_t da = __shfl_down_sync(0xffffffffu, rw.a, 1), db = __shfl_down_sync(0xffffffffu, rw.b, 1);
            const uint32_t dc = __shfl_down_sync(0xffffffffu, rw.c, 1), dd = __shfl_down_sync(0xffffffffu, rw.d, 1);
            rw.ash = (rw.a >> 1) | ((lane < 31 ? da : na) << 31);
            rw.bsh = (rw.b >> 1) | ((lane < 31 ? db : nb) << 31);
            rw.csh = (rw.c >> 1) | ((lane < 31 ? dc : nc) << 31);
            rw.dsh = (rw.d >> 1) | ((lane < 31 ? dd : nd) << 31);
            const int w = 32 * c + lane;
            count_word<MC>(rw, w, g, j, k, hasY, hasZ, trims != nullptr, rc);
            if (w < g.W) bits_out[r * g.W + w] = rw.a;
        }
        finish_row<MC>(rc, lane, r, g, rowcnt, trims, mccnt);
    }
}

// ---------------------------------------------------------------------------
// Exclusive scans of the per-row counts (vertices = x+y+z cuts, triangles,
// MC vertices) over the R = ny*nz rows, in two launches over segments of
// kSeg rows (256 threads x 4):
//   k_scan_partial  one CTA per segment: segment totals
//   k_scan_final    one CTA per segment: offset of the segment + scan inside
//                   it -> starts[3][R]; grand totals.
// ---------------------------------------------------------------------------
constexpr int kScanPer = 4;  // 4 rather than 8 rows per thread: twice the CTAs, 15.2 -> 12.9 us at 512^3
constexpr int kSeg = kThreads * kScanPer;

// Scan modes: the components scanned per row.
//   kScanFE   0: vertices (x+y+z cuts)  1: triangles
//   kScanMC   0: vertices  1: triangles  2: MC vertices
//   kScanDup  0: x cuts  1: triangles  2: y cuts  3: z cuts (the blocks of the
//             global-edge-index order; totals[4], totals[5] = all x, all y cuts)
template <int SM>
struct ScanComps {
    static constexpr int n = SM == kScanDup ? 4 : 3;
};

template <int SM>
__device__ __forceinline__ void load_counts(const uint4* __restrict__ rowcnt, const uint32_t* __restrict__ mccnt,
                                            long long R, long long b, uint32_t (&v)[4][kScanPer],
                                            unsigned long long (&s)[4])
{
    s[0] = s[1] = s[2] = s[3] = 0;
#pragma unroll
    for (int q = 0; q < kScanPer; ++q) {
        const bool ok = b + q < R;
        const uint4 c = ok ? __ldg(&rowcnt[b + q]) : make_uint4(0, 0, 0, 0);
        if (SM == kScanDup) {
            v[0][q] = c.x;
            v[2][q] = c.y;
            v[3][q] = c.z;
        } else {
            v[0][q] = c.x + c.y + c.z;
            v[2][q] = (SM == kScanMC && ok) ? __ldg(&mccnt[b + q]) : 0u;
            v[3][q] = 0u;
        }
        v[1][q] = c.w;
#pragma unroll
        for (int a = 0; a < 4; ++a) s[a] += v[a][q];
    }
}

// Segment blk of the scan: its totals into part[a * nseg + blk].
template <int SM>
__device__ __forceinline__ void scan_partial_block(const uint4* __restrict__ rowcnt,
                                                   const uint32_t* __restrict__ mccnt, long long R,
                                                   unsigned long long* __restrict__ part, int nseg, int blk)
{
    constexpr int NC = ScanComps<SM>::n;
    __shared__ unsigned long long s_w[NC][kThreads / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t v[4][kScanPer];
    unsigned long long s[4];
    load_counts<SM>(rowcnt, mccnt, R, (long long)blk * kSeg + (long long)t * kScanPer, v, s);
#pragma unroll
    for (int a = 0; a < NC; ++a) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) s[a] += __shfl_xor_sync(0xffffffffu, s[a], d);
        if (lane == 0) s_w[a][warp] = s[a];
    }
    __syncthreads();
    if (t < NC) {
        unsigned long long tot = 0;
        for (int w = 0; w < kThreads / 32; ++w) tot += s_w[t][w];
        part[t * nseg + blk] = tot;
    }
}

template <int SM>
__global__ void __launch_bounds__(kThreads) k_scan_partial(const uint4* __restrict__ rowcnt,
                                                           const uint32_t* __restrict__ mccnt, long long R,
                                                           unsigned long long* __restrict__ part, int nseg)
{
    scan_partial_block<SM>(rowcnt, mccnt, R, part, nseg, (int)blockIdx.x);
}

// Segment blk: the starts of its rows from the segments' totals; segment 0 also writes the totals.
template <int SM>
__device__ __forceinline__ void scan_final_block(const uint4* __restrict__ rowcnt,
                                                 const uint32_t* __restrict__ mccnt, long long R,
                                                 const unsigned long long* __restrict__ part, int nseg,
                                                 unsigned long long* __restrict__ starts,
                                                 unsigned long long* __restrict__ totals, int blk)
{
    constexpr int NC = ScanComps<SM>::n;
    __shared__ unsigned long long s_w[NC][kThreads / 32];
    __shared__ unsigned long long s_base[NC], s_tot[NC];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (warp < NC) {  // warp a: the segments before this one and all of them, for component a
        unsigned long long b = 0, tot = 0;
        for (int q = lane; q < nseg; q += 32) {
            const unsigned long long x = part[warp * nseg + q];
            if (q < blk) b += x;
            tot += x;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            b += __shfl_xor_sync(0xffffffffu, b, d);
            tot += __shfl_xor_sync(0xffffffffu, tot, d);
        }
        if (lane == 0) {
            s_base[warp] = b;
            s_tot[warp] = tot;
        }
    }
    const long long b = (long long)blk * kSeg + (long long)t * kScanPer;
    uint32_t v[4][kScanPer];
    unsigned long long s[4], inc[4];
    load_counts<SM>(rowcnt, mccnt, R, b, v, s);
#pragma unroll
    for (int a = 0; a < NC; ++a) {
        inc[a] = s[a];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, inc[a], d);
            if (lane >= d) inc[a] += y;
        }
        if (lane == 31) s_w[a][warp] = inc[a];
    }
    __syncthreads();
    if (blk == 0 && t == 0) {
        if (SM == kScanDup) {
            totals[0] = s_tot[0] + s_tot[2] + s_tot[3];
            totals[1] = s_tot[1];
            totals[2] = 0;
            totals[4] = s_tot[0];
            totals[5] = s_tot[2];
        } else {
            for (int a = 0; a < 3; ++a) totals[a] = s_tot[a];
        }
    }
#pragma unroll
    for (int a = 0; a < NC; ++a) {
        if (SM == kScanFE && a == 2) continue;
        unsigned long long run = s_base[a] + inc[a] - s[a];
        for (int w = 0; w < warp; ++w) run += s_w[a][w];
#pragma unroll
        for (int q = 0; q < kScanPer; ++q) {
            if (b + q < R) starts[a * R + b + q] = run;
            run += v[a][q];
        }
    }
}

template <int SM>
__global__ void __launch_bounds__(kThreads) k_scan_final(const uint4* __restrict__ rowcnt,
                                                         const uint32_t* __restrict__ mccnt, long long R,
                                                         const unsigned long long* __restrict__ part, int nseg,
                                                         unsigned long long* __restrict__ starts,
                                                         unsigned long long* __restrict__ totals)
{
    scan_final_block<SM>(rowcnt, mccnt, R, part, nseg, starts, totals, (int)blockIdx.x);
}

// The Flying Edges scans of a list of requests, one launch per phase: block x is segment
// x - first[q] of request list[q].
__global__ void __launch_bounds__(kThreads) k_scan_partial_batch(const BatchReq* __restrict__ reqs,
                                                                 const int* __restrict__ list,
                                                                 const unsigned* __restrict__ first, int m)
{
    const int q = batch_find(first, m, blockIdx.x);
    const BatchReq* d = reqs + __ldg(&list[q]);
    const int blk = (int)(blockIdx.x - __ldg(&first[q]));
    if (blk >= d->nseg) return;  // past the request's segments (the launch holds exactly first[m] blocks)
    scan_partial_block<kScanFE>(d->rowcnt, nullptr, d->g.R, d->part, d->nseg, blk);
}

__global__ void __launch_bounds__(kThreads) k_scan_final_batch(const BatchReq* __restrict__ reqs,
                                                               const int* __restrict__ list,
                                                               const unsigned* __restrict__ first, int m)
{
    const int q = batch_find(first, m, blockIdx.x);
    const BatchReq* d = reqs + __ldg(&list[q]);
    const int blk = (int)(blockIdx.x - __ldg(&first[q]));
    if (blk >= d->nseg) return;
    scan_final_block<kScanFE>(d->rowcnt, nullptr, d->g.R, d->part, d->nseg, d->starts, d->totals, blk);
}

// vfirst[q] = the vertices of requests list[0 .. q-1] whose meshes hold their counts (one CTA of 1024 threads,
// each summing a run of consecutive requests).
__global__ void __launch_bounds__(1024) k_batch_vfirst(const BatchReq* __restrict__ reqs, const int* __restrict__ list,
                                                       int m, unsigned long long* __restrict__ vfirst)
{
    __shared__ unsigned long long s_w[32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int per = (m + 1023) / 1024, q0 = t * per, q1 = min(m, q0 + per);
    auto verts = [&](int q) -> unsigned long long {
        const BatchReq* d = reqs + __ldg(&list[q]);
        const unsigned long long v = d->totals[0], tr = d->totals[1];
        return ((long long)v <= d->capV && (long long)tr <= d->capT) ? v : 0ull;
    };
    unsigned long long mine = 0;
    for (int q = q0; q < q1; ++q) mine += verts(q);
    unsigned long long inc = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += y;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    unsigned long long run = inc - mine;
    for (int w = 0; w < warp; ++w) run += s_w[w];
    for (int q = q0; q < q1; ++q) {
        vfirst[q] = run;
        run += verts(q);
    }
    if (t == 1023) vfirst[m] = run;
}

// Block-wide exclusive sums of two values per thread (one CTA of 1024 threads): returns this thread's offsets.
__device__ __forceinline__ void block_excl2(unsigned long long a, unsigned long long b, unsigned long long& ea,
                                            unsigned long long& eb, unsigned long long* s_a, unsigned long long* s_b)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long ia = a, ib = b;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long ya = __shfl_up_sync(0xffffffffu, ia, d), yb = __shfl_up_sync(0xffffffffu, ib, d);
        if (lane >= d) {
            ia += ya;
            ib += yb;
        }
    }
    if (lane == 31) {
        s_a[warp] = ia;
        s_b[warp] = ib;
    }
    __syncthreads();
    ea = ia - a;
    eb = ib - b;
    for (int w = 0; w < warp; ++w) {
        ea += s_a[w];
        eb += s_b[w];
    }
    __syncthreads();  // s_a / s_b free for the next call
}

// The packed placement (launch_place_batch): one CTA of 1024 threads, each over a run of consecutive requests.
// Request list[q] goes to vertex offset vat and triangle offset tat, the sums of the counts before it; it is
// placed when both ranges end within the capacities and, for 32-bit indices, its vertices number below 2^32.
// vfirst sums the vertices of the placed requests only.
__global__ void __launch_bounds__(1024) k_batch_place(BatchReq* __restrict__ reqs, const int* __restrict__ list, int m,
                                                      PackedOut o, unsigned long long* __restrict__ vfirst)
{
    __shared__ unsigned long long s_a[32], s_b[32];
    const int t = threadIdx.x;
    const int per = (m + 1023) / 1024, q0 = t * per, q1 = min(m, q0 + per);
    unsigned long long sv = 0, st = 0;
    for (int q = q0; q < q1; ++q) {
        const unsigned long long* tot = reqs[__ldg(&list[q])].totals;
        sv += tot[0];
        st += tot[1];
    }
    unsigned long long vat, tat;
    block_excl2(sv, st, vat, tat, s_a, s_b);
    unsigned long long placed = 0;  // vertices of this thread's placed requests
    for (int q = q0; q < q1; ++q) {
        BatchReq* d = reqs + __ldg(&list[q]);
        const unsigned long long V = d->totals[0], T = d->totals[1];
        const bool ok = vat + V <= (unsigned long long)o.cap_points && tat + T <= (unsigned long long)o.cap_tris &&
                        (o.index_bytes == 8 || V <= 0xffffffffull);
        d->points = o.points + 3 * vat;
        d->normals = o.normals + 3 * vat;
        d->tris = static_cast<char*>(o.tris) + 3 * tat * (unsigned long long)o.index_bytes;
        d->capV = ok ? (long long)V : -1;
        d->capT = ok ? (long long)T : -1;
        d->totals[4] = vat;
        d->totals[5] = tat;
        placed += ok ? V : 0ull;
        vat += V;
        tat += T;
    }
    unsigned long long at, unused;
    block_excl2(placed, 0ull, at, unused, s_a, s_b);
    for (int q = q0; q < q1; ++q) {
        const BatchReq* d = reqs + __ldg(&list[q]);
        vfirst[q] = at;
        at += d->capV >= 0 ? d->totals[0] : 0ull;
    }
    if (t == 1023) vfirst[m] = at;
}

// gridEdge records {xl, xr, xstart, ystart, zstart} and triCounter for
// inspection (counts before the scan, offsets after it).
__global__ void k_grid_edges(Grid g, RowStarts rs, const uint4* __restrict__ rowcnt, const uint2* __restrict__ trims,
                             int scanned, unsigned long long* __restrict__ ge,
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
        const unsigned long long b = rs.get(r, 0);
        o[2] = b; o[3] = b + c.x; o[4] = b + c.x + c.y;
    } else {
        o[2] = c.x; o[3] = c.y; o[4] = c.z;
    }
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    if (j < g.ny - 1 && k < g.nz - 1) tri_counter[(long long)k * (g.ny - 1) + j] = scanned ? rs.get(r, 1) : c.w;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int lanes_per_row(int W)
{
    int G = 1;
    while (G < W && G < 32) G <<= 1;
    return G;
}

CountPlan count_plan(const Grid& g, int nsm)
{
    CountPlan p;
    p.J = kCountRows;
    p.nyb = (g.ny + p.J - 1) / p.J;
    p.vec_u = 1;
    while (p.vec_u * 128 < g.nx) p.vec_u <<= 1;  // float4 per lane for one row
    // ~8 CTAs per SM in total, at least 8 planes per column
    const int nzw = g.ke - g.kr;  // planes of the window
    const long long target = (long long)nsm * 8;
    int nkc = (int)((target + p.nyb - 1) / p.nyb);
    if (nkc < 1) nkc = 1;
    p.KC = (nzw + nkc - 1) / nkc;
    if (p.KC < 8) p.KC = 8;
    if (p.KC > nzw) p.KC = nzw;
    if (p.KC < 1) p.KC = 1;
    p.nkc = (nzw + p.KC - 1) / p.KC;
    p.nseg = (int)((g.R + kSeg - 1) / kSeg);
    return p;
}

template <bool MC>
static void count_launch(const CountPlan& p, const float* vol, const Grid& g, float iso, const CaseTables* cases,
                         FeBuffers& b, cudaStream_t s)
{
    const unsigned blocks = (unsigned)(p.nyb * p.nkc);
    const bool vec4 = g.W <= 64 && (g.nx % 4 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
    uint2* trims = p.trims ? b.trims : nullptr;  // the kernels skip the trims when null
    const bool base16 = (reinterpret_cast<uintptr_t>(vol) & 15) == 0;
    if (base16 && g.W <= 32) {  // 8 rows per warp up to 4 words, 4 up to 8, 2 up to 16, else 1; planes via TMA
        const int rpw = g.W <= 4 ? 8 : (g.W <= 8 ? 4 : (g.W <= 16 ? 2 : 1));
        const bool aligned = g.nx % 4 == 0;
        const int rows = kCountRows * rpw;
        const int nyb2 = (g.ny + rows - 1) / rows;
        const unsigned blocks2 = (unsigned)(nyb2 * p.nkc);
        const int nq = g.nx >> 2;
        const size_t smem = (size_t)kCountRows * count_buffer_floats(g.nx, rpw, aligned) * sizeof(float);
#define ISO_TMA(FULL, RPW, AL)                                                                                 \
    {                                                                                                          \
        auto kern = k_count_tma<MC, FULL, RPW, AL>;                                                           \
        allow_smem(kern, smem);                                                                                \
        kern<<<blocks2, kThreads, smem, s>>>(vol, g, iso, p.KC, nyb2, b.rowcnt, trims, b.mccnt, b.bits,         \
                                             b.totals + 3);                                                    \
    }
        if (!aligned) {
            if (rpw == 8) ISO_TMA(false, 8, false)
            else if (rpw == 4) ISO_TMA(false, 4, false)
            else if (rpw == 2) ISO_TMA(false, 2, false)
            else ISO_TMA(false, 1, false)
        } else if (rpw == 1) {
            if (nq == 256) ISO_TMA(true, 1, true)
            else ISO_TMA(false, 1, true)
        } else if (rpw == 8) {
            if (nq == 32) ISO_TMA(true, 8, true)
            else ISO_TMA(false, 8, true)
        } else if (rpw == 4) {
            if (nq == 64) ISO_TMA(true, 4, true)
            else ISO_TMA(false, 4, true)
        } else {
            if (nq == 128) ISO_TMA(true, 2, true)
            else ISO_TMA(false, 2, true)
        }
#undef ISO_TMA
        return;
    }
#define ISO_COUNT(VEC, UU, NWW)                                                                                \
    k_count_warps<MC, VEC, UU, NWW><<<blocks, kThreads, 0, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt,     \
                                                                trims, b.mccnt, b.bits)
    if (vec4) {
        switch (p.vec_u) {
            case 1: ISO_COUNT(true, 1, 1); break;
            case 2: ISO_COUNT(true, 2, 1); break;
            case 4: ISO_COUNT(true, 4, 1); break;
            case 8: ISO_COUNT(true, 8, 1); break;
            default: ISO_COUNT(true, 16, 2); break;
        }
    } else if (g.W <= 32) {
        ISO_COUNT(false, 1, 1);
    } else if (g.W <= 64) {
        ISO_COUNT(false, 1, 2);
    } else {
        k_count_wide<MC><<<blocks, kThreads, 0, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt, trims, b.mccnt,
                                                     b.bits);
    }
#undef ISO_COUNT
}

void launch_count(const float* vol, const Grid& g, float iso, const CaseTables* cases, bool mc,
                  const CountPlan& p, FeBuffers& b, cudaStream_t s)
{
    cudaMemsetAsync(b.totals + 3, 0, sizeof(unsigned long long), s);  // device status
    if (mc) count_launch<true>(p, vol, g, iso, cases, b, s);
    else count_launch<false>(p, vol, g, iso, cases, b, s);
}

CountVariant count_variant(const Grid& g)
{
    CountVariant v;
    v.rpw = g.W <= 4 ? 8 : (g.W <= 8 ? 4 : 2);
    v.aligned = g.nx % 4 == 0;
    v.full = v.aligned && (g.nx >> 2) == 256 / v.rpw;  // nq = 32 * LPR / 4 points in quads
    return v;
}

size_t count_batch_smem(const Grid& g, const CountVariant& v)
{
    return (size_t)kCountRows * count_buffer_floats(g.nx, v.rpw, v.aligned) * sizeof(float);
}

void launch_count_batch(const CountVariant& v, const BatchReq* reqs, const int* list, const unsigned* first, int m,
                        unsigned blocks, size_t smem, cudaStream_t s)
{
#define ISO_TMA_BATCH(FULL, RPW, AL)                                                                           \
    {                                                                                                          \
        auto kern = k_count_tma_batch<FULL, RPW, AL>;                                                         \
        allow_smem(kern, smem);                                                                                \
        kern<<<blocks, kThreads, smem, s>>>(reqs, list, first, m);                                             \
    }
    if (!v.aligned) {
        if (v.rpw == 8) ISO_TMA_BATCH(false, 8, false)
        else if (v.rpw == 4) ISO_TMA_BATCH(false, 4, false)
        else ISO_TMA_BATCH(false, 2, false)
    } else if (v.rpw == 8) {
        if (v.full) ISO_TMA_BATCH(true, 8, true)
        else ISO_TMA_BATCH(false, 8, true)
    } else if (v.rpw == 4) {
        if (v.full) ISO_TMA_BATCH(true, 4, true)
        else ISO_TMA_BATCH(false, 4, true)
    } else {
        if (v.full) ISO_TMA_BATCH(true, 2, true)
        else ISO_TMA_BATCH(false, 2, true)
    }
#undef ISO_TMA_BATCH
}

void launch_scan_batch(const BatchReq* reqs, const int* list, const unsigned* first, int m, unsigned blocks,
                       cudaStream_t s)
{
    k_scan_partial_batch<<<blocks, kThreads, 0, s>>>(reqs, list, first, m);
    k_scan_final_batch<<<blocks, kThreads, 0, s>>>(reqs, list, first, m);
}

void launch_vfirst_batch(const BatchReq* reqs, const int* list, int m, unsigned long long* vfirst, cudaStream_t s)
{
    k_batch_vfirst<<<1, 1024, 0, s>>>(reqs, list, m, vfirst);
}

void launch_place_batch(BatchReq* reqs, const int* list, int m, const PackedOut& out, unsigned long long* vfirst,
                        cudaStream_t s)
{
    k_batch_place<<<1, 1024, 0, s>>>(reqs, list, m, out, vfirst);
}

void launch_scan(const Grid& g, const CountPlan& p, int mode, FeBuffers& b, cudaStream_t s)
{
#define ISO_SCAN(SM)                                                                                            \
    k_scan_partial<SM><<<p.nseg, kThreads, 0, s>>>(b.rowcnt, b.mccnt, g.R, b.part, p.nseg);                      \
    k_scan_final<SM><<<p.nseg, kThreads, 0, s>>>(b.rowcnt, b.mccnt, g.R, b.part, p.nseg, b.starts, b.totals)
    if (mode == kScanMC) {
        ISO_SCAN(kScanMC);
    } else if (mode == kScanDup) {
        ISO_SCAN(kScanDup);
    } else {
        ISO_SCAN(kScanFE);
    }
#undef ISO_SCAN
}

RowStarts row_starts(const Grid& g, const CountPlan& p, const FeBuffers& b)
{
    (void)p;
    RowStarts rs;
    rs.starts = b.starts;
    rs.R = g.R;
    rs.ny = g.ny;
    rs.kr = g.kr;
    rs.add[0] = rs.add[1] = rs.add[2] = rs.add[3] = 0;
    return rs;
}

// A slab's counts for the host, written by one warp straight into mapped
// pinned host memory (no copy engine: the read-back does not queue behind
// bulk copies of other streams): out[a] the totals, out[3 + a] the start of
// row rlo and out[6 + a] that of row rhi, for a = vertices, triangles, MC
// vertices.
__global__ void k_slab_readback(const unsigned long long* __restrict__ totals,
                                const unsigned long long* __restrict__ starts, long long R, long long rlo,
                                long long rhi, int has_lo, int has_hi, unsigned long long* out)
{
    const int a = threadIdx.x;
    if (a < 3) {
        out[a] = totals[a];
        if (has_lo) out[3 + a] = starts[a * R + rlo];
        if (has_hi) out[6 + a] = starts[a * R + rhi];
    }
}

void launch_slab_readback(const FeBuffers& b, const Grid& g, long long rlo, long long rhi, bool has_lo, bool has_hi,
                          unsigned long long* out, cudaStream_t s)
{
    k_slab_readback<<<1, 32, 0, s>>>(b.totals, b.starts, g.R, rlo, rhi, has_lo ? 1 : 0, has_hi ? 1 : 0, out);
}

void launch_grid_edges(const Grid& g, const CountPlan& p, const FeBuffers& b, int scanned, unsigned long long* ge,
                       unsigned long long* tri_counter, cudaStream_t s)
{
    const long long blocks = (g.R + 255) / 256;
    k_grid_edges<<<(unsigned)blocks, 256, 0, s>>>(g, row_starts(g, p, b), b.rowcnt, b.trims, scanned, ge,
                                                  tri_counter);
}

ISO_WAIT_STATS_ACCESSOR(iso_dbg_count_waits)

}  // namespace iso
