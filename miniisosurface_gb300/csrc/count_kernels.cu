// Passes 1-3 of Flying Edges (flyingEdges/serial/FlyingEdgesAlgorithm.cpp:23-269)
// on sm_103a, with pass 1 (x-edge classification, trims) fused into pass 2
// (cube cases, per-row counts):
//
//   k_count_cols   one CTA per column = block of J grid rows x KC planes.  It
//                  marches along z: classifies plane k+1 straight from the
//                  volume into a bit-per-point mask in shared memory (the
//                  reference's edgeCases bytes are never materialised), then
//                  counts, for each grid row (j,k) of the block, its cut x, y
//                  and z edges (the vertices it owns), the trims xl/xr, the
//                  triangles of cell row (j,k) and, for Marching Cubes, the
//                  vertices cell row (j,k) owns.  Per (plane, block) totals go
//                  to `groups`.
//                  Each row also gets its exclusive prefix inside its group.
//   k_scan_*       exclusive scan of the group totals; groups are in
//                  (k, block) order, which is the reference's (k, j) row order,
//                  so the first vertex / triangle / MC vertex of a row (the
//                  gridEdge xstart and triCounter offsets after pass 3) is
//                  group offset + row prefix (RowStarts).
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

// How the count pass reads a plane of its block: staged through a shared-
// memory slab ring by the TMA bulk engine (rows 16-byte aligned) or by
// cp.async, or read directly (rows too wide to stage).
enum SlabMode { kSlabBulk = 0, kSlabCpAsync = 1, kSlabDirect = 2 };

template <int G, bool MC, int MODE>
__global__ void __launch_bounds__(kThreads) k_count_cols(const float* __restrict__ vol, Grid g, float iso, int KC,
                                                         int nyb, int NS, int slab_floats,
                                                         const CaseTables* __restrict__ cases,
                                                         uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                                         uint32_t* __restrict__ mccnt, uint4* __restrict__ rowpre,
                                                         uint32_t* __restrict__ gsum, long long ngroups,
                                                         uint32_t* __restrict__ bits_out,
                                                         unsigned long long* __restrict__ totals)
{
    constexpr int J = kThreads / G;  // grid rows per block
    constexpr bool STAGED = MODE != kSlabDirect;
    extern __shared__ __align__(128) unsigned char s_raw[];
    __shared__ uint8_t s_ntris[256];
    __shared__ uint16_t s_cut[256];
    __shared__ uint32_t s_rc[3][J];
    float* slots = reinterpret_cast<float*>(s_raw);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(s_raw + (size_t)NS * slab_floats * 4);
    uint32_t* s_bits0 = reinterpret_cast<uint32_t*>(mbar + (STAGED ? NS : 0));
    uint32_t* s_bits1 = s_bits0 + (J + 1) * g.W;
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        s_ntris[c] = (uint8_t)iso_case_ntris(cases->tris[c]);
        s_cut[c] = cases->cut[c];
    }
    const int jb = blockIdx.x % nyb, kc = blockIdx.x / nyb;
    const int j0 = jb * J, JB = min(J, g.ny - j0), nbr = min(J + 1, g.ny - j0);
    const int kb = kc * KC, ke = min(kb + KC, g.nz);
    const int tid = threadIdx.x, lane = tid & 31, lig = lane & (G - 1);
    const int jj = tid / G;  // the row this group counts
    const int nchunks = (g.W + G - 1) / G;
    const int nfl = nbr * g.nx;
    const bool vec4 = (g.nx & 3) == 0 && (STAGED || (reinterpret_cast<uintptr_t>(vol) & 15) == 0);

    if (STAGED && tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&mbar[s], MODE == kSlabBulk ? 1u : (unsigned)kThreads);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t pending = 0, parity = 0;  // per slot: copy in flight / next wait parity
    auto issue = [&](int p) {
        if (!STAGED || p > ke || p >= g.nz) return;
        const int s = p % NS;
        slab_copy<MODE == kSlabBulk>(slots + (size_t)s * slab_floats, vol + ((long long)p * g.ny + j0) * g.nx, nfl,
                                     &mbar[s], tid, kThreads);
        pending |= 1u << s;
    };
    auto wait = [&](int p) -> bool {
        if (!STAGED) return true;
        const int s = p % NS;
        const bool ok = mbar_wait(&mbar[s], (parity >> s) & 1u);
        parity ^= 1u << s;
        pending &= ~(1u << s);
        return ok;
    };
    auto drain = [&]() {
        for (int s = 0; s < NS; ++s) {
            if ((pending >> s) & 1u) {
                mbar_wait(&mbar[s], (parity >> s) & 1u);
                parity ^= 1u << s;
                pending &= ~(1u << s);
            }
        }
    };
    // bit rows of plane p (slab or volume) into dst
    auto classify = [&](int p, uint32_t* dst) {
        if (STAGED) {
            const float* src = slots + (size_t)(p % NS) * slab_floats;
            if (vec4) classify_block<true, true>(src, g.nx, g.W, nbr, iso, dst);
            else classify_block<false, true>(src, g.nx, g.W, nbr, iso, dst);
        } else {
            const float* src = vol + ((long long)p * g.ny + j0) * g.nx;
            if (vec4) classify_block<true, false>(src, g.nx, g.W, nbr, iso, dst);
            else classify_block<false, false>(src, g.nx, g.W, nbr, iso, dst);
        }
    };

    for (int q = 0; q < NS; ++q) issue(kb + q);
    bool alive = __syncthreads_and(wait(kb));
    if (alive) {
        classify(kb, (kb & 1) ? s_bits1 : s_bits0);
        __syncthreads();
        issue(kb + NS);
    }
    for (int k = kb; k < ke && alive; ++k) {
        uint32_t* P0 = (k & 1) ? s_bits1 : s_bits0;  // plane k
        uint32_t* P1 = (k & 1) ? s_bits0 : s_bits1;  // plane k+1
        if (k + 1 < g.nz) {
            alive = __syncthreads_and(wait(k + 1));
            if (!alive) break;
            classify(k + 1, P1);
        }
        __syncthreads();
        issue(k + 1 + NS);  // the slot of plane k+1 is free again

        const bool valid = jj < JB;
        const int j = j0 + jj;
        const bool hasY = valid && j < g.ny - 1;
        const bool hasZ = valid && k < g.nz - 1;
        const bool cell = hasY && hasZ;
        const uint32_t* A = P0 + jj * g.W;
        const uint32_t* B = A + g.W;
        const uint32_t* Cc = P1 + jj * g.W;
        const uint32_t* D = Cc + g.W;
        uint32_t xc = 0, yc = 0, zc = 0, tc = 0, mc = 0, first = 0xffffffffu, last = 0;
        for (int ch = 0; ch < nchunks; ++ch) {
            const int w = ch * G + lig;
            const bool in = valid && w < g.W, in1 = valid && w + 1 < g.W;
            RowWords rw;
            rw.a = in ? A[w] : 0u;
            rw.b = (in && hasY) ? B[w] : 0u;
            rw.c = (in && hasZ) ? Cc[w] : 0u;
            rw.d = (in && cell) ? D[w] : 0u;
            rw.ash = (rw.a >> 1) | ((in1 ? A[w + 1] : 0u) << 31);
            rw.bsh = (rw.b >> 1) | ((in1 && hasY ? B[w + 1] : 0u) << 31);
            rw.csh = (rw.c >> 1) | ((in1 && hasZ ? Cc[w + 1] : 0u) << 31);
            rw.dsh = (rw.d >> 1) | ((in1 && cell ? D[w + 1] : 0u) << 31);
            const uint32_t evalid = validmask(w, g.nx - 1);   // x-edges / cells: i <= nx-2
            const uint32_t pvalid = validmask(w, g.nx);       // points: i <= nx-1
            const uint32_t xm = (rw.a ^ rw.ash) & evalid;
            const uint32_t ym = hasY ? ((rw.a ^ rw.b) & pvalid) : 0u;
            const uint32_t zm = hasZ ? ((rw.a ^ rw.c) & pvalid) : 0u;
            xc += __popc(xm);
            yc += __popc(ym);
            zc += __popc(zm);
            // isCutEdge (FlyingEdgesAlgorithm.cpp:515-554): edge i is marked when
            // it is cut or the y / z edge at its left point is.
            const uint32_t marked = xm | ((ym | zm) & evalid);
            if (marked) {
                first = min(first, (uint32_t)(32 * w + __ffs(marked) - 1));
                last = max(last, (uint32_t)(32 * w + 32 - __clz(marked)));
            }
            if (cell) {
                for (uint32_t act = active_cells(rw, evalid); act; act &= act - 1) {
                    const int bit = __ffs(act) - 1;
                    const int c = cube_case(rw, bit);
                    tc += s_ntris[c];
                    if (MC) mc += __popc(mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cut[c]);
                }
            }
            if (in) bits_out[((long long)k * g.ny + j) * g.W + w] = rw.a;
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
                const long long r = (long long)k * g.ny + j;
                rowcnt[r] = make_uint4(xc, yc, zc, tc);
                trims[r] = make_uint2(first == 0xffffffffu ? (uint32_t)g.nx : first, last);
                if (MC) mccnt[r] = mc;
            }
            s_rc[0][jj] = valid ? xc + yc + zc : 0u;
            s_rc[1][jj] = valid ? tc : 0u;
            s_rc[2][jj] = valid ? mc : 0u;
        }
        __syncthreads();
        // exclusive prefix of the block's rows (warp 0) and the group totals
        if (tid < 32) {
            uint32_t run[3] = {0, 0, 0};
            for (int base = 0; base < J; base += 32) {
                const int q = base + tid;
                uint32_t v[3], inc[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    v[a] = q < J ? s_rc[a][q] : 0u;
                    inc[a] = v[a];
                }
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const uint32_t t = __shfl_up_sync(0xffffffffu, inc[a], d);
                        if (tid >= d) inc[a] += t;
                    }
                }
                if (q < JB) {
                    rowpre[(long long)k * g.ny + j0 + q] =
                        make_uint4(run[0] + inc[0] - v[0], run[1] + inc[1] - v[1], run[2] + inc[2] - v[2], 0u);
                }
#pragma unroll
                for (int a = 0; a < 3; ++a) run[a] += __shfl_sync(0xffffffffu, inc[a], 31);
            }
            if (tid < 3) gsum[tid * ngroups + (long long)k * nyb + jb] = run[tid];
        }
    }
    if (!alive && tid == 0) atomicOr(&totals[3], kStatusTimeout);
    drain();
}

// Exclusive scan of the group totals (three arrays of n u32) into 64-bit
// offsets, in two launches over segments of kSeg groups (256 threads x 8):
//   k_scan_partial  one CTA per segment: segment totals
//   k_scan_final    one CTA per segment: offset of the segment (sum of the
//                   totals before it) + scan inside it; grand totals.
constexpr int kScanPer = 8;
constexpr int kSeg = kThreads * kScanPer;

__device__ __forceinline__ void load_segment(const uint32_t* __restrict__ gsum, long long n, long long b,
                                             uint32_t (&v)[3][kScanPer], unsigned long long (&s)[3])
{
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        s[a] = 0;
#pragma unroll
        for (int q = 0; q < kScanPer; ++q) {
            v[a][q] = b + q < n ? __ldg(&gsum[a * n + b + q]) : 0u;
            s[a] += v[a][q];
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_scan_partial(const uint32_t* __restrict__ gsum, long long n,
                                                           unsigned long long* __restrict__ part, int nseg)
{
    __shared__ unsigned long long s_w[3][kThreads / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t v[3][kScanPer];
    unsigned long long s[3];
    load_segment(gsum, n, (long long)blockIdx.x * kSeg + (long long)t * kScanPer, v, s);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) s[a] += __shfl_xor_sync(0xffffffffu, s[a], d);
        if (lane == 0) s_w[a][warp] = s[a];
    }
    __syncthreads();
    if (t < 3) {
        unsigned long long tot = 0;
        for (int w = 0; w < kThreads / 32; ++w) tot += s_w[t][w];
        part[t * nseg + blockIdx.x] = tot;
    }
}

__global__ void __launch_bounds__(kThreads) k_scan_final(const uint32_t* __restrict__ gsum, long long n,
                                                         const unsigned long long* __restrict__ part, int nseg,
                                                         unsigned long long* __restrict__ goff,
                                                         unsigned long long* __restrict__ totals)
{
    __shared__ unsigned long long s_w[3][kThreads / 32];
    __shared__ unsigned long long s_base[3];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t < 3) {
        unsigned long long b = 0, tot = 0;
        for (int q = 0; q < nseg; ++q) {
            const unsigned long long x = part[t * nseg + q];
            if (q < (int)blockIdx.x) b += x;
            tot += x;
        }
        s_base[t] = b;
        if (blockIdx.x == 0) totals[t] = tot;
    }
    const long long b = (long long)blockIdx.x * kSeg + (long long)t * kScanPer;
    uint32_t v[3][kScanPer];
    unsigned long long s[3], inc[3];
    load_segment(gsum, n, b, v, s);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        inc[a] = s[a];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, inc[a], d);
            if (lane >= d) inc[a] += y;
        }
        if (lane == 31) s_w[a][warp] = inc[a];
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        unsigned long long run = s_base[a] + inc[a] - s[a];
        for (int w = 0; w < warp; ++w) run += s_w[a][w];
#pragma unroll
        for (int q = 0; q < kScanPer; ++q) {
            if (b + q < n) goff[a * n + b + q] = run;
            run += v[a][q];
        }
    }
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

// Blocks of J = 256/G rows with G >= lanes per row, G doubled until the
// slab ring (3 slabs of J+1 rows) fits kCountSmem so that several CTAs share
// an SM; columns of KC planes, ~8 CTAs per SM in total.
constexpr size_t kCountSmem = 64 * 1024;
constexpr int kCountSlots = 3;

CountPlan count_plan(const Grid& g, int nsm)
{
    CountPlan p;
    int G = lanes_per_row(g.W);
    for (;;) {
        const int J = kThreads / G;
        const size_t slab = ((size_t)(J + 1) * g.nx + 31) & ~(size_t)31;
        const size_t smem = kCountSlots * slab * 4 + kCountSlots * 8 + 2 * (size_t)(J + 1) * g.W * 4;
        if (smem <= kCountSmem || G == 32) {
            p.G = G;
            p.J = J;
            p.slab_floats = (int)slab;
            p.staged = smem <= 2 * kCountSmem;
            p.NS = p.staged ? kCountSlots : 0;
            p.smem = p.staged ? smem : 2 * (size_t)(J + 1) * g.W * 4;
            if (!p.staged) p.slab_floats = 0;
            break;
        }
        G *= 2;
    }
    p.nyb = (g.ny + p.J - 1) / p.J;
    const long long target = (long long)nsm * 8;
    int nkc = (int)((target + p.nyb - 1) / p.nyb);
    if (nkc < 1) nkc = 1;
    p.KC = (g.nz + nkc - 1) / nkc;
    if (p.KC < 8) p.KC = 8;
    if (p.KC > g.nz) p.KC = g.nz;
    p.nkc = (g.nz + p.KC - 1) / p.KC;
    p.ngroups = (long long)g.nz * p.nyb;
    return p;
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

template <int G, bool MC, int MODE>
static void count_launch(const CountPlan& p, const float* vol, const Grid& g, float iso, const CaseTables* cases,
                         FeBuffers& b, cudaStream_t s)
{
    auto kern = k_count_cols<G, MC, MODE>;
    allow_smem(kern, p.smem);
    kern<<<(unsigned)(p.nyb * p.nkc), kThreads, p.smem, s>>>(vol, g, iso, p.KC, p.nyb, p.NS, p.slab_floats, cases,
                                                              b.rowcnt, b.trims, b.mccnt, b.rowpre, b.gsum,
                                                              p.ngroups, b.bits, b.totals);
}

template <int G, bool MC>
static void count_mode(const CountPlan& p, const float* vol, const Grid& g, float iso, const CaseTables* cases,
                       FeBuffers& b, cudaStream_t s)
{
    const bool bulk = (g.nx % 4 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
    if (!p.staged) count_launch<G, MC, kSlabDirect>(p, vol, g, iso, cases, b, s);
    else if (bulk) count_launch<G, MC, kSlabBulk>(p, vol, g, iso, cases, b, s);
    else count_launch<G, MC, kSlabCpAsync>(p, vol, g, iso, cases, b, s);
}

void launch_count(const float* vol, const Grid& g, float iso, const CaseTables* cases, bool mc,
                  const CountPlan& p, FeBuffers& b, cudaStream_t s)
{
    cudaMemsetAsync(b.totals + 3, 0, sizeof(unsigned long long), s);  // device status
    if (mc) {
        ISO_DISPATCH_G(p.G, (count_mode<kG, true>(p, vol, g, iso, cases, b, s)));
    } else {
        ISO_DISPATCH_G(p.G, (count_mode<kG, false>(p, vol, g, iso, cases, b, s)));
    }
}

int scan_segments(const CountPlan& p) { return (int)((p.ngroups + kSeg - 1) / kSeg); }

void launch_scan(const CountPlan& p, FeBuffers& b, cudaStream_t s)
{
    const int nseg = scan_segments(p);
    k_scan_partial<<<nseg, kThreads, 0, s>>>(b.gsum, p.ngroups, b.part, nseg);
    k_scan_final<<<nseg, kThreads, 0, s>>>(b.gsum, p.ngroups, b.part, nseg, b.goff, b.totals);
}

RowStarts row_starts(const Grid& g, const CountPlan& p, const FeBuffers& b)
{
    RowStarts rs;
    rs.goff = b.goff;
    rs.rowpre = b.rowpre;
    rs.ngroups = p.ngroups;
    rs.ny = g.ny;
    rs.nyb = p.nyb;
    int sh = 0;
    while ((1 << sh) < p.J) ++sh;
    rs.jshift = sh;
    return rs;
}

void launch_grid_edges(const Grid& g, const CountPlan& p, const FeBuffers& b, int scanned, unsigned long long* ge,
                       unsigned long long* tri_counter, cudaStream_t s)
{
    const long long blocks = (g.R + 255) / 256;
    k_grid_edges<<<(unsigned)blocks, 256, 0, s>>>(g, row_starts(g, p, b), b.rowcnt, b.trims, scanned, ge,
                                                  tri_counter);
}

}  // namespace iso

ISO_WAIT_STATS_ACCESSOR(iso_dbg_count_waits)
