// Flying Edges passes 1-4 in one kernel: k_fe_single counts, scans and
// generates a whole grid in a single launch (flyingEdges/serial/
// FlyingEdgesAlgorithm.cpp:23-497), leaving only the vertex values to
// k_vertices (vertices.cuh).
//
// The three separate kernels it replaces run back to back with opposite
// limiters: the count pass waits on HBM while its ALU idles, the generate pass
// is bound by instruction issue while HBM idles.  Here every warp alternates
// between the two kinds of work on successive items, so on each SM some warps
// stream volume rows while others issue generate instructions.
//
// Work items.  Item q = (r, p) with r = q / ngroups, p = q % ngroups: row
// group p is grid rows jw = p*RPW .. jw+RPW-1 (RPW = 2, 4 or 8 rows per warp
// for rows of up to 16, 8 or 4 words; lanes LPR*h .. LPR*h+LPR-1 hold the
// words of row jw+h), run r is planes r*KC .. r*KC+KC-1.  Items are handed out
// in increasing q by an atomic counter.  An item counts its run (r < nruns)
// and generates run r - L (r >= L): generation lags counting by L runs, more
// items than the resident warps hold at once, so the planes it needs were
// counted and scanned long before and its waits are short.
//   count  marches along its planes as k_count_tma does: volume rows jw ..
//          jw+RPW of plane k+1 come into the warp's shared buffer by one TMA
//          bulk copy (issued while plane k is counted; bounded mbarrier wait)
//          and are classified into bit words ("value >= iso", set.ge per
//          point); grid rows (jw+h, k) are counted -- cut x, y, z edges and the
//          triangles of cell row (jw+h, k) (count_word) -- and their bit words
//          and counts written.  No count waits for another item.  For each
//          plane, the warp that counts its last row group (a per-plane counter)
//          scans it: it publishes the plane's totals, finds the totals of the
//          planes before it by a decoupled look-back over the planes (the
//          single-pass scan of Merrill and Garland: 32 planes' flags at a time,
//          back to the first plane that carries its inclusive prefix), writes
//          every row's first vertex and triangle (starts[], the reference's
//          gridEdge xstart and triCounter after pass 3) and publishes the
//          plane's inclusive prefix.  Planes are scanned side by side: none
//          waits for another's scan, only for the counts of the planes before
//          it.
//   generate  run r - L of its row group, plane by plane, as k_gen_pairs does:
//          vertex records of grid rows (jw+h, k) and the triangles of cell rows
//          (jw+h, k), once the planes up to the run's end have been scanned.
// A wait is only ever for planes counted (or scanned) by warps holding
// earlier items: the waits end.  Each is bounded all the same (kWaitLimit
// polls, with a growing sleep between polls so that waiting warps do not crowd
// the memory system the counting warps need); one that runs out records
// ISO_ERR_TIMEOUT in the status word and publishes its plane's totals marked
// as failed, so that the waits after it end too.
//
// Capacity.  The totals are known only when the last plane is scanned, so
// the mesh is written as it is generated: an item writes its records and
// triangles only if their ids (all below the first ids of the next row
// group) lie inside the mesh's capacities.  A mesh that is too small is
// therefore written in part, never past its capacities, and the caller gets
// ISO_ERR_CAPACITY with the sizes needed.
//
// Used for whole grids (no z window), Flying Edges, rows of up to 16 words
// whose length is a multiple of 4 points, volumes at a 16-byte boundary.
#include "count_words.cuh"
#include "gen_pairs.cuh"

namespace iso {

constexpr int kSingleCtasPerSm = 4;

// Synchronisation words (zeroed before each launch):
//   done[plane]      row groups of the plane counted so far
//   agg[plane][2]    vertices and triangles of the plane (ready bit 63, failed bit 62)
//   incl[plane][2]   vertices and triangles of planes 0 .. plane (ready bit 63, failed bit 62)
constexpr unsigned long long kFlagReady = 1ull << 63, kFlagFailed = 1ull << 62;
constexpr unsigned long long kPrefixMask = (1ull << 62) - 1;

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Sleep between two polls of a flag, doubling up to about a microsecond.
__device__ __forceinline__ void poll_backoff(unsigned& ns)
{
    __nanosleep(ns);
    if (ns < 1024u) ns <<= 1;
}

// Per-warp shared memory: the TMA buffer of the count, then (reused) the
// generate scratch.
__host__ __device__ inline size_t single_warp_bytes(int nx, int W, int RPW)
{
    const size_t buf = (size_t)(RPW + 1) * nx * 4;
    const size_t gen = gen_pair_scratch_bytes(W, RPW, kGenFE);
    return ((buf > gen ? buf : gen) + 15) & ~(size_t)15;
}

// Row groups of RPW rows.
__host__ __device__ inline int single_groups(const Grid& g, int RPW) { return (g.ny + RPW - 1) / RPW; }

// Layout of the synchronisation words: done[nz], agg[nz][2], incl[nz][2] (u64 each).
__host__ __device__ inline size_t single_sync_words(const Grid& g) { return 5 * (size_t)g.nz; }

template <typename IndexT, int RPW>
__global__ void __launch_bounds__(kThreads, kSingleCtasPerSm) k_fe_single(
    const float* __restrict__ vol, Grid g, float iso, int KC, int L, int ws_bytes,
    const CaseTables* __restrict__ cases, uint4* __restrict__ rowcnt, uint32_t* __restrict__ bits,
    unsigned long long* __restrict__ starts, unsigned long long* __restrict__ sync,
    unsigned long long* __restrict__ totals, long long capV, long long capT, float* __restrict__ points,
    IndexT* __restrict__ tris)
{
    constexpr int LPR = 32 / RPW, NBUF = RPW + 1;
    extern __shared__ __align__(16) unsigned char s_raw[];
    // per case: each triangle corner as (mask-table row | point offset << 3), the count in bits 60..63
    __shared__ uint64_t s_tri[256];
    __shared__ uint64_t s_bar[kThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, h = lane / LPR, lw = lane % LPR;
    const int W = g.W, nx = g.nx, ny = g.ny, nz = g.nz;
    const long long R = g.R;
    for (int c = tid; c < 256; c += kThreads) {
        const uint64_t w = cases->tris[c];
        uint64_t x = w & (0xfull << 60);
        for (int q = 0; q < 15; ++q) {
            const int e = (int)((w >> (4 * q)) & 15u);
            const uint64_t nib = e < 12 ? (((0x776653524140ull >> (4 * e)) & 7u) | (((0xA22u >> e) & 1u) << 3)) : 0u;
            x |= nib << (4 * q);
        }
        s_tri[c] = x;
    }
    unsigned char* ws = s_raw + (size_t)warp * ws_bytes;
    float* buf = reinterpret_cast<float*>(ws);
    uint64_t* bar = &s_bar[warp];
    if (lane == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();  // the only CTA barrier: from here on every warp runs alone
    uint2* mb = reinterpret_cast<uint2*>(ws);                                    // [RPW][8][W]
    uint32_t* rwt = reinterpret_cast<uint32_t*>(ws + (size_t)RPW * 8 * W * 8);  // [RPW][W][8]
    uint32_t* cell = rwt + RPW * 8 * W;
    unsigned char* list = reinterpret_cast<unsigned char*>(cell + kGenCells);
    uint2* mbh = mb + h * 8 * W;
    uint32_t* rwth = rwt + h * 8 * W;

    const int ngroups = single_groups(g, RPW);
    const int nruns = (nz + KC - 1) / KC;
    unsigned long long* done = sync;
    unsigned long long* agg = sync + nz;
    unsigned long long* incl = sync + 3 * (size_t)nz;
    const long long nitems = (long long)(nruns + L) * ngroups;
    const bool in1 = lw + 1 < W;
    const uint32_t evalid = validmask(lw, nx - 1);  // x-edges / cells: i <= nx-2
    const uint32_t pvalid = validmask(lw, nx);      // points: i <= nx-1
    const int nq = nx >> 2;
    unsigned phase = 0;
    bool alive = true;  // false once a copy of this warp timed out

    // rows jw .. jw+nrows-1 of plane p -> the warp's buffer (lane 0 issues; every lane has ordered its own
    // generic accesses to the buffer before the engine's writes)
    auto issue = [&](int p, int jw) {
        const int nrows = min(NBUF, ny - jw);
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
            mbar_arrive_expect_tx(bar, (unsigned)(nrows * nx * 4));
            bulk_copy_g2s(buf, vol + ((long long)p * ny + jw) * nx, (unsigned)(nrows * nx * 4), bar);
        }
    };
    // the words of buffer rows h and h+1 once the copy has landed; false: it timed out (it is then waited
    // for once more, so that it lands before the warp stops using the buffer)
    auto take = [&](int jw, uint32_t& wa, uint32_t& wb) -> bool {
        const bool ok = mbar_wait(bar, phase);
        if (!__all_sync(0xffffffffu, ok)) {
            mbar_wait(bar, phase);
            return false;
        }
        phase ^= 1u;
        const int j = jw + h;
        wa = j < ny ? row_word<false>(buf + h * nx, nq, lw, lane & 7, iso) : 0u;
        wb = j + 1 < ny ? row_word<false>(buf + (h + 1) * nx, nq, lw, lane & 7, iso) : 0u;
        __syncwarp();  // every lane has read the buffer before it is refilled
        return true;
    };
    // bounded wait (one lane) until word *p has its ready bit; false: timed out, or marked failed
    auto wait_ready = [&](const unsigned long long* p, unsigned long long& v) -> bool {
        unsigned ns = 32;
        for (unsigned n = 0; n < kWaitLimit; ++n) {
            v = ld_acquire(p);
            if (v & kFlagReady) return !(v & kFlagFailed);
            poll_backoff(ns);
        }
        return false;
    };
    auto set_status = [&]() {
        if (lane == 0) atomicOr(&totals[3], kStatusTimeout);
    };

    for (;;) {
        unsigned long long qq = 0;
        if (lane == 0) qq = atomicAdd(&totals[7], 1ull);
        const long long q = (long long)__shfl_sync(0xffffffffu, qq, 0);
        if (q >= nitems) break;
        const int r = (int)(q / ngroups);
        const int jw = RPW * (int)(q % ngroups);
        const int j = jw + h;
        const bool row_ok = j < ny;
        const bool hasY = row_ok && j < ny - 1;
        const bool in = row_ok && lw < W;

        // ---------------- count grid rows (jw+h, k) of the planes of run r ----------------
        if (r < nruns) {
            const int k0 = r * KC, k1 = min(k0 + KC, nz);
            bool ok = alive;
            uint32_t a = 0, b = 0;
            if (ok) {
                issue(k0, jw);
                ok = take(jw, a, b);
                if (ok && k0 + 1 < nz) issue(k0 + 1, jw);
            }
            for (int k = k0; ok && k < k1; ++k) {
                const bool hasZ = k + 1 < nz;
                uint32_t c = 0, d = 0;
                if (hasZ) {  // plane k+1 was issued one step earlier
                    if (!(ok = take(jw, c, d))) break;
                    if (k + 2 < nz && k + 1 < k1) issue(k + 2, jw);
                }
                if (!row_ok) a = b = c = d = 0u;
                if (!hasY) b = d = 0u;
                RowWords rw;
                rw.a = a;
                rw.b = b;
                rw.c = c;
                rw.d = d;
                const uint32_t an = __shfl_down_sync(0xffffffffu, rw.a, 1, LPR);
                const uint32_t bn = __shfl_down_sync(0xffffffffu, rw.b, 1, LPR);
                const uint32_t cn = __shfl_down_sync(0xffffffffu, rw.c, 1, LPR);
                const uint32_t dn = __shfl_down_sync(0xffffffffu, rw.d, 1, LPR);
                rw.ash = (rw.a >> 1) | ((in1 ? an : 0u) << 31);
                rw.bsh = (rw.b >> 1) | ((in1 ? bn : 0u) << 31);
                rw.csh = (rw.c >> 1) | ((in1 ? cn : 0u) << 31);
                rw.dsh = (rw.d >> 1) | ((in1 ? dn : 0u) << 31);
                RowCounts rc;
                if (in) count_word<false>(rw, lw, g, j, k, hasY, hasZ, false, rc);
                const long long rr = (long long)k * ny + j;
                if (in) bits[rr * W + lw] = a;
                // per-row totals in the row's lanes
                uint32_t rx = 0, ry = 0, rz = 0, rt = 0;
#pragma unroll
                for (int q2 = 0; q2 < RPW; ++q2) {
                    const uint32_t sx = __reduce_add_sync(0xffffffffu, h == q2 ? rc.xc : 0u);
                    const uint32_t sy = __reduce_add_sync(0xffffffffu, h == q2 ? rc.yc : 0u);
                    const uint32_t sz = __reduce_add_sync(0xffffffffu, h == q2 ? rc.zc : 0u);
                    const uint32_t st = __reduce_add_sync(0xffffffffu, h == q2 ? rc.tc : 0u);
                    if (h == q2) {
                        rx = sx;
                        ry = sy;
                        rz = sz;
                        rt = st;
                    }
                }
                if (row_ok && lw == 0) rowcnt[rr] = make_uint4(rx, ry, rz, rt);
                a = c;
                b = d;
            }
            if (!ok) {
                alive = false;
                set_status();
            }
            __threadfence();  // the words and counts before the plane counters
            // planes of the run whose last row group this warp counted: bit k - k0
            uint32_t lastm = 0u;
            if (lane == 0) {
                for (int k = k0; k < k1; ++k)
                    if (atomicAdd(&done[k], 1ull) == (unsigned long long)(ngroups - 1)) lastm |= 1u << (k - k0);
            }
            lastm = __shfl_sync(0xffffffffu, lastm, 0);
            if (lastm) __threadfence();  // the other groups' counts (each fenced before its increment) are visible
            for (; lastm; lastm &= lastm - 1u) {
                // ---- scan plane k: this warp counted its last row group ----
                const int k = k0 + __ffs(lastm) - 1;
                const long long r0 = (long long)k * ny;
                const int per = (ny + 31) / 32;  // consecutive rows per lane
                unsigned long long lv = 0, lt = 0;
                for (int u = 0; u < per; ++u) {
                    const int jj = lane * per + u;
                    if (jj < ny) {
                        const uint4 cc = __ldcg(&rowcnt[r0 + jj]);
                        lv += (unsigned long long)cc.x + cc.y + cc.z;
                        lt += cc.w;
                    }
                }
                unsigned long long iv = lv, it = lt;
#pragma unroll
                for (int dd = 1; dd < 32; dd <<= 1) {
                    const unsigned long long yv = __shfl_up_sync(0xffffffffu, iv, dd);
                    const unsigned long long yt = __shfl_up_sync(0xffffffffu, it, dd);
                    if (lane >= dd) {
                        iv += yv;
                        it += yt;
                    }
                }
                const unsigned long long planeV = __shfl_sync(0xffffffffu, iv, 31);
                const unsigned long long planeT = __shfl_sync(0xffffffffu, it, 31);
                if (lane == 0) {
                    st_release(&agg[2 * k + 0], kFlagReady | planeV);
                    st_release(&agg[2 * k + 1], kFlagReady | planeT);
                }
                // look back over the planes before k for their totals
                unsigned long long pV = 0, pT = 0;
                bool failed = false;
                long long base = k - 1;
                unsigned spins = 0, ns = 32;
                while (base >= 0) {
                    const long long pl = base - lane;
                    int st = 2;  // 2: inclusive prefix (or before plane 0), 1: the plane's totals, 0: not ready
                    unsigned long long v = 0, t = 0;
                    bool bad = false;
                    if (pl >= 0) {
                        const unsigned long long iv2 = ld_acquire(&incl[2 * pl + 0]);
                        const unsigned long long it2 = ld_acquire(&incl[2 * pl + 1]);
                        if ((iv2 & kFlagReady) && (it2 & kFlagReady)) {
                            bad = ((iv2 | it2) & kFlagFailed) != 0;
                            v = iv2 & kPrefixMask;
                            t = it2 & kPrefixMask;
                        } else {
                            const unsigned long long av = ld_acquire(&agg[2 * pl + 0]);
                            const unsigned long long at = ld_acquire(&agg[2 * pl + 1]);
                            if ((av & kFlagReady) && (at & kFlagReady)) {
                                st = 1;
                                bad = ((av | at) & kFlagFailed) != 0;
                                v = av & kPrefixMask;
                                t = at & kPrefixMask;
                            } else {
                                st = 0;
                            }
                        }
                    }
                    const uint32_t inc = __ballot_sync(0xffffffffu, st == 2);
                    const uint32_t waiting = __ballot_sync(0xffffffffu, st == 0);
                    const int first = inc ? __ffs(inc) - 1 : 32;
                    const uint32_t upto = first == 32 ? 0xffffffffu : (0xffffffffu >> (31 - first));
                    if (__ballot_sync(0xffffffffu, bad) & upto) {
                        failed = true;
                        break;
                    }
                    if (waiting & upto) {
                        if (++spins >= kWaitLimit) {
                            failed = true;
                            break;
                        }
                        poll_backoff(ns);
                        continue;  // the same window again
                    }
                    unsigned long long sv2 = lane <= first ? v : 0ull, st2 = lane <= first ? t : 0ull;
#pragma unroll
                    for (int dd = 16; dd > 0; dd >>= 1) {
                        sv2 += __shfl_xor_sync(0xffffffffu, sv2, dd);
                        st2 += __shfl_xor_sync(0xffffffffu, st2, dd);
                    }
                    pV += sv2;
                    pT += st2;
                    if (first < 32) break;
                    base -= 32;
                }
                if (failed) {
                    set_status();
                    if (lane == 0) {
                        st_release(&incl[2 * k + 0], kFlagReady | kFlagFailed);
                        st_release(&incl[2 * k + 1], kFlagReady | kFlagFailed);
                    }
                    continue;
                }
                unsigned long long sv = pV + iv - lv, st = pT + it - lt;  // first of the lane's rows
                for (int u = 0; u < per; ++u) {
                    const int jj = lane * per + u;
                    if (jj < ny) {
                        const uint4 cc = __ldcg(&rowcnt[r0 + jj]);
                        starts[r0 + jj] = sv;
                        starts[R + r0 + jj] = st;
                        sv += (unsigned long long)cc.x + cc.y + cc.z;
                        st += cc.w;
                    }
                }
                __threadfence();
                if (lane == 0) {
                    st_release(&incl[2 * k + 0], kFlagReady | (pV + planeV));
                    st_release(&incl[2 * k + 1], kFlagReady | (pT + planeT));
                    if (k == nz - 1) {
                        totals[0] = pV + planeV;
                        totals[1] = pT + planeT;
                    }
                }
            }
        }

        // ---------------- generate the planes of run r - L, rows jw+h ----------------
        if (r < L) continue;
        const int kg0 = (r - L) * KC, kg1 = min(kg0 + KC, nz);
        {
            // planes kg0 .. kg1 (the one after the run: the cells' upper corners) scanned: their starts written
            unsigned long long v = 0;
            bool okg = true;
            const int kw = kg1 < nz ? kg1 : nz - 1;
            if (lane == 0)
                for (int k = kg0; okg && k <= kw; ++k)
                    okg = wait_ready(&incl[2 * k + 0], v) && wait_ready(&incl[2 * k + 1], v);
            if (!__shfl_sync(0xffffffffu, (int)okg, 0)) {
                set_status();
                continue;
            }
        }
        for (int k = kg0; k < kg1; ++k) {
            const bool hasZ = k + 1 < nz;
            const bool cellrow = hasY && hasZ;
            // first vertex and triangle after this row group's rows of plane k: every id the step writes
            // lies below them
            unsigned long long ev = 0, et = 0;
            if (lane == 0) {
                if (jw + RPW < ny) {
                    ev = __ldcg(&starts[(long long)k * ny + jw + RPW]);
                    et = __ldcg(&starts[R + (long long)k * ny + jw + RPW]);
                } else {
                    ev = ld_acquire(&incl[2 * k + 0]) & kPrefixMask;
                    et = ld_acquire(&incl[2 * k + 1]) & kPrefixMask;
                }
            }
            ev = __shfl_sync(0xffffffffu, ev, 0);
            et = __shfl_sync(0xffffffffu, et, 0);
            if ((long long)ev > capV || (long long)et > capT) break;  // and so do the later planes
            const long long rA = (long long)k * ny + j;
            uint32_t wA = 0, wB = 0, wC = 0, wD = 0;
            if (in) {
                wA = __ldcg(&bits[rA * W + lw]);
                wB = hasY ? __ldcg(&bits[(rA + 1) * W + lw]) : 0u;
                wC = hasZ ? __ldcg(&bits[(rA + ny) * W + lw]) : 0u;
                wD = cellrow ? __ldcg(&bits[(rA + ny + 1) * W + lw]) : 0u;
            }
            // first vertex of rows A = (j,k), B = (j+1,k), C = (j,k+1), D = (j+1,k+1), first triangle of cell
            // row A, x + y cuts of row B: in lane 0 of the row's lanes
            unsigned long long sA = 0, sB = 0, sC = 0, sD = 0, tA = 0;
            uint32_t cntB = 0;
            if (row_ok && lw == 0) {
                sA = __ldcg(&starts[rA]);
                tA = __ldcg(&starts[R + rA]);
                if (hasY) {
                    sB = __ldcg(&starts[rA + 1]);
                    const uint4 cb = __ldcg(&rowcnt[rA + 1]);
                    cntB = cb.x + cb.y;
                }
                if (hasZ) sC = __ldcg(&starts[rA + ny]);
                if (cellrow) sD = __ldcg(&starts[rA + ny + 1]);
            }
            const unsigned long long xsA = __shfl_sync(0xffffffffu, sA, LPR * h);
            const unsigned long long xs0 = __shfl_sync(0xffffffffu, sA, 0);  // row jw: the item's numbering
            const uint32_t dB = (uint32_t)(__shfl_sync(0xffffffffu, sB, LPR * h) - xsA);
            const uint32_t dC = (uint32_t)(__shfl_sync(0xffffffffu, sC, LPR * h) - xsA);
            const uint32_t dD = (uint32_t)(__shfl_sync(0xffffffffu, sD, LPR * h) - xsA);
            const uint32_t cntBr = __shfl_sync(0xffffffffu, cntB, LPR * h);
            const unsigned long long ts0 = __shfl_sync(0xffffffffu, tA, 0);

            RowWords rw;
            rw.a = wA;
            rw.b = wB;
            rw.c = wC;
            rw.d = wD;
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
            const uint32_t nxA = t0 & 0xffffu, nyA = t2 & 0xffffu, nxC = t1 & 0xffffu;
            const uint32_t off = (uint32_t)(xsA - xs0);  // the vertices of rows jw .. j-1
            __syncwarp();  // every lane has read the buffer of the count before the tables overwrite it
            if (in) {  // first ids of the word's cut edges, relative to xs0
                mbh[0 * W + lw] = make_uint2(m.xA, off + (e0 & 0xffffu));
                mbh[1 * W + lw] = make_uint2(m.xB, off + dB + (e0 >> 16));
                mbh[2 * W + lw] = make_uint2(m.xC, off + dC + (e1 & 0xffffu));
                mbh[3 * W + lw] = make_uint2(m.xD, off + dD + (e1 >> 16));
                mbh[4 * W + lw] = make_uint2(m.yA, off + nxA + (e2 & 0xffffu));
                mbh[5 * W + lw] = make_uint2(m.yC, off + dC + nxC + (e2 >> 16));
                mbh[6 * W + lw] = make_uint2(m.zA, off + nxA + nyA + (e3 & 0xffffu));
                mbh[7 * W + lw] = make_uint2(m.zB, off + dB + cntBr + (e3 >> 16));
                if (cellrow) {  // corner order of the cube case: bit v = corner v
                    uint4* t = reinterpret_cast<uint4*>(rwth + 8 * lw);
                    t[0] = make_uint4(rw.a, rw.ash, rw.bsh, rw.b);
                    t[1] = make_uint4(rw.c, rw.csh, rw.dsh, rw.d);
                }
            }
            __syncwarp();

            // ---- vertex records of grid row (j, k): the x, y, z cuts its word owns
            if (in) {
                auto records = [&](uint32_t mk, uint32_t first, uint32_t axis) {
                    unsigned long long idx = xs0 + first;
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
            for (uint32_t c0 = 0; c0 < tot; c0 += kGenCells) {
                // lane L takes active cell c0 + L: the first lane whose inclusive count passes it
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
                    const int bb = (int)(ci & 31u);
                    const uint32_t cs = ((lo4.x >> bb) & 1u) | (((lo4.y >> bb) & 1u) << 1) |
                                        (((lo4.z >> bb) & 1u) << 2) | (((lo4.w >> bb) & 1u) << 3) |
                                        (((hi4.x >> bb) & 1u) << 4) | (((hi4.y >> bb) & 1u) << 5) |
                                        (((hi4.z >> bb) & 1u) << 6) | (((hi4.w >> bb) & 1u) << 7);
                    rec = ch | (cs << 16);
                    cell[lane] = rec;
                }
                const int cs = (int)(rec >> 16);
                const uint32_t nt = live ? (uint32_t)iso_case_ntris(s_tri[cs]) : 0u;
                const uint32_t it = warp_incl_scan(nt, lane);
                const uint32_t ntb = __shfl_sync(0xffffffffu, it, 31);
                for (uint32_t q2 = 0; q2 < nt; ++q2) list[it - nt + q2] = (unsigned char)(lane | (q2 << 5));
                __syncwarp();
                for (uint32_t tb = 0; tb < ntb; tb += 32) {
                    const uint32_t t = tb + lane;
                    if (t < ntb) {
                        const uint32_t tr = list[t];
                        const uint32_t cr = cell[tr & 31u];
                        const int qt = (int)(tr >> 5);
                        const int ci = (int)(cr & 511u);
                        const uint2* mbc = mb + ((cr >> 9) & 7u) * 8 * W + (ci >> 5);
                        const uint32_t corners = (uint32_t)(s_tri[cr >> 16] >> (12 * qt)) & 0xfffu;
                        const int bit = ci & 31;
                        IndexT* o = tris + 3 * (tcur + t);
#pragma unroll
                        for (int cc = 0; cc < 3; ++cc) {  // fe_edge_rel with its table row and offset precomputed
                            const uint32_t nib = (corners >> (4 * cc)) & 15u;
                            const uint2 pm = mbc[(nib & 7u) * W];
                            // popc of the mask's bits below bit + offset (the funnel shift clamps at 32)
                            const int pos = bit + (int)(nib >> 3);
                            const uint32_t rel = pm.y + __popc(__funnelshift_lc(0u, pm.x, 32 - pos));
                            if constexpr (sizeof(IndexT) == 4)
                                o[cc] = (IndexT)((uint32_t)xs0 + rel);  // 32-bit ids: V < 2^32
                            else
                                o[cc] = (IndexT)(xs0 + rel);
                        }
                    }
                }
                tcur += ntb;
                __syncwarp();  // the next batch overwrites the lists
            }
        }
    }
}

bool fe_single_fits(const Grid& g, const float* vol)
{
    return g.kd == 0 && g.kr == 0 && g.ke == g.nz && g.nx >= 2 && g.ny >= 2 && g.nz >= 2 && g.W <= 16 &&
           (g.nx & 3) == 0 && (reinterpret_cast<uintptr_t>(vol) & 15) == 0;
}

size_t fe_single_flag_bytes(const Grid& g) { return single_sync_words(g) * sizeof(unsigned long long); }

template <typename IndexT>
void launch_fe_single(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                      unsigned long long* flags, int nsm, long long capV, long long capT, float* points, IndexT* tris,
                      cudaStream_t s)
{
    const int rpw = g.W <= 4 ? 8 : (g.W <= 8 ? 4 : 2);
    const int ngroups = single_groups(g, rpw);
    const long long wave = (long long)nsm * kSingleCtasPerSm;
    const long long warps_wave = wave * (kThreads / 32);
    // runs of KC planes: about four counting items per warp of one wave, at least 2 planes
    long long KC = ((long long)ngroups * g.nz + 4 * warps_wave - 1) / (4 * warps_wave);
    if (KC < 2) KC = 2;
    if (KC > 32) KC = 32;  // a warp's last-row-group planes fit one 32-bit mask
    if (KC > g.nz) KC = g.nz;
    const int nruns = (int)((g.nz + KC - 1) / KC);
    const long long citems = (long long)nruns * ngroups;
    long long blocks = (citems + kThreads / 32 - 1) / (kThreads / 32);
    if (blocks > wave) blocks = wave;
    // generation lags counting by more items than the launch's warps hold at once
    const long long warps = blocks * (kThreads / 32);
    int L = (int)((warps + ngroups - 1) / ngroups) + 2;
    if (L > nruns + 1) L = nruns + 1;
    // the status word, the item counter and the synchronisation words start at zero
    cudaMemsetAsync(b.totals + 3, 0, sizeof(unsigned long long), s);
    cudaMemsetAsync(b.totals + 7, 0, sizeof(unsigned long long), s);
    cudaMemsetAsync(flags, 0, single_sync_words(g) * sizeof(unsigned long long), s);
    const int ws_bytes = (int)single_warp_bytes(g.nx, g.W, rpw);
    const size_t smem = (size_t)(kThreads / 32) * ws_bytes;
    auto kern = rpw == 8 ? k_fe_single<IndexT, 8> : (rpw == 4 ? k_fe_single<IndexT, 4> : k_fe_single<IndexT, 2>);
    allow_smem(kern, smem);
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(vol, g, iso, (int)KC, L, ws_bytes, cases, b.rowcnt, b.bits,
                                                  b.starts, flags, b.totals, capV, capT, points, tris);
}

bool launch_fe_single_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, int nsm, long long capV,
                               long long capT, float* points, float* normals, cudaStream_t s)
{
    launch_vertices_impl<false, 0>(vol, g, iso, b, 0, g.nz, nsm, capV, capT, points, normals, s);
    return true;
}

template void launch_fe_single<uint32_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                         unsigned long long*, int, long long, long long, float*, uint32_t*,
                                         cudaStream_t);
template void launch_fe_single<uint64_t>(const float*, const Grid&, float, const CaseTables*, const FeBuffers&,
                                         unsigned long long*, int, long long, long long, float*, uint64_t*,
                                         cudaStream_t);

}  // namespace iso
