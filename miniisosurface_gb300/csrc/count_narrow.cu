// Passes 1+2 of Flying Edges / the Marching Cubes counts over 8- and 16-bit
// samples read as they are: the typed-volume path of iso_extract_device_typed
// without a float32 copy of the volume (flyingEdges/util/ConvertBuffer.h:
// 45-72 converts every sample to float before extracting).
//
// The reference classifies a sample s by (float)s >= iso.  For 8- and 16-bit
// integers the conversion is exact, and for an integer s and a real iso,
// s >= iso exactly when s >= ceil(iso); so the kernel compares the integer
// sample with thr = ceil(iso) (clamped to the int range; a NaN isovalue, for
// which every comparison is false, gives INT_MAX).  The bit words, counts and
// row layout are those of k_count_tma (count_kernels.cu), so the scan and the
// generate pass that follow are unchanged; the vertex pass reads the same
// narrow samples (k_vertices with a sample type, vertices.cuh).
//
// k_count_narrow is k_count_tma for rows of up to 16 words whose byte length is
// a multiple of 16 (the volume at a 16-byte boundary): a warp's rows jw ..
// jw+RPW of a plane come into its shared buffer by one TMA bulk copy (bounded
// mbarrier wait), plane k+2 in flight while plane k is counted; each lane
// builds its own 32-point word from the buffer.
#include <climits>
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "../../include/miniiso.h"
#include "count_words.cuh"
#include "iso_kernels.h"

namespace iso {

// Bit i of the result: sample i of the 16-byte chunk v >= thr.
template <typename S>
__device__ __forceinline__ uint32_t chunk_bits(uint4 v, int thr)
{
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    uint32_t b = 0u;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if constexpr (sizeof(S) == 2) {
            const int lo = std::is_signed<S>::value ? (int)(int16_t)(w[q] & 0xffffu) : (int)(w[q] & 0xffffu);
            const int hi = std::is_signed<S>::value ? ((int)w[q] >> 16) : (int)(w[q] >> 16);
            b |= (uint32_t)(lo >= thr) << (2 * q);
            b |= (uint32_t)(hi >= thr) << (2 * q + 1);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t u = (w[q] >> (8 * e)) & 0xffu;
                const int s = std::is_signed<S>::value ? (int)(int8_t)u : (int)u;
                b |= (uint32_t)(s >= thr) << (4 * q + e);
            }
        }
    }
    return b;
}

// Word wd (samples 32*wd .. 32*wd+31) of a row of nx samples in shared
// memory, built by one lane: NV chunks of 16 bytes, read starting at chunk rot
// so that neighbouring lanes read different bank groups, rotated into place at
// the end.  FULL: every lane's word lies inside the row.
template <typename S, bool FULL>
__device__ __forceinline__ uint32_t row_word_n(const S* row, int nx, int wd, int rot, int thr)
{
    constexpr int PER = 16 / (int)sizeof(S);  // samples per chunk
    constexpr int NV = 32 / PER;              // chunks per word
    const uint4* r = reinterpret_cast<const uint4*>(row + 32 * wd);
    const int nvalid = FULL ? NV : (nx - 32 * wd) / PER;  // nx is a multiple of PER
    uint32_t w = 0u;
#pragma unroll
    for (int u = 0; u < NV; ++u) {
        const int q = (u + rot) & (NV - 1);
        if (FULL || q < nvalid) w |= chunk_bits<S>(r[q], thr) << (PER * u);
    }
    return NV == 1 ? w : __funnelshift_l(w, w, PER * rot);
}

template <bool MC, typename S, int RPW, bool FULL>
__global__ void __launch_bounds__(kThreads, 4) k_count_narrow(const S* __restrict__ vol, Grid g, int thr, int KC,
                                                           int nyb, uint4* __restrict__ rowcnt,
                                                           uint32_t* __restrict__ mccnt, uint32_t* __restrict__ bits_out,
                                                           unsigned long long* __restrict__ status)
{
    constexpr int LPR = 32 / RPW, NBUF = RPW + 1;
    constexpr int NV = 2 * (int)sizeof(S);  // 16-byte chunks per 32-point word
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ uint64_t s_bar[kCountRows];
    const int jb = blockIdx.x % nyb, kc = blockIdx.x / nyb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, h = lane / LPR, lw = lane % LPR;
    const int jw = jb * kCountRows * RPW + RPW * warp;
    if (jw >= g.ny) return;  // all the warp's rows past the grid
    S* buf = reinterpret_cast<S*>(s_raw) + (size_t)warp * NBUF * g.nx;
    uint64_t* bar = &s_bar[warp];
    if (lane == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncwarp();
    const int j = jw + h;
    const bool row_ok = j < g.ny;
    const int kb = g.kr + kc * KC, ke = min(kb + KC, g.ke);
    const bool hasY = row_ok && j < g.ny - 1;
    const int nrows = min(NBUF, g.ny - jw);
    const unsigned bytes = (unsigned)(nrows * g.nx * (int)sizeof(S));
    const int rot = lane & (NV - 1);

    auto issue = [&](int p) {
        if (lane == 0) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar, bytes);
            bulk_copy_g2s(buf, vol + ((long long)(p - g.kd) * g.ny + jw) * g.nx, bytes, bar);
        }
    };
    unsigned phase = 0;
    auto take = [&](uint32_t& wa, uint32_t& wb) -> bool {
        __syncwarp();
        const bool done = mbar_wait(bar, phase);
        if (!__all_sync(0xffffffffu, done)) return false;
        phase ^= 1u;
        wa = row_ok ? row_word_n<S, FULL>(buf + h * g.nx, g.nx, lw, rot, thr) : 0u;
        wb = hasY ? row_word_n<S, FULL>(buf + (h + 1) * g.nx, g.nx, lw, rot, thr) : 0u;
        __syncwarp();  // every lane has read the buffer before it is refilled
        return true;
    };
    // per-row totals: rows 2p, 2p+1 of the warp in the two 16-bit halves of reduction p
    auto row_sum = [&](uint32_t v) -> uint32_t {
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
        if (row_ok) count_word<MC>(rw, lw, g, j, k, hasY, hasZ, false, rc);
        const long long r = (long long)(k - g.kr) * g.ny + j;
        if (row_ok && lw < g.W) bits_out[r * g.W + lw] = rw.a;
        const uint32_t sx = row_sum(rc.xc), sy = row_sum(rc.yc), sz = row_sum(rc.zc), st = row_sum(rc.tc);
        const uint32_t sm = MC ? row_sum(rc.mc) : 0u;
        if (row_ok && lw == 0) {
            rowcnt[r] = make_uint4(sx, sy, sz, st);
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

int narrow_threshold(float iso)
{
    if (std::isnan(iso)) return INT_MAX;  // (float)s >= NaN is false for every sample
    const double c = std::ceil((double)iso);
    if (c >= (double)INT_MAX) return INT_MAX;  // above every 8- and 16-bit sample
    if (c <= (double)INT_MIN) return INT_MIN;
    return (int)c;
}

bool narrow_fits(const Grid& g, const void* vol, int dtype)
{
    const size_t sb = dtype_bytes(dtype);
    return (sb == 1 || sb == 2) && g.kd == 0 && g.kr == 0 && g.ke == g.nz && g.W <= 16 &&
           ((size_t)g.nx * sb) % 16 == 0 && (reinterpret_cast<uintptr_t>(vol) & 15) == 0;
}

template <bool MC, typename S>
static void narrow_launch(const CountPlan& p, const S* vol, const Grid& g, int thr, FeBuffers& b, cudaStream_t s)
{
    const int rpw = g.W <= 4 ? 8 : (g.W <= 8 ? 4 : 2);
    const int rows = kCountRows * rpw;
    const int nyb = (g.ny + rows - 1) / rows;
    const unsigned blocks = (unsigned)(nyb * p.nkc);
    const size_t smem = (size_t)kCountRows * (rpw + 1) * g.nx * sizeof(S);
    const bool full = g.nx == 32 * (32 / rpw);
#define ISO_NARROW(RPW, FULL)                                                                               \
    {                                                                                                       \
        auto kern = k_count_narrow<MC, S, RPW, FULL>;                                                      \
        allow_smem(kern, smem);                                                                             \
        kern<<<blocks, kThreads, smem, s>>>(vol, g, thr, p.KC, nyb, b.rowcnt, b.mccnt, b.bits, b.totals + 3); \
    }
    if (rpw == 8) {
        if (full) ISO_NARROW(8, true) else ISO_NARROW(8, false)
    } else if (rpw == 4) {
        if (full) ISO_NARROW(4, true) else ISO_NARROW(4, false)
    } else {
        if (full) ISO_NARROW(2, true) else ISO_NARROW(2, false)
    }
#undef ISO_NARROW
}

void launch_count_narrow(const void* vol, int dtype, const Grid& g, float iso, bool mc, const CountPlan& p, FeBuffers& b,
                         cudaStream_t s)
{
    cudaMemsetAsync(b.totals + 3, 0, sizeof(unsigned long long), s);  // device status
    const int thr = narrow_threshold(iso);
#define ISO_TYPE(T)                                                                   \
    {                                                                                 \
        if (mc) narrow_launch<true, T>(p, static_cast<const T*>(vol), g, thr, b, s);  \
        else narrow_launch<false, T>(p, static_cast<const T*>(vol), g, thr, b, s);    \
    }
    switch (dtype) {
        case ISO_INT8: ISO_TYPE(int8_t) break;
        case ISO_UINT8: ISO_TYPE(uint8_t) break;
        case ISO_INT16: ISO_TYPE(int16_t) break;
        default: ISO_TYPE(uint16_t) break;
    }
#undef ISO_TYPE
}

}  // namespace iso
