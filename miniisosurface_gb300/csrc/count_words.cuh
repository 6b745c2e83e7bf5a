// Counting helpers shared by the count kernels (count_kernels.cu) and the
// count kernel for 8- and 16-bit samples (count_narrow.cu): a row's counts
// word by word (cut x, y, z edges, trims, triangles and Marching Cubes
// vertices of its cells) and a row's bit words built from a shared-memory
// copy of the row.
#pragma once
#include "iso_device.cuh"

namespace iso {

constexpr int kCountRows = 8;  // warps per CTA of the count kernels

// Counts of one grid row, accumulated word by word in each lane.
struct RowCounts {
    uint32_t xc = 0, yc = 0, zc = 0, tc = 0, mc = 0, first = 0xffffffffu, last = 0;
};

// Counts of word w of grid row (j,k): cut x / y / z edges the row owns, the
// trim candidates, the triangles (and MC vertices) of its cells.
// trims: whether the row trims are wanted (only the pass-by-pass interface
// reads them; an extraction skips them).
template <bool MC>
__device__ __forceinline__ void count_word(const RowWords& rw, int w, const Grid& g, int j, int k, bool hasY,
                                           bool hasZ, bool trims, RowCounts& rc)
{
    const uint32_t evalid = validmask(w, g.nx - 1);  // x-edges / cells: i <= nx-2
    const uint32_t pvalid = validmask(w, g.nx);      // points: i <= nx-1
    const uint32_t xm = (rw.a ^ rw.ash) & evalid;
    const uint32_t ym = hasY ? ((rw.a ^ rw.b) & pvalid) : 0u;
    const uint32_t zm = hasZ ? ((rw.a ^ rw.c) & pvalid) : 0u;
    rc.xc += __popc(xm);
    rc.yc += __popc(ym);
    rc.zc += __popc(zm);
    // isCutEdge (FlyingEdgesAlgorithm.cpp:515-554): edge i is marked when
    // it is cut or the y / z edge at its left point is.
    const uint32_t marked = trims ? (xm | ((ym | zm) & evalid)) : 0u;
    if (marked) {
        rc.first = min(rc.first, (uint32_t)(32 * w + __ffs(marked) - 1));
        rc.last = max(rc.last, (uint32_t)(32 * w + 32 - __clz(marked)));
    }
    if (hasY && hasZ) {  // all 32 cells at once (tris_of_word, mc_verts_of_word)
        rc.tc += tris_of_word(rw.a, rw.ash, rw.bsh, rw.b, rw.c, rw.csh, rw.dsh, rw.d, evalid);
        if (MC) rc.mc += mc_verts_of_word(rw.a, rw.ash, rw.bsh, rw.b, rw.c, rw.csh, rw.dsh, rw.d, evalid, j == 0, k == 0,
                                          w == 0);
    }
}

// All ones when v >= iso, else zero (false for NaN; -0 >= +0), one ALU op.
__device__ __forceinline__ uint32_t ge_mask(float v, float iso)
{
    uint32_t d;
    asm("set.ge.u32.f32 %0, %1, %2;" : "=r"(d) : "f"(v), "f"(iso));
    return d;
}

// Word wd (points 32*wd .. 32*wd+31) of a row of nq float4 in shared
// memory, built by one lane alone: at step u it reads float4 (u + rot) & 7 of
// its word into bits 4u .. 4u+3 (rot = the lane's place in its group of eight,
// so eight consecutive lanes read eight different bank groups), and the word
// is rotated into place at the end.  FULL: every lane's word lies inside the
// row.
template <bool FULL>
__device__ __forceinline__ uint32_t row_word(const float* row, int nq, int wd, int rot, float iso)
{
    const float4* r4 = reinterpret_cast<const float4*>(row) + 8 * wd;
    const int nv = FULL ? 8 : nq - 8 * wd;  // float4 of the word inside the row
    uint32_t w = 0u;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int q = (u + rot) & 7;
        if (FULL || q < nv) {
            const float4 v = r4[q];
            w |= ge_mask(v.x, iso) & (1u << (4 * u));
            w |= ge_mask(v.y, iso) & (2u << (4 * u));
            w |= ge_mask(v.z, iso) & (4u << (4 * u));
            w |= ge_mask(v.w, iso) & (8u << (4 * u));
        }
    }
    return __funnelshift_l(w, w, 4 * rot);
}

}  // namespace iso
