// Pass 4 vertex values from records (included by gen_warps_fe.cu through
// gen_pairs.cuh and by gen_warps_mc.cu).
//
// The generate kernels do not compute vertices: for every vertex they write a
// record into the first 8 bytes of its own 12-byte slot of the points buffer,
// and k_vertices -- one thread per slot, many warps per SM to cover the
// latency of the volume gathers -- turns each record into the vertex's point
// and normal in place.  Flying Edges records (put_vertex_record) hold the
// edge's lower point and axis; the cube that places the vertex is the edge's
// own index along the axis and the clamped one across (Image3D::getPosCube).
// Marching Cubes records (put_mc_record) add the offset of that point from the
// owner cell, whose cube places it (marchingCubes/serial/main.cpp:139-177).
#pragma once
#include "gen_warps.cuh"

namespace iso {

// Flying Edges vertex record: word 0 = i | axis << 10 | (j & 0xfffff) << 12,
// word 1 = j >> 20 | k << 8 (i < 1024, j < 2^28, k < 2^24).
__device__ __forceinline__ void put_vertex_record(float* points, unsigned long long idx, uint32_t i, uint32_t axis,
                                                  uint32_t j, uint32_t k)
{
    uint32_t* r = reinterpret_cast<uint32_t*>(points) + 3 * idx;
    r[0] = i | (axis << 10) | ((j & 0xfffffu) << 12);
    r[1] = (j >> 20) | (k << 8);
}

// edge_vertex() of iso_device.cuh for the edge from P0 = (i, j, kk) along
// axis a, placed by the cube with base (ci, cj, ck): the gradients at both
// ends from their six neighbours (grad_axis per axis, the edge's own values
// along a) and the position from the cube's corner coordinates, with the
// operations of vertex_axis<a> on the same operands, so bit-identical to it
// and to edge_vertex; written once for all three axes with the axis as data: a
// warp of consecutive vertex ids mixes axes without diverging.
// A sample as the reference sees it: converted to float by a C cast
// (flyingEdges/util/ConvertBuffer.h:45-72; exact for 8- and 16-bit samples).
template <typename S>
__device__ __forceinline__ float sample(const S* p)
{
    return (float)__ldg(p);
}

template <typename S>
__device__ __forceinline__ void vertex_any_axis(const S* __restrict__ vol, const Grid& g, const GradScale& gs,
                                                float iso, int a, int i, int j, int kk, int ci, int cj, int ck,
                                                float3& pos, float3& nrm)
{
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const S* p0 = vol + ((long long)(kk - g.kd) * g.ny + j) * g.nx + i;
    const S* p1 = p0 + (a == 0 ? 1 : (a == 1 ? sy : sz));
    const int i1 = i + (a == 0), j1 = j + (a == 1), k1 = kk + (a == 2);
    const float v0 = sample(p0), v1 = sample(p1);
    // neighbours of P0 and P1 = P0 + e_a; the edge's own values stand in along a
    const float xm0 = i > 0 ? sample(p0 - 1) : 0.f;
    const float xp0 = a == 0 ? v1 : (i < g.nx - 1 ? sample(p0 + 1) : 0.f);
    const float ym0 = j > 0 ? sample(p0 - sy) : 0.f;
    const float yp0 = a == 1 ? v1 : (j < g.ny - 1 ? sample(p0 + sy) : 0.f);
    const float zm0 = kk > 0 ? sample(p0 - sz) : 0.f;
    const float zp0 = a == 2 ? v1 : (kk < g.nz - 1 ? sample(p0 + sz) : 0.f);
    const float xm1 = a == 0 ? v0 : (i1 > 0 ? sample(p1 - 1) : 0.f);
    const float xp1 = i1 < g.nx - 1 ? sample(p1 + 1) : 0.f;
    const float ym1 = a == 1 ? v0 : (j1 > 0 ? sample(p1 - sy) : 0.f);
    const float yp1 = j1 < g.ny - 1 ? sample(p1 + sy) : 0.f;
    const float zm1 = a == 2 ? v0 : (k1 > 0 ? sample(p1 - sz) : 0.f);
    const float zp1 = k1 < g.nz - 1 ? sample(p1 + sz) : 0.f;
    const float3 g0 = grad3(xm0, xp0, ym0, yp0, zm0, zp0, v0, i, j, kk, g, gs);
    const float3 g1 = grad3(xm1, xp1, ym1, yp1, zm1, zp1, v1, i1, j1, k1, g, gs);
    const float w = fdiv(fsub(iso, v0), fsub(v1, v0));
    pos.x = lerp_ref(cube_coord(ci, i - ci, g.zp[0], g.sp[0]), cube_coord(ci, i1 - ci, g.zp[0], g.sp[0]), w);
    pos.y = lerp_ref(cube_coord(cj, j - cj, g.zp[1], g.sp[1]), cube_coord(cj, j1 - cj, g.zp[1], g.sp[1]), w);
    pos.z = lerp_ref(cube_coord(ck, kk - ck, g.zp[2], g.sp[2]), cube_coord(ck, k1 - ck, g.zp[2], g.sp[2]), w);
    nrm.x = lerp_ref(g0.x, g1.x, w);
    nrm.y = lerp_ref(g0.y, g1.y, w);
    nrm.z = lerp_ref(g0.z, g1.z, w);
}

// One wave of vertex_ctas_per_sm(MC) CTAs per SM walks the slots with a
// stride; each thread loads the record of its next slot before it works on the
// current one, so the record's trip to memory overlaps the volume gathers.
// (The Marching Cubes record takes a few more registers to decode: 5 CTAs.)
__host__ __device__ constexpr int vertex_ctas_per_sm(bool mc) { return mc ? 5 : 6; }

__device__ __forceinline__ uint2 vertex_record(const float* points, unsigned long long v)
{
    const uint32_t* r = reinterpret_cast<const uint32_t*>(points) + 3 * v;
    return make_uint2(r[0], r[1]);
}

// The vertices owned by the rows of planes [kbeg, kend) -- Flying Edges: grid
// rows (starts component COMP = 0); Marching Cubes: cell rows (COMP = 2; the
// duplicate-free order, whole grids only, counts all of them with COMP = 0)
// -- one thread each, slot v = vertex vbase + v.  MC: the records carry the
// owner cell.  The capacity test is the generate kernels': when it fails they
// wrote no record and nothing is read here.
// The vertex of slot v from its record r (k_vertices, and the batch kernel of gen_warps_fe.cu).
template <bool MC, typename S>
__device__ __forceinline__ void vertex_of_record(const S* __restrict__ vol, const Grid& g, const GradScale& gs,
                                                 float iso, int kbeg, int kend, uint2 r, unsigned long long v,
                                                 float* __restrict__ points, float* __restrict__ normals)
{
    {
        const int i = (int)(r.x & 1023u), a = (int)((r.x >> 10) & 3u);
        int j, kk, ci, cj, ck;
        if (MC) {
            const int d = (int)((r.x >> 12) & 7u);
            j = (int)((r.x >> 15) | ((r.y & 0x3ffu) << 17));
            kk = (int)(r.y >> 10);
            ci = i - (d & 1);
            cj = j - ((d >> 1) & 1);
            ck = kk - (d >> 2);
        } else {
            j = (int)((r.x >> 12) | ((r.y & 0xffu) << 20));
            kk = (int)(r.y >> 8);
            ci = a == 0 ? i : min(i, g.nx - 2);
            cj = a == 1 ? j : min(j, g.ny - 2);
            ck = a == 2 ? kk : min(kk, g.nz - 2);
        }
        // every slot holds a record of the launch's rows; anything else is left alone, never read through
        if (a > 2 || i + (a == 0) >= g.nx || j + (a == 1) >= g.ny || kk + (a == 2) >= g.nz || ci < 0 || cj < 0 ||
            ck < 0 || ci > g.nx - 2 || cj > g.ny - 2 || (MC ? (ck < kbeg || ck >= kend) : (kk < kbeg || kk >= kend)))
            return;
        float3 p, nm;
        vertex_any_axis<S>(vol, g, gs, iso, a, i, j, kk, ci, cj, ck, p, nm);
        store_vertex(points, normals, v, p, nm);
    }
}

template <bool MC, int COMP, typename S = float>
__global__ void __launch_bounds__(kThreads, vertex_ctas_per_sm(MC))
    k_vertices(const S* __restrict__ vol, Grid g, GradScale gs, float iso, int kbeg, int kend,
               const unsigned long long* __restrict__ starts, const unsigned long long* __restrict__ totals,
               long long capV, long long capT, float* __restrict__ points, float* __restrict__ normals)
{
    if ((long long)totals[0] > capV || (long long)totals[1] > capT) return;
    auto first = [&](int p) { return p < g.ke ? starts[COMP * g.R + (long long)(p - g.kr) * g.ny] : totals[COMP]; };
    const unsigned long long n = first(kend) - first(kbeg);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    uint2 next = v < n ? vertex_record(points, v) : make_uint2(0u, 0u);
    for (; v < n; v += stride) {
        const uint2 r = next;
        if (v + stride < n) next = vertex_record(points, v + stride);  // this thread's next slot
        vertex_of_record<MC, S>(vol, g, gs, iso, kbeg, kend, r, v, points, normals);
    }
}


// Vertices of the rows of planes [k0, k1) from their records.
template <bool MC, int COMP, typename S = float>
inline void launch_vertices_impl(const S* vol, const Grid& g, float iso, const FeBuffers& b, int k0, int k1,
                                 int nsm, long long capV, long long capT, float* points, float* normals,
                                 cudaStream_t s)
{
    if (k1 <= k0 || capV <= 0) return;
    // one wave, or fewer CTAs when the mesh cannot hold that many vertices (small grids in a batch)
    const long long wave = (long long)nsm * vertex_ctas_per_sm(MC);
    const unsigned blocks = (unsigned)std::min(wave, (capV + kThreads - 1) / kThreads);
    k_vertices<MC, COMP, S><<<blocks, kThreads, 0, s>>>(vol, g, make_grad_scale(g), iso, k0, k1, b.starts, b.totals, capV,
                                               capT, points, normals);
}

}  // namespace iso
