// Host-side declarations of the kernel launchers (internal to the library).
#pragma once
#include <mutex>
#include <unordered_map>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace iso {

struct Grid;
struct CaseTables;
struct RowStarts;

// Scratch of one extraction (device memory, owned by the caller of the
// launchers).  R = ny*nz grid rows, W = ceil(nx/32) words per row.
struct FeBuffers {
    uint4* rowcnt = nullptr;               // R      x/y/z cuts, triangles
    uint2* trims = nullptr;                // R      xl, xr (pass 1 trims)
    uint32_t* mccnt = nullptr;             // R      MC vertices per cell row
    unsigned long long* starts = nullptr;  // 4*R    per row: first vertex, triangle, MC vertex (or y, z cuts)
    unsigned long long* part = nullptr;    // 4*nseg scan segment totals
    unsigned long long* totals = nullptr;  // 8      vertices, triangles, mc vertices, status, x cuts, y cuts
    uint32_t* bits = nullptr;              // R*W    bit rows (row-wise kernels only)
    uint32_t* fe2mc = nullptr;             // >= V   FE vertex index -> MC index
};

// Work split of the counting pass: blocks of J = 8 grid rows (a warp per
// row), columns of KC planes, one CTA per (block, column); nseg segments of
// the row scans.
struct CountPlan {
    int J = 8, nyb = 1, KC = 1, nkc = 1;
    int vec_u = 1;  // float4 loads per lane for one row (rows up to 64 words)
    int nseg = 1;
    bool trims = false;  // write the row trims (only the pass-by-pass interface reads them)
};

// Work split of the warp-per-row generate kernels: blocks of J = 8 rows,
// columns of KC planes over planes [kbeg, kend).  For a slab: rows below
// kemit only map (MC), ids are shifted by add[] and stored at id - vbase
// (vertices) and t - tbase (triangles).
struct GenPlan {
    int J = 8, nyb = 1, KC = 1, nkc = 1;
    int kbeg = 0, kend = 0, kemit = 0;
    unsigned long long vbase = 0, tbase = 0;
    unsigned long long add[4] = {0, 0, 0, 0};
    size_t smem = 0;  // per-warp scratch of the CTA
    int nsm = 0;      // SMs of the device the plan is for
    bool fits = false;  // false: use the row-wise kernels
};

int lanes_per_row(int W);

// typed volumes (convert.cu): bytes per sample of an iso_dtype (0: unknown);
// n samples converted to float
size_t dtype_bytes(int dtype);
void launch_to_float(const void* in, int dtype, float* out, long long n, int nsm, cudaStream_t s);

// Opt a kernel into `dyn` bytes of dynamic shared memory (needed once the
// dynamic plus static shared memory passes the 48 KB default).  The limit
// belongs to the kernel, not to the calling thread, so it is only ever raised,
// under a lock: a thread setting a smaller limit for its own launch must not
// lower it under another thread's larger launch of the same kernel.
template <typename K>
inline void allow_smem(K kern, size_t dyn)
{
    if (dyn <= 16 * 1024) return;
    static std::mutex m;
    static std::unordered_map<const void*, size_t> raised;
    std::lock_guard<std::mutex> lock(m);
    size_t& cur = raised[reinterpret_cast<const void*>(kern)];
    if (dyn > cur && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) == cudaSuccess)
        cur = dyn;
}
CountPlan count_plan(const Grid& g, int nsm);
GenPlan gen_plan(const Grid& g, int nsm);
void gen_split(GenPlan& p, int nsm);  // columns over [p.kbeg, p.kend)

// passes 1-3
void launch_count(const float* vol, const Grid& g, float iso, const CaseTables* cases, bool mc,
                  const CountPlan& p, FeBuffers& b, cudaStream_t s);
enum ScanMode { kScanFE = 0, kScanMC = 1, kScanDup = 2 };
void launch_scan(const Grid& g, const CountPlan& p, int mode, FeBuffers& b, cudaStream_t s);
// totals and the starts of rows rlo / rhi into out[0..8] (device-visible host memory)
void launch_slab_readback(const FeBuffers& b, const Grid& g, long long rlo, long long rhi, bool has_lo, bool has_hi,
                          unsigned long long* out, cudaStream_t s);
// Marching Cubes in two passes (rows of up to 16 words, whole windows): owned
// vertices and FE-id triangles together, then the triangles' ids remapped
bool mc_fused(const Grid& g, const GenPlan& p);
template <typename IndexT>
void launch_mc_gen_tris(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                        const GenPlan& p, long long capV, long long capT, float* points, IndexT* tris, int reverse,
                        cudaStream_t s);
template <typename IndexT>
void launch_mc_remap(const FeBuffers& b, const GenPlan& p, long long capV, long long capT, IndexT* tris,
                     cudaStream_t s);

// learned output-size predictor (predictor.cu): 16^3-cell blocks
long long block_count(const Grid& g);
void launch_block_tris(const Grid& g, const uint32_t* bits, int* counts, cudaStream_t s);

void launch_grid_edges(const Grid& g, const CountPlan& p, const FeBuffers& b, int scanned, unsigned long long* ge,
                       unsigned long long* tri_counter, cudaStream_t s);
// Row-start accessor of a counted extraction.
RowStarts row_starts(const Grid& g, const CountPlan& p, const FeBuffers& b);

// pass 4, Flying Edges: rows of up to 16 words two per warp, writing vertex
// records that launch_fe_vertices turns into vertices (it returns false, and
// launches nothing, for the grids whose generate pass computes them itself)
template <typename IndexT>
void launch_fe_gen_warps(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                         const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                         float* normals, IndexT* tris, int reverse, cudaStream_t s);
// 8- and 16-bit samples read as they are (count_narrow.cu): whole grids of
// rows up to 16 words whose byte length is a multiple of 16, the volume at a
// 16-byte boundary.  The count pass over the samples, then the usual scan and
// generate pass, then the vertex pass over the same samples.
bool narrow_fits(const Grid& g, const void* vol, int dtype);
void launch_count_narrow(const void* vol, int dtype, const Grid& g, float iso, bool mc, const CountPlan& p,
                         FeBuffers& b, cudaStream_t s);
bool launch_fe_vertices_narrow(const void* vol, int dtype, const Grid& g, float iso, const FeBuffers& b,
                               const GenPlan& p, long long capV, long long capT, float* points, float* normals,
                               cudaStream_t s);
bool launch_mc_vertices_narrow(const void* vol, int dtype, const Grid& g, float iso, const FeBuffers& b,
                               const GenPlan& p, long long capV, long long capT, float* points, float* normals,
                               cudaStream_t s);
bool launch_fe_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                        long long capV, long long capT, float* points, float* normals, cudaStream_t s);
// Marching Cubes vertices from the records launch_mc_gen_warps wrote (false:
// nothing launched, the plan cannot run it)
bool launch_mc_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                        long long capV, long long capT, float* points, float* normals, cudaStream_t s);
// The duplicate-free order's vertices from the records launch_dup_gen_warps wrote (whole grids)
bool launch_dup_vertices(const float* vol, const Grid& g, float iso, const FeBuffers& b, const GenPlan& p,
                         long long capV, long long capT, float* points, float* normals, cudaStream_t s);
void launch_mc_gen_warps(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                         const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                         float* normals, int reverse, cudaStream_t s);
// pass 4 of the global-edge-index (duplicate-free) Marching Cubes order
template <typename IndexT>
void launch_dup_gen_warps(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                          const CountPlan& cp, const GenPlan& p, long long capV, long long capT, float* points,
                          float* normals, IndexT* tris, int reverse, cudaStream_t s);
template <typename IndexT>
void launch_mc_tri_warps(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                         const GenPlan& p, long long capV, long long capT, IndexT* tris, cudaStream_t s);

// pass 4, row-wise (bit rows from the count pass)
template <typename IndexT>
void launch_fe_gen_rows(const float* vol, const Grid& g, float iso, const CaseTables* cases, const FeBuffers& b,
                        const CountPlan& cp, long long capV, long long capT, float* points, float* normals,
                        IndexT* tris, int nsm, cudaStream_t s);
void launch_mc_vertices_rows(const float* vol, const Grid& g, float iso, const CaseTables* cases,
                             const FeBuffers& b, const CountPlan& cp, long long capV, long long capT, float* points,
                             float* normals, int nsm, cudaStream_t s);
template <typename IndexT>
void launch_mc_triangles(const Grid& g, const CaseTables* cases, const FeBuffers& b, const CountPlan& cp,
                         long long capV, long long capT, IndexT* tris, int nsm, cudaStream_t s);

}  // namespace iso
