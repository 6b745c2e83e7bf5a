// Host-side declarations of the kernel launchers (internal to the library).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace iso {

struct Grid;
struct CaseTables;

// Scratch of one extraction (device memory, owned by the caller of the
// launchers).  Sizes for R grid rows, W words per row, T = ceil(R/256) tiles.
struct FeBuffers {
    uint32_t* bits = nullptr;              // R * W   "value >= isovalue" bits
    uint4* rowcnt = nullptr;               // R       x/y/z cuts, triangles
    uint2* trims = nullptr;                // R       xl, xr (pass 1 trims)
    uint32_t* mccnt = nullptr;             // R       MC vertices per cell row
    uint4* rowpre = nullptr;               // R       in-tile prefixes
    unsigned long long* tiles = nullptr;   // 3 * T   tile totals -> offsets
    unsigned long long* totals = nullptr;  // 3       vertices, triangles, mc vertices
    uint32_t* fe2mc = nullptr;             // capV    FE vertex index -> MC index
};

int lanes_per_row(int W);
long long num_tiles(const Grid& g);

void launch_classify(const float* vol, uint32_t* bits, const Grid& g, float iso, int nsm, cudaStream_t s);
void launch_count(const uint32_t* bits, const Grid& g, const CaseTables* cases, bool mc, FeBuffers& b,
                  cudaStream_t s);
void launch_scan_tiles(const Grid& g, FeBuffers& b, cudaStream_t s);
template <typename IndexT>
void launch_fe_generate(const float* vol, const uint32_t* bits, const Grid& g, float iso, const CaseTables* cases,
                        const FeBuffers& b, long long capV, long long capT, float* points, float* normals,
                        IndexT* tris, int nsm, cudaStream_t s);
void launch_mc_vertices(const float* vol, const uint32_t* bits, const Grid& g, float iso, const CaseTables* cases,
                        const FeBuffers& b, long long capV, long long capT, float* points, float* normals, int nsm,
                        cudaStream_t s);
template <typename IndexT>
void launch_mc_triangles(const uint32_t* bits, const Grid& g, const CaseTables* cases, const FeBuffers& b,
                         long long capV, long long capT, IndexT* tris, int nsm, cudaStream_t s);
void launch_fe_grid_edges(const Grid& g, const FeBuffers& b, int scanned, unsigned long long* ge,
                          unsigned long long* tri_counter, cudaStream_t s);

}  // namespace iso
