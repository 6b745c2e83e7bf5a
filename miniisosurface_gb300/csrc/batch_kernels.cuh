// Flying Edges over many requests in one launch per pass (batch.cu plans
// them; count_kernels.cu and gen_warps_fe.cu hold the kernels).
//
// Each request's parameters and buffers are a BatchReq in device memory.  A
// launch covers a list of requests: list[q] is the request, first[q] the
// launch's first block (count, scan) or work item (generate) of it, first[m]
// the launch's total.  A block or item finds its request by a binary search
// over first[] and runs the single-request code on that request's data, so
// every request's mesh is the one its own extraction writes.  The vertex
// pass walks the concatenation of the requests' vertices, vfirst[q] being
// request list[q]'s first (requests whose mesh cannot hold their counts
// contribute none).
#pragma once
#include "gen_warps.cuh"

namespace iso {

struct BatchReq {
    const float* vol;
    uint4* rowcnt;
    uint32_t* bits;
    unsigned long long* starts;
    unsigned long long* part;
    unsigned long long* totals;  // the request's 8 counters (vertices, triangles, -, status, ...)
    float* points;
    float* normals;
    void* tris;
    long long capV, capT;
    Grid g;
    GradScale gs;
    float iso;
    int count_KC, count_nyb;                // count: blocks of count_nyb row blocks x columns of count_KC planes
    int nseg;                               // scan segments
    int gen_KC, gen_ngroups, gen_nkc;       // generate: items of (row group, run of gen_KC planes)
};

// Packed output of a batch (iso_extract_batch_packed): every request's mesh in one set of buffers.
struct PackedOut {
    float* points;
    float* normals;
    void* tris;
    int index_bytes;
    long long cap_points, cap_tris;
};

// Index of the request of block or item x: the last q in [0, m) with first[q] <= x (first[0] = 0, ascending).
__device__ __forceinline__ int batch_find(const unsigned* __restrict__ first, int m, unsigned x)
{
    int lo = 0, hi = m - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&first[mid]) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Count kernel variant of a request: rows per warp (8, 4, 2), row length a multiple of 4 points, and
// every lane's word inside the row.
struct CountVariant {
    int rpw;
    bool aligned, full;
};
CountVariant count_variant(const Grid& g);
// Rows per warp of the generate pass (rows of up to 16 words).
inline int gen_rows_per_warp(int W) { return W <= 4 ? 8 : (W <= 8 ? 4 : 2); }

void launch_count_batch(const CountVariant& v, const BatchReq* reqs, const int* list, const unsigned* first, int m,
                        unsigned blocks, size_t smem, cudaStream_t s);
void launch_scan_batch(const BatchReq* reqs, const int* list, const unsigned* first, int m, unsigned blocks,
                       cudaStream_t s);
void launch_vfirst_batch(const BatchReq* reqs, const int* list, int m, unsigned long long* vfirst, cudaStream_t s);
// Packed output: places request list[q]'s mesh after those of list[0 .. q-1] (vertices and triangles), writes its
// descriptor's mesh pointers and capacities (-1 when its range ends past a capacity, or it has 2^32 vertices or
// more with 32-bit indices: it is left out) and its offsets into totals[4] and totals[5], and vfirst over the
// placed requests.
void launch_place_batch(BatchReq* reqs, const int* list, int m, const PackedOut& out, unsigned long long* vfirst,
                        cudaStream_t s);
void launch_gen_batch(int rpw, int index_bytes, const BatchReq* reqs, const int* list, const unsigned* first, int m,
                      unsigned nitems, const CaseTables* cases, unsigned* work, int ws_bytes, int reverse, int nsm,
                      cudaStream_t s);
void launch_vertices_batch(const BatchReq* reqs, const int* list, const unsigned long long* vfirst, int m, int nsm,
                           cudaStream_t s);
// Shared memory of a count block of the variant (count_buffer_floats for kCountRows warps).
size_t count_batch_smem(const Grid& g, const CountVariant& v);
// Shared memory per warp of the generate kernel for rows of W words.
size_t gen_batch_ws_bytes(int W, int rpw);

}  // namespace iso
