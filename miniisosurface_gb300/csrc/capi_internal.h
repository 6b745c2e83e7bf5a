// Internal to the C ABI's translation units (capi.cu, batch.cu): the context
// and the helpers both use.
#pragma once
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/miniiso.h"
#include "iso_device.cuh"
#include "iso_kernels.h"

using iso::CaseTables;
using iso::FeBuffers;
using iso::Grid;

struct iso_ctx {
    int device = 0;
    int nsm = 0;
    CaseTables* d_cases = nullptr;
    // scratch of the one-shot entry points
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t* fe2mc = nullptr;
    long long fe2mc_cap = 0;
    // staging for the host entry points
    float* d_volume = nullptr;
    size_t d_volume_bytes = 0;
    float* d_points = nullptr;
    float* d_normals = nullptr;
    void* d_tris = nullptr;
    long long d_cap_points = 0, d_cap_tris = 0;
    int d_index_bytes = 0;
    unsigned long long* h_totals = nullptr;  // pinned, 4 entries
    unsigned long long* h_slab = nullptr;    // pinned and mapped, 2 x 9 entries (slab counts)
    unsigned long long* h_slab_dev = nullptr;  // its device address (written by k_slab_readback)
    void* scratch_b = nullptr;               // second scratch set (streamed path: the next slab's counts)
    size_t scratch_b_bytes = 0;
    void* d_typed = nullptr;                 // typed volume samples before conversion
    size_t d_typed_bytes = 0;
    // streamed host entry point: copy streams, events, two device staging meshes
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr, s_cnt = nullptr;  // copies in / out, slab counts
    std::vector<cudaEvent_t> sync_events;
    float* st_points[2] = {nullptr, nullptr};
    float* st_normals[2] = {nullptr, nullptr};
    void* st_tris[2] = {nullptr, nullptr};
    long long st_cap_points = 0, st_cap_tris = 0;
    int st_index_bytes = 0;
    // batched entry point (iso_extract_batch): lanes, their scratch, the captured graph
    int batch_lanes = 0;        // set by iso_batch_set_lanes; 0: the autotuner's choice
    int batch_tuned = 0;        // lanes the autotuner picked (0: not yet tuned)
    int batch_graph = 1;        // capture batches as CUDA graphs (0: launch the lanes directly)
    // iso_extract_device_async as a replayed CUDA graph (iso_ctx_set_graph)
    int one_graph = 0;
    cudaGraphExec_t one_exec = nullptr;
    std::vector<unsigned char> one_key;
    int batch_share = 0;        // set by iso_batch_set_split: a request's plans assume nsm / share SMs; 0: tuned
    int batch_tuned_share = 0;  // the autotuner's share (0: not yet tuned)
    cudaStream_t s_capture = nullptr;
    std::vector<cudaStream_t> lane_streams;
    std::vector<cudaEvent_t> lane_join;
    cudaEvent_t batch_fork = nullptr, batch_t0 = nullptr, batch_t1 = nullptr;
    void* batch_arena = nullptr;
    size_t batch_arena_bytes = 0;
    unsigned long long* h_batch = nullptr;  // pinned: 8 counters per request
    size_t h_batch_n = 0;
    // executable graphs of iso_extract_batch [0] and iso_count_batch [1], and what each was captured for
    cudaGraphExec_t batch_exec[2] = {nullptr, nullptr};
    std::vector<unsigned char> batch_key[2];
    int batch_fused = 1;  // iso_batch_set_fused: 0 lanes only, 1 fused from kFuseMin requests, 2 always fused
    int fused_kc = 0, fused_ipw = 0;  // the autotuner's fused work split (0: not yet tuned)
    unsigned char* h_fused = nullptr;  // pinned: the fused requests' descriptors and launch lists, copied in per run
    size_t h_fused_bytes = 0;
    std::vector<cudaStream_t> fused_streams;  // the fused launches of one pass side by side, and their joins
    std::vector<cudaEvent_t> fused_join;
    cudaEvent_t fused_fork = nullptr;
    int reverse = 1;  // pass 4 walks the planes backwards (the count pass leaves the last ones in L2)
    int narrow = 1;   // iso_extract_device_typed reads 8- and 16-bit samples as they are (iso_ctx_set_narrow)
    int stream_host = 1;  // iso_extract_host streams slabs (large grids)
    std::string last_error;
    // per-pass timing (iso_ctx_profile)
    bool profiling = false;
    std::vector<cudaEvent_t> event_pool;
    size_t events_used = 0;
    struct Span { int pass; cudaEvent_t begin, end; };
    std::vector<Span> spans;
};

namespace capi {

inline iso_status cuda_fail(iso_ctx* ctx, cudaError_t e, const char* what)
{
    if (ctx) {
        ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return e == cudaErrorMemoryAllocation ? ISO_ERR_OOM : ISO_ERR_CUDA;
}

#define ISO_CUDA(ctx, call)                                      \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Derived per-case tables: the packed triangle lists, the first-appearance
// edge order (marching cubes numbering) and the cut-edge masks.
inline void build_case_tables(CaseTables& t)
{
    for (int c = 0; c < 256; ++c) {
        const uint64_t w = kIsoCaseTris[c];
        t.tris[c] = w;
        uint16_t cut = 0;
        for (int e = 0; e < 12; ++e) {
            if (((c >> kIsoEdgeLo[e]) & 1) != ((c >> kIsoEdgeHi[e]) & 1)) cut |= (uint16_t)(1u << e);
        }
        t.cut[c] = cut;
        uint64_t order = 0;
        int n = 0;
        uint16_t seen = 0;
        for (int q = 0; q < 3 * iso_case_ntris(w); ++q) {
            const int e = iso_case_edge(w, q);
            if (!((seen >> e) & 1)) {
                seen |= (uint16_t)(1u << e);
                order |= (uint64_t)e << (4 * n);
                ++n;
            }
        }
        t.order[c] = order | ((uint64_t)n << 60);
    }
}

inline bool valid_algo(iso_algorithm a)
{
    return a == ISO_FLYING_EDGES || a == ISO_MARCHING_CUBES || a == ISO_MC_DUPFREE;
}

inline bool make_grid(const iso_grid* gr, Grid& g)
{
    for (int a = 0; a < 3; ++a) {
        if (gr->dims[a] < 1 || gr->dims[a] > (1ll << 30)) return false;
    }
    g.nx = (int)gr->dims[0];
    g.ny = (int)gr->dims[1];
    g.nz = (int)gr->dims[2];
    g.W = (g.nx + 31) / 32;
    g.R = (long long)g.ny * g.nz;
    if ((long long)g.W * g.R > (1ll << 40)) return false;
    g.kd = 0;
    g.kr = 0;
    g.ke = g.nz;
    for (int a = 0; a < 3; ++a) {
        g.sp[a] = gr->spacing[a];
        g.zp[a] = gr->origin[a];
    }
    return true;
}

inline bool empty_grid(const Grid& g) { return g.nx < 2 || g.ny < 2 || g.nz < 2; }

inline size_t scratch_size(const Grid& g, const iso::CountPlan& cp)
{
    const size_t R = (size_t)g.R;
    return align256(R * 16) + align256(R * 8) + align256(R * 4) + align256(4 * R * 8) +
           align256(4 * (size_t)cp.nseg * 8) + align256(8 * 8) + align256(R * (size_t)g.W * 4);
}

inline void carve(void* base, const Grid& g, const iso::CountPlan& cp, FeBuffers& b)
{
    const size_t R = (size_t)g.R;
    char* p = static_cast<char*>(base);
    b.rowcnt = reinterpret_cast<uint4*>(p); p += align256(R * 16);
    b.trims = reinterpret_cast<uint2*>(p); p += align256(R * 8);
    b.mccnt = reinterpret_cast<uint32_t*>(p); p += align256(R * 4);
    b.starts = reinterpret_cast<unsigned long long*>(p); p += align256(4 * R * 8);
    b.part = reinterpret_cast<unsigned long long*>(p); p += align256(4 * (size_t)cp.nseg * 8);
    b.totals = reinterpret_cast<unsigned long long*>(p); p += align256(8 * 8);
    b.bits = reinterpret_cast<uint32_t*>(p);
}

inline iso_status ensure_scratch(iso_ctx* ctx, const Grid& g, const iso::CountPlan& cp, FeBuffers& b, cudaStream_t s)
{
    const size_t need = scratch_size(g, cp);
    if (need > ctx->scratch_bytes) {
        if (ctx->scratch) {
            ISO_CUDA(ctx, cudaStreamSynchronize(s));
            cudaFree(ctx->scratch);
            ctx->scratch = nullptr;
            ctx->scratch_bytes = 0;
        }
        const size_t alloc = need + need / 4;
        ISO_CUDA(ctx, cudaMalloc(&ctx->scratch, alloc));
        ctx->scratch_bytes = alloc;
    }
    carve(ctx->scratch, g, cp, b);
    b.fe2mc = ctx->fe2mc;
    return ISO_OK;
}

// Device buffer for typed samples before their conversion to float.
inline iso_status ensure_typed(iso_ctx* ctx, size_t bytes, cudaStream_t s)
{
    if (bytes <= ctx->d_typed_bytes) return ISO_OK;
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    cudaFree(ctx->d_typed);
    ctx->d_typed = nullptr;
    ctx->d_typed_bytes = 0;
    ISO_CUDA(ctx, cudaMalloc(&ctx->d_typed, bytes));
    ctx->d_typed_bytes = bytes;
    return ISO_OK;
}

// The second scratch set (the streamed path counts slab q+1 while slab q
// is generated from the first).
inline iso_status ensure_scratch_b(iso_ctx* ctx, const Grid& g, const iso::CountPlan& cp, FeBuffers& b, cudaStream_t s)
{
    const size_t need = scratch_size(g, cp);
    if (need > ctx->scratch_b_bytes) {
        if (ctx->scratch_b) {
            ISO_CUDA(ctx, cudaStreamSynchronize(s));
            cudaFree(ctx->scratch_b);
            ctx->scratch_b = nullptr;
            ctx->scratch_b_bytes = 0;
        }
        const size_t alloc = need + need / 4;
        ISO_CUDA(ctx, cudaMalloc(&ctx->scratch_b, alloc));
        ctx->scratch_b_bytes = alloc;
    }
    carve(ctx->scratch_b, g, cp, b);
    b.fe2mc = ctx->fe2mc;
    return ISO_OK;
}

inline iso_status ensure_fe2mc(iso_ctx* ctx, long long cap, cudaStream_t s)
{
    if (cap > ctx->fe2mc_cap) {
        if (ctx->fe2mc) {
            ISO_CUDA(ctx, cudaStreamSynchronize(s));
            cudaFree(ctx->fe2mc);
            ctx->fe2mc = nullptr;
            ctx->fe2mc_cap = 0;
        }
        const long long alloc = cap + cap / 4 + 1024;
        ISO_CUDA(ctx, cudaMalloc(&ctx->fe2mc, (size_t)alloc * 4));
        ctx->fe2mc_cap = alloc;
    }
    return ISO_OK;
}

inline iso_status check_mesh(const iso_mesh* m)
{
    if (!m) return ISO_ERR_INVALID_ARG;
    if (m->index_bytes != 4 && m->index_bytes != 8) return ISO_ERR_INVALID_ARG;
    if (m->cap_points < 0 || m->cap_tris < 0) return ISO_ERR_INVALID_ARG;
    if (m->cap_points > 0 && (!m->points || !m->normals)) return ISO_ERR_INVALID_ARG;
    if (m->cap_tris > 0 && !m->tris) return ISO_ERR_INVALID_ARG;
    return ISO_OK;
}

// Largest vertex count a mesh may hold (32-bit indices address < 2^32).
inline long long vertex_limit(const iso_mesh* m, long long cap)
{
    const long long lim = m->index_bytes == 4 ? 0xffffffffll : (1ll << 62);
    return cap < lim ? cap : lim;
}

// Events between consecutive kernels while profiling.
inline cudaEvent_t next_event(iso_ctx* ctx)
{
    if (ctx->events_used == ctx->event_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->event_pool.push_back(e);
    }
    return ctx->event_pool[ctx->events_used++];
}

struct PassMarks {
    iso_ctx* ctx;
    cudaStream_t s;
    cudaEvent_t last = nullptr;
    PassMarks(iso_ctx* c, cudaStream_t st) : ctx(c), s(st)
    {
        if (ctx->profiling && (last = next_event(ctx))) cudaEventRecord(last, s);
    }
    void mark(int pass)
    {
        if (!ctx->profiling || !last) return;
        cudaEvent_t e = next_event(ctx);
        if (!e) return;
        cudaEventRecord(e, s);
        ctx->spans.push_back({pass, last, e});
        last = e;
    }
};

// Plans of one extraction.
struct Plans {
    iso::CountPlan cp;
    iso::GenPlan gp;
};

inline Plans make_plans(const iso_ctx* ctx, const Grid& g, int nsm = 0)
{
    Plans p;
    const int n = nsm > 0 ? nsm : ctx->nsm;
    p.cp = iso::count_plan(g, n);
    p.gp = iso::gen_plan(g, n);
    return p;
}

// Passes 1-3: counts, scan, row starts.
inline void enqueue_count(iso_ctx* ctx, iso_algorithm algo, const float* vol, const Grid& g, float iso, const Plans& pl,
                   FeBuffers& b, cudaStream_t s, PassMarks& pm)
{
    const bool mc = algo == ISO_MARCHING_CUBES;
    iso::launch_count(vol, g, iso, ctx->d_cases, mc, pl.cp, b, s);
    pm.mark(ISO_PASS_COUNT);
    iso::launch_scan(g, pl.cp, algo == ISO_MC_DUPFREE ? iso::kScanDup : (mc ? iso::kScanMC : iso::kScanFE), b, s);
    pm.mark(ISO_PASS_SCAN);
}

// Pass 4 into the mesh buffers of `out` (device memory).
inline void enqueue_generate(iso_ctx* ctx, iso_algorithm algo, const float* vol, const Grid& g, float iso, const Plans& pl,
                      const FeBuffers& b, const iso_mesh* out, cudaStream_t s, PassMarks& pm)
{
    const long long capV = vertex_limit(out, out->cap_points);
    const long long capT = out->cap_tris;
    const bool i4 = out->index_bytes == 4;
    if (algo == ISO_FLYING_EDGES) {
        if (pl.gp.fits) {
            if (i4)
                iso::launch_fe_gen_warps<uint32_t>(vol, g, iso, ctx->d_cases, b, pl.cp, pl.gp, capV, capT, out->points,
                                                   out->normals, static_cast<uint32_t*>(out->tris), ctx->reverse, s);
            else
                iso::launch_fe_gen_warps<uint64_t>(vol, g, iso, ctx->d_cases, b, pl.cp, pl.gp, capV, capT, out->points,
                                                   out->normals, static_cast<uint64_t*>(out->tris), ctx->reverse, s);
            pm.mark(ISO_PASS_FE_GENERATE);
            if (iso::launch_fe_vertices(vol, g, iso, b, pl.gp, capV, capT, out->points, out->normals, s))
                pm.mark(ISO_PASS_VERTICES);
            return;
        } else {
            if (i4)
                iso::launch_fe_gen_rows<uint32_t>(vol, g, iso, ctx->d_cases, b, pl.cp, capV, capT, out->points, out->normals,
                                                  static_cast<uint32_t*>(out->tris), ctx->nsm, s);
            else
                iso::launch_fe_gen_rows<uint64_t>(vol, g, iso, ctx->d_cases, b, pl.cp, capV, capT, out->points, out->normals,
                                                  static_cast<uint64_t*>(out->tris), ctx->nsm, s);
        }
        pm.mark(ISO_PASS_FE_GENERATE);
    } else if (algo == ISO_MC_DUPFREE) {  // vertices and triangles in one pass (make_plans checked fits)
        if (i4)
            iso::launch_dup_gen_warps<uint32_t>(vol, g, iso, ctx->d_cases, b, pl.cp, pl.gp, capV, capT, out->points,
                                                out->normals, static_cast<uint32_t*>(out->tris), ctx->reverse, s);
        else
            iso::launch_dup_gen_warps<uint64_t>(vol, g, iso, ctx->d_cases, b, pl.cp, pl.gp, capV, capT, out->points,
                                                out->normals, static_cast<uint64_t*>(out->tris), ctx->reverse, s);
        pm.mark(ISO_PASS_MC_VERTICES);
        if (iso::launch_dup_vertices(vol, g, iso, b, pl.gp, capV, capT, out->points, out->normals, s))
            pm.mark(ISO_PASS_VERTICES);
    } else {
        const long long capM = capV < 0xffffffffll ? capV : 0xffffffffll;  // fe2mc holds 32-bit ids
        if (pl.gp.fits && iso::mc_fused(g, pl.gp)) {  // owned vertices + FE-id triangles, vertices, remap
            if (i4)
                iso::launch_mc_gen_tris<uint32_t>(g, ctx->d_cases, b, pl.cp, pl.gp, capM, capT, out->points,
                                                  static_cast<uint32_t*>(out->tris), ctx->reverse, s);
            else
                iso::launch_mc_gen_tris<uint64_t>(g, ctx->d_cases, b, pl.cp, pl.gp, capM, capT, out->points,
                                                  static_cast<uint64_t*>(out->tris), ctx->reverse, s);
            pm.mark(ISO_PASS_MC_VERTICES);
            if (iso::launch_mc_vertices(vol, g, iso, b, pl.gp, capM, capT, out->points, out->normals, s))
                pm.mark(ISO_PASS_VERTICES);
            if (i4)
                iso::launch_mc_remap<uint32_t>(b, pl.gp, capM, capT, static_cast<uint32_t*>(out->tris), s);
            else
                iso::launch_mc_remap<uint64_t>(b, pl.gp, capM, capT, static_cast<uint64_t*>(out->tris), s);
            pm.mark(ISO_PASS_MC_TRIANGLES);
            return;
        }
        if (pl.gp.fits)
            iso::launch_mc_gen_warps(vol, g, iso, ctx->d_cases, b, pl.cp, pl.gp, capM, capT, out->points, out->normals,
                                     ctx->reverse, s);
        else
            iso::launch_mc_vertices_rows(vol, g, iso, ctx->d_cases, b, pl.cp, capM, capT, out->points, out->normals,
                                         ctx->nsm, s);
        pm.mark(ISO_PASS_MC_VERTICES);
        if (pl.gp.fits && iso::launch_mc_vertices(vol, g, iso, b, pl.gp, capM, capT, out->points, out->normals, s))
            pm.mark(ISO_PASS_VERTICES);
        if (pl.gp.fits) {
            if (i4)
                iso::launch_mc_tri_warps<uint32_t>(g, ctx->d_cases, b, pl.cp, pl.gp, capM, capT,
                                                   static_cast<uint32_t*>(out->tris), s);
            else
                iso::launch_mc_tri_warps<uint64_t>(g, ctx->d_cases, b, pl.cp, pl.gp, capM, capT,
                                                   static_cast<uint64_t*>(out->tris), s);
        } else {
            if (i4)
                iso::launch_mc_triangles<uint32_t>(g, ctx->d_cases, b, pl.cp, capM, capT,
                                                   static_cast<uint32_t*>(out->tris), ctx->nsm, s);
            else
                iso::launch_mc_triangles<uint64_t>(g, ctx->d_cases, b, pl.cp, capM, capT,
                                                   static_cast<uint64_t*>(out->tris), ctx->nsm, s);
        }
        pm.mark(ISO_PASS_MC_TRIANGLES);
    }
}

inline iso_status finish_counts(iso_ctx* ctx, const iso_mesh* out, long long V, long long T, long long status, int64_t* nV,
                         int64_t* nT)
{
    *nV = V;
    *nT = T;
    if (status != 0) {
        ctx->last_error = "a device-side wait timed out";
        return ISO_ERR_TIMEOUT;
    }
    if (out && out->index_bytes == 4 && V > 0xffffffffll) {
        ctx->last_error = "more than 2^32-1 vertices: use 64-bit indices";
        return ISO_ERR_OVERFLOW;
    }
    if (out && (V > out->cap_points || T > out->cap_tris)) {
        ctx->last_error = "output buffers too small";
        return ISO_ERR_CAPACITY;
    }
    return ISO_OK;
}

// iso_extract_device_async in graph mode (batch.cu).
iso_status extract_graph(iso_ctx* ctx, iso_algorithm algo, const float* volume, const Grid& g, const iso_grid* grid,
                         float isoval, const Plans& pl, FeBuffers& b, const iso_mesh* out, int64_t* result_host,
                         cudaStream_t s);

}  // namespace capi
