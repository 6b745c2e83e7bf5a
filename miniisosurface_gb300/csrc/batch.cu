// C ABI of the batched extraction and of graph mode (iso_extract_batch,
// iso_count_batch, iso_batch_*, iso_ctx_set_graph) and the exact per-block
// triangle counts of the output-size network (iso_block_tris).
#include <map>

#include "batch_kernels.cuh"
#include "capi_internal.h"

using namespace capi;

namespace capi {

// ---------------------------------------------------------------------------
// Batched extraction.  The requests are spread over L lanes (streams, each
// with its own scratch and, for Marching Cubes, its own FE -> MC map), the
// largest requests first, each to the lane with the fewest cells so far; a
// lane runs its requests one after the other (count, scan, generate,
// vertices), the lanes run side by side.  The whole batch is captured once
// as a CUDA graph: its 8-counter block per request (totals, device status,
// work counter) lives in the batch arena, so the counts stay on the device
// and the generate kernels check the capacities there; one copy at the end
// brings every request's counters back.
// ---------------------------------------------------------------------------
struct BatchItem {
    Grid g;
    Plans pl;
    int lane = 0;
};

constexpr int kMaxLanes = 64;
constexpr int kTuneLanes[] = {1, 2, 4, 8, 16, 32, 64};
// work splits: a request's count and generate plans size their grids and work
// items for nsm / share SMs (several lanes share the GPU)
constexpr int kTuneShares[] = {1, 2, 4, 8};

void replan(iso_ctx* ctx, std::vector<BatchItem>& items, const std::vector<int>& run, int share)
{
    const int nsm = std::max(1, ctx->nsm / std::max(1, share));
    for (int r : run) items[r].pl = make_plans(ctx, items[r].g, nsm);
}

// ---------------------------------------------------------------------------
// Fused requests.  Flying Edges requests whose rows fit the multi-row kernels
// (up to 16 words, the volume at a 16-byte boundary) run together, one launch
// per pass and kernel variant (batch_kernels.cuh): the count blocks of every
// request of a count variant, the two scan phases of all of them, the vertex
// prefix, the generate items of every request of a generate variant (rows
// per warp, index width), and one vertex pass over all their slots.  Each
// request has its own scratch, so nothing is shared between requests but the
// launches.  The descriptors and launch lists are written into pinned host
// memory before every run and copied in by the first node.
// ---------------------------------------------------------------------------
struct FusedGroup {
    iso::CountVariant cv{};
    int rpw = 0, index_bytes = 4;
    std::vector<int> members;  // descriptor indices
    unsigned total = 0;        // blocks (count, scan) or work items (generate)
    size_t list_at = 0, first_at = 0;
    size_t smem = 0;
    int ws_bytes = 0;
};

struct FusedPlan {
    std::vector<int> reqs;              // the batch request of descriptor d
    std::vector<iso::BatchReq> proto;   // the descriptors without their buffers
    std::vector<FusedGroup> count, gen;
    FusedGroup all;                     // every descriptor: scans (first = segments), vertex prefix and pass
    std::vector<unsigned char> meta;    // the upload block without the descriptors: lists and firsts
    size_t upload = 0;                  // bytes copied in per run: descriptors, then meta
    size_t vfirst_at = 0, work_at = 0;  // within the fused area
    std::vector<size_t> scratch_at;     // within the fused area, per descriptor
    size_t bytes = 0;                   // the fused area
    size_t at = 0;                      // its offset in the arena
    bool empty() const { return reqs.empty(); }
};

// Bytes of n descriptors at the start of the upload block (the lists and firsts follow, 256-byte aligned).
inline size_t desc_bytes(size_t n) { return (n * sizeof(iso::BatchReq) + 255) & ~(size_t)255; }

// Fewest fusable requests that run fused by default (iso_batch_set_fused 1): serving batches of 2-8 requests
// ran 4-8% faster on the lanes, the 157-request batch 11% faster fused.
constexpr int kFuseMin = 16;

bool fusable(const iso_ctx* ctx, const iso_request& r, const BatchItem& it)
{
    return ctx->batch_fused && r.algorithm == ISO_FLYING_EDGES && it.pl.gp.fits && it.g.W <= 16 &&
           (reinterpret_cast<uintptr_t>(r.volume) & 15) == 0;
}

// Groups, work split and layout of the fused requests fz (their plans are made for the whole GPU).  Returns
// an empty plan when a launch would pass 2^31 blocks or items: those requests then take the lanes.
// Work split of the fused launches: count blocks of at least kc planes, generate items for about ipw per warp
// of one wave (the autotuner's candidates; 0: the defaults).
constexpr int kFusedKC[] = {8, 16, 32};
constexpr int kFusedIPW[] = {16, 32, 64};
constexpr int kFusedKCDefault = 16, kFusedIPWDefault = 32;

FusedPlan plan_fused(iso_ctx* ctx, const iso_request* req, const iso_mesh* out, std::vector<BatchItem>& items,
                     const std::vector<int>& fz, const iso::PackedOut* pk = nullptr, int kc_min = 0, int ipw = 0)
{
    if (kc_min <= 0) kc_min = ctx->fused_kc > 0 ? ctx->fused_kc : kFusedKCDefault;
    if (ipw <= 0) ipw = ctx->fused_ipw > 0 ? ctx->fused_ipw : kFusedIPWDefault;
    const bool extract = out || pk;
    FusedPlan f;
    if (fz.empty()) return f;
    f.reqs = fz;
    const int nf = (int)fz.size();
    f.proto.resize(nf);
    std::map<int, int> ckey, gkey;
    const long long warps = (long long)ctx->nsm * 4 * 8;  // generate kernel: 4 CTAs of 8 warps per SM
    long long gen_planes = 0;                              // row groups x planes over all generate groups
    for (int d = 0; d < nf; ++d) {
        const int r = fz[d];
        BatchItem& it = items[r];
        it.pl = make_plans(ctx, it.g);
        const Grid& g = it.g;
        iso::BatchReq& x = f.proto[d];
        x = iso::BatchReq{};
        x.vol = req[r].volume;
        x.g = g;
        x.gs = iso::make_grad_scale(g);
        x.iso = req[r].isoval;
        const iso::CountVariant cv = iso::count_variant(g);
        x.count_KC = std::max(it.pl.cp.KC, kc_min);  // at least 16 planes per block: 157 small grids 2.77 -> 2.72 ms
        x.count_nyb = (g.ny + 8 * cv.rpw - 1) / (8 * cv.rpw);  // kCountRows warps of cv.rpw rows
        x.nseg = it.pl.cp.nseg;
        const int ck = cv.rpw | (cv.aligned ? 16 : 0) | (cv.full ? 32 : 0);
        if (!ckey.count(ck)) {
            ckey[ck] = (int)f.count.size();
            f.count.emplace_back();
            f.count.back().cv = cv;
        }
        FusedGroup& cg = f.count[ckey[ck]];
        cg.members.push_back(d);
        cg.smem = std::max(cg.smem, iso::count_batch_smem(g, cv));
        f.all.members.push_back(d);
        if (extract) {
            const int rpw = iso::gen_rows_per_warp(g.W);
            const int ib = out ? out[r].index_bytes : pk->index_bytes;
            const int gk = rpw | (ib << 8);
            if (!gkey.count(gk)) {
                gkey[gk] = (int)f.gen.size();
                f.gen.emplace_back();
                f.gen.back().rpw = rpw;
                f.gen.back().index_bytes = ib;
            }
            FusedGroup& gg = f.gen[gkey[gk]];
            gg.members.push_back(d);
            gg.ws_bytes = std::max(gg.ws_bytes, (int)iso::gen_batch_ws_bytes(g.W, rpw));
            x.gen_ngroups = (g.ny + rpw - 1) / rpw;
            gen_planes += (long long)x.gen_ngroups * g.nz;
        }
    }
    // generate items of KC planes: about ipw per warp of one wave over all requests, at least 2 planes
    long long KC = (gen_planes + ipw * warps - 1) / (ipw * warps);
    if (KC < 2) KC = 2;
    const long long lim = 1ll << 31;
    auto blocks_of = [&](const FusedGroup& grp, int what) -> long long {
        long long t = 0;
        for (int d : grp.members) {
            const iso::BatchReq& x = f.proto[d];
            if (what == 0) t += (long long)x.count_nyb * ((x.g.nz + x.count_KC - 1) / x.count_KC);
            else if (what == 1) t += x.nseg;
            else t += (long long)x.gen_ngroups * x.gen_nkc;
        }
        return t;
    };
    if (extract) {
        for (iso::BatchReq& x : f.proto) {
            x.gen_KC = (int)std::min<long long>(KC, x.g.nz);
            x.gen_nkc = (x.g.nz + x.gen_KC - 1) / x.gen_KC;
        }
    }
    // lists (ints) and firsts (unsigned, one more than the members) of each launch
    auto place = [&](FusedGroup& grp, int what) -> bool {
        const long long t = blocks_of(grp, what);
        if (t >= lim) return false;
        grp.total = (unsigned)t;
        const size_t m = grp.members.size();
        grp.list_at = f.meta.size();
        f.meta.resize(f.meta.size() + ((m * 4 + 15) & ~(size_t)15));
        std::memcpy(f.meta.data() + grp.list_at, grp.members.data(), m * 4);
        grp.first_at = f.meta.size();
        f.meta.resize(f.meta.size() + (((m + 1) * 4 + 15) & ~(size_t)15));
        unsigned* fs = reinterpret_cast<unsigned*>(f.meta.data() + grp.first_at);
        unsigned run = 0;
        for (size_t q = 0; q < m; ++q) {
            fs[q] = run;
            const iso::BatchReq& x = f.proto[grp.members[q]];
            run += what == 0 ? (unsigned)(x.count_nyb * ((x.g.nz + x.count_KC - 1) / x.count_KC))
                             : (what == 1 ? (unsigned)x.nseg : (unsigned)(x.gen_ngroups * x.gen_nkc));
        }
        fs[m] = run;
        return true;
    };
    bool ok = place(f.all, 1);
    for (FusedGroup& grp : f.count) ok = ok && place(grp, 0);
    for (FusedGroup& grp : f.gen) ok = ok && place(grp, 2);
    if (!ok) return FusedPlan{};
    f.upload = desc_bytes(nf) + f.meta.size();
    size_t at = align256(f.upload);
    f.vfirst_at = at;
    at += align256((size_t)(nf + 1) * 8);
    f.work_at = at;
    at += align256(f.gen.size() * 4 + 4);
    f.scratch_at.resize(nf);
    for (int d = 0; d < nf; ++d) {
        f.scratch_at[d] = at;
        at += align256(scratch_size(items[fz[d]].g, items[fz[d]].pl.cp));
    }
    f.bytes = at;
    return f;
}

// The fused requests' descriptors (buffers in the arena at f.at, meshes of out, counters of the batch) and
// launch lists into ctx->h_fused.  A packed batch's mesh pointers and capacities are set on the device.
void fill_fused(iso_ctx* ctx, const FusedPlan& f, const iso_mesh* out, const std::vector<BatchItem>& items)
{
    char* base = static_cast<char*>(ctx->batch_arena) + f.at;
    unsigned long long* counters = static_cast<unsigned long long*>(ctx->batch_arena);
    iso::BatchReq* D = reinterpret_cast<iso::BatchReq*>(ctx->h_fused);
    for (size_t d = 0; d < f.reqs.size(); ++d) {
        const int r = f.reqs[d];
        const BatchItem& it = items[r];
        FeBuffers b;
        carve(base + f.scratch_at[d], it.g, it.pl.cp, b);
        iso::BatchReq x = f.proto[d];
        x.rowcnt = b.rowcnt;
        x.bits = b.bits;
        x.starts = b.starts;
        x.part = b.part;
        x.totals = counters + 8 * (size_t)r;
        if (out) {
            x.points = out[r].points;
            x.normals = out[r].normals;
            x.tris = out[r].tris;
            x.capV = vertex_limit(&out[r], out[r].cap_points);
            x.capT = out[r].cap_tris;
        }
        D[d] = x;
    }
    std::memcpy(ctx->h_fused + desc_bytes(f.reqs.size()), f.meta.data(), f.meta.size());
}

// The launches of one pass run side by side: the largest on s, the others on streams forked from it and
// joined back into it (2.94 -> 2.77 ms on the 157-request batch against one after another).
template <typename Launch>
void fan_out(iso_ctx* ctx, const std::vector<FusedGroup>& groups, cudaStream_t s, Launch launch)
{
    std::vector<size_t> order(groups.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return groups[a].total > groups[b].total; });
    const size_t side = std::min(order.size(), ctx->fused_streams.size() + 1);
    if (side > 1) {
        cudaEventRecord(ctx->fused_fork, s);
        for (size_t i = 1; i < side; ++i) cudaStreamWaitEvent(ctx->fused_streams[i - 1], ctx->fused_fork, 0);
    }
    for (size_t i = 0; i < order.size(); ++i)
        launch(order[i], i < side && i > 0 ? ctx->fused_streams[i - 1] : s);
    for (size_t i = 1; i < side; ++i) {
        cudaEventRecord(ctx->fused_join[i - 1], ctx->fused_streams[i - 1]);
        cudaStreamWaitEvent(s, ctx->fused_join[i - 1], 0);
    }
}

// The fused chain on s: descriptors in, counts, scans and, for an extraction, the generate and vertex passes
// (pk: into one packed output, each request placed on the device after its counts).
void enqueue_fused(iso_ctx* ctx, const FusedPlan& f, bool extract, cudaStream_t s,
                   const iso::PackedOut* pk = nullptr)
{
    char* base = static_cast<char*>(ctx->batch_arena) + f.at;
    const size_t desc = desc_bytes(f.reqs.size());
    const iso::BatchReq* D = reinterpret_cast<const iso::BatchReq*>(base);
    auto L = [&](const FusedGroup& g) { return reinterpret_cast<const int*>(base + desc + g.list_at); };
    auto F = [&](const FusedGroup& g) { return reinterpret_cast<const unsigned*>(base + desc + g.first_at); };
    const int nf = (int)f.reqs.size();
    cudaMemcpyAsync(base, ctx->h_fused, f.upload, cudaMemcpyHostToDevice, s);
    fan_out(ctx, f.count, s, [&](size_t q, cudaStream_t st) {
        const FusedGroup& g = f.count[q];
        iso::launch_count_batch(g.cv, D, L(g), F(g), (int)g.members.size(), g.total, g.smem, st);
    });
    iso::launch_scan_batch(D, L(f.all), F(f.all), nf, f.all.total, s);
    if (!extract) return;
    unsigned long long* vfirst = reinterpret_cast<unsigned long long*>(base + f.vfirst_at);
    unsigned* work = reinterpret_cast<unsigned*>(base + f.work_at);
    cudaMemsetAsync(work, 0, f.gen.size() * 4, s);
    if (pk)
        iso::launch_place_batch(reinterpret_cast<iso::BatchReq*>(base), L(f.all), nf, *pk, vfirst, s);
    else
        iso::launch_vfirst_batch(D, L(f.all), nf, vfirst, s);
    fan_out(ctx, f.gen, s, [&](size_t q, cudaStream_t st) {
        const FusedGroup& g = f.gen[q];
        iso::launch_gen_batch(g.rpw, g.index_bytes, D, L(g), F(g), (int)g.members.size(), g.total, ctx->d_cases,
                              work + q, g.ws_bytes, ctx->reverse, ctx->nsm, st);
    });
    iso::launch_vertices_batch(D, L(f.all), vfirst, nf, ctx->nsm, s);
}

// Lane of every request with work and the arena layout: counters of all n
// requests, then per lane its scratch and FE -> MC map, then the fused area.
struct BatchLayout {
    int lanes = 1;
    std::vector<size_t> scratch_at, scratch_bytes, map_at;
    FusedPlan fz;
    size_t bytes = 0;
};

BatchLayout plan_batch(const iso_request* req, const iso_mesh* out, int64_t n, std::vector<BatchItem>& items,
                       const std::vector<int>& run, int lanes, const FusedPlan& fz)
{
    BatchLayout lay;
    lay.lanes = lanes;
    std::vector<int> order(run);
    auto cells = [&](int r) { return (double)(items[r].g.nx - 1) * (items[r].g.ny - 1) * (items[r].g.nz - 1); };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cells(a) > cells(b); });
    std::vector<double> load(lanes, 0.0);
    std::vector<size_t> scratch(lanes, 0), map(lanes, 0);
    for (int r : order) {
        const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        items[r].lane = l;
        load[l] += cells(r);
        scratch[l] = std::max(scratch[l], scratch_size(items[r].g, items[r].pl.cp));
        if (out && req[r].algorithm == ISO_MARCHING_CUBES) {
            const long long capV = vertex_limit(&out[r], out[r].cap_points);
            const long long capM = capV < 0xffffffffll ? capV : 0xffffffffll;
            map[l] = std::max(map[l], (size_t)(capM + 1024) * 4);
        }
    }
    size_t at = align256((size_t)n * 8 * sizeof(unsigned long long));
    for (int l = 0; l < lanes; ++l) {
        lay.scratch_at.push_back(at);
        lay.scratch_bytes.push_back(scratch[l]);
        at += align256(scratch[l]);
        lay.map_at.push_back(at);
        at += align256(map[l]);
    }
    lay.fz = fz;
    lay.fz.at = at;
    at += fz.bytes;
    lay.bytes = at;
    return lay;
}

// Captures and the batch buffers' allocations of all contexts take turns: a
// free (which synchronises the device) in one thread would invalidate a
// capture running in another.
std::mutex g_batch_mutex;

// Batch buffers (the caller holds g_batch_mutex).  Only this context's work on
// s uses them: the graphs and the lanes join back into s.
iso_status ensure_batch(iso_ctx* ctx, const BatchLayout& lay, int64_t n, cudaStream_t s)
{
    if (lay.bytes > ctx->batch_arena_bytes) {
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
        cudaFree(ctx->batch_arena);
        ctx->batch_arena = nullptr;
        ctx->batch_arena_bytes = 0;
        // a quarter more than asked: batches of varying sizes (a serving loop's) then rarely grow it again, and
        // every growth synchronises the stream
        const size_t alloc = lay.bytes + lay.bytes / 4;
        ISO_CUDA(ctx, cudaMalloc(&ctx->batch_arena, alloc));
        ctx->batch_arena_bytes = alloc;
    }
    if ((size_t)n > ctx->h_batch_n) {
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
        if (ctx->h_batch) cudaFreeHost(ctx->h_batch);
        ctx->h_batch = nullptr;
        ctx->h_batch_n = 0;
        ISO_CUDA(ctx, cudaHostAlloc(&ctx->h_batch, (size_t)n * 8 * sizeof(unsigned long long), cudaHostAllocDefault));
        ctx->h_batch_n = (size_t)n;
    }
    if (lay.fz.upload > ctx->h_fused_bytes) {
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
        if (ctx->h_fused) cudaFreeHost(ctx->h_fused);
        ctx->h_fused = nullptr;
        ctx->h_fused_bytes = 0;
        ISO_CUDA(ctx, cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_fused), lay.fz.upload, cudaHostAllocDefault));
        ctx->h_fused_bytes = lay.fz.upload;
    }
    if (!ctx->s_capture) ISO_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_capture, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&ctx->batch_fork, &ctx->batch_t0, &ctx->batch_t1})
        if (!*e) ISO_CUDA(ctx, cudaEventCreateWithFlags(e, e == &ctx->batch_fork ? cudaEventDisableTiming : 0));
    const size_t side = std::max(lay.fz.count.size(), lay.fz.gen.size());
    if (side > 1 && !ctx->fused_fork) ISO_CUDA(ctx, cudaEventCreateWithFlags(&ctx->fused_fork, cudaEventDisableTiming));
    while (ctx->fused_streams.size() + 1 < side) {
        cudaStream_t q;
        cudaEvent_t e;
        ISO_CUDA(ctx, cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
        ctx->fused_streams.push_back(q);
        ISO_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->fused_join.push_back(e);
    }
    while ((int)ctx->lane_streams.size() < lay.lanes) {
        cudaStream_t q;
        cudaEvent_t e;
        ISO_CUDA(ctx, cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
        ctx->lane_streams.push_back(q);
        ISO_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->lane_join.push_back(e);
    }
    return ISO_OK;
}

// What a captured graph depends on: lanes, buffers, requests and meshes, and the fused launches' geometry
// (each launch's grid and shared memory; the descriptors and lists are copied in by the graph at every run).
std::vector<unsigned char> batch_key(const iso_ctx* ctx, int lanes, int share, const iso_request* req,
                                     const iso_mesh* out, int64_t n, const FusedPlan& fz)
{
    std::vector<unsigned char> k;
    auto put = [&](const void* p, size_t len) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        k.insert(k.end(), c, c + len);
    };
    const unsigned char count_only = out ? 0 : 1;
    put(&count_only, 1);
    put(&lanes, sizeof lanes);
    put(&share, sizeof share);
    put(&ctx->reverse, sizeof ctx->reverse);
    put(&ctx->batch_arena, sizeof ctx->batch_arena);
    put(&ctx->h_batch, sizeof ctx->h_batch);
    put(&ctx->batch_fused, sizeof ctx->batch_fused);
    put(&ctx->h_fused, sizeof ctx->h_fused);
    put(&n, sizeof n);
    put(req, (size_t)n * sizeof(iso_request));
    const size_t nf = fz.reqs.size();
    put(&nf, sizeof nf);
    put(&fz.at, sizeof fz.at);
    put(&fz.upload, sizeof fz.upload);
    put(&fz.all.total, sizeof fz.all.total);
    for (const std::vector<FusedGroup>* gs : {&fz.count, &fz.gen}) {
        for (const FusedGroup& g : *gs) {
            put(&g.total, sizeof g.total);
            put(&g.smem, sizeof g.smem);
            put(&g.ws_bytes, sizeof g.ws_bytes);
            put(&g.rpw, sizeof g.rpw);
            put(&g.index_bytes, sizeof g.index_bytes);
            const int cv[3] = {g.cv.rpw, g.cv.aligned ? 1 : 0, g.cv.full ? 1 : 0};  // no padding bytes in the key
            put(cv, sizeof cv);
            put(&g.list_at, sizeof g.list_at);
            put(&g.first_at, sizeof g.first_at);
        }
        const size_t sep = gs->size();
        put(&sep, sizeof sep);
    }
    for (int64_t r = 0; out && r < n; ++r) {
        put(&out[r].points, sizeof out[r].points);
        put(&out[r].normals, sizeof out[r].normals);
        put(&out[r].tris, sizeof out[r].tris);
        put(&out[r].index_bytes, sizeof out[r].index_bytes);
        put(&out[r].cap_points, sizeof out[r].cap_points);
        put(&out[r].cap_tris, sizeof out[r].cap_tris);
    }
    return k;
}

// The batch's work from `origin`: fork to the lanes, each lane's requests in
// turn, join, the counters' copy to the host; all on origin's side of the join.
void enqueue_batch(iso_ctx* ctx, const iso_request* req, const iso_mesh* out, int64_t n, std::vector<BatchItem>& items,
                   const std::vector<int>& run, const BatchLayout& lay, cudaStream_t origin)
{
    char* arena = static_cast<char*>(ctx->batch_arena);
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(arena);
    const bool prof = ctx->profiling;
    ctx->profiling = false;  // no timing events between the lanes' kernels
    cudaMemsetAsync(counters, 0, (size_t)n * 8 * sizeof(unsigned long long), origin);
    cudaEventRecord(ctx->batch_fork, origin);
    for (int l = 0; l < lay.lanes; ++l) cudaStreamWaitEvent(ctx->lane_streams[l], ctx->batch_fork, 0);
    for (int r : run) {
        BatchItem& it = items[r];
        cudaStream_t ls = ctx->lane_streams[it.lane];
        FeBuffers b;
        carve(arena + lay.scratch_at[it.lane], it.g, it.pl.cp, b);
        b.totals = counters + 8 * r;
        b.fe2mc = reinterpret_cast<uint32_t*>(arena + lay.map_at[it.lane]);
        PassMarks pm(ctx, ls);
        const iso_algorithm algo = static_cast<iso_algorithm>(req[r].algorithm);
        enqueue_count(ctx, algo, req[r].volume, it.g, req[r].isoval, it.pl, b, ls, pm);
        if (out) enqueue_generate(ctx, algo, req[r].volume, it.g, req[r].isoval, it.pl, b, &out[r], ls, pm);
    }
    if (!lay.fz.empty()) enqueue_fused(ctx, lay.fz, out != nullptr, origin);  // beside the lanes
    for (int l = 0; l < lay.lanes; ++l) {
        cudaEventRecord(ctx->lane_join[l], ctx->lane_streams[l]);
        cudaStreamWaitEvent(origin, ctx->lane_join[l], 0);
    }
    cudaMemcpyAsync(ctx->h_batch, counters, (size_t)n * 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                    origin);
    ctx->profiling = prof;
}

// Capture the batch on the lanes and make ctx->batch_exec run it (updating
// the executable graph in place when the topology allows).  out == nullptr:
// passes 1-3 only (iso_count_batch).
iso_status capture_batch(iso_ctx* ctx, const iso_request* req, const iso_mesh* out, int64_t n,
                         std::vector<BatchItem>& items, const std::vector<int>& run, const BatchLayout& lay)
{
    cudaStream_t sc = ctx->s_capture;
    const int slot = out ? 0 : 1;
    cudaGraphExec_t& exec = ctx->batch_exec[slot];
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(sc, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        enqueue_batch(ctx, req, out, n, items, run, lay, sc);
        e = cudaStreamEndCapture(sc, &graph);
    }
    if (e != cudaSuccess || !graph) {
        cudaGetLastError();
        if (graph) cudaGraphDestroy(graph);
        ctx->batch_key[slot].clear();
        ctx->last_error = std::string("capturing the batch failed: ") + cudaGetErrorString(e);
        return ISO_ERR_CUDA;
    }
    if (exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(exec, graph, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    if (!exec) e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        exec = nullptr;
        ctx->batch_key[slot].clear();
        return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    return ISO_OK;
}

// Prepare (lanes, buffers, graph) for `lanes` lanes; nothing runs.
iso_status prepare_batch(iso_ctx* ctx, const iso_request* req, const iso_mesh* out, int64_t n,
                         std::vector<BatchItem>& items, const std::vector<int>& run, const FusedPlan& fz, int lanes,
                         int share, cudaStream_t s)
{
    replan(ctx, items, run, share);
    const BatchLayout lay = plan_batch(req, out, n, items, run, lanes, fz);
    std::lock_guard<std::mutex> lock(g_batch_mutex);
    iso_status st = ensure_batch(ctx, lay, n, s);
    if (st != ISO_OK) return st;
    // before every run, replayed graph or not: the staging is shared by the context's graphs
    if (!lay.fz.empty()) fill_fused(ctx, lay.fz, out, items);
    std::vector<unsigned char> key = batch_key(ctx, lanes, share, req, out, n, lay.fz);
    const int slot = out ? 0 : 1;
    if (ctx->batch_exec[slot] && key == ctx->batch_key[slot]) return ISO_OK;
    st = capture_batch(ctx, req, out, n, items, run, lay);
    if (st == ISO_OK) ctx->batch_key[slot].swap(key);
    return st;
}

// Milliseconds of one run of the prepared batch (the best of two after one warm-up run).
iso_status time_batch(iso_ctx* ctx, cudaGraphExec_t exec, cudaStream_t s, float& best)
{
    best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        ISO_CUDA(ctx, cudaEventRecord(ctx->batch_t0, s));
        ISO_CUDA(ctx, cudaGraphLaunch(exec, s));
        ISO_CUDA(ctx, cudaEventRecord(ctx->batch_t1, s));
        ISO_CUDA(ctx, cudaEventSynchronize(ctx->batch_t1));
        float ms = 0.f;
        ISO_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->batch_t0, ctx->batch_t1));
        if (rep > 0) best = std::min(best, ms);
    }
    return ISO_OK;
}

// iso_extract_device_async as a CUDA graph: the passes and the counters'
// copy to result_host captured once, relaunched while the call's arguments,
// the context's buffers and result_host stay the same (result_host must be
// pinned: a pageable one takes the stream path).
iso_status extract_graph(iso_ctx* ctx, iso_algorithm algo, const float* volume, const Grid& g, const iso_grid* grid,
                         float isoval, const Plans& pl, FeBuffers& b, const iso_mesh* out, int64_t* result_host,
                         cudaStream_t s)
{
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, result_host) != cudaSuccess || attr.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        PassMarks pm(ctx, s);
        enqueue_count(ctx, algo, volume, g, isoval, pl, b, s, pm);
        enqueue_generate(ctx, algo, volume, g, isoval, pl, b, out, s, pm);
        ISO_CUDA(ctx, cudaGetLastError());
        ISO_CUDA(ctx,
                 cudaMemcpyAsync(result_host, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        return ISO_OK;
    }
    std::vector<unsigned char> key;
    auto put = [&](const void* p, size_t len) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        key.insert(key.end(), c, c + len);
    };
    put(&algo, sizeof algo);
    put(&volume, sizeof volume);
    put(grid, sizeof *grid);
    put(&isoval, sizeof isoval);
    put(&out->points, sizeof out->points);
    put(&out->normals, sizeof out->normals);
    put(&out->tris, sizeof out->tris);
    put(&out->index_bytes, sizeof out->index_bytes);
    put(&out->cap_points, sizeof out->cap_points);
    put(&out->cap_tris, sizeof out->cap_tris);
    put(&result_host, sizeof result_host);
    put(&ctx->scratch, sizeof ctx->scratch);
    put(&ctx->fe2mc, sizeof ctx->fe2mc);
    put(&ctx->reverse, sizeof ctx->reverse);
    if (!ctx->one_exec || key != ctx->one_key) {
        std::lock_guard<std::mutex> lock(g_batch_mutex);
        if (!ctx->s_capture) ISO_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_capture, cudaStreamNonBlocking));
        cudaStream_t sc = ctx->s_capture;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(sc, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            PassMarks pm(ctx, sc);
            enqueue_count(ctx, algo, volume, g, isoval, pl, b, sc, pm);
            enqueue_generate(ctx, algo, volume, g, isoval, pl, b, out, sc, pm);
            cudaMemcpyAsync(result_host, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, sc);
            e = cudaStreamEndCapture(sc, &graph);
        }
        if (e != cudaSuccess || !graph) {
            cudaGetLastError();
            if (graph) cudaGraphDestroy(graph);
            ctx->one_key.clear();
            ctx->last_error = std::string("capturing the extraction failed: ") + cudaGetErrorString(e);
            return ISO_ERR_CUDA;
        }
        if (ctx->one_exec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(ctx->one_exec, graph, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(ctx->one_exec);
                ctx->one_exec = nullptr;
            }
        }
        if (!ctx->one_exec) e = cudaGraphInstantiate(&ctx->one_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ctx->one_exec = nullptr;
            ctx->one_key.clear();
            return cuda_fail(ctx, e, "cudaGraphInstantiate");
        }
        ctx->one_key.swap(key);
    }
    ISO_CUDA(ctx, cudaGraphLaunch(ctx->one_exec, s));
    return ISO_OK;
}

}  // namespace capi

extern "C" {

iso_status iso_ctx_set_graph(iso_ctx* ctx, int enable)
{
    if (!ctx) return ISO_ERR_INVALID_ARG;
    ctx->one_graph = enable ? 1 : 0;
    if (!enable && ctx->one_exec) {
        cudaGraphExecDestroy(ctx->one_exec);
        ctx->one_exec = nullptr;
        ctx->one_key.clear();
    }
    return ISO_OK;
}

}  // extern "C"

namespace {

// iso_extract_batch (out != nullptr) and iso_count_batch (out == nullptr, the
// counts into nV / nT): validate, tune the lanes if asked, run the graph.
iso_status run_batch(iso_ctx* ctx, int64_t n, const iso_request* req, iso_mesh* out, int64_t* nV, int64_t* nT,
                     iso_status* status, cudaStream_t s)
{
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<iso_status> st((size_t)n, ISO_OK);
    std::vector<BatchItem> items((size_t)n);
    std::vector<int> run;  // requests with work
    for (int64_t r = 0; r < n; ++r) {
        if (out) {
            if (check_mesh(&out[r]) != ISO_OK) {
                st[r] = ISO_ERR_INVALID_ARG;
                continue;
            }
            out[r].n_points = out[r].n_tris = 0;
        } else {
            nV[r] = nT[r] = 0;
        }
        Grid g;
        if (!valid_algo(static_cast<iso_algorithm>(req[r].algorithm)) || !make_grid(&req[r].grid, g)) {
            st[r] = ISO_ERR_INVALID_ARG;
            continue;
        }
        if (empty_grid(g)) continue;
        if (!req[r].volume) {
            st[r] = ISO_ERR_INVALID_ARG;
            continue;
        }
        items[r].g = g;
        items[r].pl = make_plans(ctx, g);
        if (out && req[r].algorithm == ISO_MC_DUPFREE && !items[r].pl.gp.fits) {
            ctx->last_error = "the duplicate-free order needs rows of at most 1024 points";
            st[r] = ISO_ERR_INVALID_ARG;
            continue;
        }
        run.push_back((int)r);
    }
    // the fused requests (one launch per pass) and the rest (lanes)
    std::vector<int> fused, lane_run;
    for (int r : run) (fusable(ctx, req[r], items[r]) ? fused : lane_run).push_back(r);
    if (ctx->batch_fused == 1 && (int)fused.size() < kFuseMin) {  // too few to pay for the fused launches
        fused.clear();
        lane_run = run;
    }
    FusedPlan fz = plan_fused(ctx, req, out, items, fused);
    if (ctx->batch_fused == 1 && !fz.empty() && fz.bytes > ctx->batch_arena_bytes) {
        // every fused request holds its own scratch at once: past half the free memory, the lanes instead
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            cudaGetLastError();  // the call's own error; the batch reports its own failures later
        } else if (fz.bytes > free_b / 2) {
            fz = FusedPlan{};
        }
    }
    if (fz.empty() && !fused.empty()) lane_run = run;
    iso_status rc = ISO_OK;
    if (!run.empty() && !ctx->batch_graph) {  // launched directly, no graph
        int lanes = ctx->batch_lanes > 0 ? ctx->batch_lanes : (ctx->batch_tuned > 0 ? ctx->batch_tuned : 8);
        const int share = ctx->batch_share > 0 ? ctx->batch_share : std::max(1, ctx->batch_tuned_share);
        lanes = std::min(lanes, std::max(1, (int)lane_run.size()));
        replan(ctx, items, lane_run, share);
        const BatchLayout lay = plan_batch(req, out, n, items, lane_run, lanes, fz);
        {
            std::lock_guard<std::mutex> lock(g_batch_mutex);
            rc = ensure_batch(ctx, lay, n, s);
            if (rc == ISO_OK && !lay.fz.empty()) fill_fused(ctx, lay.fz, out, items);
        }
        if (rc != ISO_OK) return rc;
        enqueue_batch(ctx, req, out, n, items, lane_run, lay, s);
        ISO_CUDA(ctx, cudaGetLastError());
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
    } else if (!run.empty()) {
        int lanes = ctx->batch_lanes > 0 ? ctx->batch_lanes : ctx->batch_tuned;
        int share = ctx->batch_share > 0 ? ctx->batch_share : ctx->batch_tuned_share;
        if (!fz.empty() && (ctx->fused_kc <= 0 || ctx->fused_ipw <= 0)) {
            // autotuner of the fused launches' work split: time the batch at each (count planes, items per
            // warp) with the lanes as they stand, keep the fastest
            const int tl = std::min(std::max(lanes, 1), std::max(1, (int)lane_run.size()));
            const int ts = std::max(share, 1);
            float best = 1e30f;
            int best_kc = kFusedKCDefault, best_ipw = kFusedIPWDefault;
            for (int kc : kFusedKC) {
                for (int ipw : kFusedIPW) {
                    const FusedPlan cand = plan_fused(ctx, req, out, items, fused, nullptr, kc, ipw);
                    if (cand.empty()) continue;
                    rc = prepare_batch(ctx, req, out, n, items, lane_run, cand, tl, ts, s);
                    if (rc != ISO_OK) return rc;
                    float ms;
                    rc = time_batch(ctx, ctx->batch_exec[out ? 0 : 1], s, ms);
                    if (rc != ISO_OK) return rc;
                    if (ms < best) {
                        best = ms;
                        best_kc = kc;
                        best_ipw = ipw;
                    }
                }
            }
            ctx->fused_kc = best_kc;
            ctx->fused_ipw = best_ipw;
            fz = plan_fused(ctx, req, out, items, fused);
        }
        if (lane_run.empty()) {  // every request fused: no lanes to tune
            lanes = std::max(lanes, 1);
            share = std::max(share, 1);
        }
        if (lanes <= 0 || share <= 0) {  // autotuner: time the batch at each (lanes, split), keep the fastest
            float best = 1e30f;
            int best_l = 1, best_s = 1;
            for (int L : kTuneLanes) {
                if (lanes > 0 && L != lanes) continue;
                if (L > 1 && L > (int)lane_run.size()) break;
                for (int S : kTuneShares) {
                    if (share > 0 && S != share) continue;
                    if (S > L) break;  // a request never has fewer SMs than nsm / lanes
                    rc = prepare_batch(ctx, req, out, n, items, lane_run, fz, L, S, s);
                    if (rc != ISO_OK) return rc;
                    float ms;
                    rc = time_batch(ctx, ctx->batch_exec[out ? 0 : 1], s, ms);
                    if (rc != ISO_OK) return rc;
                    if (ms < best) {
                        best = ms;
                        best_l = L;
                        best_s = S;
                    }
                }
            }
            lanes = best_l;
            share = best_s;
            if (ctx->batch_lanes <= 0) ctx->batch_tuned = lanes;
            if (ctx->batch_share <= 0) ctx->batch_tuned_share = share;
        }
        lanes = std::min(lanes, std::max(1, (int)lane_run.size()));
        rc = prepare_batch(ctx, req, out, n, items, lane_run, fz, lanes, share, s);
        if (rc != ISO_OK) return rc;
        ISO_CUDA(ctx, cudaGraphLaunch(ctx->batch_exec[out ? 0 : 1], s));
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
    }
    if (!run.empty()) {
        for (int r : run) {
            const unsigned long long* c = ctx->h_batch + 8 * (size_t)r;
            if (out) {
                st[r] = finish_counts(ctx, &out[r], (long long)c[0], (long long)c[1], (long long)c[3],
                                      &out[r].n_points, &out[r].n_tris);
            } else {
                st[r] = finish_counts(ctx, nullptr, (long long)c[0], (long long)c[1], (long long)c[3], &nV[r], &nT[r]);
            }
        }
    }
    for (int64_t r = 0; r < n; ++r) {
        if (status) status[r] = st[r];
        if (rc == ISO_OK && st[r] != ISO_OK) rc = st[r];
    }
    return rc;
}

// iso_extract_batch_packed: every request fused, one call, no host round trip between its counts and its mesh.
iso_status run_batch_packed(iso_ctx* ctx, int64_t n, const iso_request* req, const iso::PackedOut& pk,
                            int64_t* point_first, int64_t* tri_first, int64_t* n_points, int64_t* n_tris,
                            iso_status* status, cudaStream_t s)
{
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<iso_status> st((size_t)n, ISO_OK);
    std::vector<BatchItem> items((size_t)n);
    std::vector<int> run;
    for (int64_t r = 0; r < n; ++r) {
        point_first[r] = tri_first[r] = n_points[r] = n_tris[r] = 0;
        Grid g;
        if (!valid_algo(static_cast<iso_algorithm>(req[r].algorithm)) || !make_grid(&req[r].grid, g)) {
            st[r] = ISO_ERR_INVALID_ARG;
            continue;
        }
        if (empty_grid(g)) continue;
        items[r].g = g;
        items[r].pl = make_plans(ctx, g);
        if (!req[r].volume || req[r].algorithm != ISO_FLYING_EDGES || g.W > 16 || !items[r].pl.gp.fits ||
            (reinterpret_cast<uintptr_t>(req[r].volume) & 15) != 0) {
            ctx->last_error = "a packed batch takes Flying Edges requests of rows up to 512 points, volumes at "
                              "16-byte boundaries";
            st[r] = ISO_ERR_INVALID_ARG;
            continue;
        }
        run.push_back((int)r);
    }
    iso_status rc = ISO_OK;
    if (!run.empty()) {
        const FusedPlan fz = plan_fused(ctx, req, nullptr, items, run, &pk);
        if (fz.empty()) {
            ctx->last_error = "the packed batch is too large for one launch per pass";
            return ISO_ERR_INVALID_ARG;
        }
        const BatchLayout lay = plan_batch(req, nullptr, n, items, std::vector<int>(), 1, fz);
        {
            std::lock_guard<std::mutex> lock(g_batch_mutex);
            rc = ensure_batch(ctx, lay, n, s);
            if (rc == ISO_OK) fill_fused(ctx, lay.fz, nullptr, items);
        }
        if (rc != ISO_OK) return rc;
        unsigned long long* counters = static_cast<unsigned long long*>(ctx->batch_arena);
        const bool prof = ctx->profiling;
        ctx->profiling = false;
        cudaMemsetAsync(counters, 0, (size_t)n * 8 * sizeof(unsigned long long), s);
        enqueue_fused(ctx, lay.fz, true, s, &pk);
        cudaMemcpyAsync(ctx->h_batch, counters, (size_t)n * 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        s);
        ctx->profiling = prof;
        ISO_CUDA(ctx, cudaGetLastError());
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
        for (int r : run) {
            const unsigned long long* c = ctx->h_batch + 8 * (size_t)r;
            n_points[r] = (int64_t)c[0];
            n_tris[r] = (int64_t)c[1];
            point_first[r] = (int64_t)c[4];
            tri_first[r] = (int64_t)c[5];
            if (c[3]) {
                ctx->last_error = "a device-side wait timed out";
                st[r] = ISO_ERR_TIMEOUT;
            } else if (pk.index_bytes == 4 && c[0] > 0xffffffffull) {
                ctx->last_error = "more than 2^32-1 vertices: use 64-bit indices";
                st[r] = ISO_ERR_OVERFLOW;
            } else if ((long long)(c[4] + c[0]) > pk.cap_points || (long long)(c[5] + c[1]) > pk.cap_tris) {
                ctx->last_error = "output buffers too small";
                st[r] = ISO_ERR_CAPACITY;
            }
        }
    }
    for (int64_t r = 0; r < n; ++r) {
        if (status) status[r] = st[r];
        if (rc == ISO_OK && st[r] != ISO_OK) rc = st[r];
    }
    return rc;
}

}  // namespace

extern "C" {

iso_status iso_extract_batch_packed(iso_ctx* ctx, int64_t n, const iso_request* req, float* points, float* normals,
                                    void* tris, int32_t index_bytes, int64_t cap_points, int64_t cap_tris,
                                    int64_t* point_first, int64_t* tri_first, int64_t* n_points, int64_t* n_tris,
                                    iso_status* status, void* stream)
{
    if (!ctx || n < 0 || (n > 0 && (!req || !point_first || !tri_first || !n_points || !n_tris)) ||
        (index_bytes != 4 && index_bytes != 8) || cap_points < 0 || cap_tris < 0 ||
        (cap_points > 0 && (!points || !normals)) || (cap_tris > 0 && !tris))
        return ISO_ERR_INVALID_ARG;
    iso::PackedOut pk;
    pk.points = points;
    pk.normals = normals;
    pk.tris = tris;
    pk.index_bytes = index_bytes;
    pk.cap_points = cap_points;
    pk.cap_tris = cap_tris;
    return run_batch_packed(ctx, n, req, pk, point_first, tri_first, n_points, n_tris, status,
                            static_cast<cudaStream_t>(stream));
}

iso_status iso_extract_batch(iso_ctx* ctx, int64_t n, const iso_request* req, iso_mesh* out, iso_status* status,
                             void* stream)
{
    if (!ctx || n < 0 || (n > 0 && (!req || !out))) return ISO_ERR_INVALID_ARG;
    return run_batch(ctx, n, req, out, nullptr, nullptr, status, static_cast<cudaStream_t>(stream));
}

iso_status iso_count_batch(iso_ctx* ctx, int64_t n, const iso_request* req, int64_t* n_points, int64_t* n_tris,
                           iso_status* status, void* stream)
{
    if (!ctx || n < 0 || (n > 0 && (!req || !n_points || !n_tris))) return ISO_ERR_INVALID_ARG;
    return run_batch(ctx, n, req, nullptr, n_points, n_tris, status, static_cast<cudaStream_t>(stream));
}

iso_status iso_block_tris(iso_ctx* ctx, const float* volume, const iso_grid* grid, float isoval, int32_t* counts,
                          void* stream)
{
    if (!ctx || !grid) return ISO_ERR_INVALID_ARG;
    Grid g;
    if (!make_grid(grid, g)) return ISO_ERR_INVALID_ARG;
    if (empty_grid(g)) return ISO_OK;
    if (!volume || !counts) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const Plans pl = make_plans(ctx, g);
    FeBuffers b;
    iso_status st = ensure_scratch(ctx, g, pl.cp, b, s);
    if (st != ISO_OK) return st;
    iso::launch_count(volume, g, isoval, ctx->d_cases, false, pl.cp, b, s);  // bit rows of the whole grid
    ISO_CUDA(ctx, cudaMemsetAsync(counts, 0, sizeof(int32_t) * (size_t)iso::block_count(g), s));
    iso::launch_block_tris(g, b.bits, counts, s);
    ISO_CUDA(ctx, cudaGetLastError());
    return ISO_OK;
}

iso_status iso_batch_set_lanes(iso_ctx* ctx, int lanes)
{
    if (!ctx || lanes < 0 || lanes > kMaxLanes) return ISO_ERR_INVALID_ARG;
    ctx->batch_lanes = lanes;
    if (lanes == 0) {  // tune again on the next batch, the split and the fused work split too
        ctx->batch_tuned = 0;
        ctx->batch_tuned_share = 0;
        ctx->fused_kc = ctx->fused_ipw = 0;
    }
    return ISO_OK;
}

iso_status iso_batch_set_split(iso_ctx* ctx, int share)
{
    if (!ctx || share < 0 || share > 64) return ISO_ERR_INVALID_ARG;
    ctx->batch_share = share;
    if (share == 0) ctx->batch_tuned_share = 0;  // tune again on the next batch
    return ISO_OK;
}

int iso_batch_split(const iso_ctx* ctx)
{
    if (!ctx) return 0;
    return ctx->batch_share > 0 ? ctx->batch_share : ctx->batch_tuned_share;
}

iso_status iso_batch_set_fused(iso_ctx* ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 2) return ISO_ERR_INVALID_ARG;
    ctx->batch_fused = mode;
    return ISO_OK;
}

iso_status iso_batch_fused_split(const iso_ctx* ctx, int* count_planes, int* items_per_warp)
{
    if (!ctx || !count_planes || !items_per_warp) return ISO_ERR_INVALID_ARG;
    *count_planes = ctx->fused_kc;
    *items_per_warp = ctx->fused_ipw;
    return ISO_OK;
}

iso_status iso_batch_set_graph(iso_ctx* ctx, int enable)
{
    if (!ctx) return ISO_ERR_INVALID_ARG;
    ctx->batch_graph = enable ? 1 : 0;
    return ISO_OK;
}

int iso_batch_lanes(const iso_ctx* ctx)
{
    if (!ctx) return 0;
    return ctx->batch_lanes > 0 ? ctx->batch_lanes : ctx->batch_tuned;
}

}  // extern "C"
