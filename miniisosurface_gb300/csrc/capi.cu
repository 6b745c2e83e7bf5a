// C ABI of the extractor: contexts, scratch, the extraction entry points and
// the pass-by-pass Flying Edges object.  See include/miniiso.h.  Batches and
// graph mode live in batch.cu.
#include "capi_internal.h"
#include "case_table.h"

using namespace capi;

struct iso_fe {
    iso_ctx* ctx = nullptr;
    const float* host_volume = nullptr;
    iso_grid grid{};
    Grid g{};
    float isoval = 0.f;
    int stage = 0;
    float* d_volume = nullptr;
    void* scratch = nullptr;
    FeBuffers buf{};
    long long n_points = 0, n_tris = 0;
    float* d_points = nullptr;
    float* d_normals = nullptr;
    uint64_t* d_tris = nullptr;
};

namespace {

const char* kVersion = "miniiso-gb300 0.1 (sm_103a)";

// ---------------------------------------------------------------------------
// z-slabs [k0, k1) of a decomposition along z.  The window of a slab: the
// volume pointer holds planes max(k0-1, 0) .. min(k1+1, nz-1); the scratch
// rows are planes [kr, ke) with kr = k0 (FE) or max(k0-1, 0) (MC, whose
// triangles at plane k0 reference vertices owned by cell row k0-1) and
// ke = min(k1+1, nz) (rows of plane k1 number the vertices the slab's top
// cells reference).
// ---------------------------------------------------------------------------
bool slab_grid(const iso_grid* gr, iso_algorithm algo, int64_t k0, int64_t k1, Grid& g)
{
    if (!make_grid(gr, g)) return false;
    if (k0 < 0 || k1 <= k0 || k1 > g.nz) return false;
    g.kd = (int)(k0 > 0 ? k0 - 1 : 0);
    g.kr = algo == ISO_MARCHING_CUBES ? g.kd : (int)k0;
    g.ke = (int)(k1 + 1 < g.nz ? k1 + 1 : g.nz);
    g.R = (long long)g.ny * (g.ke - g.kr);
    return true;
}

// Counts of the window (enqueued and read back): lo[a] / hi[a] = row starts
// (vertices, triangles, MC vertices) at planes k0 and k1 (window totals for
// k1 = nz).  The slab owns [lo, hi) of each.
struct SlabCounts {
    unsigned long long lo[3], hi[3], tot[3];
};

// Enqueues the count of the window and the copies of its totals and row
// starts into h[0..8] (pinned).
// The slab-count read-back buffer: pinned host memory that kernels write.
iso_status ensure_h_slab(iso_ctx* ctx)
{
    if (ctx->h_slab) return ISO_OK;
    ISO_CUDA(ctx, cudaHostAlloc(&ctx->h_slab, 18 * sizeof(unsigned long long), cudaHostAllocMapped));
    ISO_CUDA(ctx, cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->h_slab_dev), ctx->h_slab, 0));
    return ISO_OK;
}

iso_status slab_count_enqueue(iso_ctx* ctx, iso_algorithm algo, const float* vol, const Grid& g, int64_t k0,
                              int64_t k1, float iso, const Plans& pl, FeBuffers& b, cudaStream_t s,
                              unsigned long long* h)
{
    PassMarks pm(ctx, s);
    enqueue_count(ctx, algo, vol, g, iso, pl, b, s, pm);
    ISO_CUDA(ctx, cudaGetLastError());
    // h lies in ctx->h_slab; the kernel writes it through the device address
    const long long rlo = (long long)(k0 - g.kr) * g.ny, rhi = (long long)(k1 - g.kr) * g.ny;
    iso::launch_slab_readback(b, g, rlo, rhi, rlo > 0, k1 < g.nz, ctx->h_slab_dev + (h - ctx->h_slab), s);
    ISO_CUDA(ctx, cudaGetLastError());
    return ISO_OK;
}

// The counts copied by slab_count_enqueue, once they have landed.
void slab_count_read(const Grid& g, int64_t k0, int64_t k1, const unsigned long long* h, SlabCounts& c)
{
    for (int a = 0; a < 3; ++a) {
        c.tot[a] = h[a];
        c.lo[a] = k0 - g.kr > 0 ? h[3 + a] : 0;
        c.hi[a] = k1 < g.nz ? h[6 + a] : h[a];
    }
}

iso_status slab_count(iso_ctx* ctx, iso_algorithm algo, const float* vol, const Grid& g, int64_t k0, int64_t k1,
                      float iso, const Plans& pl, FeBuffers& b, cudaStream_t s, SlabCounts& c)
{
    iso_status st = ensure_h_slab(ctx);
    if (st != ISO_OK) return st;
    st = slab_count_enqueue(ctx, algo, vol, g, k0, k1, iso, pl, b, s, ctx->h_slab);
    if (st != ISO_OK) return st;
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    slab_count_read(g, k0, k1, ctx->h_slab, c);
    return ISO_OK;
}

// Pass 4 of slab [k0, k1) into the device mesh `out` (the slab's rows),
// numbered from point_offset / tri_offset; enqueued on s.
iso_status slab_generate(iso_ctx* ctx, iso_algorithm algo, const float* volume, const Grid& g, int64_t k0, int64_t k1,
                         float isoval, const Plans& pl, const FeBuffers& b, const SlabCounts& c, int64_t point_offset,
                         int64_t tri_offset, const iso_mesh* out, cudaStream_t s)
{
    const bool mc = algo == ISO_MARCHING_CUBES;
    iso::GenPlan gp = pl.gp;
    gp.vbase = (unsigned long long)point_offset;
    gp.tbase = (unsigned long long)tri_offset;
    gp.add[0] = mc ? 0ull : (unsigned long long)point_offset - c.lo[0];
    gp.add[1] = (unsigned long long)tri_offset - c.lo[1];
    gp.add[2] = (unsigned long long)point_offset - c.lo[2];
    const long long big = 1ll << 62;  // capacities were checked above
    const bool i4 = out->index_bytes == 4;
    PassMarks pm(ctx, s);
    if (!mc) {
        gp.kbeg = (int)k0;
        gp.kend = (int)k1;
        gp.kemit = (int)k0;
        iso::gen_split(gp, ctx->nsm);
        if (i4)
            iso::launch_fe_gen_warps<uint32_t>(volume, g, isoval, ctx->d_cases, b, pl.cp, gp, big, big, out->points,
                                               out->normals, static_cast<uint32_t*>(out->tris), ctx->reverse, s);
        else
            iso::launch_fe_gen_warps<uint64_t>(volume, g, isoval, ctx->d_cases, b, pl.cp, gp, big, big, out->points,
                                               out->normals, static_cast<uint64_t*>(out->tris), ctx->reverse, s);
        pm.mark(ISO_PASS_FE_GENERATE);
        if (iso::launch_fe_vertices(volume, g, isoval, b, gp, big, big, out->points, out->normals, s))
            pm.mark(ISO_PASS_VERTICES);
    } else {
        gp.kbeg = g.kr;  // cell row k0-1 maps the edges it owns on plane k0
        gp.kend = (int)k1;
        gp.kemit = (int)k0;
        iso::gen_split(gp, ctx->nsm);
        iso::launch_mc_gen_warps(volume, g, isoval, ctx->d_cases, b, pl.cp, gp, big, big, out->points, out->normals,
                                 ctx->reverse, s);
        pm.mark(ISO_PASS_MC_VERTICES);
        if (iso::launch_mc_vertices(volume, g, isoval, b, gp, big, big, out->points, out->normals, s))
            pm.mark(ISO_PASS_VERTICES);
        gp.kbeg = (int)k0;
        iso::gen_split(gp, ctx->nsm);
        if (i4)
            iso::launch_mc_tri_warps<uint32_t>(g, ctx->d_cases, b, pl.cp, gp, big, big,
                                               static_cast<uint32_t*>(out->tris), s);
        else
            iso::launch_mc_tri_warps<uint64_t>(g, ctx->d_cases, b, pl.cp, gp, big, big,
                                               static_cast<uint64_t*>(out->tris), s);
        pm.mark(ISO_PASS_MC_TRIANGLES);
    }
    ISO_CUDA(ctx, cudaGetLastError());
    return ISO_OK;
}

iso_status slab_prepare(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid, int64_t k0,
                        int64_t k1, Grid& g, Plans& pl, FeBuffers& b, cudaStream_t s)
{
    if (!ctx || !grid) return ISO_ERR_INVALID_ARG;
    if (algo != ISO_FLYING_EDGES && algo != ISO_MARCHING_CUBES) return ISO_ERR_INVALID_ARG;  // no Dup slabs
    if (!slab_grid(grid, algo, k0, k1, g)) return ISO_ERR_INVALID_ARG;
    if (empty_grid(g)) return ISO_OK;
    if (!volume) return ISO_ERR_INVALID_ARG;
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    pl = make_plans(ctx, g);
    if (!pl.gp.fits) {
        ctx->last_error = "slabs need rows of at most 1024 points";
        return ISO_ERR_INVALID_ARG;
    }
    return ensure_scratch(ctx, g, pl.cp, b, s);
}

// ---------------------------------------------------------------------------
// Streamed host extraction: the volume goes to the device slab by slab on a
// copy stream, each slab's planes k0-1 .. k1+1 into one of kStreamWindows
// device windows (so device memory does not grow with nz: volumes larger
// than the device stream through); each slab is counted as soon as its
// planes have landed, generated with the offsets of the slabs before it into
// one of two device staging meshes, and its part of the mesh goes back on a
// second copy stream while the next slabs are copied and computed.  Host <->
// device copies of the volume and mesh overlap with each other and with the
// kernels.
// ---------------------------------------------------------------------------
constexpr int kStreamPlanes = 64;  // planes per slab of the streamed path
constexpr int kTailPlanes = 16;    // the smallest slabs, at the end of the volume
constexpr int kStreamWindows = 3;  // device windows of the volume

cudaEvent_t sync_event(iso_ctx* ctx, size_t q)
{
    while (ctx->sync_events.size() <= q) {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        ctx->sync_events.push_back(e);
    }
    return ctx->sync_events[q];
}

// Staging meshes of at least (V, T); growing waits for the streams.
iso_status ensure_stage(iso_ctx* ctx, long long V, long long T, int ib, cudaStream_t s)
{
    if (V <= ctx->st_cap_points && T <= ctx->st_cap_tris && ib == ctx->st_index_bytes) return ISO_OK;
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    ISO_CUDA(ctx, cudaStreamSynchronize(ctx->s_d2h));
    const long long cv = std::max(V + V / 4 + 1024, ctx->st_cap_points);
    const long long ct = std::max(T + T / 4 + 1024, ctx->st_index_bytes == ib ? ctx->st_cap_tris : 0ll);
    for (int q = 0; q < 2; ++q) {
        cudaFree(ctx->st_points[q]);
        cudaFree(ctx->st_normals[q]);
        cudaFree(ctx->st_tris[q]);
        ctx->st_points[q] = ctx->st_normals[q] = nullptr;
        ctx->st_tris[q] = nullptr;
    }
    ctx->st_cap_points = ctx->st_cap_tris = 0;
    for (int q = 0; q < 2; ++q) {
        ISO_CUDA(ctx, cudaMalloc(&ctx->st_points[q], (size_t)cv * 12));
        ISO_CUDA(ctx, cudaMalloc(&ctx->st_normals[q], (size_t)cv * 12));
        ISO_CUDA(ctx, cudaMalloc(&ctx->st_tris[q], (size_t)ct * 3 * ib));
    }
    ctx->st_cap_points = cv;
    ctx->st_cap_tris = ct;
    ctx->st_index_bytes = ib;
    return ISO_OK;
}

bool stream_eligible(const iso_ctx* ctx, iso_algorithm algo, const Grid& g)
{
    return algo != ISO_MC_DUPFREE && !empty_grid(g) && g.nz >= 2 * kStreamPlanes && iso::gen_plan(g, ctx->nsm).fits;
}

iso_status extract_host_streamed(iso_ctx* ctx, iso_algorithm algo, const void* volume, int dtype,
                                 const iso_grid* grid, const Grid& gfull, float isoval, iso_mesh* out, cudaStream_t s)
{
    if (!ctx->s_h2d) ISO_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_h2d, cudaStreamNonBlocking));
    if (!ctx->s_d2h) ISO_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_d2h, cudaStreamNonBlocking));
    if (!ctx->s_cnt) ISO_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_cnt, cudaStreamNonBlocking));
    const int nz = gfull.nz;
    const size_t plane = (size_t)gfull.nx * gfull.ny;
    // Slabs of at most kStreamPlanes planes; the last kStreamPlanes planes go
    // as slabs of halving size (1/2, 1/4, ... down to kTailPlanes, that one
    // twice), so that little is left to count, generate and copy back once
    // the last planes have landed.
    std::vector<int> kb;  // slab q = planes kb[q] .. kb[q + 1] - 1
    {
        const int body = nz - kStreamPlanes;  // >= kStreamPlanes (stream_eligible)
        const int nb = (body + kStreamPlanes - 1) / kStreamPlanes;
        for (int q = 0; q < nb; ++q) kb.push_back((int)((long long)q * body / nb));
        int at = body;
        for (int part = kStreamPlanes / 2; part >= kTailPlanes; part /= 2) {
            kb.push_back(at);
            at += part;
        }
        kb.push_back(at);
        kb.push_back(nz);
    }
    const int nslab = (int)kb.size() - 1;
    auto slab_k0 = [&](int q) { return kb[q]; };
    auto data_lo = [&](int q) { return std::max(slab_k0(q) - 1, 0); };
    auto data_hi = [&](int q) { return std::min(slab_k0(q + 1) + 1, nz - 1); };  // inclusive
    int wplanes = 0;
    for (int q = 0; q < nslab; ++q) wplanes = std::max(wplanes, data_hi(q) - data_lo(q) + 1);
    const size_t wbytes = (size_t)wplanes * plane * sizeof(float);
    if (kStreamWindows * wbytes > ctx->d_volume_bytes) {
        ISO_CUDA(ctx, cudaDeviceSynchronize());
        cudaFree(ctx->d_volume);
        ctx->d_volume = nullptr;
        ctx->d_volume_bytes = 0;
        ISO_CUDA(ctx, cudaMalloc(&ctx->d_volume, kStreamWindows * wbytes));
        ctx->d_volume_bytes = kStreamWindows * wbytes;
    }
    auto window = [&](int q) { return ctx->d_volume + (size_t)(q % kStreamWindows) * wplanes * plane; };
    // typed samples land in their own windows and are converted into the float ones
    const size_t elem = iso::dtype_bytes(dtype);
    const bool typed = dtype != ISO_FLOAT32;
    if (typed) {
        const iso_status ts = ensure_typed(ctx, kStreamWindows * (size_t)wplanes * plane * elem, s);
        if (ts != ISO_OK) return ts;
    }
    auto typed_window = [&](int q) {
        return static_cast<char*>(ctx->d_typed) + (size_t)(q % kStreamWindows) * wplanes * plane * elem;
    };
    {
        const iso_status e = ensure_h_slab(ctx);
        if (e != ISO_OK) return e;
    }
    {  // both scratch sets sized for the largest slab up front: none is reallocated while a stream uses it
        size_t best = 0;
        int qb = 0;
        for (int q = 0; q < nslab; ++q) {
            Grid gq;
            if (!slab_grid(grid, algo, slab_k0(q), slab_k0(q + 1), gq)) return ISO_ERR_INVALID_ARG;
            const size_t need = scratch_size(gq, make_plans(ctx, gq).cp);
            if (need > best) {
                best = need;
                qb = q;
            }
        }
        Grid gq;
        if (!slab_grid(grid, algo, slab_k0(qb), slab_k0(qb + 1), gq)) return ISO_ERR_INVALID_ARG;
        const Plans pq = make_plans(ctx, gq);
        FeBuffers unused;
        iso_status e = ensure_scratch(ctx, gq, pq.cp, unused, s);
        if (e == ISO_OK) e = ensure_scratch_b(ctx, gq, pq.cp, unused, s);
        if (e != ISO_OK) return e;
    }
    const char* src = static_cast<const char*>(volume);
    // events: 1 + q the planes of slab q have landed; 1 + nslab + w window w is
    // free again; 1 + nslab + kStreamWindows + sb slab generated into
    // staging sb; 1 + nslab + kStreamWindows + 2 + sb staging sb copied out
    const size_t ev_win = 1 + nslab, ev_gen = ev_win + kStreamWindows, ev_out = ev_gen + 2;
    if (!sync_event(ctx, ev_out + 5)) return ISO_ERR_CUDA;  // with the count and scratch events below
    ISO_CUDA(ctx, cudaEventRecord(sync_event(ctx, 0), s));  // after the caller's earlier work on s
    ISO_CUDA(ctx, cudaStreamWaitEvent(ctx->s_h2d, sync_event(ctx, 0), 0));
    ISO_CUDA(ctx, cudaStreamWaitEvent(ctx->s_cnt, sync_event(ctx, 0), 0));
    // the window slab q's samples land in (typed: converted from there)
    auto landing = [&](int q) -> char* {
        return typed ? typed_window(q) : reinterpret_cast<char*>(window(q));
    };
    auto copy_in = [&](int q) -> iso_status {
        if (q >= kStreamWindows)  // the window's previous slab is generated
            ISO_CUDA(ctx, cudaStreamWaitEvent(ctx->s_h2d, sync_event(ctx, ev_win + q % kStreamWindows), 0));
        const int lo = data_lo(q), hi = data_hi(q);
        // the planes slab q shares with slab q-1 (k0-1 .. k0+1) come from its
        // window, which is refilled only after this copy on the same stream
        const int shared = q > 0 ? std::min(data_hi(q - 1), hi) - lo + 1 : 0;
        if (shared > 0)
            ISO_CUDA(ctx, cudaMemcpyAsync(landing(q), landing(q - 1) + (size_t)(lo - data_lo(q - 1)) * plane * elem,
                                          (size_t)shared * plane * elem, cudaMemcpyDeviceToDevice, ctx->s_h2d));
        const int from = lo + std::max(shared, 0);
        if (from <= hi)
            ISO_CUDA(ctx, cudaMemcpyAsync(landing(q) + (size_t)(from - lo) * plane * elem,
                                          src + (size_t)from * plane * elem, (size_t)(hi - from + 1) * plane * elem,
                                          cudaMemcpyHostToDevice, ctx->s_h2d));
        ISO_CUDA(ctx, cudaEventRecord(sync_event(ctx, 1 + q), ctx->s_h2d));
        return ISO_OK;
    };
    for (int q = 0; q < std::min(nslab, kStreamWindows); ++q) {
        const iso_status c = copy_in(q);
        if (c != ISO_OK) return c;
    }
    const bool mc = algo == ISO_MARCHING_CUBES;
    long long V = 0, T = 0;
    bool room = true;  // the caller's buffers hold everything so far
    iso_status st = ISO_OK;
    // Slab q+1 is counted (into the other scratch set, on the count stream)
    // while slab q is generated, so the host reads counts that have already
    // landed and the generate pass of slab q never waits for the volume of
    // slab q+1.
    struct SlabRun {
        Grid g;
        Plans pl;
        FeBuffers b;
        int k0, k1;
    } run[2];
    const size_t ev_cnt = ev_out + 2;  // 2 events: counts of slab q landed in h_slab + 9 * (q & 1)
    const size_t ev_scr = ev_cnt + 2;  // 2 events: slab q generated, scratch set q & 1 free again
    auto start_count = [&](int q) -> iso_status {
        SlabRun& r = run[q & 1];
        r.k0 = slab_k0(q);
        r.k1 = slab_k0(q + 1);
        if (!slab_grid(grid, algo, r.k0, r.k1, r.g)) return ISO_ERR_INVALID_ARG;
        r.pl = make_plans(ctx, r.g);
        cudaStream_t sc = ctx->s_cnt;
        ISO_CUDA(ctx, cudaStreamWaitEvent(sc, sync_event(ctx, 1 + q), 0));
        if (q >= 2) ISO_CUDA(ctx, cudaStreamWaitEvent(sc, sync_event(ctx, ev_scr + (q & 1)), 0));
        if (typed)
            iso::launch_to_float(typed_window(q), dtype, window(q),
                                 (long long)(data_hi(q) - data_lo(q) + 1) * (long long)plane, ctx->nsm, sc);
        iso_status e =
            (q & 1) ? ensure_scratch_b(ctx, r.g, r.pl.cp, r.b, sc) : ensure_scratch(ctx, r.g, r.pl.cp, r.b, sc);
        if (e != ISO_OK) return e;
        e = slab_count_enqueue(ctx, algo, window(q), r.g, r.k0, r.k1, isoval, r.pl, r.b, sc,
                               ctx->h_slab + 9 * (q & 1));
        if (e != ISO_OK) return e;
        ISO_CUDA(ctx, cudaEventRecord(sync_event(ctx, ev_cnt + (q & 1)), sc));
        return ISO_OK;
    };
    st = start_count(0);
    for (int q = 0; q < nslab && st == ISO_OK; ++q) {
        if (q + 1 < nslab) {
            st = start_count(q + 1);
            if (st != ISO_OK) break;
        }
        SlabRun& r = run[q & 1];
        const int k0 = r.k0, k1 = r.k1;
        const Grid& g = r.g;
        const Plans& pl = r.pl;
        FeBuffers& b = r.b;
        const float* win = window(q);  // holds planes g.kd = data_lo(q) ..
        ISO_CUDA(ctx, cudaEventSynchronize(sync_event(ctx, ev_cnt + (q & 1))));
        ISO_CUDA(ctx, cudaStreamWaitEvent(s, sync_event(ctx, ev_cnt + (q & 1)), 0));
        SlabCounts c;
        slab_count_read(g, k0, k1, ctx->h_slab + 9 * (q & 1), c);
        const long long Vq = (long long)(c.hi[mc ? 2 : 0] - c.lo[mc ? 2 : 0]), Tq = (long long)(c.hi[1] - c.lo[1]);
        const long long top = V + (mc ? Vq : (long long)c.tot[0]);  // largest id the slab references
        if (out->index_bytes == 4 && top > 0xffffffffll) {
            ctx->last_error = "more than 2^32-1 vertices: use 64-bit indices";
            st = ISO_ERR_OVERFLOW;
            break;
        }
        if (V + Vq > out->cap_points || T + Tq > out->cap_tris) room = false;
        if (room && (Vq > 0 || Tq > 0)) {
            const int sb = q & 1;
            st = ensure_stage(ctx, Vq, Tq, out->index_bytes, s);
            if (st != ISO_OK) break;
            if (q >= 2) ISO_CUDA(ctx, cudaStreamWaitEvent(s, sync_event(ctx, ev_out + sb), 0));  // staging free
            if (mc) {
                st = ensure_fe2mc(ctx, (long long)c.tot[0], s);
                if (st != ISO_OK) break;
                b.fe2mc = ctx->fe2mc;
            }
            iso_mesh dm{};
            dm.points = ctx->st_points[sb];
            dm.normals = ctx->st_normals[sb];
            dm.tris = ctx->st_tris[sb];
            dm.index_bytes = out->index_bytes;
            dm.cap_points = Vq;
            dm.cap_tris = Tq;
            st = slab_generate(ctx, algo, win, g, k0, k1, isoval, pl, b, c, V, T, &dm, s);
            if (st != ISO_OK) break;
            cudaEvent_t gen_done = sync_event(ctx, ev_gen + sb);
            ISO_CUDA(ctx, cudaEventRecord(gen_done, s));
            ISO_CUDA(ctx, cudaStreamWaitEvent(ctx->s_d2h, gen_done, 0));
            if (Vq > 0) {
                ISO_CUDA(ctx, cudaMemcpyAsync(out->points + 3 * V, dm.points, (size_t)Vq * 12, cudaMemcpyDeviceToHost,
                                              ctx->s_d2h));
                ISO_CUDA(ctx, cudaMemcpyAsync(out->normals + 3 * V, dm.normals, (size_t)Vq * 12,
                                              cudaMemcpyDeviceToHost, ctx->s_d2h));
            }
            if (Tq > 0) {
                char* dst = static_cast<char*>(out->tris) + (size_t)T * 3 * out->index_bytes;
                ISO_CUDA(ctx, cudaMemcpyAsync(dst, dm.tris, (size_t)Tq * 3 * out->index_bytes, cudaMemcpyDeviceToHost,
                                              ctx->s_d2h));
            }
            ISO_CUDA(ctx, cudaEventRecord(sync_event(ctx, ev_out + sb), ctx->s_d2h));
        }
        V += Vq;
        T += Tq;
        // window q % kStreamWindows and scratch set q & 1 are free once slab q's kernels are done
        ISO_CUDA(ctx, cudaEventRecord(sync_event(ctx, ev_win + q % kStreamWindows), s));
        ISO_CUDA(ctx, cudaEventRecord(sync_event(ctx, ev_scr + (q & 1)), s));
        if (q + kStreamWindows < nslab) {
            st = copy_in(q + kStreamWindows);
            if (st != ISO_OK) break;
        }
    }
    // the mesh has landed when the copy streams, the count stream and s are done
    const iso_status sh = cudaStreamSynchronize(ctx->s_h2d) == cudaSuccess ? ISO_OK : ISO_ERR_CUDA;
    const iso_status sd = cudaStreamSynchronize(ctx->s_d2h) == cudaSuccess ? ISO_OK : ISO_ERR_CUDA;
    const iso_status sk = cudaStreamSynchronize(ctx->s_cnt) == cudaSuccess ? ISO_OK : ISO_ERR_CUDA;
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    if (st != ISO_OK) return st;
    if (sh != ISO_OK || sd != ISO_OK || sk != ISO_OK) return ISO_ERR_CUDA;
    out->n_points = V;
    out->n_tris = T;
    if (!room) {
        ctx->last_error = "output buffers too small";
        return ISO_ERR_CAPACITY;
    }
    return ISO_OK;
}


}  // namespace

extern "C" {

iso_status iso_count_slab(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid, int64_t k0,
                          int64_t k1, float isoval, int64_t* n_points, int64_t* n_tris, void* stream)
{
    if (!n_points || !n_tris) return ISO_ERR_INVALID_ARG;
    *n_points = *n_tris = 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Grid g;
    Plans pl;
    FeBuffers b;
    iso_status st = slab_prepare(ctx, algo, volume, grid, k0, k1, g, pl, b, s);
    if (st != ISO_OK || empty_grid(g)) return st;
    SlabCounts c;
    st = slab_count(ctx, algo, volume, g, k0, k1, isoval, pl, b, s, c);
    if (st != ISO_OK) return st;
    const int av = algo == ISO_MARCHING_CUBES ? 2 : 0;
    *n_points = (int64_t)(c.hi[av] - c.lo[av]);
    *n_tris = (int64_t)(c.hi[1] - c.lo[1]);
    return ISO_OK;
}

iso_status iso_extract_slab(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid, int64_t k0,
                            int64_t k1, float isoval, int64_t point_offset, int64_t tri_offset, iso_mesh* out,
                            void* stream)
{
    iso_status st = check_mesh(out);
    if (st != ISO_OK) return st;
    out->n_points = out->n_tris = 0;
    if (point_offset < 0 || tri_offset < 0) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Grid g;
    Plans pl;
    FeBuffers b;
    st = slab_prepare(ctx, algo, volume, grid, k0, k1, g, pl, b, s);
    if (st != ISO_OK || empty_grid(g)) return st;
    SlabCounts c;
    st = slab_count(ctx, algo, volume, g, k0, k1, isoval, pl, b, s, c);
    if (st != ISO_OK) return st;
    const bool mc = algo == ISO_MARCHING_CUBES;
    const long long V = (long long)(c.hi[mc ? 2 : 0] - c.lo[mc ? 2 : 0]), T = (long long)(c.hi[1] - c.lo[1]);
    out->n_points = V;
    out->n_tris = T;
    // the largest vertex id the slab's triangles reference
    const long long top = point_offset + (mc ? V : (long long)c.tot[0]);
    if (out->index_bytes == 4 && top > 0xffffffffll) {
        ctx->last_error = "more than 2^32-1 vertices: use 64-bit indices";
        return ISO_ERR_OVERFLOW;
    }
    if (V > out->cap_points || T > out->cap_tris) {
        ctx->last_error = "output buffers too small";
        return ISO_ERR_CAPACITY;
    }
    if (mc) {
        st = ensure_fe2mc(ctx, (long long)c.tot[0], s);
        if (st != ISO_OK) return st;
        b.fe2mc = ctx->fe2mc;
    }
    st = slab_generate(ctx, algo, volume, g, k0, k1, isoval, pl, b, c, point_offset, tri_offset, out, s);
    if (st != ISO_OK) return st;
    ISO_CUDA(ctx, cudaGetLastError());
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    return ISO_OK;
}


const char* iso_status_string(iso_status s)
{
    switch (s) {
        case ISO_OK: return "ok";
        case ISO_ERR_INVALID_ARG: return "invalid argument";
        case ISO_ERR_OOM: return "out of memory";
        case ISO_ERR_CUDA: return "CUDA error";
        case ISO_ERR_CAPACITY: return "output buffers too small";
        case ISO_ERR_OVERFLOW: return "index overflow";
        case ISO_ERR_TIMEOUT: return "device wait timed out";
        case ISO_ERR_IO: return "file error";
        case ISO_ERR_FORMAT: return "bad file format";
        case ISO_ERR_STATE: return "call out of order";
        case ISO_ERR_TOO_LARGE: return "grid larger than the fixed scratch of the allocation-free entry point";
    }
    return "unknown status";
}

const char* iso_version(void) { return kVersion; }

iso_status iso_ctx_create(int device, iso_ctx** out)
{
    if (!out) return ISO_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || device < 0 || device >= ndev) return e != cudaSuccess ? ISO_ERR_CUDA : ISO_ERR_INVALID_ARG;
    iso_ctx* ctx = new (std::nothrow) iso_ctx();
    if (!ctx) return ISO_ERR_OOM;
    ctx->device = device;
    iso_status st = ISO_OK;
    do {
        if ((e = cudaSetDevice(device)) != cudaSuccess) { st = cuda_fail(ctx, e, "cudaSetDevice"); break; }
        if ((e = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaDeviceGetAttribute");
            break;
        }
        CaseTables h;
        build_case_tables(h);
        if ((e = cudaMalloc(&ctx->d_cases, sizeof(CaseTables))) != cudaSuccess) { st = cuda_fail(ctx, e, "cudaMalloc"); break; }
        if ((e = cudaMemcpy(ctx->d_cases, &h, sizeof(CaseTables), cudaMemcpyHostToDevice)) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaMemcpy");
            break;
        }
        if ((e = cudaMallocHost(&ctx->h_totals, 4 * sizeof(unsigned long long))) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaMallocHost");
            break;
        }
    } while (0);
    if (st != ISO_OK) {
        iso_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return ISO_OK;
}

iso_status iso_ctx_destroy(iso_ctx* ctx)
{
    if (!ctx) return ISO_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    cudaFree(ctx->d_cases);
    cudaFree(ctx->scratch);
    cudaFree(ctx->fe2mc);
    cudaFree(ctx->d_volume);
    cudaFree(ctx->d_points);
    cudaFree(ctx->d_normals);
    cudaFree(ctx->d_tris);
    if (ctx->h_totals) cudaFreeHost(ctx->h_totals);
    if (ctx->h_slab) cudaFreeHost(ctx->h_slab);
    cudaFree(ctx->d_typed);
    cudaFree(ctx->scratch_b);
    for (int q = 0; q < 2; ++q) {
        cudaFree(ctx->st_points[q]);
        cudaFree(ctx->st_normals[q]);
        cudaFree(ctx->st_tris[q]);
    }
    for (cudaEvent_t e : ctx->sync_events) cudaEventDestroy(e);
    if (ctx->s_h2d) cudaStreamDestroy(ctx->s_h2d);
    if (ctx->s_d2h) cudaStreamDestroy(ctx->s_d2h);
    if (ctx->s_cnt) cudaStreamDestroy(ctx->s_cnt);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (cudaGraphExec_t x : ctx->batch_exec)
        if (x) cudaGraphExecDestroy(x);
    if (ctx->one_exec) cudaGraphExecDestroy(ctx->one_exec);
    for (cudaStream_t q : ctx->lane_streams) cudaStreamDestroy(q);
    for (cudaStream_t q : ctx->fused_streams) cudaStreamDestroy(q);
    for (cudaEvent_t e : ctx->fused_join) cudaEventDestroy(e);
    if (ctx->fused_fork) cudaEventDestroy(ctx->fused_fork);
    for (cudaEvent_t e : ctx->lane_join) cudaEventDestroy(e);
    for (cudaEvent_t e : {ctx->batch_fork, ctx->batch_t0, ctx->batch_t1})
        if (e) cudaEventDestroy(e);
    if (ctx->s_capture) cudaStreamDestroy(ctx->s_capture);
    cudaFree(ctx->batch_arena);
    if (ctx->h_batch) cudaFreeHost(ctx->h_batch);
    if (ctx->h_fused) cudaFreeHost(ctx->h_fused);
    delete ctx;
    return ISO_OK;
}

const char* iso_ctx_last_error(const iso_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int64_t iso_ctx_scratch_bytes(const iso_ctx* ctx)
{
    return ctx ? (int64_t)(ctx->scratch_bytes + (size_t)ctx->fe2mc_cap * 4) : 0;
}

iso_status iso_ctx_profile(iso_ctx* ctx, int enable)
{
    if (!ctx) return ISO_ERR_INVALID_ARG;
    ctx->profiling = enable != 0;
    return ISO_OK;
}

iso_status iso_ctx_profile_read(iso_ctx* ctx, double* ms, int64_t* launches)
{
    if (!ctx || !ms || !launches) return ISO_ERR_INVALID_ARG;
    for (int p = 0; p < ISO_NUM_PASSES; ++p) {
        ms[p] = 0.0;
        launches[p] = 0;
    }
    iso_status st = ISO_OK;
    for (const auto& sp : ctx->spans) {
        cudaError_t e = cudaEventSynchronize(sp.end);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, sp.begin, sp.end);
        if (e != cudaSuccess) {
            st = cuda_fail(ctx, e, "iso_ctx_profile_read");
            continue;
        }
        ms[sp.pass] += t;
        launches[sp.pass] += 1;
    }
    ctx->spans.clear();
    ctx->events_used = 0;
    return st;
}

iso_status iso_count_device(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                            float isoval, int64_t* n_points, int64_t* n_tris, void* stream)
{
    if (!ctx || !grid || !n_points || !n_tris) return ISO_ERR_INVALID_ARG;
    if (!valid_algo(algo)) return ISO_ERR_INVALID_ARG;
    Grid g;
    if (!make_grid(grid, g)) return ISO_ERR_INVALID_ARG;
    *n_points = 0;
    *n_tris = 0;
    if (empty_grid(g)) return ISO_OK;
    if (!volume) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const Plans pl = make_plans(ctx, g);
    FeBuffers b;
    iso_status st = ensure_scratch(ctx, g, pl.cp, b, s);
    if (st != ISO_OK) return st;
    PassMarks pm(ctx, s);
    enqueue_count(ctx, algo, volume, g, isoval, pl, b, s, pm);
    ISO_CUDA(ctx, cudaGetLastError());
    ISO_CUDA(ctx, cudaMemcpyAsync(ctx->h_totals, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    *n_points = (int64_t)ctx->h_totals[0];
    *n_tris = (int64_t)ctx->h_totals[1];
    return ISO_OK;
}

iso_status iso_extract_device_async(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                                    float isoval, iso_mesh* out, int64_t* result_host, void* stream)
{
    if (!ctx || !grid || !result_host) return ISO_ERR_INVALID_ARG;
    if (!valid_algo(algo)) return ISO_ERR_INVALID_ARG;
    iso_status st = check_mesh(out);
    if (st != ISO_OK) return st;
    Grid g;
    if (!make_grid(grid, g)) return ISO_ERR_INVALID_ARG;
    result_host[0] = result_host[1] = result_host[2] = result_host[3] = 0;
    if (empty_grid(g)) return ISO_OK;
    if (!volume) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const Plans pl = make_plans(ctx, g);
    if (algo == ISO_MC_DUPFREE && !pl.gp.fits) {
        ctx->last_error = "the duplicate-free order needs rows of at most 1024 points";
        return ISO_ERR_INVALID_ARG;
    }
    FeBuffers b;
    st = ensure_scratch(ctx, g, pl.cp, b, s);
    if (st != ISO_OK) return st;
    if (algo == ISO_MARCHING_CUBES) {
        st = ensure_fe2mc(ctx, out->cap_points, s);
        if (st != ISO_OK) return st;
        b.fe2mc = ctx->fe2mc;
    }
    if (ctx->one_graph && !ctx->profiling) return extract_graph(ctx, algo, volume, g, grid, isoval, pl, b, out,
                                                                result_host, s);
    PassMarks pm(ctx, s);
    enqueue_count(ctx, algo, volume, g, isoval, pl, b, s, pm);
    enqueue_generate(ctx, algo, volume, g, isoval, pl, b, out, s, pm);
    ISO_CUDA(ctx, cudaGetLastError());
    ISO_CUDA(ctx, cudaMemcpyAsync(result_host, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    return ISO_OK;
}

iso_status iso_extract_device(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                              float isoval, iso_mesh* out, void* stream)
{
    if (!ctx) return ISO_ERR_INVALID_ARG;
    iso_status st = check_mesh(out);
    if (st != ISO_OK) return st;
    out->n_points = out->n_tris = 0;
    int64_t* res = reinterpret_cast<int64_t*>(ctx->h_totals);
    st = iso_extract_device_async(ctx, algo, volume, grid, isoval, out, res, stream);
    if (st != ISO_OK) return st;
    ISO_CUDA(ctx, cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    return finish_counts(ctx, out, res[0], res[1], res[3], &out->n_points, &out->n_tris);
}

static iso_status extract_host_impl(iso_ctx* ctx, iso_algorithm algo, const void* volume, int dtype,
                                    const iso_grid* grid, float isoval, iso_mesh* out, void* stream)
{
    if (!ctx || !grid) return ISO_ERR_INVALID_ARG;
    if (!valid_algo(algo) || iso::dtype_bytes(dtype) == 0) return ISO_ERR_INVALID_ARG;
    iso_status st = check_mesh(out);
    if (st != ISO_OK) return st;
    Grid g;
    if (!make_grid(grid, g)) return ISO_ERR_INVALID_ARG;
    out->n_points = out->n_tris = 0;
    if (empty_grid(g)) return ISO_OK;
    if (!volume) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ctx->stream_host && stream_eligible(ctx, algo, g))
        return extract_host_streamed(ctx, algo, volume, dtype, grid, g, isoval, out, s);
    const size_t vbytes = (size_t)g.nx * g.ny * g.nz * sizeof(float);
    if (vbytes > ctx->d_volume_bytes) {
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
        cudaFree(ctx->d_volume);
        ctx->d_volume = nullptr;
        ctx->d_volume_bytes = 0;
        ISO_CUDA(ctx, cudaMalloc(&ctx->d_volume, vbytes));
        ctx->d_volume_bytes = vbytes;
    }
    if (dtype == ISO_FLOAT32) {
        ISO_CUDA(ctx, cudaMemcpyAsync(ctx->d_volume, volume, vbytes, cudaMemcpyHostToDevice, s));
    } else {  // narrow samples over the link, float on the device
        const long long n = (long long)g.nx * g.ny * g.nz;
        iso_status ts = ensure_typed(ctx, (size_t)n * iso::dtype_bytes(dtype), s);
        if (ts != ISO_OK) return ts;
        ISO_CUDA(ctx, cudaMemcpyAsync(ctx->d_typed, volume, (size_t)n * iso::dtype_bytes(dtype), cudaMemcpyHostToDevice,
                                      s));
        iso::launch_to_float(ctx->d_typed, dtype, ctx->d_volume, n, ctx->nsm, s);
    }
    const Plans pl = make_plans(ctx, g);
    if (algo == ISO_MC_DUPFREE && !pl.gp.fits) {
        ctx->last_error = "the duplicate-free order needs rows of at most 1024 points";
        return ISO_ERR_INVALID_ARG;
    }
    FeBuffers b;
    st = ensure_scratch(ctx, g, pl.cp, b, s);
    if (st != ISO_OK) return st;
    PassMarks pm(ctx, s);
    enqueue_count(ctx, algo, ctx->d_volume, g, isoval, pl, b, s, pm);
    ISO_CUDA(ctx, cudaGetLastError());
    ISO_CUDA(ctx, cudaMemcpyAsync(ctx->h_totals, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    const long long V = (long long)ctx->h_totals[0], T = (long long)ctx->h_totals[1];
    st = finish_counts(ctx, out, V, T, 0, &out->n_points, &out->n_tris);
    if (st != ISO_OK) return st;
    // device output staging, grown on demand
    if (V > ctx->d_cap_points || T > ctx->d_cap_tris || out->index_bytes != ctx->d_index_bytes) {
        cudaFree(ctx->d_points);
        cudaFree(ctx->d_normals);
        cudaFree(ctx->d_tris);
        ctx->d_points = ctx->d_normals = nullptr;
        ctx->d_tris = nullptr;
        ctx->d_cap_points = ctx->d_cap_tris = 0;
        const long long cv = V + V / 4 + 1024, ct = T + T / 4 + 1024;
        ISO_CUDA(ctx, cudaMalloc(&ctx->d_points, (size_t)cv * 12));
        ISO_CUDA(ctx, cudaMalloc(&ctx->d_normals, (size_t)cv * 12));
        ISO_CUDA(ctx, cudaMalloc(&ctx->d_tris, (size_t)ct * 3 * out->index_bytes));
        ctx->d_cap_points = cv;
        ctx->d_cap_tris = ct;
        ctx->d_index_bytes = out->index_bytes;
    }
    iso_mesh dm{};
    dm.points = ctx->d_points;
    dm.normals = ctx->d_normals;
    dm.tris = ctx->d_tris;
    dm.index_bytes = out->index_bytes;
    dm.cap_points = ctx->d_cap_points;
    dm.cap_tris = ctx->d_cap_tris;
    if (algo == ISO_MARCHING_CUBES) {
        st = ensure_fe2mc(ctx, dm.cap_points, s);
        if (st != ISO_OK) return st;
        b.fe2mc = ctx->fe2mc;
    }
    enqueue_generate(ctx, algo, ctx->d_volume, g, isoval, pl, b, &dm, s, pm);
    ISO_CUDA(ctx, cudaGetLastError());
    if (V > 0) {
        ISO_CUDA(ctx, cudaMemcpyAsync(out->points, dm.points, (size_t)V * 12, cudaMemcpyDeviceToHost, s));
        ISO_CUDA(ctx, cudaMemcpyAsync(out->normals, dm.normals, (size_t)V * 12, cudaMemcpyDeviceToHost, s));
    }
    if (T > 0) {
        ISO_CUDA(ctx, cudaMemcpyAsync(out->tris, dm.tris, (size_t)T * 3 * out->index_bytes, cudaMemcpyDeviceToHost, s));
    }
    ISO_CUDA(ctx, cudaMemcpyAsync(ctx->h_totals, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    return finish_counts(ctx, out, V, T, (long long)ctx->h_totals[3], &out->n_points, &out->n_tris);
}

iso_status iso_extract_host(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                            float isoval, iso_mesh* out, void* stream)
{
    return extract_host_impl(ctx, algo, volume, ISO_FLOAT32, grid, isoval, out, stream);
}

iso_status iso_extract_host_typed(iso_ctx* ctx, iso_algorithm algo, const void* volume, iso_dtype dtype,
                                  const iso_grid* grid, float isoval, iso_mesh* out, void* stream)
{
    return extract_host_impl(ctx, algo, volume, dtype, grid, isoval, out, stream);
}

// 8- and 16-bit samples read as they are (count_narrow.cu, k_vertices over the
// sample type): Flying Edges and Marching Cubes over whole grids that
// narrow_fits takes, with the scan and the generate passes of the float path.
static iso_status extract_device_narrow(iso_ctx* ctx, iso_algorithm algo, const void* volume, int dtype,
                                        const Grid& g, float isoval, iso_mesh* out, cudaStream_t s)
{
    const Plans pl = make_plans(ctx, g);
    FeBuffers b;
    iso_status st = ensure_scratch(ctx, g, pl.cp, b, s);
    if (st != ISO_OK) return st;
    const bool mc = algo == ISO_MARCHING_CUBES;
    const long long capV = vertex_limit(out, out->cap_points);
    const long long capT = out->cap_tris;
    const bool i4 = out->index_bytes == 4;
    PassMarks pm(ctx, s);
    iso::launch_count_narrow(volume, dtype, g, isoval, mc, pl.cp, b, s);
    pm.mark(ISO_PASS_COUNT);
    iso::launch_scan(g, pl.cp, mc ? iso::kScanMC : iso::kScanFE, b, s);
    pm.mark(ISO_PASS_SCAN);
    if (!mc) {
        if (i4)
            iso::launch_fe_gen_warps<uint32_t>(nullptr, g, isoval, ctx->d_cases, b, pl.cp, pl.gp, capV, capT, out->points,
                                               out->normals, static_cast<uint32_t*>(out->tris), ctx->reverse, s);
        else
            iso::launch_fe_gen_warps<uint64_t>(nullptr, g, isoval, ctx->d_cases, b, pl.cp, pl.gp, capV, capT, out->points,
                                               out->normals, static_cast<uint64_t*>(out->tris), ctx->reverse, s);
        pm.mark(ISO_PASS_FE_GENERATE);
        if (iso::launch_fe_vertices_narrow(volume, dtype, g, isoval, b, pl.gp, capV, capT, out->points, out->normals, s))
            pm.mark(ISO_PASS_VERTICES);
    } else {
        st = ensure_fe2mc(ctx, out->cap_points, s);
        if (st != ISO_OK) return st;
        b.fe2mc = ctx->fe2mc;
        const long long capM = capV < 0xffffffffll ? capV : 0xffffffffll;  // fe2mc holds 32-bit ids
        if (i4)
            iso::launch_mc_gen_tris<uint32_t>(g, ctx->d_cases, b, pl.cp, pl.gp, capM, capT, out->points,
                                              static_cast<uint32_t*>(out->tris), ctx->reverse, s);
        else
            iso::launch_mc_gen_tris<uint64_t>(g, ctx->d_cases, b, pl.cp, pl.gp, capM, capT, out->points,
                                              static_cast<uint64_t*>(out->tris), ctx->reverse, s);
        pm.mark(ISO_PASS_MC_VERTICES);
        if (iso::launch_mc_vertices_narrow(volume, dtype, g, isoval, b, pl.gp, capM, capT, out->points, out->normals, s))
            pm.mark(ISO_PASS_VERTICES);
        if (i4)
            iso::launch_mc_remap<uint32_t>(b, pl.gp, capM, capT, static_cast<uint32_t*>(out->tris), s);
        else
            iso::launch_mc_remap<uint64_t>(b, pl.gp, capM, capT, static_cast<uint64_t*>(out->tris), s);
        pm.mark(ISO_PASS_MC_TRIANGLES);
    }
    ISO_CUDA(ctx, cudaGetLastError());
    int64_t* res = reinterpret_cast<int64_t*>(ctx->h_totals);
    ISO_CUDA(ctx, cudaMemcpyAsync(res, b.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    ISO_CUDA(ctx, cudaStreamSynchronize(s));
    return finish_counts(ctx, out, res[0], res[1], res[3], &out->n_points, &out->n_tris);
}

iso_status iso_ctx_set_narrow(iso_ctx* ctx, int enable)
{
    if (!ctx) return ISO_ERR_INVALID_ARG;
    ctx->narrow = enable ? 1 : 0;
    return ISO_OK;
}

iso_status iso_extract_device_typed(iso_ctx* ctx, iso_algorithm algo, const void* volume, iso_dtype dtype,
                                    const iso_grid* grid, float isoval, iso_mesh* out, void* stream)
{
    if (!ctx || !grid || iso::dtype_bytes(dtype) == 0) return ISO_ERR_INVALID_ARG;
    if (dtype == ISO_FLOAT32) return iso_extract_device(ctx, algo, static_cast<const float*>(volume), grid, isoval,
                                                        out, stream);
    Grid g;
    if (!make_grid(grid, g)) return ISO_ERR_INVALID_ARG;
    if (empty_grid(g) || !volume) return iso_extract_device(ctx, algo, nullptr, grid, isoval, out, stream);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ctx->narrow && algo != ISO_MC_DUPFREE && iso::narrow_fits(g, volume, dtype)) {
        iso_status st = check_mesh(out);
        if (st != ISO_OK) return st;
        out->n_points = out->n_tris = 0;
        const Plans pl = make_plans(ctx, g);
        if (pl.gp.fits && (algo == ISO_FLYING_EDGES || iso::mc_fused(g, pl.gp)))
            return extract_device_narrow(ctx, algo, volume, dtype, g, isoval, out, s);
    }
    const long long n = (long long)g.nx * g.ny * g.nz;
    if ((size_t)n * 4 > ctx->d_volume_bytes) {
        ISO_CUDA(ctx, cudaStreamSynchronize(s));
        cudaFree(ctx->d_volume);
        ctx->d_volume = nullptr;
        ctx->d_volume_bytes = 0;
        ISO_CUDA(ctx, cudaMalloc(&ctx->d_volume, (size_t)n * 4));
        ctx->d_volume_bytes = (size_t)n * 4;
    }
    iso::launch_to_float(volume, dtype, ctx->d_volume, n, ctx->nsm, s);
    ISO_CUDA(ctx, cudaGetLastError());
    return iso_extract_device(ctx, algo, ctx->d_volume, grid, isoval, out, stream);
}

// ---------------------------------------------------------------------------
// Pass-by-pass Flying Edges (FlyingEdgesAlgorithm.h:29-49).  Passes 1 and 2
// run as one fused kernel here (classification feeds the counts directly):
// iso_fe_pass1 launches it, iso_fe_pass2 only advances the state.
// ---------------------------------------------------------------------------
iso_status iso_fe_create(iso_ctx* ctx, const float* host_volume, const iso_grid* grid, float isoval, iso_fe** out)
{
    if (!ctx || !grid || !out) return ISO_ERR_INVALID_ARG;
    *out = nullptr;
    Grid g;
    if (!make_grid(grid, g)) return ISO_ERR_INVALID_ARG;
    if (!empty_grid(g) && !host_volume) return ISO_ERR_INVALID_ARG;
    iso_fe* fe = new (std::nothrow) iso_fe();
    if (!fe) return ISO_ERR_OOM;
    fe->ctx = ctx;
    fe->host_volume = host_volume;
    fe->grid = *grid;
    fe->g = g;
    fe->isoval = isoval;
    *out = fe;
    return ISO_OK;
}

iso_status iso_fe_pass1(iso_fe* fe)
{
    if (!fe) return ISO_ERR_INVALID_ARG;
    if (fe->stage != 0) return ISO_ERR_STATE;
    iso_ctx* ctx = fe->ctx;
    fe->stage = 1;
    if (empty_grid(fe->g)) return ISO_OK;
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const Grid& g = fe->g;
    const size_t vbytes = (size_t)g.nx * g.ny * g.nz * sizeof(float);
    const Plans pl = make_plans(ctx, g);
    ISO_CUDA(ctx, cudaMalloc(&fe->d_volume, vbytes));
    ISO_CUDA(ctx, cudaMalloc(&fe->scratch, scratch_size(g, pl.cp)));
    carve(fe->scratch, g, pl.cp, fe->buf);
    ISO_CUDA(ctx, cudaMemcpy(fe->d_volume, fe->host_volume, vbytes, cudaMemcpyHostToDevice));
    iso::CountPlan cp = pl.cp;
    cp.trims = true;  // the gridEdge records carry them
    iso::launch_count(fe->d_volume, g, fe->isoval, ctx->d_cases, false, cp, fe->buf, 0);
    ISO_CUDA(ctx, cudaGetLastError());
    ISO_CUDA(ctx, cudaDeviceSynchronize());
    return ISO_OK;
}

iso_status iso_fe_pass2(iso_fe* fe)
{
    if (!fe) return ISO_ERR_INVALID_ARG;
    if (fe->stage != 1) return ISO_ERR_STATE;
    fe->stage = 2;
    return ISO_OK;
}

iso_status iso_fe_pass3(iso_fe* fe)
{
    if (!fe) return ISO_ERR_INVALID_ARG;
    if (fe->stage != 2) return ISO_ERR_STATE;
    fe->stage = 3;
    if (empty_grid(fe->g)) return ISO_OK;
    iso_ctx* ctx = fe->ctx;
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const Plans pl = make_plans(ctx, fe->g);
    iso::launch_scan(fe->g, pl.cp, iso::kScanFE, fe->buf, 0);
    ISO_CUDA(ctx, cudaGetLastError());
    unsigned long long tot[4];
    ISO_CUDA(ctx, cudaMemcpy(tot, fe->buf.totals, sizeof(tot), cudaMemcpyDeviceToHost));
    fe->n_points = (long long)tot[0];
    fe->n_tris = (long long)tot[1];
    // allocation of the output, as the reference does at the end of pass 3
    ISO_CUDA(ctx, cudaMalloc(&fe->d_points, (size_t)(fe->n_points + 1) * 12));
    ISO_CUDA(ctx, cudaMalloc(&fe->d_normals, (size_t)(fe->n_points + 1) * 12));
    ISO_CUDA(ctx, cudaMalloc(&fe->d_tris, (size_t)(fe->n_tris + 1) * 24));
    return ISO_OK;
}

iso_status iso_fe_pass4(iso_fe* fe)
{
    if (!fe) return ISO_ERR_INVALID_ARG;
    if (fe->stage != 3) return ISO_ERR_STATE;
    fe->stage = 4;
    if (empty_grid(fe->g)) return ISO_OK;
    iso_ctx* ctx = fe->ctx;
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const Plans pl = make_plans(ctx, fe->g);
    iso_mesh dm{};
    dm.points = fe->d_points;
    dm.normals = fe->d_normals;
    dm.tris = fe->d_tris;
    dm.index_bytes = 8;
    dm.cap_points = fe->n_points;
    dm.cap_tris = fe->n_tris;
    PassMarks pm(ctx, 0);
    enqueue_generate(ctx, ISO_FLYING_EDGES, fe->d_volume, fe->g, fe->isoval, pl, fe->buf, &dm, 0, pm);
    ISO_CUDA(ctx, cudaGetLastError());
    unsigned long long tot[4];
    ISO_CUDA(ctx, cudaMemcpy(tot, fe->buf.totals, sizeof(tot), cudaMemcpyDeviceToHost));
    if (tot[3] != 0) {
        ctx->last_error = "a device-side wait timed out";
        return ISO_ERR_TIMEOUT;
    }
    return ISO_OK;
}

iso_status iso_fe_sizes(const iso_fe* fe, int64_t* n_points, int64_t* n_tris)
{
    if (!fe || !n_points || !n_tris) return ISO_ERR_INVALID_ARG;
    if (fe->stage < 3) return ISO_ERR_STATE;
    *n_points = fe->n_points;
    *n_tris = fe->n_tris;
    return ISO_OK;
}

iso_status iso_fe_grid_edges(iso_fe* fe, uint64_t* grid_edges, uint64_t* tri_counter)
{
    if (!fe || !grid_edges || !tri_counter) return ISO_ERR_INVALID_ARG;
    if (fe->stage < 2) return ISO_ERR_STATE;
    const Grid& g = fe->g;
    if (empty_grid(g)) return ISO_OK;
    iso_ctx* ctx = fe->ctx;
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t nge = (size_t)g.R * 5, ntc = (size_t)(g.ny - 1) * (g.nz - 1);
    unsigned long long* d = nullptr;
    ISO_CUDA(ctx, cudaMalloc(&d, (nge + ntc) * 8));
    iso::launch_grid_edges(g, make_plans(ctx, g).cp, fe->buf, fe->stage >= 3 ? 1 : 0, d, d + nge, 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(grid_edges, d, nge * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(tri_counter, d + nge, ntc * 8, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "iso_fe_grid_edges");
    return ISO_OK;
}

iso_status iso_fe_move_output(iso_fe* fe, iso_mesh* out)
{
    if (!fe) return ISO_ERR_INVALID_ARG;
    iso_status st = check_mesh(out);
    if (st != ISO_OK) return st;
    if (fe->stage != 4) return ISO_ERR_STATE;
    iso_ctx* ctx = fe->ctx;
    out->n_points = fe->n_points;
    out->n_tris = fe->n_tris;
    if (fe->n_points > out->cap_points || fe->n_tris > out->cap_tris) return ISO_ERR_CAPACITY;
    if (out->index_bytes == 4 && fe->n_points > 0xffffffffll) return ISO_ERR_OVERFLOW;
    if (fe->n_points == 0 && fe->n_tris == 0) return ISO_OK;
    ISO_CUDA(ctx, cudaSetDevice(ctx->device));
    ISO_CUDA(ctx, cudaMemcpy(out->points, fe->d_points, (size_t)fe->n_points * 12, cudaMemcpyDeviceToHost));
    ISO_CUDA(ctx, cudaMemcpy(out->normals, fe->d_normals, (size_t)fe->n_points * 12, cudaMemcpyDeviceToHost));
    if (out->index_bytes == 8) {
        ISO_CUDA(ctx, cudaMemcpy(out->tris, fe->d_tris, (size_t)fe->n_tris * 24, cudaMemcpyDeviceToHost));
    } else {
        // narrow on the host: the pass-by-pass path keeps the reference's size_t
        uint64_t* tmp = new (std::nothrow) uint64_t[(size_t)fe->n_tris * 3 + 1];
        if (!tmp) return ISO_ERR_OOM;
        cudaError_t e = cudaMemcpy(tmp, fe->d_tris, (size_t)fe->n_tris * 24, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            delete[] tmp;
            return cuda_fail(ctx, e, "cudaMemcpy");
        }
        uint32_t* o = static_cast<uint32_t*>(out->tris);
        for (size_t q = 0; q < (size_t)fe->n_tris * 3; ++q) o[q] = (uint32_t)tmp[q];
        delete[] tmp;
    }
    return ISO_OK;
}

iso_status iso_fe_destroy(iso_fe* fe)
{
    if (!fe) return ISO_OK;
    cudaSetDevice(fe->ctx->device);
    cudaFree(fe->d_volume);
    cudaFree(fe->scratch);
    cudaFree(fe->d_points);
    cudaFree(fe->d_normals);
    cudaFree(fe->d_tris);
    delete fe;
    return ISO_OK;
}

}  // extern "C"
