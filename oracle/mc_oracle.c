/*
 * Marching Cubes oracle -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates marchingCubes/serial/main.cpp:42-192: cells are visited in
 * (k, j, i) order; a vertex is created the first time a triangle corner
 * references its global edge (marchingCubes/util/Image3D.cpp:168-256), using
 * the cube of the referencing cell for position and gradient
 * (marchingCubes/util/Image3D.cpp:22-166, util.h:24-54).  The reference's
 * std::unordered_map is replaced by an open-addressing table with the same
 * lookup semantics.
 */
#include "oracle.h"
#include "case_table.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const unsigned char kLo[12] = {0, 1, 3, 0, 4, 5, 7, 4, 0, 1, 3, 2};
static const unsigned char kHi[12] = {1, 2, 2, 3, 5, 6, 6, 7, 4, 5, 7, 6};

static double g_mc_wall;

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
    size_t* keys;   /* key+1, 0 = empty */
    size_t* vals;
    size_t cap, size;
} edge_map;

static size_t mix(size_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

static void map_init(edge_map* m, size_t cap)
{
    m->cap = 1024;
    while (m->cap < cap) m->cap <<= 1;
    m->keys = (size_t*)calloc(m->cap, sizeof(size_t));
    m->vals = (size_t*)malloc(m->cap * sizeof(size_t));
    m->size = 0;
}

static void map_grow(edge_map* m);

/* Returns 1 and sets *val when present, else inserts (key -> val_if_new). */
static int map_find_or_insert(edge_map* m, size_t key, size_t val_if_new, size_t* val)
{
    if (2 * (m->size + 1) > m->cap) map_grow(m);
    size_t mask = m->cap - 1, h = mix(key) & mask;
    for (;;) {
        if (m->keys[h] == 0) {
            m->keys[h] = key + 1;
            m->vals[h] = val_if_new;
            m->size++;
            *val = val_if_new;
            return 0;
        }
        if (m->keys[h] == key + 1) { *val = m->vals[h]; return 1; }
        h = (h + 1) & mask;
    }
}

static void map_grow(edge_map* m)
{
    edge_map n;
    map_init(&n, m->cap * 2);
    for (size_t s = 0; s < m->cap; ++s) {
        if (m->keys[s]) {
            size_t v;
            map_find_or_insert(&n, m->keys[s] - 1, m->vals[s], &v);
        }
    }
    free(m->keys); free(m->vals);
    *m = n;
}

typedef struct {
    float* p; size_t n, cap;
} fvec;
typedef struct {
    size_t* p; size_t n, cap;
} svec;

static void fpush3(fvec* v, const float x[3])
{
    if (v->n + 3 > v->cap) {
        v->cap = v->cap ? 2 * v->cap : 3 * 1024;
        v->p = (float*)realloc(v->p, v->cap * sizeof(float));
    }
    v->p[v->n++] = x[0]; v->p[v->n++] = x[1]; v->p[v->n++] = x[2];
}
static void spush(svec* v, size_t x)
{
    if (v->n + 1 > v->cap) {
        v->cap = v->cap ? 2 * v->cap : 1024;
        v->p = (size_t*)realloc(v->p, v->cap * sizeof(size_t));
    }
    v->p[v->n++] = x;
}

/* The cells of z-section [zbeg, zend) x all y x all x, visited in (k, j, i)
 * order, appended to a running mesh whose edge map persists across the
 * sections one thread runs: sectionOfMarchingCubes
 * (marchingCubes/openmp/main.cpp:44-154); with one section over the whole
 * grid it is MarchingCubes() of marchingCubes/serial/main.cpp:42-192. */
typedef struct {
    edge_map map;
    fvec pts, nrm;
    svec tris, eov;
    size_t pt_idx;
} mc_part;

static void mc_section(const float* data, const size_t dims[3], const float spacing[3], const float origin[3],
                       float iso, size_t zbeg, size_t zend, mc_part* part)
{
    size_t nx = dims[0], ny = dims[1], nz = dims[2];
    size_t nX = (nx - 1) * ny * nz, nY = nx * (ny - 1) * nz;
    static const int dx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    static const int dy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    static const int dz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    /* per cube edge: offset of the edge's low end, and axis */
    static const int ex[12] = {0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 1};
    static const int ey[12] = {0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1};
    static const int ez[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0};
    static const int axis[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};
#define V(i, j, k) data[(k) * nx * ny + (j) * nx + (i)]
    for (size_t k = zbeg; k < zend; ++k)
    for (size_t j = 0; j + 1 < ny; ++j)
    for (size_t i = 0; i + 1 < nx; ++i) {
        float vals[8];
        int c = 0;
        for (int v = 0; v < 8; ++v) {
            vals[v] = V(i + dx[v], j + dy[v], k + dz[v]);
            if (vals[v] >= iso) c |= 1 << v;   /* util::findCaseId, util.h:24-42 */
        }
        if (c == 0 || c == 255) continue;
        /* getPosCube (marchingCubes/util/Image3D.cpp:22-65) */
        float xpos = origin[0] + (float)i * spacing[0];
        float ypos = origin[1] + (float)j * spacing[1];
        float zpos = origin[2] + (float)k * spacing[2];
        float x1 = xpos + spacing[0], y1 = ypos + spacing[1], z1 = zpos + spacing[2];
        float pc[8][3] = {{xpos, ypos, zpos}, {x1, ypos, zpos}, {x1, y1, zpos}, {xpos, y1, zpos},
                          {xpos, ypos, z1}, {x1, ypos, z1}, {x1, y1, z1}, {xpos, y1, z1}};
        /* getGradCube / computeGradient (Image3D.cpp:67-166) */
        float gc[8][3];
        for (int v = 0; v < 8; ++v) {
            size_t p[3] = {i + dx[v], j + dy[v], k + dz[v]};
            size_t n[3] = {nx, ny, nz};
            for (int a = 0; a < 3; ++a) {
                size_t q0[3] = {p[0], p[1], p[2]}, q1[3] = {p[0], p[1], p[2]};
                float run;
                if (p[a] == 0) { q0[a] = 1; q1[a] = 0; run = spacing[a]; }
                else if (p[a] == n[a] - 1) { q1[a] = p[a] - 1; run = spacing[a]; }
                else { q0[a] = p[a] + 1; q1[a] = p[a] - 1; run = 2 * spacing[a]; }
                gc[v][a] = (V(q1[0], q1[1], q1[2]) - V(q0[0], q0[1], q0[2])) / run;
            }
        }
        int ntri = (int)strlen(kOracleCases[c]) / 3;
        for (int t = 0; t < ntri; ++t) {
            size_t tri[3];
            for (int q = 0; q < 3; ++q) {
                char ch = kOracleCases[c][3 * t + q];
                int e = ch <= '9' ? ch - '0' : ch - 'a' + 10;
                size_t x = i + ex[e], y = j + ey[e], z = k + ez[e];
                size_t gid;
                if (axis[e] == 0) gid = x + (nx - 1) * y + ny * (nx - 1) * z;
                else if (axis[e] == 1) gid = nX + x + nx * y + nx * (ny - 1) * z;
                else gid = nX + nY + x + nx * y + nx * ny * z;
                size_t found;
                if (map_find_or_insert(&part->map, gid, part->pt_idx, &found)) {
                    tri[q] = found;
                } else {
                    tri[q] = part->pt_idx++;
                    int v1 = kLo[e], v2 = kHi[e];
                    float w = (iso - vals[v1]) / (vals[v2] - vals[v1]);
                    float np[3], nn[3];
                    for (int a = 0; a < 3; ++a) {
                        np[a] = pc[v1][a] + (w * (pc[v2][a] - pc[v1][a]));
                        nn[a] = gc[v1][a] + (w * (gc[v2][a] - gc[v1][a]));
                    }
                    fpush3(&part->pts, np);
                    fpush3(&part->nrm, nn);
                    spush(&part->eov, gid);
                }
            }
            if (tri[0] != tri[1] && tri[1] != tri[2] && tri[2] != tri[0]) {
                spush(&part->tris, tri[0]); spush(&part->tris, tri[1]); spush(&part->tris, tri[2]);
            }
        }
    }
#undef V
}

static void part_to_mesh(mc_part* part, oracle_mesh* out)
{
    out->n_points = part->pt_idx;
    out->n_tris = part->tris.n / 3;
    out->points = part->pts.p ? part->pts.p : (float*)calloc(1, sizeof(float));
    out->normals = part->nrm.p ? part->nrm.p : (float*)calloc(1, sizeof(float));
    out->tris = part->tris.p ? part->tris.p : (size_t*)calloc(1, sizeof(size_t));
    out->edge_of_vertex = part->eov.p ? part->eov.p : (size_t*)calloc(1, sizeof(size_t));
}

int oracle_mc_run(const float* data, const size_t dims[3], const float spacing[3],
                  const float origin[3], float iso, oracle_mesh* out)
{
    memset(out, 0, sizeof(*out));
    size_t nx = dims[0], ny = dims[1], nz = dims[2];
    if (nx < 2 || ny < 2 || nz < 2) { g_mc_wall = 0.0; return 0; }
    double t0 = now_s();
    mc_part part;
    memset(&part, 0, sizeof(part));
    map_init(&part.map, 1 << 16);
    mc_section(data, dims, spacing, origin, iso, 0, nz - 1, &part);
    free(part.map.keys); free(part.map.vals);
    part_to_mesh(&part, out);
    g_mc_wall = now_s() - t0;
    return 0;
}

/* util::Indexer (marchingCubes/util/util.h:56-78): the first index of section
 * idx when n elements are split into nsec sections of grain or grain + 1. */
static size_t section_begin(size_t n, size_t nsec, size_t idx)
{
    const size_t grain = n / nsec, split = (grain + 1) * nsec - n;
    return idx <= split ? grain * idx : grain * split + (grain + 1) * (idx - split);
}

/* MarchingCubes() of marchingCubes/openmp/main.cpp:156-296 with its default
 * sections (main.cpp:308-322, 405-410): nthreads z-sections (at most nz - 1),
 * one x and one y section; each thread runs its sections with its own edge
 * map, so a vertex on a seam between two threads' sections is made by both;
 * the threads' meshes are appended one after another with their triangle
 * indices offset.  The reference appends them in the order the threads
 * finish (an omp critical section); this port appends them in thread order,
 * so its output is deterministic. */
int oracle_mc_openmp_run(const float* data, const size_t dims[3], const float spacing[3],
                         const float origin[3], float iso, int nthreads, oracle_mesh* out)
{
    memset(out, 0, sizeof(*out));
    size_t nx = dims[0], ny = dims[1], nz = dims[2];
    if (nx < 2 || ny < 2 || nz < 2) { g_mc_wall = 0.0; return 0; }
    double t0 = now_s();
    int nt = nthreads > 0 ? nthreads : 1;
    size_t nsec = (size_t)nt;
    if (nsec > nz - 1) nsec = nz - 1;
    mc_part* parts = (mc_part*)calloc((size_t)nt, sizeof(mc_part));
    if (!parts) return 1;
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        mc_part* part = &parts[t];
        map_init(&part->map, 1 << 16);
        long s;
#pragma omp for schedule(static) nowait
        for (s = 0; s < (long)nsec; ++s) {
            const size_t zb = section_begin(nz - 1, nsec, (size_t)s), ze = section_begin(nz - 1, nsec, (size_t)s + 1);
            mc_section(data, dims, spacing, origin, iso, zb, ze, part);
        }
        free(part->map.keys); free(part->map.vals);
    }
    size_t nv = 0, ntr = 0;
    for (int t = 0; t < nt; ++t) { nv += parts[t].pt_idx; ntr += parts[t].tris.n / 3; }
    out->n_points = nv;
    out->n_tris = ntr;
    out->points = (float*)malloc(sizeof(float) * (3 * nv + 1));
    out->normals = (float*)malloc(sizeof(float) * (3 * nv + 1));
    out->tris = (size_t*)malloc(sizeof(size_t) * (3 * ntr + 1));
    out->edge_of_vertex = (size_t*)malloc(sizeof(size_t) * (nv + 1));
    size_t ov = 0, ot = 0;
    for (int t = 0; t < nt; ++t) {
        mc_part* p = &parts[t];
        if (p->pt_idx) {
            memcpy(out->points + 3 * ov, p->pts.p, sizeof(float) * 3 * p->pt_idx);
            memcpy(out->normals + 3 * ov, p->nrm.p, sizeof(float) * 3 * p->pt_idx);
            memcpy(out->edge_of_vertex + ov, p->eov.p, sizeof(size_t) * p->pt_idx);
        }
        for (size_t q = 0; q < p->tris.n; ++q) out->tris[3 * ot + q] = p->tris.p[q] + ov;
        ov += p->pt_idx;
        ot += p->tris.n / 3;
        free(p->pts.p); free(p->nrm.p); free(p->tris.p); free(p->eov.p);
    }
    free(parts);
    g_mc_wall = now_s() - t0;
    return 0;
}

double oracle_mc_last_wall_seconds(void) { return g_mc_wall; }

/* util::duplicateRemover (marchingCubes/util/DuplicateRemover.h:38-103) for a
 * mesh made by one section: the vertices sorted by global edge index (each
 * edge appears once), triangles renumbered.  This is what
 * marchingCubes/openmpDupFree returns with one thread. */
typedef struct {
    size_t gid, idx;
} gid_pair;

static int cmp_gid(const void* a, const void* b)
{
    const size_t x = ((const gid_pair*)a)->gid, y = ((const gid_pair*)b)->gid;
    return x < y ? -1 : (x > y ? 1 : 0);
}

int oracle_mc_dupfree_run(const float* data, const size_t dims[3], const float spacing[3], const float origin[3],
                          float isoval, oracle_mesh* out)
{
    int st = oracle_mc_run(data, dims, spacing, origin, isoval, out);
    if (st != 0 || out->n_points == 0) return st;
    const size_t n = out->n_points;
    gid_pair* pr = (gid_pair*)malloc(n * sizeof(gid_pair));
    size_t* newidx = (size_t*)malloc(n * sizeof(size_t));
    float* pts = (float*)malloc(3 * n * sizeof(float));
    float* nrm = (float*)malloc(3 * n * sizeof(float));
    size_t* eov = (size_t*)malloc(n * sizeof(size_t));
    if (!pr || !newidx || !pts || !nrm || !eov) return 1;
    for (size_t i = 0; i < n; ++i) {
        pr[i].gid = out->edge_of_vertex[i];
        pr[i].idx = i;
    }
    qsort(pr, n, sizeof(gid_pair), cmp_gid);
    for (size_t r = 0; r < n; ++r) {
        const size_t o = pr[r].idx;
        newidx[o] = r;
        memcpy(pts + 3 * r, out->points + 3 * o, 3 * sizeof(float));
        memcpy(nrm + 3 * r, out->normals + 3 * o, 3 * sizeof(float));
        eov[r] = pr[r].gid;
    }
    for (size_t t = 0; t < 3 * out->n_tris; ++t) out->tris[t] = newidx[out->tris[t]];
    free(out->points);
    free(out->normals);
    free(out->edge_of_vertex);
    out->points = pts;
    out->normals = nrm;
    out->edge_of_vertex = eov;
    free(pr);
    free(newidx);
    return 0;
}
