/*
 * Flying Edges oracle -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates flyingEdges/serial/FlyingEdgesAlgorithm.cpp pass by pass, with the
 * OpenMP loop structure of flyingEdges/openmp/FlyingEdgesAlgorithm.cpp
 * (parallel over rows in pass 1, 2 and 4), whose output is byte-identical to
 * the serial one.  nthreads == 1 gives the serial algorithm.
 */
#include "oracle.h"
#include "case_table.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    size_t xl, xr, xstart, ystart, zstart;
} grid_edge;

struct oracle_fe {
    const float* data;
    size_t nx, ny, nz;
    float sp[3], zp[3];
    float iso;
    int nthreads;
    grid_edge* ge;          /* ny*nz            FlyingEdgesAlgorithm.h:81 */
    size_t* tri_counter;    /* (ny-1)*(nz-1)    :82 */
    unsigned char* edge_cases; /* (nx-1)*ny*nz  :84 */
    unsigned char* cube_cases; /* (nx-1)*(ny-1)*(nz-1) :85 */
    size_t n_points, n_tris;
    float* points;
    float* normals;
    size_t* tris;
    size_t* edge_of_vertex;
};

static double g_last_wall = 0.0;

/* Pass 3 of the reference (openmp/FlyingEdgesAlgorithm.cpp:329-331) builds
 * the output vectors with std::vector<T>(n), which zero-fills them on one
 * thread inside the timed extraction (its YAML shows pass 3 at about 0.2 s on
 * a 512^3 volume); the oracle allocates its outputs the same way.  The
 * constructor's work arrays cost the reference no measurable time, so they
 * come from calloc. */
static void* zeroed(size_t n, size_t size)
{
    void* p = malloc(n * size);
    if (p) memset(p, 0, n * size);
    return p;
}
double oracle_last_wall_seconds(void) { return g_last_wall; }

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Cube edge endpoints (flyingEdges/util/MarchingCubesTables.h:563). */
static const unsigned char kLo[12] = {0, 1, 3, 0, 4, 5, 7, 4, 0, 1, 3, 2};
static const unsigned char kHi[12] = {1, 2, 2, 3, 5, 6, 6, 7, 4, 5, 7, 6};

static int case_ntris(int c) { return (int)strlen(kOracleCases[c]) / 3; }
static int case_edge(int c, int t)
{
    char ch = kOracleCases[c][t];
    return ch <= '9' ? ch - '0' : ch - 'a' + 10;
}
static int is_cut(int c, int e) { return ((c >> kLo[e]) & 1) != ((c >> kHi[e]) & 1); }

oracle_fe* oracle_fe_create(const float* data, const size_t dims[3],
                            const float spacing[3], const float origin[3],
                            float isoval, int nthreads)
{
    oracle_fe* fe = (oracle_fe*)calloc(1, sizeof(oracle_fe));
    size_t nx = dims[0], ny = dims[1], nz = dims[2];
    fe->data = data;
    fe->nx = nx; fe->ny = ny; fe->nz = nz;
    for (int a = 0; a < 3; ++a) { fe->sp[a] = spacing[a]; fe->zp[a] = origin[a]; }
    fe->iso = isoval;
    fe->nthreads = nthreads > 0 ? nthreads : 1;
    fe->ge = (grid_edge*)calloc(ny * nz, sizeof(grid_edge));
    fe->tri_counter = (size_t*)calloc((ny - 1) * (nz - 1) + 1, sizeof(size_t));
    fe->edge_cases = (unsigned char*)calloc((nx - 1) * ny * nz + 1, 1);
    fe->cube_cases = (unsigned char*)calloc((nx - 1) * (ny - 1) * (nz - 1) + 1, 1);
    return fe;
}

/* calcCaseEdge (FlyingEdgesAlgorithm.cpp:556-574). */
static unsigned char calc_case_edge(int prev_ge, int curr_ge)
{
    if (prev_ge && curr_ge) return 0;
    if (!prev_ge && curr_ge) return 1;
    if (prev_ge && !curr_ge) return 2;
    return 3;
}

/* isCutEdge (FlyingEdgesAlgorithm.cpp:515-554). */
static int is_cut_edge(const oracle_fe* fe, size_t i, size_t j, size_t k)
{
    size_t nx = fe->nx, ny = fe->ny, nz = fe->nz;
    size_t idx = k * (nx - 1) * ny + j * (nx - 1) + i;
    unsigned char ec = fe->edge_cases[idx];
    if (ec == 1 || ec == 2) return 1;
    if (j != ny - 1) {
        size_t iy = k * (nx - 1) * ny + (j + 1) * (nx - 1) + i;
        if ((ec + fe->edge_cases[iy]) % 2 == 1) return 1;
    }
    if (k != nz - 1) {
        size_t iz = (k + 1) * (nx - 1) * ny + j * (nx - 1) + i;
        if ((ec + fe->edge_cases[iz]) % 2 == 1) return 1;
    }
    return 0;
}

/* pass1 (FlyingEdgesAlgorithm.cpp:23-66): x-edge cases, then row trims. */
void oracle_fe_pass1(oracle_fe* fe)
{
    long nrows = (long)(fe->ny * fe->nz);
    size_t nx = fe->nx, ny = fe->ny;
    long r;
#pragma omp parallel for num_threads(fe->nthreads) schedule(static)
    for (r = 0; r < nrows; ++r) {
        size_t k = (size_t)r / ny, j = (size_t)r % ny;
        unsigned char* ec = fe->edge_cases + (nx - 1) * (k * ny + j);
        const float* row = fe->data + nx * (k * ny + j);
        int prev = row[0] >= fe->iso;
        for (size_t i = 1; i < nx; ++i) {
            int cur = row[i] >= fe->iso;
            ec[i - 1] = calc_case_edge(prev, cur);
            prev = cur;
        }
    }
#pragma omp parallel for num_threads(fe->nthreads) schedule(static)
    for (r = 0; r < nrows; ++r) {
        size_t k = (size_t)r / ny, j = (size_t)r % ny;
        grid_edge* g = &fe->ge[k * ny + j];
        g->xl = nx;
        for (size_t i = 1; i < nx; ++i) {
            if (is_cut_edge(fe, i - 1, j, k)) {
                if (g->xl == nx) g->xl = i - 1;
                g->xr = i;
            }
        }
    }
}

/* calcCubeCase (FlyingEdgesAlgorithm.cpp:576-604). */
static int calc_cube_case(unsigned char e0, unsigned char e1, unsigned char e2, unsigned char e3)
{
    int c = 0;
    if (e0 == 0 || e0 == 2) c |= 1;
    if (e0 == 0 || e0 == 1) c |= 2;
    if (e1 == 0 || e1 == 1) c |= 4;
    if (e1 == 0 || e1 == 2) c |= 8;
    if (e2 == 0 || e2 == 2) c |= 16;
    if (e2 == 0 || e2 == 1) c |= 32;
    if (e3 == 0 || e3 == 1) c |= 64;
    if (e3 == 0 || e3 == 2) c |= 128;
    return c;
}

/* calcTrimValues (FlyingEdgesAlgorithm.cpp:606-621). */
static void calc_trim(const oracle_fe* fe, size_t j, size_t k, size_t* xl, size_t* xr)
{
    size_t ny = fe->ny;
    const grid_edge* g0 = &fe->ge[k * ny + j];
    const grid_edge* g1 = &fe->ge[k * ny + j + 1];
    const grid_edge* g2 = &fe->ge[(k + 1) * ny + j];
    const grid_edge* g3 = &fe->ge[(k + 1) * ny + j + 1];
    size_t l = g0->xl, rr = g0->xr;
    if (g1->xl < l) l = g1->xl;
    if (g2->xl < l) l = g2->xl;
    if (g3->xl < l) l = g3->xl;
    if (g1->xr > rr) rr = g1->xr;
    if (g2->xr > rr) rr = g2->xr;
    if (g3->xr > rr) rr = g3->xr;
    if (l > rr) l = rr;
    *xl = l; *xr = rr;
}

/* pass2 (FlyingEdgesAlgorithm.cpp:72-190): cube cases, per-row counts. */
void oracle_fe_pass2(oracle_fe* fe)
{
    size_t nx = fe->nx, ny = fe->ny, nz = fe->nz;
    if (ny < 2 || nz < 2 || nx < 2) return;
    long nrows = (long)((ny - 1) * (nz - 1));
    long r;
#pragma omp parallel for num_threads(fe->nthreads) schedule(static)
    for (r = 0; r < nrows; ++r) {
        size_t k = (size_t)r / (ny - 1), j = (size_t)r % (ny - 1);
        size_t xl, xr;
        calc_trim(fe, j, k, &xl, &xr);
        grid_edge* g0 = &fe->ge[k * ny + j];
        grid_edge* g1 = &fe->ge[k * ny + j + 1];
        grid_edge* g2 = &fe->ge[(k + 1) * ny + j];
        grid_edge* g3 = &fe->ge[(k + 1) * ny + j + 1];
        const unsigned char* ec0 = fe->edge_cases + (nx - 1) * (k * ny + j);
        const unsigned char* ec1 = fe->edge_cases + (nx - 1) * (k * ny + j + 1);
        const unsigned char* ec2 = fe->edge_cases + (nx - 1) * ((k + 1) * ny + j);
        const unsigned char* ec3 = fe->edge_cases + (nx - 1) * ((k + 1) * ny + j + 1);
        size_t* tc = &fe->tri_counter[k * (ny - 1) + j];
        unsigned char* cc = fe->cube_cases + (nx - 1) * (k * (ny - 1) + j);
        int y_end = (j == ny - 2), z_end = (k == nz - 2);
        for (size_t i = xl; i != xr; ++i) {
            int x_end = (i == nx - 2);
            int c = calc_cube_case(ec0[i], ec1[i], ec2[i], ec3[i]);
            cc[i] = (unsigned char)c;
            if (c == 0 || c == 255) continue;
            *tc += (size_t)case_ntris(c);
            g0->xstart += is_cut(c, 0);
            g0->ystart += is_cut(c, 3);
            g0->zstart += is_cut(c, 8);
            /* boundary rows/columns (FlyingEdgesAlgorithm.cpp:160-187) */
            if (x_end) { g0->ystart += is_cut(c, 1); g0->zstart += is_cut(c, 9); }
            if (y_end) { g1->xstart += is_cut(c, 2); g1->zstart += is_cut(c, 10); }
            if (z_end) { g2->xstart += is_cut(c, 4); g2->ystart += is_cut(c, 7); }
            if (x_end && y_end) g1->zstart += is_cut(c, 11);
            if (x_end && z_end) g2->ystart += is_cut(c, 5);
            if (y_end && z_end) g3->xstart += is_cut(c, 6);
        }
    }
}

/* pass3 (FlyingEdgesAlgorithm.cpp:196-269): exclusive scans, allocation. */
void oracle_fe_pass3(oracle_fe* fe)
{
    size_t ny = fe->ny, nz = fe->nz;
    size_t acc = 0, tmp;
    if (ny >= 2 && nz >= 2) {
        for (size_t r = 0; r < (ny - 1) * (nz - 1); ++r) {
            tmp = fe->tri_counter[r];
            fe->tri_counter[r] = acc;
            acc += tmp;
        }
    }
    fe->n_tris = acc;
    acc = 0;
    for (size_t r = 0; r < ny * nz; ++r) {
        grid_edge* g = &fe->ge[r];
        tmp = g->xstart; g->xstart = acc; acc += tmp;
        tmp = g->ystart; g->ystart = acc; acc += tmp;
        tmp = g->zstart; g->zstart = acc; acc += tmp;
    }
    fe->n_points = acc;
    fe->points = (float*)zeroed(3 * fe->n_points + 1, sizeof(float));
    fe->normals = (float*)zeroed(3 * fe->n_points + 1, sizeof(float));
    fe->tris = (size_t*)zeroed(3 * fe->n_tris + 1, sizeof(size_t));
    /* the vertices' edge ids are the oracle's own bookkeeping (no reference counterpart) */
    fe->edge_of_vertex = (size_t*)malloc((fe->n_points + 1) * sizeof(size_t));
}

/* Image3D::getPosCube (flyingEdges/util/Image3D.cpp:45-87). */
static void pos_cube(const oracle_fe* fe, size_t i, size_t j, size_t k, float pos[8][3])
{
    float xpos = fe->zp[0] + (float)i * fe->sp[0];
    float ypos = fe->zp[1] + (float)j * fe->sp[1];
    float zpos = fe->zp[2] + (float)k * fe->sp[2];
    float x1 = xpos + fe->sp[0], y1 = ypos + fe->sp[1], z1 = zpos + fe->sp[2];
    float px[8] = {xpos, x1, x1, xpos, xpos, x1, x1, xpos};
    float py[8] = {ypos, ypos, y1, y1, ypos, ypos, y1, y1};
    float pz[8] = {zpos, zpos, zpos, zpos, z1, z1, z1, z1};
    for (int v = 0; v < 8; ++v) { pos[v][0] = px[v]; pos[v][1] = py[v]; pos[v][2] = pz[v]; }
}

static float at(const oracle_fe* fe, size_t i, size_t j, size_t k)
{
    return fe->data[k * fe->nx * fe->ny + j * fe->nx + i];
}

/* Image3D::computeGradient (flyingEdges/util/Image3D.cpp:116-188): per axis
 * x0 = the forward neighbour (or the point itself on the last plane), x1 =
 * the backward one (or the point itself on the first), g = (x1 - x0) / run
 * with run = spacing at a face and 2 * spacing inside. */
static void gradient(const oracle_fe* fe, size_t i, size_t j, size_t k, float g[3])
{
    const size_t n[3] = {fe->nx, fe->ny, fe->nz};
    const size_t p[3] = {i, j, k};
    const size_t stride[3] = {1, fe->nx, fe->nx * fe->ny};
    const float* here = fe->data + k * stride[2] + j * stride[1] + i;
    for (int a = 0; a < 3; ++a) {
        const ptrdiff_t s = (ptrdiff_t)stride[a];
        float x0, x1, run;
        if (p[a] == 0) {
            x0 = here[s]; x1 = here[0]; run = fe->sp[a];
        } else if (p[a] == n[a] - 1) {
            x0 = here[0]; x1 = here[-s]; run = fe->sp[a];
        } else {
            x0 = here[s]; x1 = here[-s]; run = 2 * fe->sp[a];
        }
        g[a] = (x1 - x0) / run;
    }
}

static void grad_cube(const oracle_fe* fe, size_t i, size_t j, size_t k, float g[8][3])
{
    static const int dx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    static const int dy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    static const int dz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    for (int v = 0; v < 8; ++v) gradient(fe, i + dx[v], j + dy[v], k + dz[v], g[v]);
}

/* interpolateOnCube + interpolate (FlyingEdgesAlgorithm.cpp:623-647). */
static void interp_on_cube(float iso, float pts[8][3], const float vals[8], int e, float out[3])
{
    int i0 = kLo[e], i1 = kHi[e];
    float w = (iso - vals[i0]) / (vals[i1] - vals[i0]);
    for (int a = 0; a < 3; ++a) out[a] = pts[i0][a] + (w * (pts[i1][a] - pts[i0][a]));
}

/* Global edge id of cube edge e of cell (i,j,k), numbered as in
 * marchingCubes/util/Image3D.cpp:168-256 (used only for error reporting). */
static size_t global_edge(const oracle_fe* fe, size_t i, size_t j, size_t k, int e)
{
    size_t nx = fe->nx, ny = fe->ny, nz = fe->nz;
    size_t nX = (nx - 1) * ny * nz, nY = nx * (ny - 1) * nz;
    static const int ox[12] = {0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 1};
    static const int oy[12] = {0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1};
    static const int oz[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0};
    size_t x = i + ox[e], y = j + oy[e], z = k + oz[e];
    if (e == 0 || e == 2 || e == 4 || e == 6) return x + (nx - 1) * (y + ny * z);
    if (e == 1 || e == 3 || e == 5 || e == 7) return nX + x + nx * (y + (ny - 1) * z);
    return nX + nY + x + nx * (y + ny * z);
}

/* pass4 (FlyingEdgesAlgorithm.cpp:275-497). */
void oracle_fe_pass4(oracle_fe* fe)
{
    size_t nx = fe->nx, ny = fe->ny, nz = fe->nz;
    if (ny < 2 || nz < 2 || nx < 2) return;
    long nrows = (long)((ny - 1) * (nz - 1));
    long r;
#pragma omp parallel for num_threads(fe->nthreads) schedule(static)
    for (r = 0; r < nrows; ++r) {
        size_t k = (size_t)r / (ny - 1), j = (size_t)r % (ny - 1);
        size_t xl, xr;
        calc_trim(fe, j, k, &xl, &xr);
        if (xl == xr) continue;
        size_t tri_idx = fe->tri_counter[k * (ny - 1) + j];
        const unsigned char* cc = fe->cube_cases + (nx - 1) * (k * (ny - 1) + j);
        const grid_edge* g0 = &fe->ge[k * ny + j];
        const grid_edge* g1 = &fe->ge[k * ny + j + 1];
        const grid_edge* g2 = &fe->ge[(k + 1) * ny + j];
        const grid_edge* g3 = &fe->ge[(k + 1) * ny + j + 1];
        size_t x0c = 0, y0c = 0, z0c = 0, x1c = 0, z1c = 0, x2c = 0, y2c = 0, x3c = 0;
        int y_end = (j == ny - 2), z_end = (k == nz - 2);
        for (size_t i = xl; i != xr; ++i) {
            int x_end = (i == nx - 2);
            int c = cc[i];
            if (c == 0 || c == 255) continue;
            float pc[8][3], gc[8][3], vc[8];
            pos_cube(fe, i, j, k, pc);
            {
                static const int dx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
                static const int dy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
                static const int dz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
                for (int v = 0; v < 8; ++v) vc[v] = at(fe, i + dx[v], j + dy[v], k + dz[v]);
            }
            grad_cube(fe, i, j, k, gc);
            size_t gid[12];
            /* (edge, owner row start, counter, write?, advance counter?) in
             * the order of FlyingEdgesAlgorithm.cpp:340-484 */
#define ORACLE_EMIT(E, START, CNT, WRITE, ADV)                                   \
            if (is_cut(c, E)) {                                                 \
                size_t idx = (START) + (CNT);                                   \
                if (WRITE) {                                                    \
                    interp_on_cube(fe->iso, pc, vc, E, fe->points + 3 * idx);   \
                    interp_on_cube(fe->iso, gc, vc, E, fe->normals + 3 * idx);  \
                    fe->edge_of_vertex[idx] = global_edge(fe, i, j, k, E);      \
                }                                                               \
                gid[E] = idx;                                                   \
                if (ADV) ++(CNT);                                               \
            }
            ORACLE_EMIT(0, g0->xstart, x0c, 1, 1)
            ORACLE_EMIT(3, g0->ystart, y0c, 1, 1)
            ORACLE_EMIT(8, g0->zstart, z0c, 1, 1)
            ORACLE_EMIT(1, g0->ystart, y0c, x_end, 0)
            ORACLE_EMIT(9, g0->zstart, z0c, x_end, 0)
            ORACLE_EMIT(2, g1->xstart, x1c, y_end, 1)
            ORACLE_EMIT(10, g1->zstart, z1c, y_end, 1)
            ORACLE_EMIT(4, g2->xstart, x2c, z_end, 1)
            ORACLE_EMIT(7, g2->ystart, y2c, z_end, 1)
            ORACLE_EMIT(11, g1->zstart, z1c, x_end && y_end, 0)
            ORACLE_EMIT(5, g2->ystart, y2c, x_end && z_end, 0)
            ORACLE_EMIT(6, g3->xstart, x3c, y_end && z_end, 1)
#undef ORACLE_EMIT
            int nt = case_ntris(c);
            for (int t = 0; t < nt; ++t) {
                fe->tris[3 * tri_idx + 0] = gid[case_edge(c, 3 * t + 0)];
                fe->tris[3 * tri_idx + 1] = gid[case_edge(c, 3 * t + 1)];
                fe->tris[3 * tri_idx + 2] = gid[case_edge(c, 3 * t + 2)];
                ++tri_idx;
            }
        }
    }
}

void oracle_fe_grid_edges(const oracle_fe* fe, size_t* out)
{
    for (size_t r = 0; r < fe->ny * fe->nz; ++r) {
        out[5 * r + 0] = fe->ge[r].xl;
        out[5 * r + 1] = fe->ge[r].xr;
        out[5 * r + 2] = fe->ge[r].xstart;
        out[5 * r + 3] = fe->ge[r].ystart;
        out[5 * r + 4] = fe->ge[r].zstart;
    }
}

void oracle_fe_tri_counter(const oracle_fe* fe, size_t* out)
{
    if (fe->ny < 2 || fe->nz < 2) return;
    memcpy(out, fe->tri_counter, (fe->ny - 1) * (fe->nz - 1) * sizeof(size_t));
}

void oracle_fe_cube_cases(const oracle_fe* fe, unsigned char* out)
{
    memcpy(out, fe->cube_cases, (fe->nx - 1) * (fe->ny - 1) * (fe->nz - 1));
}

void oracle_fe_take(oracle_fe* fe, oracle_mesh* out)
{
    out->n_points = fe->n_points;
    out->n_tris = fe->n_tris;
    out->points = fe->points;
    out->normals = fe->normals;
    out->tris = fe->tris;
    out->edge_of_vertex = fe->edge_of_vertex;
    fe->points = fe->normals = NULL;
    fe->tris = fe->edge_of_vertex = NULL;
    fe->n_points = fe->n_tris = 0;
}

void oracle_fe_destroy(oracle_fe* fe)
{
    if (!fe) return;
    free(fe->ge); free(fe->tri_counter); free(fe->edge_cases); free(fe->cube_cases);
    free(fe->points); free(fe->normals); free(fe->tris); free(fe->edge_of_vertex);
    free(fe);
}

int oracle_fe_run(const float* data, const size_t dims[3], const float spacing[3],
                  const float origin[3], float isoval, int nthreads, oracle_mesh* out)
{
    memset(out, 0, sizeof(*out));
    if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2) { g_last_wall = 0.0; return 0; }
    double t0 = now_s();
    oracle_fe* fe = oracle_fe_create(data, dims, spacing, origin, isoval, nthreads);
    oracle_fe_pass1(fe);
    oracle_fe_pass2(fe);
    oracle_fe_pass3(fe);
    oracle_fe_pass4(fe);
    oracle_fe_take(fe, out);
    oracle_fe_destroy(fe);
    g_last_wall = now_s() - t0;
    return 0;
}

void oracle_mesh_free(oracle_mesh* m)
{
    if (!m) return;
    free(m->points); free(m->normals); free(m->tris); free(m->edge_of_vertex);
    memset(m, 0, sizeof(*m));
}

void oracle_block_tris(const float* data, const size_t dims[3], float iso, int block, int* counts)
{
    const size_t nx = dims[0], ny = dims[1], nz = dims[2];
    if (nx < 2 || ny < 2 || nz < 2) return;
    const size_t nbx = (nx - 2) / block + 1, nby = (ny - 2) / block + 1, nbz = (nz - 2) / block + 1;
    memset(counts, 0, sizeof(int) * nbx * nby * nbz);
    /* corner v: (i + dx[v], j + dy[v], k + dz[v]) */
    static const int dx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, dy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    for (size_t k = 0; k + 1 < nz; ++k)
        for (size_t j = 0; j + 1 < ny; ++j)
            for (size_t i = 0; i + 1 < nx; ++i) {
                int c = 0;
                for (int v = 0; v < 8; ++v)
                    if (data[((k + dz[v]) * ny + (j + dy[v])) * nx + (i + dx[v])] >= iso) c |= 1 << v;
                const int n = case_ntris(c);
                if (n) counts[((k / block) * nby + j / block) * nbx + i / block] += n;
            }
}
