/*
 * Oracle for the isosurface hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of miniIsosurface's serial Flying Edges
 * (flyingEdges/serial/FlyingEdgesAlgorithm.cpp) and serial Marching Cubes
 * (marchingCubes/serial/main.cpp:42-192).  It is used by the tests, by
 * smoke() and by the CPU-baseline leg of bench.py as the checker and as the
 * CPU timing baseline.  Nothing in the product links or calls it.
 *
 * Parity pin: the restatement is checked against the reference executables
 * themselves (compiled from the reference sources by oracle/build_ref.sh)
 * and against the committed golden fixtures in tests/golden/.
 *
 * Floating point follows the reference exactly: float32 arithmetic, no FMA
 * contraction (this library is compiled with -ffp-contract=off).
 */
#ifndef ISO_ORACLE_H
#define ISO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One output mesh: points / normals V x 3 float (AoS), tris T x 3 size_t.
 * edge_of_vertex[v] is the global edge id the vertex lies on, numbered like
 * marchingCubes/util/Image3D.cpp:210-256 (x-edges, then y-edges, then z). */
typedef struct oracle_mesh {
    size_t n_points;
    size_t n_tris;
    float* points;
    float* normals;
    size_t* tris;
    size_t* edge_of_vertex;
} oracle_mesh;

typedef struct oracle_fe oracle_fe;

/* Flying Edges, pass by pass (flyingEdges/serial/FlyingEdgesAlgorithm.h:29-49). */
oracle_fe* oracle_fe_create(const float* data, const size_t dims[3],
                            const float spacing[3], const float origin[3],
                            float isoval, int nthreads);
void oracle_fe_pass1(oracle_fe* fe);
void oracle_fe_pass2(oracle_fe* fe);
void oracle_fe_pass3(oracle_fe* fe);
void oracle_fe_pass4(oracle_fe* fe);
/* gridEdges as ny*nz records {xl, xr, xstart, ystart, zstart}. */
void oracle_fe_grid_edges(const oracle_fe* fe, size_t* out);
/* triCounter, (ny-1)*(nz-1) entries (counts after pass 2, offsets after pass 3). */
void oracle_fe_tri_counter(const oracle_fe* fe, size_t* out);
/* cubeCases, (nx-1)*(ny-1)*(nz-1) bytes (only trimmed ranges are written). */
void oracle_fe_cube_cases(const oracle_fe* fe, unsigned char* out);
/* moveOutput(): hands the mesh over; the oracle keeps nothing. */
void oracle_fe_take(oracle_fe* fe, oracle_mesh* out);
void oracle_fe_destroy(oracle_fe* fe);

/* All four passes in one call. */
int oracle_fe_run(const float* data, const size_t dims[3], const float spacing[3],
                  const float origin[3], float isoval, int nthreads, oracle_mesh* out);

/* Serial marching cubes with first-reference vertex numbering. */
int oracle_mc_run(const float* data, const size_t dims[3], const float spacing[3],
                  const float origin[3], float isoval, oracle_mesh* out);

/* The same mesh with its vertices in global-edge-index order
 * (util::duplicateRemover, marchingCubes/util/DuplicateRemover.h:38-103):
 * marchingCubes/openmpDupFree's output with one thread. */
int oracle_mc_dupfree_run(const float* data, const size_t dims[3], const float spacing[3],
                          const float origin[3], float isoval, oracle_mesh* out);

/* The OpenMP Marching Cubes of marchingCubes/openmp/main.cpp:156-296 with
 * its default sections (nthreads z-sections): vertices on the seams between
 * threads' sections appear once per section.  The threads' meshes are
 * appended in thread order. */
int oracle_mc_openmp_run(const float* data, const size_t dims[3], const float spacing[3],
                         const float origin[3], float isoval, int nthreads, oracle_mesh* out);

void oracle_mesh_free(oracle_mesh* m);

/* Triangles per block of `block`^3 cells at isovalue iso: each cell's case
 * from its eight corners (v0..v7 of Image3D::getValsCube,
 * flyingEdges/util/Image3D.cpp:26-43; corner bit set when value >= iso, the
 * test of calcCaseEdge, FlyingEdgesAlgorithm.cpp:31-45) and that case's
 * triangle count (numTris, flyingEdges/util/MarchingCubesTables.h:23),
 * summed over the block's cells.  counts has nbx*nby*nbz entries, block
 * (bx, by, bz) at (bz*nby + by)*nbx + bx, nb = ceil((n-1)/block). */
void oracle_block_tris(const float* data, const size_t dims[3], float iso, int block, int* counts);

/* The seeded benchmark volumes (oracle/volgen_oracle.c), x fastest:
 * Gaussian blobs and octaves of trilinear value noise.  Return 0 on success. */
int oracle_generate_blobs(const size_t dims[3], int nblobs, uint64_t seed, float* out);
int oracle_generate_value_noise(const size_t dims[3], int octaves, int period, uint64_t seed, float* out);

/* Seconds of wall time of the last oracle_fe_run / oracle_mc_run (or
 * oracle_mc_openmp_run) call
 * (extraction only, like the reference's "Total Program WALL Time"). */
double oracle_last_wall_seconds(void);
double oracle_mc_last_wall_seconds(void);

#ifdef __cplusplus
}
#endif

#endif
