/*
 * miniiso.h -- C ABI of the GB300 isosurface extractor.
 *
 * Drop-in boundary for miniIsosurface's serial extraction calls:
 *
 *   Flying Edges  FlyingEdgesAlgorithm(image, isoval); pass1(); pass2();
 *                 pass3(); pass4(); moveOutput()
 *                 (flyingEdges/serial/FlyingEdgesAlgorithm.h:29-49,
 *                  called from flyingEdges/serial/main.cpp:114-155)
 *   Marching Cubes  MarchingCubes(image, isoval) -> TriangleMesh
 *                 (marchingCubes/serial/main.cpp:42-44, called at :287)
 *
 * Input: a float32 volume, x fastest (data[k*nx*ny + j*nx + i]), its
 * spacing and origin (util::Image3D, flyingEdges/util/Image3D.h:26-85).
 * Output: points and normals (V x 3 float, AoS) and triangles (T x 3 vertex
 * indices, 32- or 64-bit), as util::TriangleMesh (TriangleMesh.h:24-90).
 * Triangle count, order, connectivity and vertex numbering are identical to
 * the reference; points and normals are bit-identical float32.
 *
 * Plain pointers and sizes only; no exceptions cross this boundary; every
 * call returns an iso_status.  One iso_ctx per host thread (a context is not
 * thread-safe; distinct contexts are).  All device work runs on the CUDA
 * stream passed in (NULL = legacy default stream).
 */
#ifndef MINIISO_H
#define MINIISO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum iso_status {
    ISO_OK = 0,
    ISO_ERR_INVALID_ARG = 1, /* bad pointer, dimension, algorithm or index width */
    ISO_ERR_OOM = 2,         /* device or pinned host allocation failed */
    ISO_ERR_CUDA = 3,        /* a CUDA call failed; see iso_ctx_last_error */
    ISO_ERR_CAPACITY = 4,    /* output buffers too small; n_points/n_tris hold the sizes needed */
    ISO_ERR_OVERFLOW = 5,    /* more than 2^32-1 vertices with 32-bit indices */
    ISO_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
    ISO_ERR_IO = 7,          /* file cannot be opened / read / written (util::file_not_found) */
    ISO_ERR_FORMAT = 8,      /* malformed VTK file (util::bad_format, LoadImage.h:45-133) */
    ISO_ERR_STATE = 9,       /* pass called out of order */
    ISO_ERR_TOO_LARGE = 10   /* grid beyond the fixed scratch of iso_count_device_noalloc */
} iso_status;

typedef enum iso_algorithm {
    ISO_FLYING_EDGES = 0,    /* vertex order of flyingEdges/serial */
    ISO_MARCHING_CUBES = 1,  /* vertex order of marchingCubes/serial */
    ISO_MC_DUPFREE = 2       /* Marching Cubes with the vertices in global-edge-index order, the order
                                util::duplicateRemover gives marchingCubes/openmpDupFree
                                (marchingCubes/util/DuplicateRemover.h:38-103); rows of at most
                                1024 points, whole-volume entry points only */
} iso_algorithm;

/* Geometry of a structured-points volume (Image3D's dims, spacing, zeroPos). */
/* Sample types of a volume: the VTK scalar types the reference reads
 * (flyingEdges/util/ConvertBuffer.h:45-72, TypeInfo.h) plus unsigned char. */
typedef enum iso_dtype {
    ISO_FLOAT32 = 0, /* float */
    ISO_INT8 = 1,    /* char (signed, as the reference's x86 hosts read it) */
    ISO_UINT8 = 2,   /* unsigned_char */
    ISO_INT16 = 3,   /* short */
    ISO_UINT16 = 4,  /* unsigned_short */
    ISO_INT32 = 5,   /* int */
    ISO_FLOAT64 = 6  /* double */
} iso_dtype;

typedef struct iso_grid {
    int64_t dims[3];
    float spacing[3];
    float origin[3];
} iso_grid;

/* Output mesh.  The caller owns the buffers (device or host, depending on
 * the call) and states their capacities in elements (points, triangles);
 * the library fills n_points / n_tris.  tris holds 3 indices per triangle of
 * index_bytes bytes each (4 or 8; 8 matches the reference's size_t). */
typedef struct iso_mesh {
    float* points;
    float* normals;
    void* tris;
    int32_t index_bytes;
    int64_t cap_points;
    int64_t cap_tris;
    int64_t n_points;
    int64_t n_tris;
} iso_mesh;

typedef struct iso_ctx iso_ctx;

const char* iso_status_string(iso_status s);
/* Library version string. */
const char* iso_version(void);

/* Context: device, case tables, scratch, pinned staging. */
iso_status iso_ctx_create(int device, iso_ctx** out);
iso_status iso_ctx_destroy(iso_ctx* ctx);
const char* iso_ctx_last_error(const iso_ctx* ctx);
/* Device-memory bytes currently held by the context's scratch. */
int64_t iso_ctx_scratch_bytes(const iso_ctx* ctx);

/* Per-pass device timing of the one-shot entry points (no counterpart in
 * the reference, whose util::Timer brackets each pass on the host,
 * flyingEdges/serial/main.cpp:120-158).  While enabled, CUDA events are
 * recorded on the extraction stream between consecutive kernels.
 * iso_ctx_profile_read synchronises on them, returns the summed
 * milliseconds and launch counts per pass (ISO_PASS_*) and clears them. */
enum {
    ISO_PASS_CLASSIFY = 0,     /* pass 1: fused into ISO_PASS_COUNT, never reported */
    ISO_PASS_COUNT = 1,        /* passes 1+2: classification and counts */
    ISO_PASS_SCAN = 2,         /* pass 3: offsets */
    ISO_PASS_FE_GENERATE = 3,  /* pass 4, Flying Edges */
    ISO_PASS_MC_VERTICES = 4,  /* pass 4, Marching Cubes vertices */
    ISO_PASS_MC_TRIANGLES = 5, /* pass 4, Marching Cubes triangles */
    ISO_PASS_VERTICES = 6,     /* pass 4, vertex points and normals from the generate pass's records */
    ISO_NUM_PASSES = 7
};
iso_status iso_ctx_profile(iso_ctx* ctx, int enable);
iso_status iso_ctx_profile_read(iso_ctx* ctx, double* ms, int64_t* launches);

/* Count only: passes 1-3 (FlyingEdgesAlgorithm.cpp:23-269).  Returns the
 * exact output sizes.  volume is a device pointer. */
iso_status iso_count_device(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                            float isoval, int64_t* n_points, int64_t* n_tris, void* stream);

/* Allocation-free count (no counterpart in the reference): the sizes
 * iso_count_device returns, for callers that must not allocate device memory
 * while they size a mesh (a solver that reserved the device for its own
 * pool, an allocator sizing a mesh before carving it from its arena, loops
 * that a device-wide cudaFree would stall).  No context: all scratch is one
 * fixed 16 MiB device array, which a device holds from the time the
 * library's module for this call loads until the process exits.  CUDA loads
 * modules lazily by default, so the first call on a device loads it: make
 * that call (a one-point grid will do) before reserving the device's memory,
 * and before any stream capture.  Grids of more than ISO_NOALLOC_MAX_ROWS
 * rows (ny * nz), or with rows of more than ISO_NOALLOC_MAX_ROW_POINTS
 * points, are rejected with ISO_ERR_TOO_LARGE before anything is enqueued.
 * ISO_MC_DUPFREE gives the ISO_MARCHING_CUBES counts (the same vertices in
 * another order).  Runs on the calling thread's current device; volume and
 * counts are device pointers on it.  Enqueues the count on `stream` and
 * returns: counts[0] = vertices, counts[1] = triangles once the stream gets
 * there.  Nothing is cached between calls.  Calls on one device must not
 * overlap (other streams or host threads): they share the scratch. */
#define ISO_NOALLOC_MAX_ROW_POINTS 858993459
#define ISO_NOALLOC_MAX_ROWS (1 << 20)
iso_status iso_count_device_noalloc(iso_algorithm algo, const float* volume, const iso_grid* grid, float isoval,
                                    int64_t* counts, void* stream);

/* Full extraction, volume and output in device memory.  Synchronises the
 * stream before returning.  If the buffers are too small nothing is written,
 * ISO_ERR_CAPACITY is returned and out->n_points / n_tris hold the sizes
 * needed.  Replaces the four passes + moveOutput() of
 * flyingEdges/serial/main.cpp:114-155 (ISO_FLYING_EDGES) and the
 * MarchingCubes() call of marchingCubes/serial/main.cpp:287
 * (ISO_MARCHING_CUBES). */
iso_status iso_extract_device(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                              float isoval, iso_mesh* out, void* stream);

/* Same, without the final synchronisation: all work is queued on `stream`;
 * result_host (4 x int64) receives, when the stream reaches that point, the
 * vertex count, the triangle count, a reserved value and the device status
 * (0, or ISO_ERR_TIMEOUT when a bounded device-side wait gave up).  Nothing
 * is written to the mesh when the counts exceed its capacities.  result_host
 * must stay valid until then (pinned memory gives a true asynchronous copy).
 * Calls on one context share its scratch: queue them on one stream. */
iso_status iso_extract_device_async(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                                    float isoval, iso_mesh* out, int64_t* result_host, void* stream);

/* Graph mode of iso_extract_device / iso_extract_device_async (no
 * counterpart in the reference; off by default): the first call captures its
 * kernels and the copy of the counts to result_host as a CUDA graph, and
 * later calls with the same arguments (volume, grid, isovalue, mesh,
 * result_host) relaunch it -- no per-kernel launch overhead between the
 * passes; a call with other arguments captures again (updating the graph in
 * place where possible).  result_host must be pinned for the graph path;
 * while per-pass profiling (iso_ctx_profile) is on, calls take the stream
 * path.  The same capture rules as iso_extract_batch apply. */
iso_status iso_ctx_set_graph(iso_ctx* ctx, int enable);

/* Batched extraction (no counterpart in the reference, which extracts one
 * volume per call).  n requests -- each a volume in device memory with its
 * own grid, isovalue and algorithm (an iso_algorithm value) -- into n
 * device meshes out[0..n); each mesh is exactly what iso_extract_device
 * gives for its request.  The requests are spread over lanes (streams with
 * their own scratch, largest requests first) and the whole batch is captured
 * once as a CUDA graph, launched on `stream`: no host round trip between
 * requests, and a repeated call with the same requests and meshes only
 * relaunches the graph (a changed batch is captured again and the graph
 * updated in place).  Capacities are checked on the device: a request whose
 * mesh is too small writes nothing and gets ISO_ERR_CAPACITY with the sizes
 * it needs in out[r].n_points / n_tris, as from iso_extract_device.
 * status (n entries, may be NULL) receives each request's status; the call
 * returns ISO_OK when every request succeeded, else the first failing
 * request's status.  Synchronises the stream.  Calls on one context must not
 * overlap, and none may run while a stream is being captured. */
typedef struct iso_request {
    const float* volume;
    iso_grid grid;
    float isoval;
    int32_t algorithm;
} iso_request;
iso_status iso_extract_batch(iso_ctx* ctx, int64_t n, const iso_request* req, iso_mesh* out, iso_status* status,
                             void* stream);
/* Batched extraction into one packed output, with no host round trip
 * between a request's counts and its mesh: request r's vertices go to
 * points / normals [point_first[r], point_first[r] + n_points[r]) and its
 * triangles to tris [tri_first[r], tri_first[r] + n_tris[r]) (index_bytes 4
 * or 8 per index, three per triangle), each request's indices counting from
 * its own first vertex, as in its own mesh.  point_first / tri_first are the
 * sums of the counts of the requests before it, so the meshes lie one after
 * another.  A request placed past cap_points or cap_tris (or with 2^32
 * vertices or more and 32-bit indices) writes nothing and gets
 * ISO_ERR_CAPACITY (ISO_ERR_OVERFLOW) with its sizes; the others complete.
 * Every request must be Flying Edges with rows of at most 512 points and its
 * volume at a 16-byte boundary (else ISO_ERR_INVALID_ARG for it).  All passes
 * of all requests run as one launch per pass and kernel variant, each request
 * with its own scratch held at once (about 60 + 4 * ceil(nx / 32) bytes per
 * grid row), so a batch too large for the device's free memory fails with
 * ISO_ERR_OOM: split it.  The five output arrays have n entries; status may be
 * NULL.  Synchronises the stream; returns ISO_OK or the first failing
 * request's status. */
iso_status iso_extract_batch_packed(iso_ctx* ctx, int64_t n, const iso_request* req, float* points, float* normals,
                                    void* tris, int32_t index_bytes, int64_t cap_points, int64_t cap_tris,
                                    int64_t* point_first, int64_t* tri_first, int64_t* n_points, int64_t* n_tris,
                                    iso_status* status, void* stream);

/* Counts only (passes 1-3) of a batch of requests, the same lanes and graph
 * as iso_extract_batch without the generate passes: n_points[r] / n_tris[r]
 * receive what iso_count_device returns for request r, for all requests with
 * one synchronisation (sizing meshes, admitting requests by output bytes). */
iso_status iso_count_batch(iso_ctx* ctx, int64_t n, const iso_request* req, int64_t* n_points, int64_t* n_tris,
                           iso_status* status, void* stream);

/* Learned output-size predictor (no counterpart in the reference): a small
 * network that predicts how many triangles an isovalue gives in each block of
 * 16^3 cells, from statistics of the block's samples.  Blocks are numbered
 * (bz * nby + by) * nbx + bx with nbx = ceil((nx - 1) / 16) and so on.
 *   iso_block_count     blocks of a grid.
 *   iso_block_stats     per block (ISO_MLP_IN floats): min, max and a 32-bin
 *                       histogram of its 17^3 point values over [min, max]
 *                       (fractions of its points); independent of the
 *                       isovalue, so computed once per resident volume.
 *   iso_block_tris      exact triangles of every block at isoval (the count
 *                       pass's bit rows, summed per block): the training
 *                       labels, and what the predictor's error is measured against.
 *   iso_mlp_forward     the network (ISO_MLP_IN -> 64 -> 64 -> 1, ReLU,
 *                       float32, ISO_MLP_PARAMS parameters) on n samples:
 *                       inputs of sample i are (min - iso[i]) / (max - min),
 *                       (max - iso[i]) / (max - min) and the 32 fractions of
 *                       stats row i; y[i] predicts the block's triangles
 *                       (the package trains it on triangles / 256).  It is
 *                       meant for blocks with min < iso <= max (the others
 *                       have no triangles).
 *   iso_mlp_gradient    gradient of (1/n) sum (y - target)^2 with respect to
 *                       the parameters (grads, ISO_MLP_PARAMS floats) and the
 *                       loss, for the same inputs.
 *   iso_mlp_adam        one Adam step (step counts from 1).
 *   iso_mlp_predict     for each of n_sets (block statistics, isovalue)
 *                       sets -- a volume's iso_block_stats and one isovalue
 *                       -- totals[s] = the sum of max(y, 0) over the set's
 *                       blocks with min < iso <= max: the predicted
 *                       triangles of a whole extraction (in the units the
 *                       network was trained on), all sets in one launch per
 *                       128 sets; totals (n_sets floats, device) is zeroed
 *                       first; `sets` is a host array.
 * All pointers are device memory; the calls enqueue on `stream`. */
#define ISO_BLOCK 16
#define ISO_MLP_IN 34
#define ISO_MLP_HIDDEN 64
#define ISO_MLP_PARAMS (ISO_MLP_IN * ISO_MLP_HIDDEN + ISO_MLP_HIDDEN + ISO_MLP_HIDDEN * ISO_MLP_HIDDEN + 2 * ISO_MLP_HIDDEN + 1)
int64_t iso_block_count(const iso_grid* grid);
iso_status iso_block_stats(const float* volume, const iso_grid* grid, float* stats, void* stream);
iso_status iso_block_tris(iso_ctx* ctx, const float* volume, const iso_grid* grid, float isoval, int32_t* counts,
                          void* stream);
iso_status iso_mlp_forward(const float* params, const float* stats, const float* isovals, int64_t n, float* y,
                           void* stream);
iso_status iso_mlp_gradient(const float* params, const float* stats, const float* isovals, const float* target,
                            int64_t n, float* grads, float* loss, void* stream);
iso_status iso_mlp_adam(float* params, float* m, float* v, const float* grads, int64_t step, float lr, void* stream);
typedef struct iso_block_set {
    const float* stats; /* n_blocks x ISO_MLP_IN, device */
    int64_t n_blocks;
    float isoval;
} iso_block_set;
iso_status iso_mlp_predict(const float* params, int64_t n_sets, const iso_block_set* sets, float* totals,
                           void* stream);

/* Lanes of iso_extract_batch / iso_count_batch: a fixed count (1..64), or 0
 * (the default).  Work split: a request's count and generate passes size
 * their grids and work items for nsm / share SMs (1..64; the lanes share the
 * GPU), or 0 (the default).  Whatever is 0 the autotuner picks: it times the
 * context's next batch at 1, 2, 4, ..., 64 lanes and shares 1, 2, 4, 8 (at
 * most the lanes; each run writes the same meshes) and keeps the fastest for
 * that batch and the ones after it.  iso_batch_lanes / iso_batch_split
 * return the values in use (0 before the autotuner has run). */
iso_status iso_batch_set_lanes(iso_ctx* ctx, int lanes);
iso_status iso_batch_set_split(iso_ctx* ctx, int share);
int iso_batch_split(const iso_ctx* ctx);
/* Whether the context's batches are captured as CUDA graphs (1, the default:
 * a repeated batch only relaunches its graph) or their lanes are launched
 * directly each call (0: no capture, for batches that change every call, as
 * in a serving loop; the lanes default to 8, or the autotuner's count once it
 * has run).  While a batch is being captured, no other thread may free device
 * memory or synchronise the device: that would invalidate the capture (the
 * library's own calls take turns with captures). */
iso_status iso_batch_set_graph(iso_ctx* ctx, int enable);
int iso_batch_lanes(const iso_ctx* ctx);
/* How the context's batches run their Flying Edges requests of rows up to
 * 512 points (volume at a 16-byte boundary): fused, one kernel launch per
 * pass and kernel variant covering all of them, each request with its own
 * scratch, or each request's passes on a lane.  The other requests take the
 * lanes beside the fused launches.  The meshes are the same either way.
 * mode 0: every request on the lanes; 1 (the default): fused when a batch
 * holds at least 16 such requests (fewer run faster on the lanes); 2: always
 * fused.  Other modes: ISO_ERR_INVALID_ARG. */
iso_status iso_batch_set_fused(iso_ctx* ctx, int mode);
/* The fused launches' work split: count blocks of at least *count_planes
 * planes, generate work items sized for about *items_per_warp per warp of
 * one wave.  The context's first graph-mode batch with fused requests times
 * 8, 16, 32 planes x 16, 32, 64 items per warp and keeps the fastest (both 0
 * before that; the defaults 16 and 32 are used meanwhile).
 * iso_batch_set_lanes(ctx, 0) also makes it tune again. */
iso_status iso_batch_fused_split(const iso_ctx* ctx, int* count_planes, int* items_per_warp);

/* z-slabs: the grid split along z into slabs of planes [k0, k1), for
 * sharding over GPUs or streaming a volume that does not fit (no counterpart
 * in the serial reference; marchingCubes/mpi/mpiutil.h:197-203 splits the
 * MPI version the same way).  A slab owns the Flying Edges vertices of the
 * grid rows of planes k0 .. k1-1, the cells between planes k0 and k1 (their
 * triangles) and, for Marching Cubes, the vertices those cells own.
 * `volume` (device memory) holds planes max(k0-1, 0) .. min(k1+1, nz-1) of
 * the grid only; `grid` describes the whole volume.  Rows must be at most
 * 1024 points long.
 * iso_count_slab: the slab's vertex and triangle counts.
 * iso_extract_slab: the slab's vertices and triangles, numbered exactly as in
 * the whole-volume extraction: the slab's first vertex has id point_offset
 * and its first triangle index tri_offset (the sums of the counts of the
 * slabs below: an exclusive scan of iso_count_slab over the slabs); `out`
 * receives the slab's part only (out->points row 0 is vertex point_offset).
 * Concatenating the slabs' parts gives the whole extraction's mesh, bit for
 * bit.  Both synchronise the stream. */
iso_status iso_count_slab(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid, int64_t k0,
                          int64_t k1, float isoval, int64_t* n_points, int64_t* n_tris, void* stream);
iso_status iso_extract_slab(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid, int64_t k0,
                            int64_t k1, float isoval, int64_t point_offset, int64_t tri_offset, iso_mesh* out,
                            void* stream);

/* Typed volumes: samples of `dtype`, converted to float32 on the device with
 * the reference's C cast to scalar_t (ConvertBuffer.h:45-72), then extracted
 * as float32 -- the same mesh as converting on the host first.  The narrow
 * types cross the host -> device link in 1/4 (8-bit) or 1/2 (16-bit) of the
 * bytes.  volume is a device pointer (_device_typed) or a host pointer
 * (_host_typed); otherwise as iso_extract_device / iso_extract_host. */
iso_status iso_extract_device_typed(iso_ctx* ctx, iso_algorithm algo, const void* volume, iso_dtype dtype,
                                    const iso_grid* grid, float isoval, iso_mesh* out, void* stream);
/* Narrow reads for iso_extract_device_typed (no counterpart in the reference;
 * on by default): 8- and 16-bit samples are read as they are by the count and
 * vertex passes -- no float32 copy of the volume -- for Flying Edges and
 * Marching Cubes over grids of rows of at most 512 points whose byte length is
 * a multiple of 16, with the volume at a 16-byte boundary.  The samples are
 * classified as the reference classifies their float conversion, so the mesh
 * is the one the converted volume gives.  enable = 0 converts first. */
iso_status iso_ctx_set_narrow(iso_ctx* ctx, int enable);
iso_status iso_extract_host_typed(iso_ctx* ctx, iso_algorithm algo, const void* volume, iso_dtype dtype,
                                  const iso_grid* grid, float isoval, iso_mesh* out, void* stream);

/* Host in, host out: copies the volume to the device, extracts, and copies
 * the mesh back into the caller's host buffers (pinned buffers give the full
 * link bandwidth).  This is the whole reference call, util::Image3D in and
 * util::TriangleMesh out. */
iso_status iso_extract_host(iso_ctx* ctx, iso_algorithm algo, const float* volume, const iso_grid* grid,
                            float isoval, iso_mesh* out, void* stream);

/* Flying Edges pass by pass, mirroring FlyingEdgesAlgorithm
 * (flyingEdges/serial/FlyingEdgesAlgorithm.h:29-49).  The volume is a host
 * pointer that must stay valid until iso_fe_pass4 (the reference keeps a
 * reference to the image); it is uploaded by iso_fe_pass1. */
typedef struct iso_fe iso_fe;
iso_status iso_fe_create(iso_ctx* ctx, const float* host_volume, const iso_grid* grid, float isoval,
                         iso_fe** out);
iso_status iso_fe_pass1(iso_fe* fe);  /* classification + trims      (:23-66)   */
iso_status iso_fe_pass2(iso_fe* fe);  /* cube cases, per-row counts   (:72-190)  */
iso_status iso_fe_pass3(iso_fe* fe);  /* prefix sums, output sizes    (:196-269) */
iso_status iso_fe_pass4(iso_fe* fe);  /* points, normals, triangles   (:275-497) */
/* Sizes known after pass 3. */
iso_status iso_fe_sizes(const iso_fe* fe, int64_t* n_points, int64_t* n_tris);
/* gridEdges {xl, xr, xstart, ystart, zstart} x ny*nz (after pass 2: counts;
 * after pass 3: offsets) and triCounter x (ny-1)*(nz-1), into host arrays. */
iso_status iso_fe_grid_edges(iso_fe* fe, uint64_t* grid_edges, uint64_t* tri_counter);
/* moveOutput() (:503-508): copies the mesh into the caller's host buffers. */
iso_status iso_fe_move_output(iso_fe* fe, iso_mesh* out);
iso_status iso_fe_destroy(iso_fe* fe);

/* ---- VTK legacy IO (flyingEdges/util/LoadImage.h, SaveTriangleMesh.h) ---- */

/* Reads a BINARY STRUCTURED_POINTS file (char, short, unsigned_short, int,
 * float or double scalars, big-endian) into float32.  Call with data == NULL
 * to get the grid only; then again with a buffer of dims product floats. */
iso_status iso_vtk_read_image(const char* path, iso_grid* grid, float* data);
/* Writes a mesh in the reference's POLYDATA layout (big-endian floats,
 * POLYGONS with 8-byte indices, NORMALS) -- byte-identical to
 * util::saveTriangleMesh.  Host buffers. */
iso_status iso_vtk_write_mesh(const char* path, const iso_mesh* mesh);
/* Writes a float32 volume as BINARY STRUCTURED_POINTS (big-endian). */
iso_status iso_vtk_write_image(const char* path, const iso_grid* grid, const float* data);

/* ---- synthetic volumes of the benchmark configurations ---- */

/* Sum of nblobs isotropic Gaussians exp(-|x-c|^2 / (2 s^2)), amplitude 1,
 * centres uniform in the box, s uniform in [0.05, 0.15] x mean side. */
iso_status iso_generate_blobs(const int64_t dims[3], int nblobs, uint64_t seed, float* host_out);
/* Octave value noise: trilinear interpolation of a seeded uniform[-1,1]
 * lattice, base period `period` cells, halved per octave, gain 0.5. */
iso_status iso_generate_value_noise(const int64_t dims[3], int octaves, int period, uint64_t seed,
                                    float* host_out);

#ifdef __cplusplus
}
#endif

#endif /* MINIISO_H */
