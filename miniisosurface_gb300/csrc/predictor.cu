// Learned output-size predictor (no counterpart in the reference): per-block
// statistics of a volume, exact per-block triangle counts, and a small MLP
// (34 -> 64 -> 64 -> 1, ReLU, float32) with hand-written forward, backward
// and Adam kernels.
//
// Blocks are 16^3 cells (17^3 points, clipped at the grid's far faces),
// numbered (bz * nby + by) * nbx + bx.  A block's statistics (34 floats):
// min, max and a 32-bin histogram of its point values over [min, max]
// (fractions of its points).  They do not depend on the isovalue, so they are
// computed once per resident volume; the network's 34 inputs for an
// isovalue are (min - iso) / (max - min), (max - iso) / (max - min) and the
// 32 fractions.  A block has triangles only when min < iso <= max (some
// corner below, some at or above); the network is trained on and applied to
// those blocks; the package trains its output on triangles / 256.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "../../include/miniiso.h"
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

constexpr int kBlock = ISO_BLOCK;  // cells per block edge
constexpr int kIn = ISO_MLP_IN, kHid = ISO_MLP_HIDDEN;
// parameter layout: W1 [kIn][kHid], b1 [kHid], W2 [kHid][kHid], b2 [kHid], W3 [kHid], b3
constexpr int kOffB1 = kIn * kHid, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid,
              kOffB3 = kOffW3 + kHid, kParams = kOffB3 + 1;
static_assert(kParams == ISO_MLP_PARAMS, "parameter count");

struct BlockDims {
    int nbx, nby, nbz;
};

inline BlockDims block_dims(const Grid& g)
{
    auto nb = [](int n) { return n < 2 ? 0 : (n - 1 + kBlock - 1) / kBlock; };
    return {nb(g.nx), nb(g.ny), nb(g.nz)};
}

// ---- per-block statistics: one CTA per block ------------------------------
__global__ void __launch_bounds__(256) k_block_stats(const float* __restrict__ vol, Grid g, BlockDims bd,
                                                     float* __restrict__ stats)
{
    __shared__ float s_min[8], s_max[8];
    __shared__ unsigned s_hist[32];
    const int b = blockIdx.x;
    const int bx = b % bd.nbx, by = (b / bd.nbx) % bd.nby, bz = b / (bd.nbx * bd.nby);
    const int x0 = bx * kBlock, y0 = by * kBlock, z0 = bz * kBlock;
    const int ex = min(kBlock, g.nx - 1 - x0) + 1, ey = min(kBlock, g.ny - 1 - y0) + 1,
              ez = min(kBlock, g.nz - 1 - z0) + 1;  // points per edge
    const int npts = ex * ey * ez;
    auto value = [&](int p) {
        const int dx = p % ex, dy = (p / ex) % ey, dz = p / (ex * ey);
        return __ldg(vol + ((long long)(z0 + dz) * g.ny + (y0 + dy)) * g.nx + (x0 + dx));
    };
    float lo = 3.402823466e38f, hi = -3.402823466e38f;
    for (int p = threadIdx.x; p < npts; p += blockDim.x) {
        const float v = value(p);
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
    }
    for (int d = 16; d > 0; d >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, d));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, d));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_min[warp] = lo;
        s_max[warp] = hi;
    }
    if (threadIdx.x < 32) s_hist[threadIdx.x] = 0u;
    __syncthreads();
    lo = s_min[0];
    hi = s_max[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
        lo = fminf(lo, s_min[w]);
        hi = fmaxf(hi, s_max[w]);
    }
    const float range = hi - lo;
    const float scale = range > 0.f ? 32.f / range : 0.f;
    for (int p = threadIdx.x; p < npts; p += blockDim.x) {
        const int bin = min(31, max(0, (int)((value(p) - lo) * scale)));
        atomicAdd(&s_hist[bin], 1u);
    }
    __syncthreads();
    float* o = stats + (size_t)b * kIn;
    if (threadIdx.x == 0) {
        o[0] = lo;
        o[1] = hi;
    }
    if (threadIdx.x < 32) o[2 + threadIdx.x] = (float)s_hist[threadIdx.x] / (float)npts;
}

// ---- exact triangles per block from the count pass's bit rows -------------
// One thread per (cell row (j, k), word w): the triangles of the word's 32
// cells (tris_of_word, the count pass's formula) split into its two
// 16-cell halves, each half one block's.
__global__ void k_block_tris(const uint32_t* __restrict__ bits, Grid g, BlockDims bd, int* __restrict__ counts)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)(g.ny - 1) * (g.nz - 1);
    if (t >= rows * g.W) return;
    const int w = (int)(t % g.W);
    const long long cr = t / g.W;
    const int j = (int)(cr % (g.ny - 1)), k = (int)(cr / (g.ny - 1));
    auto word = [&](int jj, int kk, int ww) -> uint32_t {
        return ww < g.W ? __ldg(&bits[((long long)kk * g.ny + jj) * g.W + ww]) : 0u;
    };
    const uint32_t a = word(j, k, w), b = word(j + 1, k, w), c = word(j, k + 1, w), d = word(j + 1, k + 1, w);
    const uint32_t ash = (a >> 1) | (word(j, k, w + 1) << 31), bsh = (b >> 1) | (word(j + 1, k, w + 1) << 31);
    const uint32_t csh = (c >> 1) | (word(j, k + 1, w + 1) << 31), dsh = (d >> 1) | (word(j + 1, k + 1, w + 1) << 31);
    const uint32_t cells = validmask(w, g.nx - 1);
    const int by = j / kBlock, bz = k / kBlock;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const uint32_t m = cells & (half ? 0xffff0000u : 0x0000ffffu);
        if (!m) continue;
        const uint32_t n = tris_of_word(a, ash, bsh, b, c, csh, dsh, d, m);
        if (n) atomicAdd(&counts[((long long)bz * bd.nby + by) * bd.nbx + 2 * w + half], (int)n);
    }
}

// ---- the network -----------------------------------------------------------
// A CTA of 256 threads takes tiles of 64 samples.  Thread t works on sample
// row r = t / 4 and the 16 hidden units u0 .. u0 + 15, u0 = 16 * (t % 4), for
// the layer products; the weight gradients accumulate in registers over all
// tiles of the CTA (dW2 row i = t / 4, dW1 row k = t / 4 for t < 4 * kIn)
// and are added to `grads` once at the end.  Shared rows are padded to 65
// floats so that columns spread over the banks.
constexpr int kTile = 64, kPad = kHid + 1, kXPad = kIn + 1;

struct MlpSmem {
    float w1[kIn * kHid], b1[kHid], w2[kHid * kPad], b2[kHid], w3[kHid], b3;
    float x[kTile * kXPad], h1[kTile * kPad], h2[kTile * kPad], d2[kTile * kPad], d1[kTile * kPad];
    float dy[kTile], y[kTile];
};

__device__ __forceinline__ void load_params(MlpSmem& s, const float* __restrict__ p)
{
    for (int i = threadIdx.x; i < kIn * kHid; i += blockDim.x) s.w1[i] = p[i];
    for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) s.w2[(i / kHid) * kPad + i % kHid] = p[kOffW2 + i];
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
        s.b1[i] = p[kOffB1 + i];
        s.b2[i] = p[kOffB2 + i];
        s.w3[i] = p[kOffW3 + i];
    }
    if (threadIdx.x == 0) s.b3 = p[kOffB3];
}

// Inputs of sample n for the isovalue iso[n] from its block statistics.
__device__ __forceinline__ void load_tile(MlpSmem& s, const float* __restrict__ stats, const float* __restrict__ iso,
                                          long long base, long long n)
{
    for (int i = threadIdx.x; i < kTile * kIn; i += blockDim.x) {
        const int r = i / kIn, c = i % kIn;
        const long long q = base + r;
        float v = 0.f;
        if (q < n) {
            const float* st = stats + q * kIn;
            if (c < 2) {
                const float range = st[1] - st[0];
                v = range > 0.f ? (st[c] - iso[q]) / range : 0.f;
            } else {
                v = st[c];
            }
        }
        s.x[r * kXPad + c] = v;
    }
}

// h1, h2 and the output y of the tile.
__device__ __forceinline__ void forward_tile(MlpSmem& s)
{
    const int r = threadIdx.x >> 2, u0 = 16 * (threadIdx.x & 3);
    float acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = s.b1[u0 + q];
    for (int k = 0; k < kIn; ++k) {
        const float xv = s.x[r * kXPad + k];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] += xv * s.w1[k * kHid + u0 + q];
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) s.h1[r * kPad + u0 + q] = fmaxf(acc[q], 0.f);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = s.b2[u0 + q];
    for (int i = 0; i < kHid; ++i) {
        const float hv = s.h1[r * kPad + i];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] += hv * s.w2[i * kPad + u0 + q];
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) s.h2[r * kPad + u0 + q] = fmaxf(acc[q], 0.f);
    __syncthreads();
    if (threadIdx.x < kTile) {
        float y = s.b3;
        for (int u = 0; u < kHid; ++u) y += s.h2[threadIdx.x * kPad + u] * s.w3[u];
        s.y[threadIdx.x] = y;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256) k_mlp_forward(const float* __restrict__ params, const float* __restrict__ stats,
                                                     const float* __restrict__ iso, long long n, float* __restrict__ y)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>(s_raw);
    load_params(s, params);
    __syncthreads();
    for (long long base = (long long)blockIdx.x * kTile; base < n; base += (long long)gridDim.x * kTile) {
        load_tile(s, stats, iso, base, n);
        __syncthreads();
        forward_tile(s);
        if (threadIdx.x < kTile && base + threadIdx.x < n) y[base + threadIdx.x] = s.y[threadIdx.x];
        __syncthreads();
    }
}

// Prediction for many (block statistics, isovalue) sets in one launch: the
// samples are the sets' blocks one after another; a block counts when
// min < iso <= max, and max(y, 0) of those is added to its set's total.
constexpr int kMaxSets = 128;
struct PredictSets {
    int n;
    long long start[kMaxSets + 1];  // first sample of each set; start[n] = all samples
    const float* stats[kMaxSets];
    float iso[kMaxSets];
};

__global__ void __launch_bounds__(256) k_mlp_predict(const float* __restrict__ params, PredictSets sets,
                                                     float* __restrict__ totals)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>(s_raw);
    __shared__ int s_set[kTile];
    load_params(s, params);
    __syncthreads();
    const long long n = sets.start[sets.n];
    for (long long base = (long long)blockIdx.x * kTile; base < n; base += (long long)gridDim.x * kTile) {
        if (threadIdx.x < kTile) {  // the set of sample base + t (-1: past the end or an inactive block)
            const long long q = base + threadIdx.x;
            int set = -1;
            if (q < n) {
                int lo = 0, hi = sets.n - 1;  // last set with start <= q
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sets.start[mid] <= q) lo = mid;
                    else hi = mid - 1;
                }
                const float* st = sets.stats[lo] + (q - sets.start[lo]) * kIn;
                if (st[0] < sets.iso[lo] && st[1] >= sets.iso[lo]) set = lo;
            }
            s_set[threadIdx.x] = set;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kTile * kIn; i += blockDim.x) {
            const int r = i / kIn, c = i % kIn;
            const int set = s_set[r];
            float v = 0.f;
            if (set >= 0) {
                const float* st = sets.stats[set] + (base + r - sets.start[set]) * kIn;
                if (c < 2) {
                    const float range = st[1] - st[0];
                    v = range > 0.f ? (st[c] - sets.iso[set]) / range : 0.f;
                } else {
                    v = st[c];
                }
            }
            s.x[r * kXPad + c] = v;
        }
        __syncthreads();
        forward_tile(s);
        if (threadIdx.x < kTile && s_set[threadIdx.x] >= 0)
            atomicAdd(&totals[s_set[threadIdx.x]], fmaxf(s.y[threadIdx.x], 0.f));
        __syncthreads();
    }
}

// Gradient of the mean squared error (1/n) sum (y - target)^2 with respect
// to every parameter, added into grads (zeroed by the caller); the loss
// into *loss.
__global__ void __launch_bounds__(256) k_mlp_gradient(const float* __restrict__ params,
                                                      const float* __restrict__ stats, const float* __restrict__ iso,
                                                      const float* __restrict__ target, long long n,
                                                      float* __restrict__ grads, float* __restrict__ loss)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>(s_raw);
    load_params(s, params);
    __syncthreads();
    const int t = threadIdx.x, r = t >> 2, u0 = 16 * (t & 3);
    float gw2[16], gw1[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) gw2[q] = gw1[q] = 0.f;
    float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, lsum = 0.f;
    const float inv_n = 1.f / (float)n;
    for (long long base = (long long)blockIdx.x * kTile; base < n; base += (long long)gridDim.x * kTile) {
        load_tile(s, stats, iso, base, n);
        __syncthreads();
        forward_tile(s);
        if (t < kTile) {
            const long long q = base + t;
            float dy = 0.f;
            if (q < n) {
                const float e = s.y[t] - target[q];
                lsum += e * e;
                dy = 2.f * e * inv_n;
            }
            s.dy[t] = dy;
        }
        __syncthreads();
        // d2 = dy * w3 where h2 > 0
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int u = u0 + q;
            s.d2[r * kPad + u] = s.h2[r * kPad + u] > 0.f ? s.dy[r] * s.w3[u] : 0.f;
        }
        __syncthreads();
        // d1[r][i] = sum_u d2[r][u] w2[i][u] where h1 > 0
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int i = u0 + q;
            float acc = 0.f;
            for (int u = 0; u < kHid; ++u) acc += s.d2[r * kPad + u] * s.w2[i * kPad + u];
            s.d1[r * kPad + i] = s.h1[r * kPad + i] > 0.f ? acc : 0.f;
        }
        __syncthreads();
        // weight gradients of the tile
        {
            const int i = r;  // dW2 row
            for (int rr = 0; rr < kTile; ++rr) {
                const float hv = s.h1[rr * kPad + i];
#pragma unroll
                for (int q = 0; q < 16; ++q) gw2[q] += hv * s.d2[rr * kPad + u0 + q];
            }
        }
        if (r < kIn) {
            const int k = r;  // dW1 row
            for (int rr = 0; rr < kTile; ++rr) {
                const float xv = s.x[rr * kXPad + k];
#pragma unroll
                for (int q = 0; q < 16; ++q) gw1[q] += xv * s.d1[rr * kPad + u0 + q];
            }
        }
        if (t < kHid) {
            for (int rr = 0; rr < kTile; ++rr) {
                gb1 += s.d1[rr * kPad + t];
                gb2 += s.d2[rr * kPad + t];
                gw3 += s.h2[rr * kPad + t] * s.dy[rr];
            }
        }
        if (t == 0)
            for (int rr = 0; rr < kTile; ++rr) gb3 += s.dy[rr];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) atomicAdd(&grads[kOffW2 + r * kHid + u0 + q], gw2[q]);
    if (r < kIn) {
#pragma unroll
        for (int q = 0; q < 16; ++q) atomicAdd(&grads[r * kHid + u0 + q], gw1[q]);
    }
    if (t < kHid) {
        atomicAdd(&grads[kOffB1 + t], gb1);
        atomicAdd(&grads[kOffB2 + t], gb2);
        atomicAdd(&grads[kOffW3 + t], gw3);
    }
    if (t == 0) atomicAdd(&grads[kOffB3], gb3);
    for (int d = 16; d > 0; d >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, d);
    if ((t & 31) == 0) atomicAdd(loss, lsum * inv_n);
}

// Adam (Kingma & Ba 2015) with bias correction; step counts from 1.
__global__ void k_mlp_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ g, float lr, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

size_t mlp_smem() { return sizeof(MlpSmem); }

int mlp_blocks(long long n, int nsm)
{
    const long long tiles = (n + kTile - 1) / kTile;
    return (int)std::min<long long>(tiles, (long long)nsm * 2);
}

int device_sms()
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return nsm > 0 ? nsm : 1;
}

void launch_block_tris(const Grid& g, const uint32_t* bits, int* counts, cudaStream_t s)
{
    const BlockDims bd = block_dims(g);
    const long long threads = (long long)(g.ny - 1) * (g.nz - 1) * g.W;
    if (threads <= 0) return;
    k_block_tris<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(bits, g, bd, counts);
}

long long block_count(const Grid& g)
{
    const BlockDims bd = block_dims(g);
    return (long long)bd.nbx * bd.nby * bd.nbz;
}

}  // namespace iso

namespace {
using iso::Grid;

iso_status launch_status(cudaError_t e) { return e == cudaSuccess ? ISO_OK : ISO_ERR_CUDA; }

bool grid_of(const iso_grid* gr, Grid& g)
{
    if (!gr) return false;
    for (int a = 0; a < 3; ++a)
        if (gr->dims[a] < 1 || gr->dims[a] > (1ll << 30)) return false;
    g = Grid{};
    g.nx = (int)gr->dims[0];
    g.ny = (int)gr->dims[1];
    g.nz = (int)gr->dims[2];
    g.W = (g.nx + 31) / 32;
    g.kd = g.kr = 0;
    g.ke = g.nz;
    g.R = (long long)g.ny * g.nz;
    return true;
}
}  // namespace

extern "C" {

int64_t iso_block_count(const iso_grid* grid)
{
    Grid g;
    if (!grid_of(grid, g)) return -1;
    return iso::block_count(g);
}

iso_status iso_block_stats(const float* volume, const iso_grid* grid, float* stats, void* stream)
{
    Grid g;
    if (!grid_of(grid, g)) return ISO_ERR_INVALID_ARG;
    const long long nb = iso::block_count(g);
    if (nb == 0) return ISO_OK;
    if (!volume || !stats) return ISO_ERR_INVALID_ARG;
    iso::k_block_stats<<<(unsigned)nb, 256, 0, static_cast<cudaStream_t>(stream)>>>(volume, g, iso::block_dims(g),
                                                                                   stats);
    return launch_status(cudaGetLastError());
}

iso_status iso_mlp_forward(const float* params, const float* stats, const float* isovals, int64_t n, float* y,
                           void* stream)
{
    if (n < 0 || (n > 0 && (!params || !stats || !isovals || !y))) return ISO_ERR_INVALID_ARG;
    if (n == 0) return ISO_OK;
    const size_t smem = iso::mlp_smem();
    cudaFuncSetAttribute(iso::k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    iso::k_mlp_forward<<<iso::mlp_blocks(n, iso::device_sms()), 256, smem, static_cast<cudaStream_t>(stream)>>>(
        params, stats, isovals, n, y);
    return launch_status(cudaGetLastError());
}

iso_status iso_mlp_predict(const float* params, int64_t n_sets, const iso_block_set* sets, float* totals,
                           void* stream)
{
    if (n_sets < 0 || (n_sets > 0 && (!params || !sets || !totals))) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_sets == 0) return ISO_OK;
    if (cudaMemsetAsync(totals, 0, sizeof(float) * (size_t)n_sets, s) != cudaSuccess) return ISO_ERR_CUDA;
    const size_t smem = iso::mlp_smem();
    cudaFuncSetAttribute(iso::k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int nsm = iso::device_sms();
    for (int64_t s0 = 0; s0 < n_sets; s0 += iso::kMaxSets) {  // kMaxSets sets per launch
        iso::PredictSets ps{};
        ps.n = (int)std::min<int64_t>(iso::kMaxSets, n_sets - s0);
        long long at = 0;
        for (int q = 0; q < ps.n; ++q) {
            const iso_block_set& b = sets[s0 + q];
            if (b.n_blocks < 0 || (b.n_blocks > 0 && !b.stats)) return ISO_ERR_INVALID_ARG;
            ps.start[q] = at;
            ps.stats[q] = b.stats;
            ps.iso[q] = b.isoval;
            at += b.n_blocks;
        }
        ps.start[ps.n] = at;
        if (at == 0) continue;
        iso::k_mlp_predict<<<iso::mlp_blocks(at, nsm), 256, smem, s>>>(params, ps, totals + s0);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    return ISO_OK;
}

iso_status iso_mlp_gradient(const float* params, const float* stats, const float* isovals, const float* target,
                            int64_t n, float* grads, float* loss, void* stream)
{
    if (n <= 0 || !params || !stats || !isovals || !target || !grads || !loss) return ISO_ERR_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(grads, 0, sizeof(float) * ISO_MLP_PARAMS, s) != cudaSuccess ||
        cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess)
        return ISO_ERR_CUDA;
    const size_t smem = iso::mlp_smem();
    cudaFuncSetAttribute(iso::k_mlp_gradient, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    iso::k_mlp_gradient<<<iso::mlp_blocks(n, iso::device_sms()), 256, smem, s>>>(params, stats, isovals, target, n,
                                                                                grads, loss);
    return launch_status(cudaGetLastError());
}

iso_status iso_mlp_adam(float* params, float* m, float* v, const float* grads, int64_t step, float lr, void* stream)
{
    if (!params || !m || !v || !grads || step < 1) return ISO_ERR_INVALID_ARG;
    const double c1 = 1.0 - std::pow(0.9, (double)step), c2 = 1.0 - std::pow(0.999, (double)step);
    iso::k_mlp_adam<<<(ISO_MLP_PARAMS + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, m, v, grads, lr, (float)c1, (float)c2);
    return launch_status(cudaGetLastError());
}

}  // extern "C"
