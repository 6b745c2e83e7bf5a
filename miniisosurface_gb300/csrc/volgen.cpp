// Seeded synthetic scalar fields of the benchmark workloads (no dataset is
// shipped with miniIsosurface; these stand in for its inputs):
//   blobs        sum of isotropic Gaussians exp(-|x-c|^2 / (2 s^2)), amplitude 1
//   value noise  octaves of trilinearly interpolated uniform[-1,1] lattices
// Both are evaluated in double and rounded to float32 once, with no libm call
// (the exponential below is our own), so a seed gives bit-identical volumes on
// every host (compiled with -ffp-contract=off).  Work is split over OpenMP
// threads by z-plane; the result does not depend on the thread count.
#include <cstdint>
#include <vector>

#include "../../include/miniiso.h"

namespace {

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

// Lattice value in [-1, 1) of lattice point (x, y, z) of one octave.
double lattice(uint64_t seed, int octave, int64_t x, int64_t y, int64_t z)
{
    uint64_t h = seed * 0x9E3779B97F4A7C15ull ^ (uint64_t)(octave + 1) * 0xD6E8FEB86659FD93ull;
    h ^= (uint64_t)x * 0xA0761D6478BD642Full;
    h = (h ^ (h >> 32)) * 0xE7037ED1A0B428DBull;
    h ^= (uint64_t)y * 0x8EBC6AF09C88C6E3ull;
    h = (h ^ (h >> 32)) * 0x589965CC75374CC3ull;
    h ^= (uint64_t)z * 0x1D8E4E27C47D124Full;
    h = (h ^ (h >> 29)) * 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// exp(x) for x <= 0 in plain double arithmetic: x = n ln2 + r with
// |r| <= ln2/2 (Cody-Waite split of ln2 into a short high part and a
// correction), exp(r) by its Taylor series to 18 terms (truncation error below
// 1e-20 there), then scaling by 2^n.  Values below 2^-1000 flush to zero.
double exp_nonpositive(double x)
{
    if (x < -690.0) return 0.0;
    const double ln2_hi = 0.693145751953125;           // 22 significant bits
    const double ln2_lo = 1.42860682030941723212e-6;   // ln2 - ln2_hi
    const double inv_ln2 = 1.44269504088896338700;
    const double t = x * inv_ln2;
    const long long n = (long long)(t < 0 ? t - 0.5 : t + 0.5);
    const double r = (x - (double)n * ln2_hi) - (double)n * ln2_lo;
    double term = 1.0, sum = 1.0;
    for (int q = 1; q <= 18; ++q) {
        term = term * r / (double)q;
        sum += term;
    }
    // sum * 2^n, n in [-996, 0]
    long long e = n;
    double scale = 1.0;
    while (e < -60) { scale *= 8.673617379884035e-19; e += 60; }  // 2^-60
    uint64_t bits = (uint64_t)(1023 + e) << 52;
    double p2;
    static_assert(sizeof(p2) == sizeof(bits), "double is 64-bit");
    __builtin_memcpy(&p2, &bits, sizeof p2);
    return sum * p2 * scale;
}

}  // namespace

extern "C" {

iso_status iso_generate_blobs(const int64_t dims[3], int nblobs, uint64_t seed, float* out)
{
    if (!dims || !out || nblobs < 0) return ISO_ERR_INVALID_ARG;
    const int64_t nx = dims[0], ny = dims[1], nz = dims[2];
    if (nx < 1 || ny < 1 || nz < 1) return ISO_ERR_INVALID_ARG;
    const double mean_side = (double)(nx + ny + nz) / 3.0;
    uint64_t s = seed;
    std::vector<double> cx(nblobs), cy(nblobs), cz(nblobs), sg(nblobs);
    for (int b = 0; b < nblobs; ++b) {
        cx[b] = uniform01(s) * (double)nx;
        cy[b] = uniform01(s) * (double)ny;
        cz[b] = uniform01(s) * (double)nz;
        sg[b] = (0.05 + 0.10 * uniform01(s)) * mean_side;
    }
    // separable: exp(-(dx^2+dy^2+dz^2)/(2s^2)) = ex(i) * ey(j) * ez(k)
    std::vector<double> ex((size_t)nblobs * nx), ey((size_t)nblobs * ny), ez((size_t)nblobs * nz);
    for (int b = 0; b < nblobs; ++b) {
        const double inv = 1.0 / (2.0 * sg[b] * sg[b]);
        for (int64_t i = 0; i < nx; ++i) ex[(size_t)b * nx + i] = exp_nonpositive(-((double)i - cx[b]) * ((double)i - cx[b]) * inv);
        for (int64_t j = 0; j < ny; ++j) ey[(size_t)b * ny + j] = exp_nonpositive(-((double)j - cy[b]) * ((double)j - cy[b]) * inv);
        for (int64_t k = 0; k < nz; ++k) ez[(size_t)b * nz + k] = exp_nonpositive(-((double)k - cz[b]) * ((double)k - cz[b]) * inv);
    }
    long long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; ++k) {
        for (int64_t j = 0; j < ny; ++j) {
            float* row = out + ((size_t)k * ny + j) * nx;
            for (int64_t i = 0; i < nx; ++i) {
                double v = 0.0;
                for (int b = 0; b < nblobs; ++b) v += ex[(size_t)b * nx + i] * ey[(size_t)b * ny + j] * ez[(size_t)b * nz + k];
                row[i] = (float)v;
            }
        }
    }
    return ISO_OK;
}

iso_status iso_generate_value_noise(const int64_t dims[3], int octaves, int period, uint64_t seed, float* out)
{
    if (!dims || !out || octaves < 1 || octaves > 16 || period < 1) return ISO_ERR_INVALID_ARG;
    const int64_t nx = dims[0], ny = dims[1], nz = dims[2];
    if (nx < 1 || ny < 1 || nz < 1) return ISO_ERR_INVALID_ARG;
    struct Octave {
        int64_t P, lx, ly, lz;
        double amp;
        std::vector<double> lat;  // (lz+2) x (ly+2) x (lx+2) lattice values
    };
    std::vector<Octave> oct(octaves);
    double amp = 1.0;
    for (int o = 0; o < octaves; ++o) {
        Octave& q = oct[o];
        q.P = period >> o;
        if (q.P < 1) q.P = 1;
        q.amp = amp;
        amp *= 0.5;
        q.lx = (nx - 1) / q.P + 2;
        q.ly = (ny - 1) / q.P + 2;
        q.lz = (nz - 1) / q.P + 2;
        q.lat.resize((size_t)q.lx * q.ly * q.lz);
        for (int64_t z = 0; z < q.lz; ++z)
            for (int64_t y = 0; y < q.ly; ++y)
                for (int64_t x = 0; x < q.lx; ++x)
                    q.lat[((size_t)z * q.ly + y) * q.lx + x] = lattice(seed, o, x, y, z);
    }
    long long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; ++k) {
        for (int64_t j = 0; j < ny; ++j) {
            float* row = out + ((size_t)k * ny + j) * nx;
            for (int64_t i = 0; i < nx; ++i) {
                double v = 0.0;
                for (int o = 0; o < octaves; ++o) {
                    const Octave& q = oct[o];
                    const int64_t x0 = i / q.P, y0 = j / q.P, z0 = k / q.P;
                    const double fx = (double)(i % q.P) / (double)q.P;
                    const double fy = (double)(j % q.P) / (double)q.P;
                    const double fz = (double)(k % q.P) / (double)q.P;
                    const double* L = q.lat.data();
                    auto at = [&](int64_t x, int64_t y, int64_t z) { return L[((size_t)z * q.ly + y) * q.lx + x]; };
                    const double c00 = at(x0, y0, z0) + fx * (at(x0 + 1, y0, z0) - at(x0, y0, z0));
                    const double c10 = at(x0, y0 + 1, z0) + fx * (at(x0 + 1, y0 + 1, z0) - at(x0, y0 + 1, z0));
                    const double c01 = at(x0, y0, z0 + 1) + fx * (at(x0 + 1, y0, z0 + 1) - at(x0, y0, z0 + 1));
                    const double c11 = at(x0, y0 + 1, z0 + 1) + fx * (at(x0 + 1, y0 + 1, z0 + 1) - at(x0, y0 + 1, z0 + 1));
                    const double c0 = c00 + fy * (c10 - c00);
                    const double c1 = c01 + fy * (c11 - c01);
                    v += q.amp * (c0 + fz * (c1 - c0));
                }
                row[i] = (float)v;
            }
        }
    }
    return ISO_OK;
}

}  // extern "C"
