/*
 * Seeded benchmark volumes for the oracle side -- TEST INFRASTRUCTURE ONLY.
 *
 * miniIsosurface ships no input data; the benchmark inputs are seeded
 * synthetic fields (Gaussian blobs and 4-octave value noise).  The product
 * generates them in miniisosurface_gb300/csrc/volgen.cpp.  This file states
 * the same generators a second time, in C, so that the CPU reference arm of
 * bench.py and the oracle tests can build the same volumes without loading
 * the product library.  tests/test_oracle.py checks the two bit for bit and
 * against the volume digests pinned in tests/golden/golden.json.
 *
 *   blobs        sum over b of exp(-|x - c_b|^2 / (2 s_b^2)), c_b uniform in
 *                the box, s_b uniform in [0.05, 0.15] x the mean side
 *   value noise  sum over octaves o of 0.5^o x trilinear interpolation of a
 *                hashed uniform[-1, 1) lattice of period (period >> o)
 *
 * Everything is evaluated in double with no libm call (the exponential is a
 * Cody-Waite reduction plus a Taylor series) and rounded to float once, so a
 * seed gives the same bits on every host (built with -ffp-contract=off).
 */
#include "oracle.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t next_u64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double next_unit(uint64_t* s) { return (double)(next_u64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* Lattice value in [-1, 1) at lattice point (x, y, z) of octave o. */
static double lattice_value(uint64_t seed, int o, int64_t x, int64_t y, int64_t z)
{
    uint64_t h = seed * 0x9E3779B97F4A7C15ull ^ (uint64_t)(o + 1) * 0xD6E8FEB86659FD93ull;
    h ^= (uint64_t)x * 0xA0761D6478BD642Full;
    h = (h ^ (h >> 32)) * 0xE7037ED1A0B428DBull;
    h ^= (uint64_t)y * 0x8EBC6AF09C88C6E3ull;
    h = (h ^ (h >> 32)) * 0x589965CC75374CC3ull;
    h ^= (uint64_t)z * 0x1D8E4E27C47D124Full;
    h = (h ^ (h >> 29)) * 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

/* exp(x) for x <= 0: x = n ln2 + r, |r| <= ln2 / 2, exp(r) by 18 Taylor
 * terms, times 2^n built from its exponent bits. */
static double exp_neg(double x)
{
    if (x < -690.0) return 0.0;
    const double ln2_hi = 0.693145751953125, ln2_lo = 1.42860682030941723212e-6;
    const double t = x * 1.44269504088896338700;
    const long long n = (long long)(t < 0 ? t - 0.5 : t + 0.5);
    const double r = (x - (double)n * ln2_hi) - (double)n * ln2_lo;
    double term = 1.0, sum = 1.0;
    for (int q = 1; q <= 18; ++q) {
        term = term * r / (double)q;
        sum += term;
    }
    long long e = n;
    double scale = 1.0;
    while (e < -60) {
        scale *= 8.673617379884035e-19; /* 2^-60 */
        e += 60;
    }
    const uint64_t bits = (uint64_t)(1023 + e) << 52;
    double p2;
    memcpy(&p2, &bits, sizeof p2);
    return sum * p2 * scale;
}

int oracle_generate_blobs(const size_t dims[3], int nblobs, uint64_t seed, float* out)
{
    const int64_t nx = (int64_t)dims[0], ny = (int64_t)dims[1], nz = (int64_t)dims[2];
    if (nx < 1 || ny < 1 || nz < 1 || nblobs < 0 || !out) return 1;
    const double mean_side = (double)(nx + ny + nz) / 3.0;
    uint64_t s = seed;
    const int nb = nblobs > 0 ? nblobs : 1;
    double* fx = (double*)malloc(sizeof(double) * (size_t)nb * (size_t)nx);
    double* fy = (double*)malloc(sizeof(double) * (size_t)nb * (size_t)ny);
    double* fz = (double*)malloc(sizeof(double) * (size_t)nb * (size_t)nz);
    if (!fx || !fy || !fz) {
        free(fx); free(fy); free(fz);
        return 1;
    }
    for (int b = 0; b < nblobs; ++b) {
        const double cx = next_unit(&s) * (double)nx;
        const double cy = next_unit(&s) * (double)ny;
        const double cz = next_unit(&s) * (double)nz;
        const double sg = (0.05 + 0.10 * next_unit(&s)) * mean_side;
        const double inv = 1.0 / (2.0 * sg * sg);
        /* the Gaussian is separable: one factor per axis */
        for (int64_t i = 0; i < nx; ++i) fx[(size_t)b * nx + i] = exp_neg(-((double)i - cx) * ((double)i - cx) * inv);
        for (int64_t j = 0; j < ny; ++j) fy[(size_t)b * ny + j] = exp_neg(-((double)j - cy) * ((double)j - cy) * inv);
        for (int64_t k = 0; k < nz; ++k) fz[(size_t)b * nz + k] = exp_neg(-((double)k - cz) * ((double)k - cz) * inv);
    }
    long long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; ++k) {
        for (int64_t j = 0; j < ny; ++j) {
            float* row = out + ((size_t)k * ny + j) * nx;
            for (int64_t i = 0; i < nx; ++i) {
                double v = 0.0;
                for (int b = 0; b < nblobs; ++b) v += fx[(size_t)b * nx + i] * fy[(size_t)b * ny + j] * fz[(size_t)b * nz + k];
                row[i] = (float)v;
            }
        }
    }
    free(fx); free(fy); free(fz);
    return 0;
}

typedef struct {
    int64_t period, lx, ly, lz;
    double amp;
    double* lat; /* lz x ly x lx lattice values */
} noise_octave;

int oracle_generate_value_noise(const size_t dims[3], int octaves, int period, uint64_t seed, float* out)
{
    const int64_t nx = (int64_t)dims[0], ny = (int64_t)dims[1], nz = (int64_t)dims[2];
    if (nx < 1 || ny < 1 || nz < 1 || octaves < 1 || octaves > 16 || period < 1 || !out) return 1;
    noise_octave oct[16];
    double amp = 1.0;
    int ok = 1;
    for (int o = 0; o < octaves; ++o) {
        noise_octave* q = &oct[o];
        q->period = (period >> o) < 1 ? 1 : (period >> o);
        q->amp = amp;
        amp *= 0.5;
        q->lx = (nx - 1) / q->period + 2;
        q->ly = (ny - 1) / q->period + 2;
        q->lz = (nz - 1) / q->period + 2;
        q->lat = (double*)malloc(sizeof(double) * (size_t)(q->lx * q->ly * q->lz));
        if (!q->lat) { ok = 0; continue; }
        for (int64_t z = 0; z < q->lz; ++z)
            for (int64_t y = 0; y < q->ly; ++y)
                for (int64_t x = 0; x < q->lx; ++x)
                    q->lat[((size_t)z * q->ly + y) * q->lx + x] = lattice_value(seed, o, x, y, z);
    }
    if (ok) {
        long long k;
#pragma omp parallel for schedule(static)
        for (k = 0; k < nz; ++k) {
            for (int64_t j = 0; j < ny; ++j) {
                float* row = out + ((size_t)k * ny + j) * nx;
                for (int64_t i = 0; i < nx; ++i) {
                    double v = 0.0;
                    for (int o = 0; o < octaves; ++o) {
                        const noise_octave* q = &oct[o];
                        const int64_t P = q->period, x0 = i / P, y0 = j / P, z0 = k / P;
                        const double fx = (double)(i % P) / (double)P;
                        const double fy = (double)(j % P) / (double)P;
                        const double fz = (double)(k % P) / (double)P;
#define L(x, y, z) q->lat[((size_t)(z) * q->ly + (y)) * q->lx + (x)]
                        const double c00 = L(x0, y0, z0) + fx * (L(x0 + 1, y0, z0) - L(x0, y0, z0));
                        const double c10 = L(x0, y0 + 1, z0) + fx * (L(x0 + 1, y0 + 1, z0) - L(x0, y0 + 1, z0));
                        const double c01 = L(x0, y0, z0 + 1) + fx * (L(x0 + 1, y0, z0 + 1) - L(x0, y0, z0 + 1));
                        const double c11 =
                            L(x0, y0 + 1, z0 + 1) + fx * (L(x0 + 1, y0 + 1, z0 + 1) - L(x0, y0 + 1, z0 + 1));
#undef L
                        const double c0 = c00 + fy * (c10 - c00);
                        const double c1 = c01 + fy * (c11 - c01);
                        v += q->amp * (c0 + fz * (c1 - c0));
                    }
                    row[i] = (float)v;
                }
            }
        }
    }
    for (int o = 0; o < octaves; ++o) free(oct[o].lat);
    return ok ? 0 : 1;
}
