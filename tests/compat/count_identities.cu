// Host check of the bit-parallel counts of iso_device.cuh (tris_of_word,
// mc_verts_of_word) against the per-cell tables: every cube case alone, and
// words of 32 random cases.  Prints "ok" or the first mismatch; exit code 0/1.
#include <cstdio>
#include <random>

#include "iso_device.cuh"

using namespace iso;

static uint32_t cut_mask(int c)
{
    uint32_t m = 0;
    for (int e = 0; e < 12; ++e)
        if (((c >> kIsoEdgeLo[e]) & 1) != ((c >> kIsoEdgeHi[e]) & 1)) m |= 1u << e;
    return m;
}

static uint32_t owned(bool i0, bool j0, bool k0)
{
    uint32_t m = (1u << 5) | (1u << 6) | (1u << 11);
    if (k0) m |= (1u << 1) | (1u << 2);
    if (j0) m |= (1u << 4) | (1u << 9);
    if (j0 && k0) m |= 1u;
    if (i0) m |= (1u << 7) | (1u << 10);
    if (i0 && k0) m |= 1u << 3;
    if (i0 && j0) m |= 1u << 8;
    return m;
}

int main()
{
    std::mt19937 rng(7);
    for (int trial = 0; trial < 20000; ++trial) {
        int cs[32];
        uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int b = 0; b < 32; ++b) {
            cs[b] = trial < 256 ? (b == 0 ? trial : 0) : (int)(rng() & 255u);
            for (int v = 0; v < 8; ++v) w[v] |= (uint32_t)((cs[b] >> v) & 1) << b;
        }
        const uint32_t cells = trial < 256 ? 1u : (uint32_t)rng();
        for (int flags = 0; flags < 8; ++flags) {
            const bool j0 = flags & 1, k0 = flags & 2, first0 = flags & 4;
            uint32_t want_t = 0, want_m = 0;
            for (int b = 0; b < 32; ++b) {
                if (!((cells >> b) & 1)) continue;
                want_t += (uint32_t)iso_case_ntris(kIsoCaseTris[cs[b]]);
                want_m += __builtin_popcount(owned(first0 && b == 0, j0, k0) & cut_mask(cs[b]));
            }
            const uint32_t got_t = tris_of_word(w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7], cells);
            const uint32_t got_m = mc_verts_of_word(w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7], cells, j0, k0,
                                                    first0);
            if (got_t != want_t || got_m != want_m) {
                std::printf("mismatch trial %d flags %d: tris %u/%u mc %u/%u\n", trial, flags, got_t, want_t, got_m,
                            want_m);
                return 1;
            }
        }
    }
    std::printf("ok\n");
    return 0;
}
