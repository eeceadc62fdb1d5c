// Seeded synthetic worlds.  Every probability is an integer threshold on a
// 32-bit PCG32 draw (XSH-RR 64/32, O'Neill 2014) so the grids are identical on
// every host; the dune height field uses double-precision improved noise
// (Perlin 2002) compiled without FMA contraction.
#include <math.h>
#include <string.h>

#include <vector>

#include "fs3d_common.h"
#include "pcg.h"

namespace {

using fs3d::Pcg32;
using fs3d::kP05;
using fs3d::kP10;
using fs3d::kP20;
using fs3d::kP25;
using fs3d::kP30;
using fs3d::kP35;
using fs3d::kP40;

bool dims_ok(int X, int Y, int Z, const uint8_t* g) { return g && X > 0 && Y > 0 && Z > 0; }

void clear_with_floor(uint8_t* g, int X, int Y, int Z) {
    const size_t layer = (size_t)X * Z;
    memset(g, 0, layer * (size_t)Y);
    for (int y = 0; y < 2 && y < Y; ++y) memset(g + layer * y, 1, layer);
}

double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
double mix(double t, double a, double b) { return a + t * (b - a); }
double gradient(int hash, double x, double y, double z) {
    const int h = hash & 15;
    const double u = h < 8 ? x : y;
    const double v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}

double improved_noise(const uint8_t* p, double x, double y, double z) {
    const double fx = floor(x), fy = floor(y), fz = floor(z);
    const int xi = (int)fx & 255, yi = (int)fy & 255, zi = (int)fz & 255;
    x -= fx;
    y -= fy;
    z -= fz;
    const double u = fade(x), v = fade(y), w = fade(z);
    const int a = p[xi] + yi, aa = p[a] + zi, ab = p[a + 1] + zi;
    const int b = p[xi + 1] + yi, ba = p[b] + zi, bb = p[b + 1] + zi;
    const double l0 = mix(u, gradient(p[aa], x, y, z), gradient(p[ba], x - 1, y, z));
    const double l1 = mix(u, gradient(p[ab], x, y - 1, z), gradient(p[bb], x - 1, y - 1, z));
    const double l2 = mix(u, gradient(p[aa + 1], x, y, z - 1), gradient(p[ba + 1], x - 1, y, z - 1));
    const double l3 =
        mix(u, gradient(p[ab + 1], x, y - 1, z - 1), gradient(p[bb + 1], x - 1, y - 1, z - 1));
    return mix(w, mix(v, l0, l1), mix(v, l2, l3));
}

}  // namespace

extern "C" {

fs3d_status fs3d_gen_parity(uint64_t seed, int X, int Y, int Z, uint8_t* g) {
    if (!dims_ok(X, Y, Z, g)) return fs3d::set_error(FS3D_ERR_INVALID_ARG, "gen_parity: bad args");
    clear_with_floor(g, X, Y, Z);
    Pcg32 r(seed, 0xC1u);
    const size_t n = (size_t)X * Y * Z;
    for (size_t i = (size_t)X * Z * (Y / 2); i < n; ++i) {
        if (g[i]) continue;
        const uint32_t u = r.next();
        g[i] = u < kP25 ? 2 : (u < kP40 ? 3 : 0);
    }
    return FS3D_OK;
}

fs3d_status fs3d_gen_pillars(uint64_t seed, int X, int Y, int Z, uint8_t* g) {
    if (!dims_ok(X, Y, Z, g)) return fs3d::set_error(FS3D_ERR_INVALID_ARG, "gen_pillars: bad args");
    clear_with_floor(g, X, Y, Z);
    Pcg32 r(seed, 0xC2u);
    for (int p = 0; p < 256; ++p) {
        const int cx = (int)r.bounded((uint32_t)X), cz = (int)r.bounded((uint32_t)Z);
        const int rad = 2 + (int)r.bounded(7u), h = 10 + (int)r.bounded(291u);
        const int ytop = 2 + h < Y ? 2 + h : Y;
        for (int z = cz - rad; z <= cz + rad; ++z)
            for (int x = cx - rad; x <= cx + rad; ++x) {
                if (x < 0 || x >= X || z < 0 || z >= Z) continue;
                if ((x - cx) * (x - cx) + (z - cz) * (z - cz) > rad * rad) continue;
                for (int y = 2; y < ytop; ++y) g[(size_t)x + (size_t)X * ((size_t)z + (size_t)Z * y)] = 1;
            }
    }
    const size_t n = (size_t)X * Y * Z;
    for (size_t i = (size_t)X * Z * ((2 * Y + 4) / 5); i < n; ++i) {
        if (g[i]) continue;
        const uint32_t u = r.next();
        g[i] = u < kP30 ? 2 : (u < kP40 ? 3 : 0);
    }
    return FS3D_OK;
}

fs3d_status fs3d_gen_batch_dims(uint64_t master, int count, int* dims, uint64_t* seeds) {
    if (count < 0 || (count > 0 && (!dims || !seeds)))
        return fs3d::set_error(FS3D_ERR_INVALID_ARG, "gen_batch_dims: bad args");
    static const int kChoices[7] = {16, 24, 32, 48, 64, 96, 128};
    Pcg32 r(master, 0xC3u);
    for (int w = 0; w < count; ++w) {
        for (int a = 0; a < 3; ++a) dims[3 * w + a] = kChoices[r.bounded(7u)];
        seeds[w] = fs3d::fmix64(master ^ (uint64_t)w);
    }
    return FS3D_OK;
}

fs3d_status fs3d_gen_batch_world(uint64_t world_seed, int X, int Y, int Z, uint8_t* g) {
    if (!dims_ok(X, Y, Z, g)) return fs3d::set_error(FS3D_ERR_INVALID_ARG, "gen_batch_world: bad args");
    clear_with_floor(g, X, Y, Z);
    const fs3d::BatchWorldGen p = fs3d::batch_world_gen(world_seed);
    Pcg32 r(0, 0);
    r.state = p.fill_state;
    r.inc = p.inc;
    const uint32_t sand_thr = p.sand_thr, water_thr = p.water_thr;
    const size_t n = (size_t)X * Y * Z;
    for (size_t i = (size_t)X * Z * (Y / 2); i < n; ++i) {
        if (g[i]) continue;
        const uint32_t u = r.next();
        g[i] = u < sand_thr ? 2 : (u < water_thr ? 3 : 0);
    }
    return FS3D_OK;
}

fs3d_status fs3d_gen_dunes(uint64_t seed, int X, int Y, int Z, uint8_t* g) {
    if (!dims_ok(X, Y, Z, g)) return fs3d::set_error(FS3D_ERR_INVALID_ARG, "gen_dunes: bad args");
    uint8_t perm[512];
    Pcg32 r(seed, 0xC5u);
    for (int a = 0; a < 256; ++a) perm[a] = (uint8_t)a;
    for (int a = 255; a > 0; --a) {
        const int b = (int)r.bounded((uint32_t)(a + 1));
        const uint8_t t = perm[a];
        perm[a] = perm[b];
        perm[b] = t;
    }
    for (int a = 0; a < 256; ++a) perm[256 + a] = perm[a];
    std::vector<int> hf((size_t)X * Z);
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            double sum = 0.0, amp = 1.0, freq = 1.0, norm = 0.0;
            for (int oct = 0; oct < 4; ++oct) {
                sum += amp * improved_noise(perm, (double)x / 256.0 * freq, 0.5, (double)z / 256.0 * freq);
                norm += amp;
                amp *= 0.5;
                freq *= 2.0;
            }
            double h = round(0.3 * (double)Y * (0.5 + 0.5 * (sum / norm)));
            h = h < 0.0 ? 0.0 : (h > (double)Y ? (double)Y : h);
            hf[(size_t)z * X + x] = (int)h;
        }
    Pcg32 rw(seed, 0xC5Au);
    for (int y = 0; y < Y; ++y)
        for (int z = 0; z < Z; ++z) {
            uint8_t* row = g + (size_t)X * ((size_t)z + (size_t)Z * y);
            const int* hrow = hf.data() + (size_t)z * X;
            for (int x = 0; x < X; ++x) {
                if (y < hrow[x]) {
                    row[x] = 2;
                } else {
                    row[x] = rw.next() < kP10 ? 3 : 0;
                }
            }
        }
    return FS3D_OK;
}

}  // extern "C"
