/*
 * fs3d oracle — CPU restatement (test infrastructure only; see fs3d_oracle.h).
 *
 * FS3D-rule v1 — the voxel update step, stated in full
 * ----------------------------------------------------
 * State.  A world is a dense uint8 grid of X*Y*Z cells, idx = x + X*(z + Z*y),
 *   gravity along -y.  0 EMPTY, 1 STONE, 2 SAND, 3 WATER; every value >= 4 is
 *   static and solid.  Cells outside the grid are solid and never written.
 *
 * Partition.  Step t (a per-world 64-bit counter) uses offset o = t & 1 on all
 *   three axes.  Blocks are 2x2x2 with lattice index (i,j,k), min corner
 *   (bx,by,bz) = (2i-o, 2j-o, 2k-o), i in [0, (X+o+1)/2) and likewise for j
 *   (over Y) and k (over Z).  Partial blocks at the faces are included; their
 *   missing cells are solid.  Blocks are disjoint, so they may be visited in
 *   any order; the canonical order is j, then k, then i.
 *
 * Slots.  Slot s in 0..7 is visited in increasing s.  L = s>>2 is the layer
 *   (0 = top, dy=1; 1 = bottom, dy=0), q = s&3 the column, dz = q>>1, dx = q&1.
 *   Every slot holding SAND or WATER that has not yet moved in this block tries:
 *   (a) top layer only: straight down into the bottom cell of its column, if
 *       that cell is EMPTY;
 *   (b) top layer only: diagonal-down: candidates are the other three bottom
 *       cells that are EMPTY, in increasing column order;
 *   (c) WATER only, either layer, only if (a) and (b) found nothing: sideways:
 *       candidates are the other three cells of its own layer that are EMPTY.
 *   With n candidates the r-th is taken, r = draw(n).  A move swaps the
 *   particle with the EMPTY cell and marks the destination as moved.  Sand
 *   never displaces water.
 *
 * Randomness (counter-based, shared by CPU and GPU):
 *   sk  = stepkey(seed, t)  = fmix32 chain over 0x243F6A88, seed_lo, seed_hi,
 *                             t_lo, t_hi
 *   rk  = rowkey(sk, j, k)  = fmix32(fmix32(sk ^ 0x85EBCA77*(j+1)) ^ 0xC2B2AE3D*(k+1))
 *   P_w = plane(rk, g, s, w) = fmix32(rk + 0x9E3779B9*(1 + w + 8s + 64g))
 *   For block i let g = i>>5, b = i&31 and p_w = bit b of P_w.
 *   draw(1) = 0;  draw(2) = p_0;
 *   draw(3): u = sum_w p_w << w (w = 0..7); r = u<85 ? 0 : (u<170 ? 1 : 2).
 *   fmix32 / fmix64 are the MurmurHash3 finalizers (Appleby, public domain).
 *   Every draw depends only on the world's seed, its step and the block, so a
 *   world's trajectory does not depend on where or with whom it is stepped.
 *
 * Stability.  A block changes under a step iff some SAND/WATER slot has a
 *   non-empty candidate set when visited; the first such slot sees the
 *   block's initial state, so "the block does not change" does not depend on
 *   the random draws.  (The first move puts a particle into a cell that was
 *   EMPTY at the start; a moved particle never moves again, so the block ends
 *   different from how it started.)
 *
 * Whole-grid hash: H = sum_i fmix64(i*256 + v_i) mod 2^64 (order-free).
 */
#include "fs3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* primitives                                                          */
/* ------------------------------------------------------------------ */
uint32_t orc_fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

uint64_t orc_fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

uint32_t orc_stepkey(uint64_t seed, uint64_t t) {
    uint32_t h = orc_fmix32(0x243F6A88u ^ (uint32_t)seed);
    h = orc_fmix32(h ^ (uint32_t)(seed >> 32));
    h = orc_fmix32(h ^ (uint32_t)t);
    h = orc_fmix32(h ^ (uint32_t)(t >> 32));
    return h;
}

uint32_t orc_rowkey(uint32_t sk, uint32_t j, uint32_t k) {
    uint32_t h = orc_fmix32(sk ^ (0x85EBCA77u * (j + 1u)));
    return orc_fmix32(h ^ (0xC2B2AE3Du * (k + 1u)));
}

uint32_t orc_plane(uint32_t rk, uint32_t g, uint32_t s, uint32_t w) {
    return orc_fmix32(rk + 0x9E3779B9u * (1u + w + 8u * s + 64u * g));
}

/* PCG32 XSH-RR 64/32 (O'Neill 2014, pcg32_srandom_r / pcg32_random_r /
 * pcg32_boundedrand_r as published). */
uint32_t orc_pcg32_next(orc_pcg32* r) {
    uint64_t old = r->state;
    r->state = old * 6364136223846793005ULL + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

void orc_pcg32_seed(orc_pcg32* r, uint64_t initstate, uint64_t initseq) {
    r->state = 0u;
    r->inc = (initseq << 1u) | 1u;
    orc_pcg32_next(r);
    r->state += initstate;
    orc_pcg32_next(r);
}

uint32_t orc_pcg32_bounded(orc_pcg32* r, uint32_t bound) {
    uint32_t threshold = (0u - bound) % bound;
    for (;;) {
        uint32_t v = orc_pcg32_next(r);
        if (v >= threshold) return v % bound;
    }
}

/* ------------------------------------------------------------------ */
/* the step                                                            */
/* ------------------------------------------------------------------ */
static int draw(int n, uint32_t rk, int i, int s) {
    if (n <= 1) return 0;
    uint32_t g = (uint32_t)i >> 5, b = (uint32_t)i & 31u;
    if (n == 2) return (int)((orc_plane(rk, g, (uint32_t)s, 0) >> b) & 1u);
    uint32_t u = 0;
    for (uint32_t w = 0; w < 8; ++w) u |= ((orc_plane(rk, g, (uint32_t)s, w) >> b) & 1u) << w;
    return u < 85u ? 0 : (u < 170u ? 1 : 2);
}

/* The rule on one block held as 8 values v[s] (slot s; out-of-grid slots
 * have inb[s] = 0 and hold 1, solid).  Updates v in place; returns 1 if
 * anything moved (with `dry`, returns at the first move without applying it). */
static int block_rule8(uint8_t* v, const int* inb, uint32_t rk, int i, int dry) {
    unsigned moved = 0;
    int changed = 0;
    for (int s = 0; s < 8; ++s) {
        const uint8_t m = v[s];
        if (!(m == 2 || m == 3) || ((moved >> s) & 1u)) continue;
        const int q = s & 3;
        int dst = -1;
        int cand[3], n;
        if (s < 4) {
            if (v[4 + q] == 0 && inb[4 + q]) {
                dst = 4 + q;
            } else {
                n = 0;
                for (int q2 = 0; q2 < 4; ++q2)
                    if (q2 != q && inb[4 + q2] && v[4 + q2] == 0) cand[n++] = 4 + q2;
                if (n) dst = cand[draw(n, rk, i, s)];
            }
        }
        if (dst < 0 && m == 3) {
            const int base = s & 4;
            n = 0;
            for (int q2 = 0; q2 < 4; ++q2)
                if (q2 != q && inb[base + q2] && v[base + q2] == 0) cand[n++] = base + q2;
            if (n) dst = cand[draw(n, rk, i, s)];
        }
        if (dst >= 0) {
            if (dry) return 1;
            v[dst] = m;
            v[s] = 0;
            moved |= 1u << dst;
            changed = 1;
        }
    }
    return changed;
}

/* Update block (i,j,k) of step t in place.  Returns 1 if anything moved. */
static int block_update(uint8_t* grid, int X, int Y, int Z, int o, uint32_t rk, int i, int j,
                        int k, int dry) {
    const int bx = 2 * i - o, by = 2 * j - o, bz = 2 * k - o;
    int64_t idx[8];
    int inb[8];
    uint8_t v[8];
    for (int s = 0; s < 8; ++s) {
        const int L = s >> 2, q = s & 3;
        const int x = bx + (q & 1), y = by + (1 - L), z = bz + (q >> 1);
        inb[s] = (x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z);
        idx[s] = inb[s] ? (int64_t)x + (int64_t)X * ((int64_t)z + (int64_t)Z * (int64_t)y) : -1;
        v[s] = inb[s] ? grid[idx[s]] : (uint8_t)1; /* out of bounds acts as solid */
    }
    const int changed = block_rule8(v, inb, rk, i, dry);
    if (changed && !dry)
        for (int s = 0; s < 8; ++s)
            if (inb[s]) grid[idx[s]] = v[s];
    return changed;
}

static inline int nblocks(int n, int o) { return (n + o + 1) / 2; }

/* One block row (j, k) of step t: the same rule as block_update for every i,
 * with the four rows addressed once.  A block changes only if it holds a
 * particle (2 or 3) and an empty cell (the stability property above), so
 * blocks without both are passed over. */
static void block_row(uint8_t* grid, int X, int Y, int Z, int o, uint32_t sk, int j, int k) {
    const int by = 2 * j - o, bz = 2 * k - o;
    uint8_t* row[4]; /* slot column q = dz*2 + dx: rows (layer, dz) -> index (1-L)*2 + dz */
    int rin[4];
    for (int r = 0; r < 4; ++r) {
        const int L = r >> 1, dz = r & 1;
        const int y = by + (1 - L), z = bz + dz;
        rin[r] = y >= 0 && y < Y && z >= 0 && z < Z;
        row[r] = rin[r] ? grid + (int64_t)X * ((int64_t)z + (int64_t)Z * (int64_t)y) : NULL;
    }
    const uint32_t rk = orc_rowkey(sk, (uint32_t)j, (uint32_t)k);
    const int NBX = nblocks(X, o);
    for (int i = 0; i < NBX; ++i) {
        const int x0 = 2 * i - o;
        if ((i & 3) == 0 && x0 >= 0 && x0 + 8 <= X) {
            /* four blocks at once (x0 .. x0+7 of the four rows): none can change
             * unless their cells hold both a particle and an empty cell */
            int part = 0, empty = 0;
            for (int r = 0; r < 4; ++r) {
                if (!rin[r]) continue; /* outside the grid: solid */
                uint64_t c;
                memcpy(&c, row[r] + x0, 8);
                const uint64_t lo = 0x0101010101010101ull, hi = 0x8080808080808080ull;
                const uint64_t p = (c & 0xFEFEFEFEFEFEFEFEull) ^ 0x0202020202020202ull; /* 0 byte: 2 or 3 */
                part |= ((p - lo) & ~p & hi) != 0;
                empty |= ((c - lo) & ~c & hi) != 0;
            }
            if (!part || !empty) {
                i += 3;
                continue;
            }
        }
        uint8_t v[8];
        int inb[8];
        int part = 0, empty = 0;
        for (int s = 0; s < 8; ++s) {
            const int L = s >> 2, q = s & 3;
            const int r = L * 2 + (q >> 1), x = x0 + (q & 1);
            inb[s] = rin[r] && x >= 0 && x < X;
            v[s] = inb[s] ? row[r][x] : (uint8_t)1;
            part |= v[s] == 2 || v[s] == 3;
            empty |= v[s] == 0;
        }
        if (!part || !empty) continue;
        if (block_rule8(v, inb, rk, i, 0))
            for (int s = 0; s < 8; ++s) {
                const int L = s >> 2, q = s & 3;
                if (inb[s]) row[L * 2 + (q >> 1)][x0 + (q & 1)] = v[s];
            }
    }
}

void orc_step(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t) {
    const int o = (int)(t & 1u);
    const uint32_t sk = orc_stepkey(seed, t);
    const int NBY = nblocks(Y, o), NBZ = nblocks(Z, o);
    for (int j = 0; j < NBY; ++j)
        for (int k = 0; k < NBZ; ++k) block_row(grid, X, Y, Z, o, sk, j, k);
}

void orc_step_shuffled(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t,
                       uint64_t order_seed) {
    const int o = (int)(t & 1u);
    const uint32_t sk = orc_stepkey(seed, t);
    const int NBX = nblocks(X, o), NBY = nblocks(Y, o), NBZ = nblocks(Z, o);
    const int64_t nb = (int64_t)NBX * NBY * NBZ;
    int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * (size_t)nb);
    if (!perm) return;
    for (int64_t a = 0; a < nb; ++a) perm[a] = a;
    orc_pcg32 r;
    orc_pcg32_seed(&r, order_seed, 0x5EEDu);
    for (int64_t a = nb - 1; a > 0; --a) {
        uint64_t hi = orc_pcg32_next(&r), lo = orc_pcg32_next(&r);
        int64_t b = (int64_t)(((hi << 32) | lo) % (uint64_t)(a + 1));
        int64_t tmp = perm[a];
        perm[a] = perm[b];
        perm[b] = tmp;
    }
    for (int64_t a = 0; a < nb; ++a) {
        const int64_t p = perm[a];
        const int i = (int)(p % NBX);
        const int k = (int)((p / NBX) % NBZ);
        const int j = (int)(p / ((int64_t)NBX * NBZ));
        block_update(grid, X, Y, Z, o, orc_rowkey(sk, (uint32_t)j, (uint32_t)k), i, j, k, 0);
    }
    free(perm);
}

void orc_step_omp(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t, int nthreads) {
    const int o = (int)(t & 1u);
    const uint32_t sk = orc_stepkey(seed, t);
    const int NBY = nblocks(Y, o), NBZ = nblocks(Z, o);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads) collapse(2)
#else
    (void)nthreads;
#endif
    for (int j = 0; j < NBY; ++j)
        for (int k = 0; k < NBZ; ++k) block_row(grid, X, Y, Z, o, sk, j, k);
}

void orc_run(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t0, int n,
             uint64_t* hashes, int nthreads) {
    const int64_t cells = (int64_t)X * Y * Z;
    for (int a = 0; a < n; ++a) {
        if (nthreads == 1)
            orc_step(grid, X, Y, Z, seed, t0 + (uint64_t)a);
        else
            orc_step_omp(grid, X, Y, Z, seed, t0 + (uint64_t)a, nthreads);
        if (hashes) hashes[a] = orc_hash(grid, cells);
    }
}

int orc_block_would_change(const uint8_t* grid, int X, int Y, int Z, uint64_t t, int i, int j,
                           int k) {
    /* dry run: stability does not depend on the draws, so any row key will do */
    return block_update((uint8_t*)grid, X, Y, Z, (int)(t & 1u), 0u, i, j, k, 1);
}

/* ------------------------------------------------------------------ */
/* hash / diff                                                         */
/* ------------------------------------------------------------------ */
uint64_t orc_hash(const uint8_t* grid, int64_t n) {
    uint64_t h = 0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : h) schedule(static)
#endif
    for (int64_t i = 0; i < n; ++i) h += orc_fmix64((uint64_t)i * 256u + grid[i]);
    return h;
}

int64_t orc_first_diff(const uint8_t* a, const uint8_t* b, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (a[i] != b[i]) return i;
    return -1;
}

/* ------------------------------------------------------------------ */
/* generators                                                          */
/* ------------------------------------------------------------------ */
#define THR_P05 214748364u   /* floor(0.05 * 2^32) */
#define THR_P10 429496729u   /* floor(0.10 * 2^32) */
#define THR_P20 858993459u   /* floor(0.20 * 2^32) */
#define THR_P25 1073741824u  /* floor(0.25 * 2^32) */
#define THR_P30 1288490188u  /* floor(0.30 * 2^32) */
#define THR_P35 1503238553u  /* floor(0.35 * 2^32) */
#define THR_P40 1717986918u  /* floor(0.40 * 2^32) */

static inline int64_t cidx(int X, int Z, int x, int y, int z) {
    return (int64_t)x + (int64_t)X * ((int64_t)z + (int64_t)Z * (int64_t)y);
}

static void stone_floor(uint8_t* grid, int X, int Y, int Z) {
    const int64_t layer = (int64_t)X * Z;
    for (int y = 0; y < 2 && y < Y; ++y) memset(grid + layer * y, 1, (size_t)layer);
}

/* Parity workload: stone at y<2; for y >= Y/2 each cell iid, drawn in idx
 * order: sand p=0.25, water p=0.15, else empty. */
void orc_gen_c1(uint64_t seed, int X, int Y, int Z, uint8_t* grid) {
    const int64_t n = (int64_t)X * Y * Z, layer = (int64_t)X * Z;
    memset(grid, 0, (size_t)n);
    stone_floor(grid, X, Y, Z);
    orc_pcg32 r;
    orc_pcg32_seed(&r, seed, 0xC1u);
    for (int64_t i = layer * (Y / 2); i < n; ++i) {
        if (grid[i]) continue;
        uint32_t u = orc_pcg32_next(&r);
        grid[i] = u < THR_P25 ? 2 : (u < THR_P40 ? 3 : 0);
    }
}

/* Pillar workload: stone floor, 256 stone pillars (centre uniform, radius
 * 2..8, height 10..300), then for y >= ceil(2Y/5) every non-stone cell iid:
 * sand p=0.30, water p=0.10. */
void orc_gen_c2(uint64_t seed, int X, int Y, int Z, uint8_t* grid) {
    const int64_t n = (int64_t)X * Y * Z, layer = (int64_t)X * Z;
    memset(grid, 0, (size_t)n);
    stone_floor(grid, X, Y, Z);
    orc_pcg32 r;
    orc_pcg32_seed(&r, seed, 0xC2u);
    for (int p = 0; p < 256; ++p) {
        const int cx = (int)orc_pcg32_bounded(&r, (uint32_t)X);
        const int cz = (int)orc_pcg32_bounded(&r, (uint32_t)Z);
        const int rad = 2 + (int)orc_pcg32_bounded(&r, 7u);
        const int h = 10 + (int)orc_pcg32_bounded(&r, 291u);
        const int ytop = (2 + h < Y) ? 2 + h : Y;
        for (int z = cz - rad; z <= cz + rad; ++z) {
            if (z < 0 || z >= Z) continue;
            for (int x = cx - rad; x <= cx + rad; ++x) {
                if (x < 0 || x >= X) continue;
                if ((x - cx) * (x - cx) + (z - cz) * (z - cz) > rad * rad) continue;
                for (int y = 2; y < ytop; ++y) grid[cidx(X, Z, x, y, z)] = 1;
            }
        }
    }
    const int y0 = (2 * Y + 4) / 5;
    for (int64_t i = layer * y0; i < n; ++i) {
        if (grid[i]) continue;
        uint32_t u = orc_pcg32_next(&r);
        grid[i] = u < THR_P30 ? 2 : (u < THR_P40 ? 3 : 0);
    }
}

/* Mixed-size batch: per world X, Y, Z drawn (in that order) uniformly from
 * {16,24,32,48,64,96,128} with the master generator; world seed =
 * fmix64(master ^ world index). */
void orc_gen_c3_dims(uint64_t master, int count, int* dims, uint64_t* seeds) {
    static const int choices[7] = {16, 24, 32, 48, 64, 96, 128};
    orc_pcg32 r;
    orc_pcg32_seed(&r, master, 0xC3u);
    for (int w = 0; w < count; ++w) {
        for (int a = 0; a < 3; ++a) dims[3 * w + a] = choices[orc_pcg32_bounded(&r, 7u)];
        seeds[w] = orc_fmix64(master ^ (uint64_t)w);
    }
}

/* One batch world: sand fraction U[0.05,0.40], water U[0,0.20] (integer
 * thresholds from two draws), stone at y<2, cells with y >= Y/2 filled iid. */
void orc_gen_c3_world(uint64_t world_seed, int X, int Y, int Z, uint8_t* grid) {
    const int64_t n = (int64_t)X * Y * Z, layer = (int64_t)X * Z;
    memset(grid, 0, (size_t)n);
    stone_floor(grid, X, Y, Z);
    orc_pcg32 r;
    orc_pcg32_seed(&r, world_seed, 0xC3Du);
    const uint32_t u1 = orc_pcg32_next(&r), u2 = orc_pcg32_next(&r);
    const uint32_t sand_thr = THR_P05 + (uint32_t)(((uint64_t)u1 * THR_P35) >> 32);
    const uint32_t water_thr = sand_thr + (uint32_t)(((uint64_t)u2 * THR_P20) >> 32);
    for (int64_t i = layer * (Y / 2); i < n; ++i) {
        if (grid[i]) continue;
        uint32_t u = orc_pcg32_next(&r);
        grid[i] = u < sand_thr ? 2 : (u < water_thr ? 3 : 0);
    }
}

/* Improved noise (Perlin 2002), restated from the published algorithm. */
static double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
static double lerp_d(double t, double a, double b) { return a + t * (b - a); }
static double grad(int hash, double x, double y, double z) {
    const int h = hash & 15;
    const double u = h < 8 ? x : y;
    const double v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}

double orc_perlin(const uint8_t* p, double x, double y, double z) {
    const double fx = floor(x), fy = floor(y), fz = floor(z);
    const int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
    x -= fx;
    y -= fy;
    z -= fz;
    const double u = fade(x), v = fade(y), w = fade(z);
    const int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
    const int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
    const double x1 = lerp_d(u, grad(p[AA], x, y, z), grad(p[BA], x - 1, y, z));
    const double x2 = lerp_d(u, grad(p[AB], x, y - 1, z), grad(p[BB], x - 1, y - 1, z));
    const double x3 = lerp_d(u, grad(p[AA + 1], x, y, z - 1), grad(p[BA + 1], x - 1, y, z - 1));
    const double x4 =
        lerp_d(u, grad(p[AB + 1], x, y - 1, z - 1), grad(p[BB + 1], x - 1, y - 1, z - 1));
    return lerp_d(w, lerp_d(v, x1, x2), lerp_d(v, x3, x4));
}

/* Dune world: height h(x,z) = clamp(round(0.3*Y*(0.5+0.5*fbm)), 0, Y) with a
 * 4-octave fbm (lacunarity 2, gain 0.5, normalised by the amplitude sum) of
 * improved noise at (x/256, 0.5, z/256) over a seeded permutation; sand for
 * y < h, water iid p=0.1 (drawn in idx order) for y >= h. */
void orc_gen_c5(uint64_t seed, int X, int Y, int Z, uint8_t* grid) {
    uint8_t perm[512];
    orc_pcg32 r;
    orc_pcg32_seed(&r, seed, 0xC5u);
    for (int a = 0; a < 256; ++a) perm[a] = (uint8_t)a;
    for (int a = 255; a > 0; --a) {
        const int b = (int)orc_pcg32_bounded(&r, (uint32_t)(a + 1));
        const uint8_t tmp = perm[a];
        perm[a] = perm[b];
        perm[b] = tmp;
    }
    for (int a = 0; a < 256; ++a) perm[256 + a] = perm[a];
    int* hf = (int*)malloc(sizeof(int) * (size_t)X * (size_t)Z);
    if (!hf) return;
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            double sum = 0.0, amp = 1.0, freq = 1.0, norm = 0.0;
            for (int oct = 0; oct < 4; ++oct) {
                sum += amp * orc_perlin(perm, (double)x / 256.0 * freq, 0.5,
                                        (double)z / 256.0 * freq);
                norm += amp;
                amp *= 0.5;
                freq *= 2.0;
            }
            const double fbm = sum / norm;
            double h = round(0.3 * (double)Y * (0.5 + 0.5 * fbm));
            if (h < 0.0) h = 0.0;
            if (h > (double)Y) h = (double)Y;
            hf[(size_t)z * (size_t)X + (size_t)x] = (int)h;
        }
    orc_pcg32 rw;
    orc_pcg32_seed(&rw, seed, 0xC5Au);
    for (int y = 0; y < Y; ++y)
        for (int z = 0; z < Z; ++z) {
            uint8_t* row = grid + cidx(X, Z, 0, y, z);
            const int* hrow = hf + (size_t)z * (size_t)X;
            for (int x = 0; x < X; ++x) {
                if (y < hrow[x]) {
                    row[x] = 2;
                } else {
                    const uint32_t u = orc_pcg32_next(&rw);
                    row[x] = u < THR_P10 ? 3 : 0;
                }
            }
        }
    free(hf);
}

/* ------------------------------------------------------------------ */
/* render (build with -ffp-contract=off: every op is a single IEEE op)  */
/* ------------------------------------------------------------------ */
static inline float dot3(const float* a, const float* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void normalize3(float* v) {
    const float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] = v[0] / len;
    v[1] = v[1] / len;
    v[2] = v[2] / len;
}

/* pixel -> uv of the fullscreen quad (renderer.cpp:1253-1267): vertex x=+1
 * carries u=0, x=-1 carries u=1; v grows with NDC y, which points down. */
static inline void pixel_uv2(int px, int py, int W, int H, float* ux, float* uy) {
    const float u = 1.0f - ((float)px + 0.5f) / (float)W;
    const float v = ((float)py + 0.5f) / (float)H;
    *ux = u * 2.0f - 1.0f;
    *uy = v * 2.0f - 1.0f;
}

/* fs_raymarch.frag:10-26 — map_the_world = sphereSDF(p, 0, 0.5) */
static inline float sdf_world(float x, float y, float z) {
    return sqrtf(x * x + y * y + z * z) - 0.5f;
}

void orc_render_sdf(const orc_camera* cam, int W, int H, float* rgba) {
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            float ux, uy;
            pixel_uv2(px, py, W, H, &ux, &uy);
            uy = uy * (1.0f / cam->aspect); /* fs_raymarch.frag:72 */
            float dir[3] = {ux, uy, 1.0f};
            normalize3(dir);
            const float* o = cam->origin;
            float col = 0.0f;
            float t = 0.0f;
            for (int it = 0; it < 64; ++it) { /* fs_raymarch.frag:41 */
                const float p[3] = {o[0] + t * dir[0], o[1] + t * dir[1], o[2] + t * dir[2]};
                const float d = sdf_world(p[0], p[1], p[2]);
                if (d < 0.001f) {
                    const float h = 0.001f; /* calculate_normal, :28-36 */
                    float n[3] = {
                        sdf_world(p[0] + h, p[1], p[2]) - sdf_world(p[0] - h, p[1], p[2]),
                        sdf_world(p[0], p[1] + h, p[2]) - sdf_world(p[0], p[1] - h, p[2]),
                        sdf_world(p[0], p[1], p[2] + h) - sdf_world(p[0], p[1], p[2] - h)};
                    normalize3(n);
                    /* the upstream shader points this vector away from the light */
                    float l[3] = {p[0] - cam->light_pos[0], p[1] - cam->light_pos[1],
                                  p[2] - cam->light_pos[2]};
                    normalize3(l);
                    col = fmaxf(0.05f, dot3(n, l));
                    break;
                } else if (t > 1000.0f) {
                    break;
                }
                t += d;
            }
            float* out = rgba + 4 * ((size_t)py * (size_t)W + (size_t)px);
            out[0] = col;
            out[1] = 0.0f;
            out[2] = 0.0f;
            out[3] = 1.0f;
        }
}

static const float k_palette[5][3] = {
    {0.0f, 0.0f, 0.0f},    /* empty (never shaded) */
    {0.50f, 0.50f, 0.52f}, /* stone */
    {0.86f, 0.74f, 0.46f}, /* sand */
    {0.20f, 0.42f, 0.90f}, /* water */
    {0.65f, 0.35f, 0.30f}, /* any static material >= 4 */
};

/* Voxel DDA: per pixel a ray from the camera, clipped to the grid's box
 * (slab test per axis in x, y, z order), walks cell by cell (Amanatides &
 * Woo): at each cell the axis whose next boundary comes first is stepped
 * (on equal keys z, then y, then x).  Axis a's key after n steps is
 * fmaf(n, |1/d_a|, b_a), b_a its first boundary's t: one rounding per key,
 * so a walker may jump over cells and land on the same keys.  The first
 * non-empty cell is shaded by its material colour times max(0.05, n.l),
 * n the normal of the face the ray entered through, l towards the light. */
void orc_render_dda(const uint8_t* grid, int X, int Y, int Z, const orc_camera* cam, int W,
                    int H, float* rgba) {
    const int N[3] = {X, Y, Z};
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            float ux, uy;
            pixel_uv2(px, py, W, H, &ux, &uy);
            const float sx = ux * cam->tan_half_fov * cam->aspect;
            const float sy = uy * cam->tan_half_fov;
            float d[3];
            for (int a = 0; a < 3; ++a)
                d[a] = cam->forward[a] + cam->right[a] * sx + cam->up[a] * sy;
            normalize3(d);
            const float* o = cam->origin;
            float out4[4] = {0.0f, 0.0f, 0.0f, 1.0f};
            float inv[3];
            float tmin = 0.0f, tmax = INFINITY;
            int entry_axis = -1, miss = 0;
            for (int a = 0; a < 3; ++a) {
                if (d[a] == 0.0f) {
                    inv[a] = INFINITY;
                    if (o[a] < 0.0f || o[a] >= (float)N[a]) miss = 1;
                    continue;
                }
                inv[a] = 1.0f / d[a];
                float t0 = (0.0f - o[a]) * inv[a];
                float t1 = ((float)N[a] - o[a]) * inv[a];
                if (t0 > t1) {
                    const float tmp = t0;
                    t0 = t1;
                    t1 = tmp;
                }
                if (t0 > tmin) {
                    tmin = t0;
                    entry_axis = a;
                }
                if (t1 < tmax) tmax = t1;
            }
            if (!miss && tmin <= tmax) {
                int v[3], step[3], nst[3] = {0, 0, 0};
                float tmx[3], tdl[3], tb0[3];
                for (int a = 0; a < 3; ++a) {
                    const float p = o[a] + d[a] * tmin;
                    int c = (int)floorf(p);
                    if (c < 0) c = 0;
                    if (c > N[a] - 1) c = N[a] - 1;
                    v[a] = c;
                    step[a] = d[a] > 0.0f ? 1 : (d[a] < 0.0f ? -1 : 0);
                    if (d[a] == 0.0f) {
                        tb0[a] = INFINITY;
                        tdl[a] = INFINITY;
                    } else {
                        tb0[a] = ((float)(c + (step[a] > 0 ? 1 : 0)) - o[a]) * inv[a];
                        tdl[a] = fabsf(inv[a]);
                    }
                    tmx[a] = tb0[a];
                }
                int last = entry_axis;
                float tcur = tmin;
                const int max_iter = X + Y + Z + 3;
                for (int it = 0; it < max_iter; ++it) {
                    const uint8_t m =
                        grid[(int64_t)v[0] + (int64_t)X * ((int64_t)v[2] + (int64_t)Z * v[1])];
                    if (m != 0) {
                        float n[3] = {0.0f, 0.0f, 0.0f};
                        if (last >= 0) n[last] = step[last] > 0 ? -1.0f : 1.0f;
                        float l[3] = {o[0] + d[0] * tcur - cam->light_pos[0],
                                      o[1] + d[1] * tcur - cam->light_pos[1],
                                      o[2] + d[2] * tcur - cam->light_pos[2]};
                        normalize3(l);
                        const float diff = fmaxf(0.05f, dot3(n, l));
                        const float* c = k_palette[m < 4 ? m : 4];
                        out4[0] = c[0] * diff;
                        out4[1] = c[1] * diff;
                        out4[2] = c[2] * diff;
                        break;
                    }
                    int a;
                    if (tmx[0] < tmx[1])
                        a = tmx[0] < tmx[2] ? 0 : 2;
                    else
                        a = tmx[1] < tmx[2] ? 1 : 2;
                    tcur = tmx[a];
                    v[a] += step[a];
                    if (v[a] < 0 || v[a] >= N[a]) break;
                    nst[a] += 1;
                    tmx[a] = fmaf((float)nst[a], tdl[a], tb0[a]);
                    last = a;
                }
            }
            memcpy(rgba + 4 * ((size_t)py * (size_t)W + (size_t)px), out4, sizeof(out4));
        }
}

/* ---- raymarch_sphere material: the object the upstream scene draws --------
 * Matrices follow materials.cpp:531-545 (view = rotY(camRot.y) * translate(camPos),
 * glm::perspective with an OpenGL depth range and proj[1][1] negated) and
 * raymarch_sphere.vert:30-45 (clip = viewproj*model*v; the fragment origin is
 * invModel*(-camPos), the fragment position the object-space vertex, both
 * noperspective).  Between the stages sit the fixed-function steps the
 * pipeline configures: no culling (pipelines.cpp:114), depth LESS_OR_EQUAL
 * against a buffer cleared to 1 (renderer.cpp:502-503, 1233), pixel centres
 * at (px+0.5, py+0.5), and a top-left rule on shared edges.  The fragment
 * stage is raymarch_sphere.frag:18-51.  Matrices are column-major,
 * m[c*4 + r]; every sum runs left to right. */
static void mat4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int i = 0; i < 4; ++i)
            r[c * 4 + i] = a[0 * 4 + i] * b[c * 4 + 0] + a[1 * 4 + i] * b[c * 4 + 1] +
                           a[2 * 4 + i] * b[c * 4 + 2] + a[3 * 4 + i] * b[c * 4 + 3];
    memcpy(out, r, sizeof(r));
}

/* inverse by 2x2 minors of the top and bottom row pairs (Laplace expansion,
 * D. Eberly, "The Laplace Expansion Theorem", 2008); 0 if singular */
static int mat4_inverse(const float* m, float* out) {
#define A(r, c) m[(c) * 4 + (r)]
    const float s0 = A(0, 0) * A(1, 1) - A(1, 0) * A(0, 1), s1 = A(0, 0) * A(1, 2) - A(1, 0) * A(0, 2);
    const float s2 = A(0, 0) * A(1, 3) - A(1, 0) * A(0, 3), s3 = A(0, 1) * A(1, 2) - A(1, 1) * A(0, 2);
    const float s4 = A(0, 1) * A(1, 3) - A(1, 1) * A(0, 3), s5 = A(0, 2) * A(1, 3) - A(1, 2) * A(0, 3);
    const float c5 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3), c4 = A(2, 1) * A(3, 3) - A(3, 1) * A(2, 3);
    const float c3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2), c2 = A(2, 0) * A(3, 3) - A(3, 0) * A(2, 3);
    const float c1 = A(2, 0) * A(3, 2) - A(3, 0) * A(2, 2), c0 = A(2, 0) * A(3, 1) - A(3, 0) * A(2, 1);
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0f || det != det) return 0;
    const float k = 1.0f / det;
    float b[16];
#define B(r, c) b[(c) * 4 + (r)]
    B(0, 0) = (A(1, 1) * c5 - A(1, 2) * c4 + A(1, 3) * c3) * k;
    B(0, 1) = (-A(0, 1) * c5 + A(0, 2) * c4 - A(0, 3) * c3) * k;
    B(0, 2) = (A(3, 1) * s5 - A(3, 2) * s4 + A(3, 3) * s3) * k;
    B(0, 3) = (-A(2, 1) * s5 + A(2, 2) * s4 - A(2, 3) * s3) * k;
    B(1, 0) = (-A(1, 0) * c5 + A(1, 2) * c2 - A(1, 3) * c1) * k;
    B(1, 1) = (A(0, 0) * c5 - A(0, 2) * c2 + A(0, 3) * c1) * k;
    B(1, 2) = (-A(3, 0) * s5 + A(3, 2) * s2 - A(3, 3) * s1) * k;
    B(1, 3) = (A(2, 0) * s5 - A(2, 2) * s2 + A(2, 3) * s1) * k;
    B(2, 0) = (A(1, 0) * c4 - A(1, 1) * c2 + A(1, 3) * c0) * k;
    B(2, 1) = (-A(0, 0) * c4 + A(0, 1) * c2 - A(0, 3) * c0) * k;
    B(2, 2) = (A(3, 0) * s4 - A(3, 1) * s2 + A(3, 3) * s0) * k;
    B(2, 3) = (-A(2, 0) * s4 + A(2, 1) * s2 - A(2, 3) * s0) * k;
    B(3, 0) = (-A(1, 0) * c3 + A(1, 1) * c1 - A(1, 2) * c0) * k;
    B(3, 1) = (A(0, 0) * c3 - A(0, 1) * c1 + A(0, 2) * c0) * k;
    B(3, 2) = (-A(3, 0) * s3 + A(3, 1) * s1 - A(3, 2) * s0) * k;
    B(3, 3) = (A(2, 0) * s3 - A(2, 1) * s1 + A(2, 2) * s0) * k;
#undef A
#undef B
    memcpy(out, b, sizeof(b));
    return 1;
}

void orc_object_mvp(const orc_object_view* v, float* mvp) {
    const float fovy = v->fovy_deg * 0.0174532925199432957692f;
    const float th = tanf(fovy * 0.5f);
    float P[16] = {0};
    P[0] = 1.0f / (v->aspect * th);
    P[5] = -(1.0f / th); /* proj[1][1] *= -1 */
    P[10] = -(v->zfar + v->znear) / (v->zfar - v->znear);
    P[11] = -1.0f;
    P[14] = -(2.0f * v->zfar * v->znear) / (v->zfar - v->znear);
    const float ang = v->cam_rot_y_deg * 0.0174532925199432957692f;
    const float c = cosf(ang), s = sinf(ang);
    float R[16] = {c, 0, -s, 0, 0, 1, 0, 0, s, 0, c, 0, 0, 0, 0, 1};
    float T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, v->cam_pos[0], v->cam_pos[1], v->cam_pos[2], 1};
    float V[16];
    mat4_mul(R, T, V);
    mat4_mul(P, V, mvp);
    mat4_mul(mvp, v->model, mvp);
}

/* edge function of p against a->b (y down: > 0 on the interior side of a
 * positively oriented triangle) */
static inline float edge_fn(const float* a, const float* b, float px, float py) {
    return (b[0] - a[0]) * (py - a[1]) - (b[1] - a[1]) * (px - a[0]);
}
static inline int top_left(const float* a, const float* b) {
    return b[1] < a[1] || (b[1] == a[1] && b[0] > a[0]);
}

/* raymarch_sphere.frag:13-16 (box of half-extent 0.5) */
static inline float box_sdf(float x, float y, float z) {
    const float qx = fabsf(x) - 0.5f, qy = fabsf(y) - 0.5f, qz = fabsf(z) - 0.5f;
    const float mx = fmaxf(qx, 0.0f), my = fmaxf(qy, 0.0f), mz = fmaxf(qz, 0.0f);
    return sqrtf(mx * mx + my * my + mz * mz) + fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f);
}

int orc_render_object(const orc_object_view* v, const float* tri, int ntri, int W, int H, float* rgba) {
    if (ntri < 0 || ntri > ORC_OBJECT_MAX_TRIS) return -1;
    float mvp[16], inv[16];
    orc_object_mvp(v, mvp);
    if (!mat4_inverse(v->model, inv)) return -1;
    const float ncp[3] = {-v->cam_pos[0], -v->cam_pos[1], -v->cam_pos[2]};
    float o[3];
    for (int i = 0; i < 3; ++i) o[i] = inv[0 * 4 + i] * ncp[0] + inv[1 * 4 + i] * ncp[1] + inv[2 * 4 + i] * ncp[2] + inv[3 * 4 + i];
    /* triangle set-up: screen positions, orientation, top-left edges */
    float sv[ORC_OBJECT_MAX_TRIS][3][3], at[ORC_OBJECT_MAX_TRIS][3][3], area[ORC_OBJECT_MAX_TRIS];
    int tl[ORC_OBJECT_MAX_TRIS][3];
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    for (int t = 0; t < ntri; ++t) {
        for (int k = 0; k < 3; ++k) {
            const float* p = tri + 9 * t + 3 * k;
            float cl[4];
            for (int i = 0; i < 4; ++i) cl[i] = mvp[0 * 4 + i] * p[0] + mvp[1 * 4 + i] * p[1] + mvp[2 * 4 + i] * p[2] + mvp[3 * 4 + i];
            if (!(cl[3] > 0.0f)) return -1;
            const float nx = cl[0] / cl[3], ny = cl[1] / cl[3], nz = cl[2] / cl[3];
            if (!(nz >= 0.0f && nz <= 1.0f)) return -1; /* clipping is not restated */
            sv[t][k][0] = nx * hw + hw;
            sv[t][k][1] = ny * hh + hh;
            sv[t][k][2] = nz;
            memcpy(at[t][k], p, 3 * sizeof(float));
        }
        area[t] = edge_fn(sv[t][0], sv[t][1], sv[t][2][0], sv[t][2][1]);
        if (area[t] < 0.0f) {
            float tmp[3];
            memcpy(tmp, sv[t][1], sizeof(tmp));
            memcpy(sv[t][1], sv[t][2], sizeof(tmp));
            memcpy(sv[t][2], tmp, sizeof(tmp));
            memcpy(tmp, at[t][1], sizeof(tmp));
            memcpy(at[t][1], at[t][2], sizeof(tmp));
            memcpy(at[t][2], tmp, sizeof(tmp));
            area[t] = edge_fn(sv[t][0], sv[t][1], sv[t][2][0], sv[t][2][1]);
        }
        tl[t][0] = top_left(sv[t][1], sv[t][2]);
        tl[t][1] = top_left(sv[t][2], sv[t][0]);
        tl[t][2] = top_left(sv[t][0], sv[t][1]);
    }
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
            float best = 1.0f, pos[3];
            int hit = 0;
            for (int t = 0; t < ntri; ++t) {
                if (!(area[t] > 0.0f)) continue;
                const float w0 = edge_fn(sv[t][1], sv[t][2], fx, fy);
                const float w1 = edge_fn(sv[t][2], sv[t][0], fx, fy);
                const float w2 = edge_fn(sv[t][0], sv[t][1], fx, fy);
                if (!(w0 > 0.0f || (w0 == 0.0f && tl[t][0]))) continue;
                if (!(w1 > 0.0f || (w1 == 0.0f && tl[t][1]))) continue;
                if (!(w2 > 0.0f || (w2 == 0.0f && tl[t][2]))) continue;
                const float l0 = w0 / area[t], l1 = w1 / area[t], l2 = w2 / area[t];
                const float z = l0 * sv[t][0][2] + l1 * sv[t][1][2] + l2 * sv[t][2][2];
                if (!(z <= best)) continue;
                best = z;
                hit = 1;
                for (int i = 0; i < 3; ++i) pos[i] = l0 * at[t][0][i] + l1 * at[t][1][i] + l2 * at[t][2][i];
            }
            float* out = rgba + 4 * ((size_t)py * (size_t)W + (size_t)px);
            if (!hit) {
                memcpy(out, v->clear, 4 * sizeof(float));
                continue;
            }
            float d[3] = {pos[0] - o[0], pos[1] - o[1], pos[2] - o[2]};
            normalize3(d);
            float col = 0.0f, t = 0.0f, density = 1.0f;
            for (int it = 0; it < 64; ++it) { /* ray_march, raymarch_sphere.frag:18-43 */
                const float dist = box_sdf(o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t);
                if (dist < 0.001f) {
                    col = fmaxf(0.05f, density);
                    break;
                } else if (t > 1000.0f) {
                    break;
                }
                t += dist;
                density -= 0.05f;
            }
            out[0] = col;
            out[1] = 0.0f;
            out[2] = 0.0f;
            out[3] = 1.0f;
        }
    return 0;
}

/* assets/cube2.obj: the +-1 cube of the scene, its 12 faces in file order */
int orc_mesh_cube(float* tri) {
    static const float vtx[8][3] = {{1, 1, -1}, {1, -1, -1}, {1, 1, 1}, {1, -1, 1},
                                    {-1, 1, -1}, {-1, -1, -1}, {-1, 1, 1}, {-1, -1, 1}};
    static const int face[12][3] = {{5, 3, 1}, {3, 8, 4}, {7, 6, 8}, {2, 8, 6}, {1, 4, 2}, {5, 2, 6},
                                    {5, 7, 3}, {3, 7, 8}, {7, 5, 6}, {2, 4, 8}, {1, 3, 4}, {5, 1, 2}};
    for (int t = 0; t < 12; ++t)
        for (int k = 0; k < 3; ++k) memcpy(tri + 9 * t + 3 * k, vtx[face[t][k] - 1], 3 * sizeof(float));
    return 12;
}

/* ---- mesh materials basic_mat / textured_mat / tri --------------------------
 * Restates basic_mat.{vert,frag}, textured_mat.{vert,frag} and tri.{vert,frag}
 * with the fixed-function state the pipelines set (no culling, depth
 * LESS_OR_EQUAL against 1, one sample per pixel, NEAREST filtering with
 * REPEAT addressing, R8G8B8A8_SRGB textures: materials.cpp:438,
 * initializers.cpp:49-58, pipelines.cpp:114,131, renderer.cpp:1233).
 * Stages: clip = P*V*model*(x,y,z,1); Sutherland-Hodgman clipping of each
 * triangle against 0 <= z <= w (Vulkan's depth range), fan triangulation;
 * screen position (x/w, y/w) to pixels, depth z/w; coverage by edge functions
 * at pixel centres with the top-left rule; per pixel the nearest fragment,
 * ties going to the later primitive; texture coordinates interpolated
 * perspective-correctly; texel i = floor(u*width) wrapped (likewise v);
 * sRGB-decoded through a 256-entry table; the result clamped to [0,1] as the
 * 8-bit attachment stores it. */
void orc_srgb_table(float* lut) {
    for (int i = 0; i < 256; ++i) {
        const double c = i / 255.0;
        lut[i] = (float)(c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4));
    }
}

/* floor to int, saturating, NaN -> 0 (the same on every platform) */
static int floor_to_int(float x) {
    if (x != x) return 0;
    x = floorf(x);
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return -2147483647 - 1;
    return (int)x;
}

typedef struct {
    float x, y, z, w, u, v;
} clip_vtx;

static clip_vtx clip_lerp(const clip_vtx* a, const clip_vtx* b, float t) {
    clip_vtx r;
    r.x = a->x + t * (b->x - a->x);
    r.y = a->y + t * (b->y - a->y);
    r.z = a->z + t * (b->z - a->z);
    r.w = a->w + t * (b->w - a->w);
    r.u = a->u + t * (b->u - a->u);
    r.v = a->v + t * (b->v - a->v);
    return r;
}

/* keeps the part with d >= 0, d = z (plane 0) or w - z (plane 1) */
static int clip_plane(const clip_vtx* in, int n, clip_vtx* out, int plane) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const clip_vtx* a = &in[i];
        const clip_vtx* b = &in[(i + 1) % n];
        const float da = plane ? a->w - a->z : a->z, db = plane ? b->w - b->z : b->z;
        if (da >= 0.0f) out[m++] = *a;
        if ((da >= 0.0f) != (db >= 0.0f)) out[m++] = clip_lerp(a, b, da / (da - db));
    }
    return m;
}

/* screen triangle: positions, depth, 1/w and u/w, v/w per vertex */
typedef struct {
    float sx[3], sy[3], sz[3], iw[3], uw[3], vw[3];
    float area;
    int tl;
    int valid;
} scr_tri;

/* up to three screen triangles of primitive p (vertices v: 3 x {x,y,z,u,v}) */
static void setup_prim(const float* mvp, const float* v, int W, int H, scr_tri* out) {
    clip_vtx a[8], b[8];
    for (int k = 0; k < 3; ++k) {
        const float* p = v + 5 * k;
        a[k].x = mvp[0] * p[0] + mvp[4] * p[1] + mvp[8] * p[2] + mvp[12];
        a[k].y = mvp[1] * p[0] + mvp[5] * p[1] + mvp[9] * p[2] + mvp[13];
        a[k].z = mvp[2] * p[0] + mvp[6] * p[1] + mvp[10] * p[2] + mvp[14];
        a[k].w = mvp[3] * p[0] + mvp[7] * p[1] + mvp[11] * p[2] + mvp[15];
        a[k].u = p[3];
        a[k].v = p[4];
    }
    int n = clip_plane(a, 3, b, 0);
    n = clip_plane(b, n, a, 1);
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    for (int t = 0; t < 3; ++t) {
        scr_tri* s = &out[t];
        s->valid = 0;
        if (t + 2 >= n) continue;
        const int idx[3] = {0, t + 1, t + 2};
        for (int k = 0; k < 3; ++k) {
            const clip_vtx* c = &a[idx[k]];
            if (!(c->w > 0.0f)) goto next;
            s->sx[k] = (c->x / c->w) * hw + hw;
            s->sy[k] = (c->y / c->w) * hh + hh;
            s->sz[k] = c->z / c->w;
            s->iw[k] = 1.0f / c->w;
            s->uw[k] = c->u * s->iw[k];
            s->vw[k] = c->v * s->iw[k];
        }
        s->area = edge_fn((float[]){s->sx[0], s->sy[0]}, (float[]){s->sx[1], s->sy[1]}, s->sx[2], s->sy[2]);
        if (s->area == 0.0f || s->area != s->area) continue;
        if (s->area < 0.0f) {
            float* f[6] = {s->sx, s->sy, s->sz, s->iw, s->uw, s->vw};
            for (int q = 0; q < 6; ++q) {
                const float x = f[q][1];
                f[q][1] = f[q][2];
                f[q][2] = x;
            }
            s->area = -s->area;
        }
        s->tl = top_left((float[]){s->sx[1], s->sy[1]}, (float[]){s->sx[2], s->sy[2]}) |
                top_left((float[]){s->sx[2], s->sy[2]}, (float[]){s->sx[0], s->sy[0]}) << 1 |
                top_left((float[]){s->sx[0], s->sy[0]}, (float[]){s->sx[1], s->sy[1]}) << 2;
        s->valid = 1;
    next:;
    }
}

/* barycentric weights of pixel centre (fx, fy); 0 if not covered */
static int tri_cover(const scr_tri* s, float fx, float fy, float* l) {
    const float w0 = edge_fn((float[]){s->sx[1], s->sy[1]}, (float[]){s->sx[2], s->sy[2]}, fx, fy);
    const float w1 = edge_fn((float[]){s->sx[2], s->sy[2]}, (float[]){s->sx[0], s->sy[0]}, fx, fy);
    const float w2 = edge_fn((float[]){s->sx[0], s->sy[0]}, (float[]){s->sx[1], s->sy[1]}, fx, fy);
    if (!(w0 > 0.0f || (w0 == 0.0f && (s->tl & 1)))) return 0;
    if (!(w1 > 0.0f || (w1 == 0.0f && (s->tl & 2)))) return 0;
    if (!(w2 > 0.0f || (w2 == 0.0f && (s->tl & 4)))) return 0;
    l[0] = w0 / s->area;
    l[1] = w1 / s->area;
    l[2] = w2 / s->area;
    return 1;
}

static float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

int orc_render_meshes(const orc_object_view* view, const orc_mesh_draw* draws, int n_draws, int W, int H,
                      float* rgba) {
    float lut[256];
    orc_srgb_table(lut);
    orc_object_view cam = *view;
    for (int i = 0; i < 16; ++i) cam.model[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    float vp[16];
    orc_object_mvp(&cam, vp);
    const size_t npx = (size_t)W * H;
    uint64_t* key = (uint64_t*)malloc(npx * sizeof(uint64_t));
    if (!key) return -1;
    for (size_t i = 0; i < npx; ++i) key[i] = ~0ull;
    /* pass 1: nearest fragment per pixel, keyed (depth, primitive) */
    int64_t prim0 = 0;
    for (int d = 0; d < n_draws; ++d) {
        float mvp[16];
        mat4_mul(vp, draws[d].model, mvp);
        const int nt = draws[d].n_vertices / 3;
        for (int t = 0; t < nt; ++t) {
            scr_tri st[3];
            setup_prim(mvp, draws[d].vertices + 15 * t, W, H, st);
            const uint32_t prim = (uint32_t)(prim0 + t);
            for (int q = 0; q < 3; ++q) {
                if (!st[q].valid) continue;
                float xmin = st[q].sx[0], xmax = xmin, ymin = st[q].sy[0], ymax = ymin;
                for (int k = 1; k < 3; ++k) {
                    xmin = fminf(xmin, st[q].sx[k]);
                    xmax = fmaxf(xmax, st[q].sx[k]);
                    ymin = fminf(ymin, st[q].sy[k]);
                    ymax = fmaxf(ymax, st[q].sy[k]);
                }
                int x0 = floor_to_int(xmin), x1 = floor_to_int(ceilf(xmax));
                int y0 = floor_to_int(ymin), y1 = floor_to_int(ceilf(ymax));
                x0 = x0 < 0 ? 0 : x0;
                y0 = y0 < 0 ? 0 : y0;
                x1 = x1 > W - 1 ? W - 1 : x1;
                y1 = y1 > H - 1 ? H - 1 : y1;
                for (int py = y0; py <= y1; ++py)
                    for (int px = x0; px <= x1; ++px) {
                        float l[3];
                        if (!tri_cover(&st[q], (float)px + 0.5f, (float)py + 0.5f, l)) continue;
                        const float z = l[0] * st[q].sz[0] + l[1] * st[q].sz[1] + l[2] * st[q].sz[2];
                        if (!(z >= 0.0f && z <= 1.0f)) continue;
                        uint32_t zb;
                        memcpy(&zb, &z, 4);
                        const uint64_t k = ((uint64_t)zb << 32) | (uint64_t)(0xFFFFFFFFu - (prim * 4u + (uint32_t)q));
                        size_t i = (size_t)py * W + px;
                        if (k < key[i]) key[i] = k;
                    }
            }
        }
        prim0 += nt;
    }
    /* pass 2: shade the winners */
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            float* out = rgba + 4 * ((size_t)py * W + px);
            const uint64_t k = key[(size_t)py * W + px];
            if (k == ~0ull) {
                memcpy(out, view->clear, 4 * sizeof(float));
                continue;
            }
            const uint32_t code = 0xFFFFFFFFu - (uint32_t)(k & 0xFFFFFFFFu);
            const uint32_t prim = code >> 2, q = code & 3u;
            int d = 0;
            int64_t base = 0;
            while (prim >= base + draws[d].n_vertices / 3) {
                base += draws[d].n_vertices / 3;
                ++d;
            }
            float mvp[16];
            mat4_mul(vp, draws[d].model, mvp);
            scr_tri st[3];
            setup_prim(mvp, draws[d].vertices + 15 * (prim - base), W, H, st);
            float l[3] = {0.0f, 0.0f, 0.0f}; /* the winner covers this pixel centre: tri_cover sets them */
            tri_cover(&st[q], (float)px + 0.5f, (float)py + 0.5f, l);
            const orc_mesh_draw* dr = &draws[d];
            float r = dr->color[0], g = dr->color[1], b = dr->color[2], a = dr->color[3];
            if (dr->material != ORC_MAT_BASIC) {
                const float den = l[0] * st[q].iw[0] + l[1] * st[q].iw[1] + l[2] * st[q].iw[2];
                const float u = (l[0] * st[q].uw[0] + l[1] * st[q].uw[1] + l[2] * st[q].uw[2]) / den;
                const float v = (l[0] * st[q].vw[0] + l[1] * st[q].vw[1] + l[2] * st[q].vw[2]) / den;
                int ti = floor_to_int(u * (float)dr->tex_width), tj = floor_to_int(v * (float)dr->tex_height);
                ti %= dr->tex_width;
                if (ti < 0) ti += dr->tex_width;
                tj %= dr->tex_height;
                if (tj < 0) tj += dr->tex_height;
                const uint8_t* tx = dr->texture + 4 * ((size_t)tj * dr->tex_width + ti);
                const float tr = lut[tx[0]], tg = lut[tx[1]], tb = lut[tx[2]];
                if (dr->material == ORC_MAT_TEXTURED) {
                    r += tr;
                    g += tg;
                    b += tb;
                    a += 1.0f;
                } else {
                    r = tr;
                    g = tg;
                    b = tb;
                    a = 1.0f;
                }
            }
            out[0] = clamp01(r);
            out[1] = clamp01(g);
            out[2] = clamp01(b);
            out[3] = clamp01(a);
        }
    free(key);
    return 0;
}
