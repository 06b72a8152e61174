/*
 * bh_model.c -- CPU model of the GPU Barnes-Hut tree build.  TEST
 * INFRASTRUCTURE ONLY (the shipped library never links it).
 *
 * The GPU build (physim_gb300/csrc/bh.cu) quantises f64 positions to Morton
 * keys, sorts them with a stable radix sort and builds a level-by-level,
 * non-path-compressed tree.  This file does the same steps with the same f64
 * operations, sequentially, so keys, sort order and tree topology (node body
 * ranges, children, levels, geometric centres) can be compared bit for bit.
 *
 * The octant rule and centre arithmetic are the reference's
 * (astro/src/octree.rs:160-215, astro/src/quadtree.rs:161-194); the root box
 * is centred at the origin with half-width X = max |coordinate|
 * (astro/src/transformers.rs:126-132).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct BhEntity {
    double x, y, z, vx, vy, vz, radius, mass;
    uintptr_t id;
    _Bool fixed;
} BhEntity;

static int levels(int nchild) { return nchild == 8 ? 21 : 31; }
static int bits(int nchild) { return nchild == 8 ? 3 : 2; }

static uint32_t axis_cell(double p, double X, double scale, int D)
{
    const double lim = (double)((1u << D) - 1u);
    double u = (p + X) * scale;
    double r = rint(u);
    const double margin = ldexp(1.0, D - 40);
    if (fabs(u - r) >= margin || !(u == u)) {
        double q = ceil(u) - 1.0;
        q = fmin(fmax(q, 0.0), lim);
        return (uint32_t)q;
    }
    double c = 0.0, ext = X;
    uint32_t q = 0;
    for (int d = 0; d < D; ++d) {
        int hi = p > c;
        double h = ext / 2.0;
        c = hi ? c + h : c - h;
        ext = h;
        q = (q << 1) | (hi ? 1u : 0u);
    }
    return q;
}

static uint64_t interleave(const uint32_t *q, int nchild)
{
    const int D = levels(nchild), B = bits(nchild);
    uint64_t key = 0;
    for (int b = 0; b < D; ++b)
        for (int a = 0; a < B; ++a) key |= (uint64_t)((q[a] >> b) & 1u) << (B * b + a);
    return key;
}

double bh_model_extent(const BhEntity *s, size_t n)
{
    double m = 0.0;
    for (size_t i = 0; i < n; ++i) {
        m = fmax(m, fabs(s[i].x));
        m = fmax(m, fabs(s[i].y));
        m = fmax(m, fabs(s[i].z));
    }
    return m;
}

void bh_model_keys(const BhEntity *s, size_t n, int nchild, uint64_t *keys)
{
    const double X = bh_model_extent(s, n);
    const int D = levels(nchild);
    for (size_t i = 0; i < n; ++i) {
        if (!(X > 0.0)) {
            keys[i] = 0;
            continue;
        }
        const double scale = ldexp(1.0, D - 1) / X;
        uint32_t q[3] = {axis_cell(s[i].x, X, scale, D), axis_cell(s[i].y, X, scale, D),
                         axis_cell(s[i].z, X, scale, D)};
        keys[i] = interleave(q, nchild);
    }
}

/* Stable LSD radix sort of (key, index) by key. */
static void stable_sort(uint64_t *keys, uint32_t *order, size_t n, int key_bits)
{
    uint64_t *k2 = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    uint32_t *o2 = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (int shift = 0; shift < key_bits; shift += 8) {
        size_t cnt[257] = {0};
        for (size_t i = 0; i < n; ++i) cnt[((keys[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (size_t i = 0; i < n; ++i) {
            size_t p = cnt[(keys[i] >> shift) & 255u]++;
            k2[p] = keys[i];
            o2[p] = order[i];
        }
        memcpy(keys, k2, n * sizeof(uint64_t));
        memcpy(order, o2, n * sizeof(uint32_t));
    }
    free(k2);
    free(o2);
}

/* Builds the model tree.  keys/order: [n]; node arrays: [cap]; centre: 4
 * planes of length cap (cx, cy, cz, half-width).  Returns the node count, or
 * -1 if cap is too small. */
long bh_model_build(const BhEntity *s, size_t n, int nchild, int leaf, uint64_t *keys,
                    uint32_t *order, int32_t *nbegin, int32_t *ncount, int32_t *nchildidx,
                    uint8_t *nnchild, uint8_t *nlevel, double *centre, size_t cap)
{
    const int D = levels(nchild), B = bits(nchild);
    bh_model_keys(s, n, nchild, keys);
    for (size_t i = 0; i < n; ++i) order[i] = (uint32_t)i;
    stable_sort(keys, order, n, D * B);
    if (n == 0) return 0;
    if (cap < 1) return -1;
    const double X = bh_model_extent(s, n);
    size_t total = 1;
    nbegin[0] = 0;
    ncount[0] = (int32_t)n;
    nchildidx[0] = -1;
    nnchild[0] = 0;
    nlevel[0] = 0;
    centre[0] = centre[cap] = centre[2 * cap] = 0.0;
    centre[3 * cap] = X;
    size_t lvl_begin = 0, lvl_end = 1;
    for (int level = 0; level < D && lvl_begin < lvl_end; ++level) {
        const int shift = B * (D - level - 1);
        const uint32_t mask = (uint32_t)nchild - 1u;
        for (size_t node = lvl_begin; node < lvl_end; ++node) {
            const int32_t b = nbegin[node], c = ncount[node];
            if (!(c > leaf && keys[b] != keys[b + c - 1])) continue;
            int32_t bounds[9];
            int32_t j = b;
            for (int q = 0; q < nchild; ++q) {
                bounds[q] = j;
                while (j < b + c && ((keys[j] >> shift) & mask) == (uint32_t)q) ++j;
            }
            bounds[nchild] = b + c;
            const double h = centre[3 * cap + node] / 2.0;
            int nc = 0;
            for (int q = 0; q < nchild; ++q) {
                if (bounds[q + 1] <= bounds[q]) continue;
                if (total >= cap) return -1;
                size_t ci = total++;
                if (nc == 0) nchildidx[node] = (int32_t)ci;
                ++nc;
                nbegin[ci] = bounds[q];
                ncount[ci] = bounds[q + 1] - bounds[q];
                nchildidx[ci] = -1;
                nnchild[ci] = 0;
                nlevel[ci] = (uint8_t)(level + 1);
                centre[ci] = (q & 1) ? centre[node] + h : centre[node] - h;
                centre[cap + ci] = (q & 2) ? centre[cap + node] + h : centre[cap + node] - h;
                centre[2 * cap + ci] =
                    nchild == 8 ? ((q & 4) ? centre[2 * cap + node] + h : centre[2 * cap + node] - h)
                                : centre[2 * cap + node];
                centre[3 * cap + ci] = h;
            }
            nnchild[node] = (uint8_t)nc;
        }
        lvl_begin = lvl_end;
        lvl_end = total;
    }
    return (long)total;
}
