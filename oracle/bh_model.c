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

/* ------------------------------------------------------------------------ */
/* The accuracy options of the GPU traversal (not reference behaviour), in   */
/* f64, per body: a cell is accepted when the reference's rule               */
/* extent / |x - centre| < theta holds (astro/src/octree.rs:137-144) and,    */
/* with com_theta > 0, b_max < com_theta |x - c| with c the cell's centre of */
/* mass and b_max = sqrt(3) extent + |c - centre|.  Accepted cells add their */
/* monopole and, with quad != 0, the quadrupole term of the reference law    */
/* a = sum m d / (|d| (|d|^2 + e)) expanded about c (second moments S about  */
/* c):  a_2 = h S D + (h tr S + (h'/r) D.S.D) D / 2, D = c - x,              */
/* h = g'/r, g(r) = 1/(r (r^2 + e)).  Opened leaves add their bodies         */
/* exactly, skipping bodies at the same position.  out[k] = acceleration of  */
/* body idx[k].  Returns 0, or -1 when out of memory.                         */
/* ------------------------------------------------------------------------ */
static void model_pair(const double x[3], const double p[3], double m, double e, double a[3])
{
    const double d0 = p[0] - x[0], d1 = p[1] - x[1], d2 = p[2] - x[2];
    const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
    if (r2 == 0.0) return;
    const double f = m / (sqrt(r2) * (r2 + e));
    a[0] += d0 * f;
    a[1] += d1 * f;
    a[2] += d2 * f;
}

int bh_model_accel(const BhEntity *s, size_t n, int nchild, int leaf, double theta, double e,
                   int quad, double com_theta, const int64_t *idx, size_t n_idx, double *out)
{
    const size_t cap = 4 * (n > 64 ? n : 64) + 64 * 31;
    uint64_t *keys = malloc((n ? n : 1) * sizeof *keys);
    uint32_t *order = malloc((n ? n : 1) * sizeof *order);
    int32_t *nb = malloc(cap * sizeof *nb), *nc = malloc(cap * sizeof *nc);
    int32_t *ch = malloc(cap * sizeof *ch);
    uint8_t *nn = malloc(cap), *lvl = malloc(cap);
    double *cen = malloc(4 * cap * sizeof *cen);
    double *mom = malloc(10 * cap * sizeof *mom); /* M, cx, cy, cz, Sxx Syy Szz Sxy Sxz Syz */
    int64_t *rank = malloc((n ? n : 1) * sizeof *rank);
    int32_t *stack = malloc(cap * sizeof *stack);
    int rc = -1;
    if (!keys || !order || !nb || !nc || !ch || !nn || !lvl || !cen || !mom || !rank || !stack)
        goto done;
    long total = bh_model_build(s, n, nchild, leaf, keys, order, nb, nc, ch, nn, lvl, cen, cap);
    if (total < 0) goto done;
    for (size_t k = 0; k < n; ++k) rank[order[k]] = (int64_t)k;
    /* moments by direct summation over each node's sorted bodies */
    for (long i = 0; i < total; ++i) {
        double M = 0, c[3] = {0, 0, 0};
        for (int32_t j = nb[i]; j < nb[i] + nc[i]; ++j) {
            const BhEntity *b = &s[order[j]];
            M += b->mass;
            c[0] += b->mass * b->x;
            c[1] += b->mass * b->y;
            c[2] += b->mass * b->z;
        }
        if (M != 0.0)
            for (int a = 0; a < 3; ++a) c[a] /= M;
        else
            for (int a = 0; a < 3; ++a) c[a] = cen[a * cap + i];
        double S[6] = {0, 0, 0, 0, 0, 0};
        for (int32_t j = nb[i]; j < nb[i] + nc[i]; ++j) {
            const BhEntity *b = &s[order[j]];
            const double dx = b->x - c[0], dy = b->y - c[1], dz = b->z - c[2];
            S[0] += b->mass * dx * dx;
            S[1] += b->mass * dy * dy;
            S[2] += b->mass * dz * dz;
            S[3] += b->mass * dx * dy;
            S[4] += b->mass * dx * dz;
            S[5] += b->mass * dy * dz;
        }
        double *o = &mom[10 * i];
        o[0] = M;
        o[1] = c[0];
        o[2] = c[1];
        o[3] = c[2];
        for (int a = 0; a < 6; ++a) o[4 + a] = S[a];
    }
    for (size_t k = 0; k < n_idx; ++k) {
        const BhEntity *bi = &s[idx[k]];
        const double x[3] = {bi->x, bi->y, bi->z};
        double a[3] = {0, 0, 0};
        size_t sp = 0;
        if (n) stack[sp++] = 0;
        while (sp) {
            const int32_t i = stack[--sp];
            const double *o = &mom[10 * i];
            const double g0 = x[0] - cen[i], g1 = x[1] - cen[cap + i], g2 = x[2] - cen[2 * cap + i];
            const double r = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
            const double ext = cen[3 * cap + i];
            int accept = ext / r < theta;
            if (accept && com_theta > 0.0) {
                const double o0 = o[1] - cen[i], o1 = o[2] - cen[cap + i], o2 = o[3] - cen[2 * cap + i];
                const double bmax = sqrt(3.0) * ext + sqrt(o0 * o0 + o1 * o1 + o2 * o2);
                const double D0 = o[1] - x[0], D1 = o[2] - x[1], D2 = o[3] - x[2];
                accept = bmax < com_theta * sqrt(D0 * D0 + D1 * D1 + D2 * D2);
            }
            if (accept) {
                model_pair(x, &o[1], o[0], e, a);
                if (quad) {
                    const double D0 = o[1] - x[0], D1 = o[2] - x[1], D2 = o[3] - x[2];
                    const double r2 = D0 * D0 + D1 * D1 + D2 * D2;
                    if (r2 > 0.0) {
                        const double rr = sqrt(r2), u = rr * (r2 + e), A = 3.0 * r2 + e;
                        const double h = -A / (rr * u * u);
                        const double hp = (-6.0 / (u * u) + A * (u + 2.0 * rr * A) / (r2 * u * u * u)) / rr;
                        const double *S = &o[4];
                        const double sd0 = S[0] * D0 + S[3] * D1 + S[4] * D2;
                        const double sd1 = S[3] * D0 + S[1] * D1 + S[5] * D2;
                        const double sd2 = S[4] * D0 + S[5] * D1 + S[2] * D2;
                        const double dsd = D0 * sd0 + D1 * sd1 + D2 * sd2;
                        const double kk = 0.5 * (h * (S[0] + S[1] + S[2]) + hp * dsd);
                        a[0] += h * sd0 + kk * D0;
                        a[1] += h * sd1 + kk * D1;
                        a[2] += h * sd2 + kk * D2;
                    }
                }
            } else if (ch[i] < 0) {
                for (int32_t j = nb[i]; j < nb[i] + nc[i]; ++j) {
                    const BhEntity *b = &s[order[j]];
                    const double p[3] = {b->x, b->y, b->z};
                    model_pair(x, p, b->mass, e, a);
                }
            } else {
                for (int c = 0; c < nn[i]; ++c) stack[sp++] = ch[i] + c;
            }
        }
        out[3 * k] = a[0];
        out[3 * k + 1] = a[1];
        out[3 * k + 2] = a[2];
    }
    rc = 0;
done:
    free(keys); free(order); free(nb); free(nc); free(ch); free(nn); free(lvl);
    free(cen); free(mom); free(rank); free(stack);
    return rc;
}
