/*
 * physim_oracle.c -- CPU restatement of physim's gravity + integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file.  It is what the CUDA path's results are compared against
 * (tests/, __graft_entry__.smoke(), and bench.py's CPU-baseline leg).
 *
 * Every function restates the reference algorithm in plain C with f64
 * arithmetic, in the reference's operation order, so that the results are the
 * ones physim computes on the same input arrays:
 *
 *   law             astro/src/lib.rs:84-113   (Star::newtons_law_of_universal_gravitation)
 *   centre_of_mass  astro/src/lib.rs:40-50
 *   fake            astro/src/lib.rs:64-76    (panics on a NaN x -> reported as status 2)
 *   tree push       astro/src/octree.rs:59-128, astro/src/quadtree.rs:59-128
 *   traversal       astro/src/octree.rs:130-158, astro/src/quadtree.rs:130-159
 *   octant ids      astro/src/octree.rs:160-215, astro/src/quadtree.rs:161-194
 *   astro2          astro/src/transformers.rs:122-160
 *   astro           astro/src/transformers.rs:31-69
 *   simple_astro    astro/src/transformers.rs:219-244
 *   verlet          integrators/src/verlet.rs:24-107
 *   euler           integrators/src/euler.rs:17-49
 *   rk4             integrators/src/rk4.rs:24-178
 *   cube, plummer   astro/src/initialisers.rs:81-106, :286-330 (own variates)
 *   pipeline step   physim-core/src/pipeline.rs:137-141,166-173
 *
 * Parity status: the reference is Rust and cannot be built here, and its own
 * tests hold no force, acceleration or trajectory values.  The tree structure
 * is pinned by the reference's leaf-count tests (ported in tests/); the force
 * arithmetic is pinned only by analytic known-answer cases derived from the
 * formula in astro/src/lib.rs:84-113.  Force/trajectory parity with the Rust
 * binary itself is therefore "parity unpinned".
 *
 * Notes on restating Rust f64 arithmetic in C:
 *   - x.powi(2) is x*x (LLVM lowers powi with exponent 2 to one multiply).
 *   - x.powf(0.5) is evaluated as sqrt(x); LLVM rewrites pow(x, 0.5) to sqrt
 *     for the finite non-negative arguments that occur here.
 *   - Rust does not contract a*b+c into an FMA, so this file must be compiled
 *     with -ffp-contract=off (the build recipe does so).
 *   - f64::max ignores a NaN operand, as C's fmax does.
 */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* physim-core/src/lib.rs:16-29, c_plugin/physim.h:37-48 (80 bytes). */
typedef struct Entity {
    double x, y, z, vx, vy, vz, radius, mass;
    uintptr_t id;
    bool fixed;
} Entity;

/* physim-core/src/lib.rs:31-37 (24 bytes). */
typedef struct Acceleration {
    double x, y, z;
} Acceleration;

#define ORACLE_G 1.0 /* astro/src/lib.rs:27 */

int oracle_sizeof_entity(void) { return (int)sizeof(Entity); }
int oracle_sizeof_acceleration(void) { return (int)sizeof(Acceleration); }

/* astro/src/lib.rs:84-113.  a = self, b = other, e = easing factor. */
void oracle_law(const Entity *a, const Entity *b, double e, double out[3])
{
    double ac0 = a->x, ac1 = a->y, ac2 = a->z;
    double bc0 = b->x, bc1 = b->y, bc2 = b->z;
    double d0 = ac0 - bc0, d1 = ac1 - bc1, d2 = ac2 - bc2;
    double r_norm = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    double r_easing = d0 * d0 + d1 * d1 + d2 * d2 + e;
    double r0 = (bc0 - ac0) / r_norm;
    double r1 = (bc1 - ac1) / r_norm;
    double r2 = (bc2 - ac2) / r_norm;
    double am = a->mass, bm = b->mass;
    out[0] = r0 * ORACLE_G * am * bm / r_easing;
    out[1] = r1 * ORACLE_G * am * bm / r_easing;
    out[2] = r2 * ORACLE_G * am * bm / r_easing;
}

/* astro/src/lib.rs:40-50 */
static void centre_of_mass(const Entity *self, const Entity *other, double out[3])
{
    double total_mass = self->mass + other->mass;
    double inv_total_mass = 1.0 / total_mass;
    out[0] = (self->mass * self->x + other->mass * other->x) * inv_total_mass;
    out[1] = (self->mass * self->y + other->mass * other->y) * inv_total_mass;
    out[2] = (self->mass * self->z + other->mass * other->z) * inv_total_mass;
}

/* astro/src/lib.rs:64-76.  Returns 0, or 2 where the reference panics. */
static int fake(const double c[3], double mass, Entity *out)
{
    if (isnan(c[0])) return 2;
    memset(out, 0, sizeof *out);
    out->x = c[0];
    out->y = c[1];
    out->z = c[2];
    out->radius = 0.0;
    out->mass = mass;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Pointer octree / quadtree in an index arena (astro/src/octree.rs,        */
/* astro/src/quadtree.rs).  `nchild` is 8 for the octree, 4 for the quadtree. */
/* ------------------------------------------------------------------------ */
typedef struct Node {
    double centre[3];
    double extent;
    int has_entity;
    Entity entity;
    int32_t child[8];
} Node;

typedef struct Tree {
    int nchild;
    Node *nodes;
    size_t len, cap;
} Tree;

static int32_t tree_new_node(Tree *t, const double c[3], double extent)
{
    if (t->len == t->cap) {
        size_t cap = t->cap ? t->cap * 2 : 64;
        Node *p = (Node *)realloc(t->nodes, cap * sizeof(Node));
        if (!p) return -1;
        t->nodes = p;
        t->cap = cap;
    }
    Node *n = &t->nodes[t->len];
    memset(n, 0, sizeof *n);
    n->centre[0] = c[0];
    n->centre[1] = c[1];
    n->centre[2] = c[2];
    n->extent = extent;
    for (int i = 0; i < 8; ++i) n->child[i] = -1;
    return (int32_t)t->len++;
}

Tree *oracle_tree_new(int nchild, const double centre[3], double extent)
{
    if (nchild != 8 && nchild != 4) return NULL;
    Tree *t = (Tree *)calloc(1, sizeof(Tree));
    if (!t) return NULL;
    t->nchild = nchild;
    if (tree_new_node(t, centre, extent) != 0) {
        free(t);
        return NULL;
    }
    return t;
}

void oracle_tree_free(Tree *t)
{
    if (!t) return;
    free(t->nodes);
    free(t);
}

size_t oracle_tree_node_count(const Tree *t) { return t->len; }

/* Node geometry of the arena (centre x,y,z and half-width per node, and the
 * number of children), for comparing tree topologies.  Returns the count. */
size_t oracle_tree_dump(const Tree *t, double *geom4, int32_t *nchildren, size_t cap)
{
    for (size_t i = 0; i < t->len && i < cap; ++i) {
        const Node *n = &t->nodes[i];
        geom4[4 * i + 0] = n->centre[0];
        geom4[4 * i + 1] = n->centre[1];
        geom4[4 * i + 2] = n->centre[2];
        geom4[4 * i + 3] = n->extent;
        int k = 0;
        for (int c = 0; c < t->nchild; ++c) k += n->child[c] >= 0;
        nchildren[i] = k;
    }
    return t->len;
}

static int node_is_leaf(const Tree *t, const Node *n)
{
    for (int i = 0; i < t->nchild; ++i)
        if (n->child[i] >= 0) return 0;
    return 1;
}

/* octree.rs:160-165 / quadtree.rs:161-165 */
static int octant_id(const Tree *t, const Node *n, const double p[3])
{
    int xb = p[0] > n->centre[0];
    int yb = p[1] > n->centre[1];
    if (t->nchild == 4) return xb | (yb << 1);
    int zb = p[2] > n->centre[2];
    return xb | (yb << 1) | (zb << 2);
}

/* octree.rs:167-215 / quadtree.rs:167-194 */
static void octant_centre(const Tree *t, const Node *n, const double p[3], double out[3])
{
    int id = octant_id(t, n, p);
    double h = n->extent / 2.0;
    out[0] = (id & 1) ? n->centre[0] + h : n->centre[0] - h;
    out[1] = (id & 2) ? n->centre[1] + h : n->centre[1] - h;
    if (t->nchild == 4)
        out[2] = n->centre[2];
    else
        out[2] = (id & 4) ? n->centre[2] + h : n->centre[2] - h;
}

/* octree.rs:59-128 (same body in quadtree.rs).  Returns 0 on success,
 * 1 where the reference panics with "Recursion too deep", 2 where it panics
 * in fake() on a NaN centre of mass, -1 on allocation failure. */
int oracle_tree_push(Tree *t, const Entity *item_in)
{
    Entity item = *item_in;
    int32_t ni = 0;
    for (int count = 0;; ++count) {
        if (count > 64) return 1;
        Node *node = &t->nodes[ni];
        if (!node->has_entity) {
            node->entity = item;
            node->has_entity = 1;
            return 0;
        }
        Entity current = node->entity;
        int leaf = node_is_leaf(t, node);
        if (leaf && fabs(current.x - item.x) < 1e-9 && fabs(current.y - item.y) < 1e-9 &&
            fabs(current.z - item.z) < 1e-9) {
            double c[3] = {item.x, item.y, item.z};
            Entity f;
            if (fake(c, current.mass + item.mass, &f)) return 2;
            node->entity = f;
            return 0;
        }
        double com[3];
        centre_of_mass(&current, &item, com);
        Entity f;
        if (fake(com, current.mass + item.mass, &f)) return 2;
        node->entity = f;
        if (leaf) {
            double pc[3] = {current.x, current.y, current.z};
            int idx = octant_id(t, node, pc);
            double cc[3];
            octant_centre(t, node, pc, cc);
            double ext = node->extent / 2.0;
            int32_t c = tree_new_node(t, cc, ext);
            if (c < 0) return -1;
            node = &t->nodes[ni]; /* realloc may move the arena */
            t->nodes[c].entity = current;
            t->nodes[c].has_entity = 1;
            node->child[idx] = c;
        }
        double ip[3] = {item.x, item.y, item.z};
        int idx = octant_id(t, node, ip);
        if (node->child[idx] >= 0) {
            ni = node->child[idx];
            continue;
        }
        double cc[3];
        octant_centre(t, node, ip, cc);
        double ext = node->extent / 2.0;
        int32_t c = tree_new_node(t, cc, ext);
        if (c < 0) return -1;
        node = &t->nodes[ni];
        t->nodes[c].entity = item;
        t->nodes[c].has_entity = 1;
        node->child[idx] = c;
        return 0;
    }
}

/* octree.rs:130-158.  Writes at most `cap` entities to `out` (may be NULL)
 * and returns the full length of the list. */
size_t oracle_tree_leaves(const Tree *t, const double loc[3], double theta, Entity *out, size_t cap)
{
    size_t n_out = 0;
    size_t sp = 0, scap = 256;
    int32_t *stack = (int32_t *)malloc(scap * sizeof(int32_t));
    stack[sp++] = 0;
    while (sp > 0) {
        const Node *node = &t->nodes[stack[--sp]];
        if (node->has_entity) {
            double d0 = loc[0] - node->centre[0];
            double d1 = loc[1] - node->centre[1];
            double d2 = loc[2] - node->centre[2];
            double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            if (node->extent / r < theta) {
                if (out && n_out < cap) out[n_out] = node->entity;
                ++n_out;
                continue;
            }
        }
        if (!node->has_entity) continue;
        if (node_is_leaf(t, node)) {
            if (out && n_out < cap) out[n_out] = node->entity;
            ++n_out;
        } else {
            for (int i = 0; i < t->nchild; ++i) {
                if (node->child[i] < 0) continue;
                if (sp == scap) {
                    scap *= 2;
                    stack = (int32_t *)realloc(stack, scap * sizeof(int32_t));
                }
                stack[sp++] = node->child[i];
            }
        }
    }
    free(stack);
    return n_out;
}

/* The per-body force loop shared by astro / astro2 (transformers.rs:138-159)
 * and simple_astro (transformers.rs:224-243). */
static void accumulate_list(const Entity *a, const Entity *list, size_t len, double e, Acceleration *acc)
{
    double f[3] = {0.0, 0.0, 0.0};
    for (size_t k = 0; k < len; ++k) {
        const Entity *b = &list[k];
        if (a->x == b->x && a->y == b->y && a->z == b->z) continue;
        double fij[3];
        oracle_law(a, b, e, fij);
        f[0] += fij[0];
        f[1] += fij[1];
        f[2] += fij[2];
    }
    acc->x += f[0] / a->mass;
    acc->y += f[1] / a->mass;
    acc->z += f[2] / a->mass;
}

/* transformers.rs:219-244 (simple_astro).  `+=` into acc. */
void oracle_simple_astro(const Entity *state, size_t n, double e, Acceleration *acc)
{
    for (size_t i = 0; i < n; ++i) {
        if (state[i].fixed) continue;
        accumulate_list(&state[i], state, n, e, &acc[i]);
    }
}

/* simple_astro restricted to the bodies listed in idx (a sample), with the
 * per-body loop spread over OpenMP threads (`threads` <= 0: all).  Each body's
 * sum is the same serial sum as oracle_simple_astro, so results are identical.
 * acc_out[k] receives (not accumulates) body idx[k]'s acceleration. */
void oracle_simple_astro_sample(const Entity *state, size_t n, double e, const int64_t *idx,
                                size_t n_idx, Acceleration *acc_out, int threads)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (long k = 0; k < (long)n_idx; ++k) {
        Acceleration a = {0.0, 0.0, 0.0};
        const Entity *s = &state[idx[k]];
        if (!s->fixed) accumulate_list(s, state, n, e, &a);
        acc_out[k] = a;
    }
    (void)threads;
}

static double state_extent(const Entity *state, size_t n)
{
    /* transformers.rs:126-131: max over |x|,|y|,|z|, 1.0 for an empty state. */
    if (n == 0) return 1.0;
    double m = fabs(state[0].x);
    for (size_t i = 0; i < n; ++i) {
        if (i > 0) m = fmax(m, fabs(state[i].x));
        m = fmax(m, fabs(state[i].y));
        m = fmax(m, fabs(state[i].z));
    }
    return m;
}

double oracle_state_extent(const Entity *state, size_t n) { return state_extent(state, n); }

/* astro2 (nchild 8, transformers.rs:122-160) and astro (nchild 4,
 * transformers.rs:31-69), restricted to the bodies in idx (NULL: all bodies,
 * accumulated with `+=` into acc[i]; else acc[k] += for body idx[k]).
 * Returns 0 or the tree's panic status. */
int oracle_barnes_hut(int nchild, const Entity *state, size_t n, double theta, double e,
                      const int64_t *idx, size_t n_idx, Acceleration *acc, int threads)
{
    double extent = state_extent(state, n);
    double c0[3] = {0.0, 0.0, 0.0};
    Tree *t = oracle_tree_new(nchild, c0, 1.0 * extent);
    if (!t) return -1;
    for (size_t i = 0; i < n; ++i) {
        int st = oracle_tree_push(t, &state[i]);
        if (st) {
            oracle_tree_free(t);
            return st;
        }
    }
    size_t count = idx ? n_idx : n;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
    {
        size_t cap = 1024;
        Entity *list = (Entity *)malloc(cap * sizeof(Entity));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (long k = 0; k < (long)count; ++k) {
            size_t i = idx ? (size_t)idx[k] : (size_t)k;
            const Entity *a = &state[i];
            if (a->fixed) continue;
            double loc[3] = {a->x, a->y, a->z};
            size_t len = oracle_tree_leaves(t, loc, theta, list, cap);
            if (len > cap) {
                while (cap < len) cap *= 2;
                list = (Entity *)realloc(list, cap * sizeof(Entity));
                len = oracle_tree_leaves(t, loc, theta, list, cap);
            }
            accumulate_list(a, list, len, e, &acc[idx ? (size_t)k : i]);
        }
        free(list);
    }
    (void)threads;
    oracle_tree_free(t);
    return 0;
}

int oracle_astro2(const Entity *state, size_t n, double theta, double e, Acceleration *acc)
{
    return oracle_barnes_hut(8, state, n, theta, e, NULL, 0, acc, 1);
}

int oracle_astro(const Entity *state, size_t n, double theta, double e, Acceleration *acc)
{
    return oracle_barnes_hut(4, state, n, theta, e, NULL, 0, acc, 1);
}

/* ------------------------------------------------------------------------ */
/* Verlet (integrators/src/verlet.rs:19-107).                                */
/* ------------------------------------------------------------------------ */
typedef struct Verlet {
    Entity *previous_state;
    size_t len;
} Verlet;

Verlet *oracle_verlet_new(void) { return (Verlet *)calloc(1, sizeof(Verlet)); }

void oracle_verlet_free(Verlet *v)
{
    if (!v) return;
    free(v->previous_state);
    free(v);
}

static void verlet_store_previous(Verlet *v, const Entity *entities, size_t n)
{
    if (v->len != n) {
        free(v->previous_state);
        v->previous_state = (Entity *)malloc((n ? n : 1) * sizeof(Entity));
        v->len = n;
    }
    memcpy(v->previous_state, entities, n * sizeof(Entity));
}

/* verlet.rs:85-107 with the accelerations already evaluated by acc_fn.
 * Returns 1 when the Taylor first step (initial_integration) was taken. */
int oracle_verlet_step(Verlet *v, const Entity *entities, Entity *new_state, size_t n,
                       const Acceleration *a, double dt)
{
    double dt2 = dt * dt;
    if (v->len != n) {
        /* verlet.rs:24-50 (previous_state is stored first) */
        verlet_store_previous(v, entities, n);
        for (size_t i = 0; i < n; ++i) {
            const Entity *en = &entities[i];
            double x = en->x + en->vx * dt + 0.5 * a[i].x * dt2;
            double y = en->y + en->vy * dt + 0.5 * a[i].y * dt2;
            double z = en->z + en->vz * dt + 0.5 * a[i].z * dt2;
            double vx = en->vx + a[i].x * dt;
            double vy = en->vy + a[i].y * dt;
            double vz = en->vz + a[i].z * dt;
            Entity ne = *en;
            ne.x = x; ne.y = y; ne.z = z;
            ne.vx = vx; ne.vy = vy; ne.vz = vz;
            new_state[i] = ne;
        }
        return 1;
    }
    /* verlet.rs:52-82 */
    for (size_t i = 0; i < n; ++i) {
        const Entity *en = &entities[i];
        const Entity *prev = &v->previous_state[i];
        double x = 2.0 * en->x - prev->x + a[i].x * dt2;
        double y = 2.0 * en->y - prev->y + a[i].y * dt2;
        double z = 2.0 * en->z - prev->z + a[i].z * dt2;
        double vx = (x - en->x) / dt;
        double vy = (y - en->y) / dt;
        double vz = (z - en->z) / dt;
        Entity ne = *en;
        ne.x = x; ne.y = y; ne.z = z;
        ne.vx = vx; ne.vy = vy; ne.vz = vz;
        new_state[i] = ne;
    }
    verlet_store_previous(v, entities, n);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Euler (integrators/src/euler.rs:17-49): one acc_fn call, the Taylor step  */
/* x + v dt + 0.5 a dt^2, v + a dt for every body (fixed ones included).     */
/* ------------------------------------------------------------------------ */
void oracle_euler_step(const Entity *entities, Entity *new_state, size_t n, const Acceleration *a,
                       double dt)
{
    double dt2 = dt * dt; /* dt.powi(2) */
    for (size_t i = 0; i < n; ++i) {
        const Entity *en = &entities[i];
        Entity ne = *en;
        ne.x = en->x + en->vx * dt + 0.5 * a[i].x * dt2;
        ne.y = en->y + en->vy * dt + 0.5 * a[i].y * dt2;
        ne.z = en->z + en->vz * dt + 0.5 * a[i].z * dt2;
        ne.vx = en->vx + a[i].x * dt;
        ne.vy = en->vy + a[i].y * dt;
        ne.vz = en->vz + a[i].z * dt;
        new_state[i] = ne;
    }
}

/* ------------------------------------------------------------------------ */
/* RK4 (integrators/src/rk4.rs:24-178): four acc_fn calls per step, at the   */
/* state, at state + k1/2, at state + k2/2 and at state + k3, where          */
/* k = (dt v, dt a) of the stage state.  The combination is evaluated left   */
/* to right, (k1 + 2 k2 + 2 k3 + k4) / 6, as the reference writes it; fixed  */
/* bodies keep their position and get zero velocity (rk4.rs:165-171).       */
/* acc_fn receives zeroed accelerations (rk4.rs:33,57,82,108).               */
/* ------------------------------------------------------------------------ */
typedef void (*oracle_acc_fn)(void *user, const Entity *state, size_t n, Acceleration *acc);

typedef struct Stage6 {
    double x, y, z, vx, vy, vz;
} Stage6;

/* k of a stage state and its accelerations (rk4.rs:36-47 and the later copies) */
static void rk4_k(const Entity *t, const Acceleration *f, size_t n, double dt, Stage6 *k)
{
    for (size_t i = 0; i < n; ++i) {
        k[i].x = dt * t[i].vx;
        k[i].y = dt * t[i].vy;
        k[i].z = dt * t[i].vz;
        k[i].vx = dt * f[i].x;
        k[i].vy = dt * f[i].y;
        k[i].vz = dt * f[i].z;
    }
}

/* the next stage state: entities + c k (rk4.rs:50-62, c = 0.5 or 1) */
static void rk4_shift(const Entity *e, const Stage6 *k, size_t n, int half, Entity *t)
{
    for (size_t i = 0; i < n; ++i) {
        t[i] = e[i];
        if (half) {
            t[i].x = e[i].x + 0.5 * k[i].x;
            t[i].y = e[i].y + 0.5 * k[i].y;
            t[i].z = e[i].z + 0.5 * k[i].z;
            t[i].vx = e[i].vx + 0.5 * k[i].vx;
            t[i].vy = e[i].vy + 0.5 * k[i].vy;
            t[i].vz = e[i].vz + 0.5 * k[i].vz;
        } else {
            t[i].x = e[i].x + k[i].x;
            t[i].y = e[i].y + k[i].y;
            t[i].z = e[i].z + k[i].z;
            t[i].vx = e[i].vx + k[i].vx;
            t[i].vy = e[i].vy + k[i].vy;
            t[i].vz = e[i].vz + k[i].vz;
        }
    }
}

int oracle_rk4_step(const Entity *entities, Entity *new_state, size_t n, oracle_acc_fn acc_fn,
                    void *user, double dt)
{
    size_t m = n ? n : 1;
    Acceleration *f = (Acceleration *)calloc(m, sizeof(Acceleration));
    Entity *t = (Entity *)malloc(m * sizeof(Entity));
    Stage6 *k1 = (Stage6 *)malloc(m * sizeof(Stage6));
    Stage6 *k2 = (Stage6 *)malloc(m * sizeof(Stage6));
    Stage6 *k3 = (Stage6 *)malloc(m * sizeof(Stage6));
    Stage6 *k4 = (Stage6 *)malloc(m * sizeof(Stage6));
    if (!f || !t || !k1 || !k2 || !k3 || !k4) {
        free(f); free(t); free(k1); free(k2); free(k3); free(k4);
        return 1;
    }
    acc_fn(user, entities, n, f);
    rk4_k(entities, f, n, dt, k1);
    rk4_shift(entities, k1, n, 1, t);
    memset(f, 0, m * sizeof(Acceleration));
    acc_fn(user, t, n, f);
    rk4_k(t, f, n, dt, k2);
    rk4_shift(entities, k2, n, 1, t);
    memset(f, 0, m * sizeof(Acceleration));
    acc_fn(user, t, n, f);
    rk4_k(t, f, n, dt, k3);
    rk4_shift(entities, k3, n, 0, t);
    memset(f, 0, m * sizeof(Acceleration));
    acc_fn(user, t, n, f);
    rk4_k(t, f, n, dt, k4);
    for (size_t i = 0; i < n; ++i) {
        const Entity *e = &entities[i];
        Entity *ns = &new_state[i];
        if (!e->fixed) {
            ns->x = e->x + (k1[i].x + 2.0 * k2[i].x + 2.0 * k3[i].x + k4[i].x) / 6.0;
            ns->y = e->y + (k1[i].y + 2.0 * k2[i].y + 2.0 * k3[i].y + k4[i].y) / 6.0;
            ns->z = e->z + (k1[i].z + 2.0 * k2[i].z + 2.0 * k3[i].z + k4[i].z) / 6.0;
            ns->vx = e->vx + (k1[i].vx + 2.0 * k2[i].vx + 2.0 * k3[i].vx + k4[i].vx) / 6.0;
            ns->vy = e->vy + (k1[i].vy + 2.0 * k2[i].vy + 2.0 * k3[i].vy + k4[i].vy) / 6.0;
            ns->vz = e->vz + (k1[i].vz + 2.0 * k2[i].vz + 2.0 * k3[i].vz + k4[i].vz) / 6.0;
        } else {
            ns->x = e->x;
            ns->y = e->y;
            ns->z = e->z;
            ns->vx = 0.0;
            ns->vy = 0.0;
            ns->vz = 0.0;
        }
        ns->mass = e->mass;
        ns->radius = e->radius;
        ns->id = e->id;
        ns->fixed = e->fixed;
    }
    free(f); free(t); free(k1); free(k2); free(k3); free(k4);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Pipeline loop (pipeline.rs:137-141,166-173) with one gravity transform    */
/* and one integrator.  element: 0 simple_astro, 1 astro2, 2 astro;          */
/* integrator: 0 verlet, 1 euler, 2 rk4.  state is advanced in place by      */
/* `steps` steps.  Returns 0 or a panic status.                              */
/* ------------------------------------------------------------------------ */
typedef struct GravityFn {
    int element;
    double theta, e;
    int threads;
    const int64_t *all;
    int status;
} GravityFn;

/* transform_fn (pipeline.rs:137-141) with the single gravity element */
static void gravity_acc(void *user, const Entity *state, size_t n, Acceleration *acc)
{
    GravityFn *g = (GravityFn *)user;
    if (g->status) return;
    if (g->element == 0)
        oracle_simple_astro_sample(state, n, g->e, g->all, n, acc, g->threads);
    else
        g->status = oracle_barnes_hut(g->element == 1 ? 8 : 4, state, n, g->theta, g->e, NULL, 0,
                                      acc, g->threads);
}

int oracle_run_pipeline_with(Entity *state, size_t n, int element, int integrator, double theta,
                             double e, double dt, int steps, int threads)
{
    Verlet *v = oracle_verlet_new();
    Entity *new_state = (Entity *)malloc((n ? n : 1) * sizeof(Entity));
    Acceleration *acc = (Acceleration *)malloc((n ? n : 1) * sizeof(Acceleration));
    int64_t *all = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
    for (size_t i = 0; i < n; ++i) all[i] = (int64_t)i;
    GravityFn g = {element, theta, e, threads, all, 0};
    for (int s = 0; s < steps && g.status == 0; ++s) {
        if (integrator == 2) {
            if (oracle_rk4_step(state, new_state, n, gravity_acc, &g, dt)) g.status = 1;
        } else {
            memset(acc, 0, n * sizeof(Acceleration));
            gravity_acc(&g, state, n, acc);
            if (g.status) break;
            if (integrator == 1)
                oracle_euler_step(state, new_state, n, acc, dt);
            else
                oracle_verlet_step(v, state, new_state, n, acc, dt);
        }
        if (g.status) break;
        memcpy(state, new_state, n * sizeof(Entity));
    }
    free(all);
    free(acc);
    free(new_state);
    oracle_verlet_free(v);
    return g.status;
}

int oracle_run_pipeline(Entity *state, size_t n, int element, double theta, double e, double dt,
                        int steps, int threads)
{
    return oracle_run_pipeline_with(state, n, element, 0, theta, e, dt, steps, threads);
}

/* Number of OpenMP threads the oracle library uses (1 without OpenMP). */
int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Initialisers `cube` (astro/src/initialisers.rs:81-106, with Entity::random */
/* physim-core/src/lib.rs:115-128) and `plummer` (initialisers.rs:286-330),  */
/* with the uniform variates of the GPU generator (the reference's ChaCha8    */
/* stream cannot be reproduced): variate k of body i is the SplitMix64        */
/* finaliser of seed + (3i + k + 1) * 0x9E3779B97F4A7C15, times 2^-53.        */
/* ------------------------------------------------------------------------ */
static double oracle_uniform53(uint64_t seed, uint64_t i, int k)
{
    uint64_t z = seed + (3ull * i + (uint64_t)k + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

void oracle_cube(uint64_t seed, double spin, double size, double mass, const double centre[3],
                 uint64_t id, size_t n, Entity *out)
{
    const double entity_mass = mass / (double)n;
    for (size_t i = 0; i < n; ++i) {
        Entity e;
        memset(&e, 0, sizeof e);
        e.x = -1.0 + 2.0 * oracle_uniform53(seed, i, 0); /* random_range(-1.0..1.0) */
        e.y = -1.0 + 2.0 * oracle_uniform53(seed, i, 1);
        e.z = oracle_uniform53(seed, i, 2);               /* random_range(0.0..1.0) */
        e.radius = 0.02;
        e.x *= size;
        e.y *= size;
        e.z *= size;
        e.vx = e.y * spin;
        e.vy = -e.x * spin;
        e.x += centre[0];
        e.y += centre[1];
        e.z += centre[2];
        e.mass = entity_mass;
        e.id = (uintptr_t)id;
        out[i] = e;
    }
}

void oracle_plummer(uint64_t seed, double mass, double a, double spin, const double centre[3],
                    const double v[3], uint64_t id, size_t n, Entity *out)
{
    const double PI = 3.14159265358979311600;
    const double m = mass / (double)n;
    for (size_t i = 0; i < n; ++i) {
        const double c0 = oracle_uniform53(seed, i, 0);
        const double c1 = oracle_uniform53(seed, i, 1);
        const double c2 = oracle_uniform53(seed, i, 2);
        const double r = a * sqrt(pow(c0, -2.0 / 3.0) - 1.0);
        const double theta = PI * c2;
        const double phi = 2.0 * PI * c1;
        Entity e;
        memset(&e, 0, sizeof e);
        e.x = r * sin(theta) * cos(phi) + centre[0];
        e.y = r * sin(theta) * sin(phi) + centre[1];
        e.z = r * cos(theta) + centre[2];
        e.mass = m;
        e.radius = 0.01; /* Entity::new2(x, y, z, m, 0.01) */
        const double r2 = r * r;
        const double a2 = a * a;
        const double v_phi = spin * sqrt(mass * r2 / pow(r2 + a2, 1.5));
        e.vx = -v_phi * sin(phi) + v[0];
        e.vy = v_phi * cos(phi) + v[1];
        e.vz = 0.0 + v[2];
        e.id = (uintptr_t)id;
        out[i] = e;
    }
}
