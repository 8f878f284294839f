/*
 * bh_oracle.c -- CPU restatement of the reference's single-rank `--fc tree`
 * Barnes-Hut path (YonatanGM/Barnes-Hut), in plain C11 + OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the GPU engine's parity
 * tests compare against it, `bench.py` times it as the CPU baseline, and
 * `bench.py --impl reference` runs it as the reference arm where the
 * reference's own sources are not available.  No product code path calls it.
 *
 * Pinning: every function here is checked against the reference's own
 * sources compiled unmodified into oracle/_ref/libbhref.so (see
 * oracle/Makefile) and against the golden fixtures under tests/golden/ that
 * the compiled reference produced (tests/golden/make_golden.py).
 *
 * Arithmetic is strict IEEE binary64: the Makefile compiles this file with
 * -ffp-contract=off -fno-fast-math, so every product and sum below rounds
 * exactly where the reference's (strict-IEEE-built) C++ rounds.
 *
 * Layout: positions, velocities and accelerations are AoS (x,y,z per body)
 * like the reference's Vec3 (include/body.h:4-10).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_DEPTH 21
#define ORC_STACK_MAX 256

enum { ORC_OK = 0, ORC_ERR_OOM = 3, ORC_ERR_STACK = 5 };

/* ------------------------------------------------------------------ */
/* Bounding box -- compute_local_bbox, src/bounding_box.cpp:23-44.      */
/* std::min(a,b) is (b<a)?b:a and std::max(a,b) is (a<b)?b:a, so the    */
/* first of two equal values (e.g. +0/-0) is kept, as written here.     */
/* ------------------------------------------------------------------ */
void orc_bbox(const double *pos, int64_t n, double out[6])
{
    if (n <= 0) {
        out[0] = out[1] = out[2] = INFINITY;
        out[3] = out[4] = out[5] = -INFINITY;
        return;
    }
    double lo[3] = {pos[0], pos[1], pos[2]};
    double hi[3] = {pos[0], pos[1], pos[2]};
    for (int64_t i = 1; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            double v = pos[3 * i + a];
            if (v < lo[a]) lo[a] = v;
            if (hi[a] < v) hi[a] = v;
        }
    }
    for (int a = 0; a < 3; ++a) { out[a] = lo[a]; out[3 + a] = hi[a]; }
}

/* ------------------------------------------------------------------ */
/* Morton keys -- generateMortonCodes, src/morton_keys.cpp:65-98, with  */
/* spread21/morton63 (:11-25).  The interleave is written bit by bit    */
/* here, independently of the reference's magic-mask form.              */
/* ------------------------------------------------------------------ */
uint64_t orc_spread21(uint32_t v)
{
    uint64_t r = 0;
    for (int b = 0; b < 21; ++b) r |= (uint64_t)((v >> b) & 1u) << (3 * b);
    return r;
}

uint64_t orc_morton63(uint32_t xi, uint32_t yi, uint32_t zi)
{
    return orc_spread21(xi) | (orc_spread21(yi) << 1) | (orc_spread21(zi) << 2);
}

/* mortonPrefix, src/morton_keys.cpp:28-32 */
uint64_t orc_prefix(uint64_t key, int depth)
{
    if (depth == 0) return 0;
    return key & (~0ULL << (63 - 3 * depth));
}

static double orc_norm(double v, double lo, double span)
{
    double t = (v - lo) / span;
    if (t <= 0.0) return 0.0;
    if (t >= 1.0) return nextafter(1.0, 0.0);
    return t;
}

void orc_keys(const double *pos, int64_t n, const double bb[6], uint64_t *out)
{
    double span[3];
    for (int a = 0; a < 3; ++a) span[a] = (bb[3 + a] == bb[a]) ? 1.0 : (bb[3 + a] - bb[a]);
    const double Q = 2097152.0; /* 2^21 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t c[3];
        for (int a = 0; a < 3; ++a) c[a] = (uint32_t)(orc_norm(pos[3 * i + a], bb[a], span[a]) * Q);
        out[i] = orc_morton63(c[0], c[1], c[2]);
    }
}

/* ------------------------------------------------------------------ */
/* Sort + permute -- sortBodiesByMortonKey, include/utility.h:23-52.    */
/* The reference's std::sort is not stable; keys are unique in every    */
/* input it was run on, and there any comparison sort yields the same   */
/* permutation.  Ties are broken here by original index.                */
/* ------------------------------------------------------------------ */
typedef struct { uint64_t key; int64_t idx; } orc_kidx;

static int orc_kidx_cmp(const void *a, const void *b)
{
    const orc_kidx *x = (const orc_kidx *)a, *y = (const orc_kidx *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

/* perm_out (optional): perm_out[i] = original index of the body now at i */
int orc_sort_bodies(int64_t n, uint64_t *keys, double *pos, double *mass, double *vel,
                    uint64_t *ids, int64_t *perm_out)
{
    if (n <= 0) return ORC_OK;
    orc_kidx *o = (orc_kidx *)malloc(sizeof(orc_kidx) * (size_t)n);
    double *tmp = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    if (!o || !tmp) { free(o); free(tmp); return ORC_ERR_OOM; }
    for (int64_t i = 0; i < n; ++i) { o[i].key = keys[i]; o[i].idx = i; }
    qsort(o, (size_t)n, sizeof(orc_kidx), orc_kidx_cmp);
    for (int64_t i = 0; i < n; ++i) memcpy(tmp + 3 * i, pos + 3 * o[i].idx, 24);
    memcpy(pos, tmp, 24 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) memcpy(tmp + 3 * i, vel + 3 * o[i].idx, 24);
    memcpy(vel, tmp, 24 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) tmp[i] = mass[o[i].idx];
    memcpy(mass, tmp, 8 * (size_t)n);
    uint64_t *ut = (uint64_t *)tmp;
    for (int64_t i = 0; i < n; ++i) ut[i] = ids[o[i].idx];
    memcpy(ids, ut, 8 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) keys[i] = o[i].key;
    if (perm_out)
        for (int64_t i = 0; i < n; ++i) perm_out[i] = o[i].idx;
    free(o);
    free(tmp);
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* Linear octree as a hash map keyed by (prefix, depth).                */
/* OctreeKey/OctreeKeyHash/OctreeNode: include/linear_octree.h:15-53.   */
/* Open addressing with linear probing; the key mix is the splitmix64   */
/* finaliser the reference applies to prefix ^ depth*golden.            */
/* ------------------------------------------------------------------ */
typedef struct {
    uint64_t prefix;
    int32_t depth; /* -1 = empty slot */
    int32_t pad;
    double mass, cx, cy, cz;
} orc_node;

typedef struct {
    orc_node *slot;
    uint64_t cap; /* power of two */
    uint64_t count;
} orc_tree;

static uint64_t orc_hash(uint64_t prefix, int depth)
{
    uint64_t x = prefix ^ ((uint64_t)depth * 0x9e3779b97f4a7c15ULL);
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

static int orc_tree_init(orc_tree *t, uint64_t want)
{
    uint64_t cap = 16;
    while (cap < 2 * want) cap <<= 1;
    t->slot = (orc_node *)malloc(sizeof(orc_node) * cap);
    if (!t->slot) return ORC_ERR_OOM;
    for (uint64_t i = 0; i < cap; ++i) t->slot[i].depth = -1;
    t->cap = cap;
    t->count = 0;
    return ORC_OK;
}

static orc_node *orc_tree_find(const orc_tree *t, uint64_t prefix, int depth)
{
    uint64_t m = t->cap - 1, h = orc_hash(prefix, depth) & m;
    for (;;) {
        orc_node *s = &t->slot[h];
        if (s->depth < 0) return NULL;
        if (s->depth == depth && s->prefix == prefix) return s;
        h = (h + 1) & m;
    }
}

static int orc_tree_grow(orc_tree *t);

/* operator[] of the reference's map: find, or insert a zeroed node */
static orc_node *orc_tree_get(orc_tree *t, uint64_t prefix, int depth)
{
    if (2 * (t->count + 1) > t->cap && orc_tree_grow(t) != ORC_OK) return NULL;
    uint64_t m = t->cap - 1, h = orc_hash(prefix, depth) & m;
    for (;;) {
        orc_node *s = &t->slot[h];
        if (s->depth < 0) {
            s->prefix = prefix;
            s->depth = depth;
            s->mass = s->cx = s->cy = s->cz = 0.0;
            t->count++;
            return s;
        }
        if (s->depth == depth && s->prefix == prefix) return s;
        h = (h + 1) & m;
    }
}

static int orc_tree_grow(orc_tree *t)
{
    orc_tree nt;
    if (orc_tree_init(&nt, t->cap) != ORC_OK) return ORC_ERR_OOM;
    for (uint64_t i = 0; i < t->cap; ++i) {
        orc_node *s = &t->slot[i];
        if (s->depth < 0) continue;
        uint64_t m = nt.cap - 1, h = orc_hash(s->prefix, s->depth) & m;
        while (nt.slot[h].depth >= 0) h = (h + 1) & m;
        nt.slot[h] = *s;
        nt.count++;
    }
    free(t->slot);
    *t = nt;
    return ORC_OK;
}

static int orc_u64_cmp(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

static int64_t orc_sort_unique(uint64_t *v, int64_t n)
{
    if (n <= 0) return 0;
    qsort(v, (size_t)n, sizeof(uint64_t), orc_u64_cmp);
    int64_t w = 1;
    for (int64_t i = 1; i < n; ++i)
        if (v[i] != v[w - 1]) v[w++] = v[i];
    return w;
}

/*
 * buildOctreeBottomUp, src/linear_octree.cpp:13-107, followed (merge != 0)
 * by the single-rank full-tree exchange of src/exchange.cpp:9-29, which
 * re-inserts every node into an empty map through mergeRecordsIntoTree
 * (src/linear_octree.cpp:178-204): mass' = 0 + m, com' = (0*0 + m*c)/mass',
 * and a node whose mass' is 0 is left as an all-zero node.
 */
void *orc_build_tree(int64_t n, const uint64_t *keys, const double *pos, const double *mass, int merge)
{
    orc_tree *t = (orc_tree *)calloc(1, sizeof(orc_tree));
    if (!t) return NULL;
    if (orc_tree_init(t, (uint64_t)(n > 0 ? n : 1) * 2) != ORC_OK) { free(t); return NULL; }
    if (n <= 0) return t;

    /* 1. leaves, accumulated in body order */
    uint64_t *cur = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *par = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    if (!cur || !par) goto oom;
    for (int64_t i = 0; i < n; ++i) {
        orc_node *s = orc_tree_get(t, keys[i], ORC_MAX_DEPTH);
        if (!s) goto oom;
        double m = mass[i];
        s->mass += m;
        s->cx += pos[3 * i + 0] * m;
        s->cy += pos[3 * i + 1] * m;
        s->cz += pos[3 * i + 2] * m;
        cur[i] = keys[i];
    }
    int64_t ncur = orc_sort_unique(cur, n);

    /* 2. parents level by level, children summed in octant order 0..7 */
    for (int depth = ORC_MAX_DEPTH - 1; depth >= 0 && ncur > 0; --depth) {
        for (int64_t j = 0; j < ncur; ++j) par[j] = orc_prefix(cur[j], depth);
        int64_t npar = orc_sort_unique(par, ncur);
        for (int64_t j = 0; j < npar; ++j) {
            orc_node *p = orc_tree_get(t, par[j], depth);
            if (!p) goto oom;
            uint64_t pfx = p->prefix;
            for (int oc = 0; oc < 8; ++oc) {
                uint64_t cp = pfx | ((uint64_t)oc << (63 - 3 * (depth + 1)));
                const orc_node *c = orc_tree_find(t, cp, depth + 1);
                if (!c) continue;
                p->mass += c->mass;
                p->cx += c->cx;
                p->cy += c->cy;
                p->cz += c->cz;
            }
        }
        uint64_t *sw = cur; cur = par; par = sw;
        ncur = npar;
    }

    /* 3. finalise centre of mass */
    for (uint64_t i = 0; i < t->cap; ++i) {
        orc_node *s = &t->slot[i];
        if (s->depth < 0) continue;
        if (s->mass > 0) {
            s->cx /= s->mass;
            s->cy /= s->mass;
            s->cz /= s->mass;
        }
    }

    /* 4. single-rank exchange: each record merged into a fresh node */
    if (merge) {
        for (uint64_t i = 0; i < t->cap; ++i) {
            orc_node *s = &t->slot[i];
            if (s->depth < 0) continue;
            double m0 = 0.0, c0 = 0.0;
            double m1 = s->mass;
            double tot = m0 + m1;
            if (tot == 0) {
                s->mass = s->cx = s->cy = s->cz = 0.0;
                continue;
            }
            s->cx = (m0 * c0 + m1 * s->cx) / tot;
            s->cy = (m0 * c0 + m1 * s->cy) / tot;
            s->cz = (m0 * c0 + m1 * s->cz) / tot;
            s->mass = tot;
        }
    }
    free(cur);
    free(par);
    return t;
oom:
    free(cur);
    free(par);
    free(t->slot);
    free(t);
    return NULL;
}

int64_t orc_tree_size(void *h) { return (int64_t)((orc_tree *)h)->count; }

void orc_tree_free(void *h)
{
    if (!h) return;
    free(((orc_tree *)h)->slot);
    free(h);
}

static int orc_rec_cmp(const void *a, const void *b)
{
    const orc_node *x = (const orc_node *)a, *y = (const orc_node *)b;
    if (x->depth != y->depth) return x->depth < y->depth ? -1 : 1;
    return (x->prefix > y->prefix) - (x->prefix < y->prefix);
}

/* All nodes sorted by (depth, prefix). */
int orc_tree_records(void *h, uint64_t *prefix, uint8_t *depth, double *mass, double *com)
{
    orc_tree *t = (orc_tree *)h;
    orc_node *v = (orc_node *)malloc(sizeof(orc_node) * (t->count ? t->count : 1));
    if (!v) return ORC_ERR_OOM;
    uint64_t k = 0;
    for (uint64_t i = 0; i < t->cap; ++i)
        if (t->slot[i].depth >= 0) v[k++] = t->slot[i];
    qsort(v, (size_t)k, sizeof(orc_node), orc_rec_cmp);
    for (uint64_t i = 0; i < k; ++i) {
        prefix[i] = v[i].prefix;
        depth[i] = (uint8_t)v[i].depth;
        mass[i] = v[i].mass;
        com[3 * i + 0] = v[i].cx;
        com[3 * i + 1] = v[i].cy;
        com[3 * i + 2] = v[i].cz;
    }
    free(v);
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* Traversal -- computeAccelerations, src/traversal.cpp:13-103.         */
/* Per body: DFS with an explicit stack, children pushed in octant      */
/* order 0..7 and popped LIFO; a node is skipped when absent or         */
/* massless, the body's own leaf is skipped by key equality, and a      */
/* node is accepted when it is a leaf or side(d)^2 < theta^2 r^2 with   */
/* side(d) = maxspan/2^d.  Summation order equals the reference's.      */
/* n_inter (optional): accepted interactions per body.                  */
/* ------------------------------------------------------------------ */
typedef struct {
    double theta2;
    double side2[ORC_MAX_DEPTH + 1];
    uint64_t stride[ORC_MAX_DEPTH + 1];
} orc_walk_params;

static void orc_walk_init(orc_walk_params *w, double theta, const double bb[6])
{
    w->theta2 = theta * theta;
    double dx = bb[3] - bb[0], dy = bb[4] - bb[1], dz = bb[5] - bb[2];
    double L = dx;
    if (L < dy) L = dy;
    if (L < dz) L = dz;
    for (int d = 0; d <= ORC_MAX_DEPTH; ++d) {
        double side = L / (double)(1ULL << d);
        w->side2[d] = side * side;
        w->stride[d] = 1ULL << (63 - 3 * d);
    }
}

/* One body's walk (traversal.cpp:57-101): its acceleration into a[3] and
 * its accepted interactions into *cnt_out; returns ORC_ERR_STACK when the
 * 256-entry stack would overflow. */
static int orc_walk_one(const orc_tree *t, const orc_walk_params *w, uint64_t key, const double p[3], double G,
                        double soft2, double a[3], int64_t *cnt_out)
{
    uint64_t sp[ORC_STACK_MAX];
    int sd[ORC_STACK_MAX];
    int top = 0, err = ORC_OK;
    double ax = 0.0, ay = 0.0, az = 0.0;
    int64_t cnt = 0;
    const double px = p[0], py = p[1], pz = p[2];
    sp[top] = 0;
    sd[top] = 0;
    top++;
    while (top) {
        --top;
        uint64_t pref = sp[top];
        int dep = sd[top];
        const orc_node *nd = orc_tree_find(t, pref, dep);
        if (!nd || nd->mass == 0.0) continue;
        if (dep == ORC_MAX_DEPTH && pref == key) continue;
        double ex = nd->cx - px, ey = nd->cy - py, ez = nd->cz - pz;
        double r2 = ex * ex + ey * ey + ez * ez + soft2;
        if (dep == ORC_MAX_DEPTH || w->side2[dep] < w->theta2 * r2) {
            double invR = 1.0 / sqrt(r2);
            double invR3 = invR * invR * invR;
            double s = G * nd->mass * invR3;
            ax += s * ex;
            ay += s * ey;
            az += s * ez;
            cnt++;
        } else {
            int cd = dep + 1;
            for (int oc = 0; oc < 8; ++oc) {
                uint64_t c = pref + w->stride[cd] * (uint64_t)oc;
                if (!orc_tree_find(t, c, cd)) continue;
                if (top >= ORC_STACK_MAX) {
                    err = ORC_ERR_STACK;
                    top = 0;
                    break;
                }
                sp[top] = c;
                sd[top] = cd;
                top++;
            }
        }
    }
    a[0] = ax;
    a[1] = ay;
    a[2] = az;
    *cnt_out = cnt;
    return err;
}

int orc_accelerations(void *h, int64_t n, const uint64_t *key, const double *pos, double theta,
                      double G, double soft2, const double bb[6], double *acc, int64_t *n_inter)
{
    const orc_tree *t = (const orc_tree *)h;
    orc_walk_params w;
    orc_walk_init(&w, theta, bb);
    int err = ORC_OK;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int64_t cnt;
        if (orc_walk_one(t, &w, key[i], pos + 3 * i, G, soft2, acc + 3 * i, &cnt) != ORC_OK) {
#pragma omp atomic write
            err = ORC_ERR_STACK;
        }
        if (n_inter) n_inter[i] = cnt;
    }
    return err;
}

/* The same walk for a sample of bodies: body targets[k] (an index into
 * key/pos) gives acc[3k..3k+2] and n_inter[k] (optional). */
int orc_accelerations_at(void *h, int64_t ns, const int64_t *targets, const uint64_t *key, const double *pos,
                         double theta, double G, double soft2, const double bb[6], double *acc, int64_t *n_inter)
{
    const orc_tree *t = (const orc_tree *)h;
    orc_walk_params w;
    orc_walk_init(&w, theta, bb);
    int err = ORC_OK;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t k = 0; k < ns; ++k) {
        const int64_t i = targets[k];
        int64_t cnt;
        if (orc_walk_one(t, &w, key[i], pos + 3 * i, G, soft2, acc + 3 * k, &cnt) != ORC_OK) {
#pragma omp atomic write
            err = ORC_ERR_STACK;
        }
        if (n_inter) n_inter[k] = cnt;
    }
    return err;
}

/* ------------------------------------------------------------------ */
/* createInteractionListForRank, src/exchange.cpp:117-179: the cells of */
/* a rank's tree that a remote rank (domain = `nb` boxes, 6 doubles     */
/* each) needs.  Depth-first from the root; a cell is opened when       */
/* s^2 >= theta2 * d^2 for any remote box (s the largest side of the    */
/* cell's box, getBoundingBoxForCell in src/bounding_box.cpp:55-75; d^2 */
/* min_distance_sq of :10-18) and its depth is below max_depth; it is  */
/* kept otherwise.  Children are pushed in octant order while the       */
/* 256-entry stack has room.  A failing cell at depth 21 with           */
/* max_depth > 21 has no children in the map and is dropped.  Writes up */
/* to `cap` records in visiting order; returns the count.              */
/* ------------------------------------------------------------------ */
static double orc_max2(double a, double b) { return (a < b) ? b : a; }

int64_t orc_let_export(void *h, const double *boxes, int64_t nb, const double bb[6], double theta2, int max_depth,
                       uint64_t *prefix, uint8_t *depth, double *mass, double *com, int64_t cap)
{
    const orc_tree *t = (const orc_tree *)h;
    if (t->count == 0 || nb <= 0 || !orc_tree_find(t, 0, 0)) return 0;
    const double span[3] = {bb[3] - bb[0], bb[4] - bb[1], bb[5] - bb[2]};
    uint64_t sp[ORC_STACK_MAX];
    int sd[ORC_STACK_MAX];
    int top = 0;
    int64_t out = 0;
    sp[top] = 0;
    sd[top] = 0;
    top++;
    while (top) {
        --top;
        const uint64_t pref = sp[top];
        const int dep = sd[top];
        /* the cell's box: integer coordinates from the prefix's bits */
        uint32_t ic[3] = {0, 0, 0};
        if (dep > 0) {
            const uint64_t bits = pref >> (63 - 3 * dep);
            for (int b = 0; b < dep; ++b)
                for (int a = 0; a < 3; ++a) ic[a] |= (uint32_t)((bits >> (3 * b + a)) & 1u) << b;
        }
        const double scale = 1.0 / (double)(1ULL << dep);
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const double size = span[a] / (double)(1 << dep);
            lo[a] = bb[a] + ((double)ic[a] * scale) * span[a];
            hi[a] = lo[a] + size;
        }
        double s = hi[0] - lo[0];
        s = orc_max2(s, hi[1] - lo[1]);
        s = orc_max2(s, hi[2] - lo[2]);
        const double s2 = s * s;
        int opens = 0;
        for (int64_t k = 0; k < nb && !opens; ++k) {
            const double *r = boxes + 6 * k;
            double e[3];
            for (int a = 0; a < 3; ++a) e[a] = orc_max2(0.0, orc_max2(lo[a] - r[3 + a], r[a] - hi[a]));
            const double d2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
            opens = s2 >= theta2 * d2;
        }
        if (opens && dep < max_depth) {
            if (dep >= ORC_MAX_DEPTH) continue; /* no deeper cells exist */
            const int cd = dep + 1;
            const uint64_t stride = 1ULL << (63 - 3 * cd);
            for (int oc = 0; oc < 8; ++oc) {
                const uint64_t c = pref | (uint64_t)oc * stride;
                if (orc_tree_find(t, c, cd) && top < ORC_STACK_MAX) {
                    sp[top] = c;
                    sd[top] = cd;
                    top++;
                }
            }
        } else {
            const orc_node *nd = orc_tree_find(t, pref, dep);
            if (out < cap) {
                prefix[out] = pref;
                depth[out] = (uint8_t)dep;
                mass[out] = nd->mass;
                com[3 * out] = nd->cx;
                com[3 * out + 1] = nd->cy;
                com[3 * out + 2] = nd->cz;
            }
            out++;
        }
    }
    return out;
}

/* ------------------------------------------------------------------ */
/* buildTreeFromPseudoLeaves, src/linear_octree.cpp:242-322: a map of   */
/* the given records (mass > 0 and finite; depth clamped to 21; prefix  */
/* masked to it) and all their ancestors.  A record adds m and c * m to */
/* its cell, in input order; every cell then adds its children's sums,  */
/* deepest level first; com = sum / mass where mass > 1e-12.  Children  */
/* are added in octant order here; the reference adds them in the      */
/* iteration order of its hash map, so sums over several children agree */
/* with it to rounding only.  Returns a tree handle (orc_tree_records). */
/* ------------------------------------------------------------------ */
typedef struct { uint64_t prefix; int depth; } orc_cell;

static int orc_cell_cmp(const void *a, const void *b)
{
    const orc_cell *x = (const orc_cell *)a, *y = (const orc_cell *)b;
    if (x->depth != y->depth) return (x->depth > y->depth) - (x->depth < y->depth);
    return (x->prefix > y->prefix) - (x->prefix < y->prefix);
}

void *orc_pseudo_tree(const uint64_t *prefix, const uint8_t *depth, const double *mass, const double *com, int64_t m)
{
    orc_tree *t = (orc_tree *)malloc(sizeof(orc_tree));
    if (!t || orc_tree_init(t, (uint64_t)(m > 0 ? m : 1) * 4) != ORC_OK) {
        free(t);
        return NULL;
    }
    for (int64_t k = 0; k < m; ++k) {
        const double w = mass[k];
        if (!(w > 0.0) || !isfinite(w)) continue;
        const int d = depth[k] > ORC_MAX_DEPTH ? ORC_MAX_DEPTH : depth[k];
        orc_node *nd = orc_tree_get(t, orc_prefix(prefix[k], d), d);
        if (!nd) goto fail;
        nd->mass += w;
        nd->cx += com[3 * k] * w;
        nd->cy += com[3 * k + 1] * w;
        nd->cz += com[3 * k + 2] * w;
    }
    {
        /* ancestors */
        uint64_t nrec = t->count;
        orc_cell *own = (orc_cell *)malloc(sizeof(orc_cell) * (nrec ? nrec : 1));
        if (!own) goto fail;
        uint64_t w = 0;
        for (uint64_t i = 0; i < t->cap; ++i)
            if (t->slot[i].depth >= 0) own[w++] = (orc_cell){t->slot[i].prefix, t->slot[i].depth};
        for (uint64_t i = 0; i < w; ++i)
            for (int d = own[i].depth - 1; d >= 0; --d)
                if (!orc_tree_get(t, orc_prefix(own[i].prefix, d), d)) {
                    free(own);
                    goto fail;
                }
        free(own);
        /* bottom-up sums in octant order */
        orc_cell *all = (orc_cell *)malloc(sizeof(orc_cell) * (t->count ? t->count : 1));
        if (!all) goto fail;
        w = 0;
        for (uint64_t i = 0; i < t->cap; ++i)
            if (t->slot[i].depth >= 0) all[w++] = (orc_cell){t->slot[i].prefix, t->slot[i].depth};
        qsort(all, (size_t)w, sizeof(orc_cell), orc_cell_cmp);
        for (int64_t i = (int64_t)w - 1; i >= 0; --i) {
            const int d = all[i].depth;
            if (d >= ORC_MAX_DEPTH) continue;
            orc_node *p = orc_tree_find(t, all[i].prefix, d);
            const uint64_t stride = 1ULL << (63 - 3 * (d + 1));
            for (int oc = 0; oc < 8; ++oc) {
                const orc_node *c = orc_tree_find(t, all[i].prefix | (uint64_t)oc * stride, d + 1);
                if (!c) continue;
                p->mass += c->mass;
                p->cx += c->cx;
                p->cy += c->cy;
                p->cz += c->cz;
            }
        }
        free(all);
    }
    for (uint64_t i = 0; i < t->cap; ++i) {
        orc_node *n = &t->slot[i];
        if (n->depth < 0 || !(n->mass > 1e-12)) continue;
        n->cx /= n->mass;
        n->cy /= n->mass;
        n->cz /= n->mass;
    }
    return t;
fail:
    free(t->slot);
    free(t);
    return NULL;
}

/* ------------------------------------------------------------------ */
/* computeAccelerationsWithLET, src/traversal.cpp:107-127: the records'  */
/* pseudo-leaf map (orc_pseudo_tree) merged into a copy of the local map */
/* as mergeRecordsIntoTree (src/linear_octree.cpp:178-204) merges -- a   */
/* cell in both gets com = (m0 c0 + m1 c1) / (m0 + m1), nothing when   */
/* that mass is 0; a new cell enters with m0 = c0 = 0 -- then the       */
/* ordinary traversal over the merged map.  `direct` selects            */
/* computeAccelerationsWithRemoteDirectSum (:149-221): the traversal of */
/* the local map plus, per body, the records summed in order (rm =     */
/* mass * G; pairs with r^2 <= 1e-12 skipped).                          */
/* ------------------------------------------------------------------ */
static orc_tree *orc_tree_clone(const orc_tree *t)
{
    orc_tree *c = (orc_tree *)malloc(sizeof(orc_tree));
    if (!c) return NULL;
    c->slot = (orc_node *)malloc(sizeof(orc_node) * t->cap);
    if (!c->slot) {
        free(c);
        return NULL;
    }
    memcpy(c->slot, t->slot, sizeof(orc_node) * t->cap);
    c->cap = t->cap;
    c->count = t->count;
    return c;
}

int orc_let_accelerations(void *h, const uint64_t *prefix, const uint8_t *depth, const double *mass,
                          const double *com, int64_t m, int64_t n, const uint64_t *key, const double *pos,
                          double theta, double G, double soft2, const double bb[6], int direct, double *acc)
{
    const orc_tree *local = (const orc_tree *)h;
    if (direct) {
        int rc = orc_accelerations(h, n, key, pos, theta, G, soft2, bb, acc, NULL);
        if (rc) return rc;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double ax = 0.0, ay = 0.0, az = 0.0;
            const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
            for (int64_t j = 0; j < m; ++j) {
                const double dx = com[3 * j] - px, dy = com[3 * j + 1] - py, dz = com[3 * j + 2] - pz;
                const double r2 = dx * dx + dy * dy + dz * dz + soft2;
                if (r2 <= 1e-12) continue;
                const double inv = 1.0 / sqrt(r2);
                const double inv3 = inv * inv * inv;
                const double s = (mass[j] * G) * inv3;
                ax += s * dx;
                ay += s * dy;
                az += s * dz;
            }
            acc[3 * i] += ax;
            acc[3 * i + 1] += ay;
            acc[3 * i + 2] += az;
        }
        return ORC_OK;
    }
    orc_tree *merged = orc_tree_clone(local);
    orc_tree *pt = (orc_tree *)orc_pseudo_tree(prefix, depth, mass, com, m);
    if (!merged || !pt) {
        if (merged) orc_tree_free(merged);
        if (pt) orc_tree_free(pt);
        return ORC_ERR_OOM;
    }
    for (uint64_t i = 0; i < pt->cap; ++i) {
        const orc_node *r = &pt->slot[i];
        if (r->depth < 0) continue;
        orc_node *nd = orc_tree_get(merged, r->prefix, r->depth);
        if (!nd) {
            orc_tree_free(merged);
            orc_tree_free(pt);
            return ORC_ERR_OOM;
        }
        const double m0 = nd->mass, tot = m0 + r->mass;
        if (tot == 0) continue;
        nd->cx = (m0 * nd->cx + r->mass * r->cx) / tot;
        nd->cy = (m0 * nd->cy + r->mass * r->cy) / tot;
        nd->cz = (m0 * nd->cz + r->mass * r->cz) / tot;
        nd->mass = tot;
    }
    int rc = orc_accelerations(merged, n, key, pos, theta, G, soft2, bb, acc, NULL);
    orc_tree_free(merged);
    orc_tree_free(pt);
    return rc;
}

/* ------------------------------------------------------------------ */
/* The step loop of src/main.cpp:191-282 for `--fc tree` on one rank.   */
/* The half kick at :193-200 runs only when t > 0; t is accumulated in  */
/* double (t += dt), as the reference's loop header does.  The MPI      */
/* layers are identities on one rank (global bbox = local bbox,          */
/* rebalance keeps the order) and are omitted.                          */
/* phase_s (7 doubles, accumulated): kdk, bbox, keys, sort, build,       */
/* merge (folded into build here: 0), traversal.                        */
/* ------------------------------------------------------------------ */
static double orc_now(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

int orc_simulate(int64_t n, double *pos, double *vel, double *mass, uint64_t *ids, double *acc,
                 double dt, double theta, double G, int64_t nsteps, double *t_io, double *phase_s)
{
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
    if (!keys) return ORC_ERR_OOM;
    double t = *t_io;
    int err = ORC_OK;
    const double h = 0.5 * dt;
    for (int64_t s = 0; s < nsteps && err == ORC_OK; ++s, t += dt) {
        double t0 = orc_now();
        if (t > 0) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < 3 * n; ++i) vel[i] += h * acc[i];
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < 3 * n; ++i) pos[i] += dt * vel[i];
        double t1 = orc_now();
        double bb[6];
        orc_bbox(pos, n, bb);
        double t2 = orc_now();
        orc_keys(pos, n, bb, keys);
        double t3 = orc_now();
        err = orc_sort_bodies(n, keys, pos, mass, vel, ids, NULL);
        if (err) break;
        /* acceleration follows its body through the permutation only by
         * being recomputed below; the reference's stale local_acc is
         * overwritten by computeAccelerations before it is read again. */
        double t4 = orc_now();
        void *tree = orc_build_tree(n, keys, pos, mass, 1);
        if (!tree) { err = ORC_ERR_OOM; break; }
        double t5 = orc_now();
        err = orc_accelerations(tree, n, keys, pos, theta, G, 0.0, bb, acc, NULL);
        orc_tree_free(tree);
        double t6 = orc_now();
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < 3 * n; ++i) vel[i] += h * acc[i];
        double t7 = orc_now();
        if (phase_s) {
            phase_s[0] += (t1 - t0) + (t7 - t6);
            phase_s[1] += t2 - t1;
            phase_s[2] += t3 - t2;
            phase_s[3] += t4 - t3;
            phase_s[4] += t5 - t4;
            phase_s[6] += t6 - t5;
        }
    }
    *t_io = t;
    free(keys);
    return err;
}

/* ------------------------------------------------------------------ */
/* FP64 direct sum over all sources for a sample of target bodies       */
/* (no reference counterpart; the yardstick of every force error).      */
/* Self-exclusion is by index.                                          */
/* ------------------------------------------------------------------ */
void orc_direct_sum(int64_t n, const double *pos, const double *mass, int64_t ns, const int64_t *targets,
                    double G, double *acc_out)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t k = 0; k < ns; ++k) {
        int64_t j = targets[k];
        double ax = 0.0, ay = 0.0, az = 0.0;
        const double px = pos[3 * j], py = pos[3 * j + 1], pz = pos[3 * j + 2];
        for (int64_t i = 0; i < n; ++i) {
            if (i == j) continue;
            double ex = pos[3 * i] - px, ey = pos[3 * i + 1] - py, ez = pos[3 * i + 2] - pz;
            double r2 = ex * ex + ey * ey + ez * ez;
            if (r2 == 0.0) continue;
            double invR = 1.0 / sqrt(r2);
            double s = G * mass[i] * (invR * invR * invR);
            ax += s * ex;
            ay += s * ey;
            az += s * ez;
        }
        acc_out[3 * k] = ax;
        acc_out[3 * k + 1] = ay;
        acc_out[3 * k + 2] = az;
    }
}

/* Total energy (exact pairwise potential, O(n^2): small n only), linear
 * and angular momentum.  out = {E, K, U, Lx, Ly, Lz, Px, Py, Pz}. */
void orc_invariants(int64_t n, const double *pos, const double *vel, const double *mass, double G, double out[9])
{
    double K = 0.0, U = 0.0, L[3] = {0, 0, 0}, P[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        const double *x = pos + 3 * i, *v = vel + 3 * i;
        double m = mass[i];
        K += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        L[0] += m * (x[1] * v[2] - x[2] * v[1]);
        L[1] += m * (x[2] * v[0] - x[0] * v[2]);
        L[2] += m * (x[0] * v[1] - x[1] * v[0]);
        for (int a = 0; a < 3; ++a) P[a] += m * v[a];
    }
#pragma omp parallel for reduction(+ : U) schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        double u = 0.0;
        for (int64_t j = i + 1; j < n; ++j) {
            double ex = pos[3 * j] - pos[3 * i], ey = pos[3 * j + 1] - pos[3 * i + 1],
                   ez = pos[3 * j + 2] - pos[3 * i + 2];
            double r = sqrt(ex * ex + ey * ey + ez * ez);
            if (r > 0) u -= G * mass[i] * mass[j] / r;
        }
        U += u;
    }
    out[0] = K + U;
    out[1] = K;
    out[2] = U;
    out[3] = L[0]; out[4] = L[1]; out[5] = L[2];
    out[6] = P[0]; out[7] = P[1]; out[8] = P[2];
}

/* ------------------------------------------------------------------ */
/* convertKeplerToCartesian, src/kepler_to_cartesian.cpp:13-107:        */
/* propagate M to J2000 (JD 2451544.5), Newton on Kepler's equation     */
/* (tol 1e-8, <= 100 iterations), true anomaly, perifocal state and     */
/* the 3-1-3 rotation.  el = {e, a, i, omega, Omega, M, epoch, mu}.     */
/* ------------------------------------------------------------------ */
void orc_kepler_to_cartesian(const double *el, int64_t n, double *out)
{
    for (int64_t k = 0; k < n; ++k) {
        const double *q = el + 8 * k;
        double e = q[0], a = q[1], inc = q[2], w = q[3], Om = q[4], M = q[5], epoch = q[6], mu = q[7];
        double nmot = sqrt(mu / pow(a, 3));
        M += nmot * (2451544.5 - epoch);
        M = fmod(M, 2 * M_PI);
        if (M < 0) M += 2 * M_PI;
        double E = M;
        for (int it = 0; it < 100; ++it) {
            double f = E - e * sin(E) - M;
            double fp = 1 - e * cos(E);
            double d = -f / fp;
            E += d;
            if (fabs(d) < 1e-8) break;
        }
        double nu = 2 * atan2(sqrt(1 + e) * sin(E / 2), sqrt(1 - e) * cos(E / 2));
        double r = a * (1 - e * cos(E));
        double xo = r * cos(nu), yo = r * sin(nu);
        double hh = sqrt(mu * a) / r;
        double vxo = hh * (-sin(E)), vyo = hh * sqrt(1 - e * e) * cos(E);
        double cO = cos(Om), sO = sin(Om), ci = cos(inc), si = sin(inc), cw = cos(w), sw = sin(w);
        double R11 = cO * cw - sO * sw * ci, R12 = -cO * sw - sO * cw * ci;
        double R21 = sO * cw + cO * sw * ci, R22 = -sO * sw + cO * cw * ci;
        double R31 = sw * si, R32 = cw * si;
        double *o = out + 6 * k;
        o[0] = R11 * xo + R12 * yo;
        o[1] = R21 * xo + R22 * yo;
        o[2] = R31 * xo + R32 * yo;
        o[3] = R11 * vxo + R12 * vyo;
        o[4] = R21 * vxo + R22 * vyo;
        o[5] = R31 * vxo + R32 * vyo;
    }
}

/* ------------------------------------------------------------------ */
/* The seeded synthetic solar system the configurations name (no        */
/* reference counterpart: the reference reads CSV files).  Restates the */
/* engine's generator draw for draw so the reference arm of the bench    */
/* and the tests can make the same inputs without the engine's library: */
/* the Sun at rest at the origin; the eight planets on circular          */
/* coplanar orbits (mass and a from the reference's                      */
/* data/orbital_elements_raw_csvs/planets_and_moons.csv:2-9), mean       */
/* anomaly U[0,2pi); then inner-belt, outer-belt and trojan asteroids    */
/* (a, e, i, Omega, omega, M as documented in include/bh_gpu.h), mass    */
/* log-uniform on [1e12, 1e20] kg; each converted by the Kepler          */
/* conversion above with mu = G M_sun and epoch J2000.  Uniform draws    */
/* are the top 53 bits of one mt19937_64 output (Matsumoto-Nishimura     */
/* 64-bit Mersenne Twister, seeded by its standard linear recurrence)    */
/* scaled by 2^-53.                                                     */
/* ------------------------------------------------------------------ */
typedef struct {
    uint64_t mt[312];
    int idx;
} orc_mt64;

static void orc_mt64_seed(orc_mt64 *g, uint64_t seed)
{
    g->mt[0] = seed;
    for (int i = 1; i < 312; ++i)
        g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
    g->idx = 312;
}

static uint64_t orc_mt64_next(orc_mt64 *g)
{
    if (g->idx >= 312) {
        for (int i = 0; i < 312; ++i) {
            uint64_t y = (g->mt[i] & 0xFFFFFFFF80000000ULL) | (g->mt[(i + 1) % 312] & 0x7FFFFFFFULL);
            uint64_t v = g->mt[(i + 156) % 312] ^ (y >> 1);
            if (y & 1ULL) v ^= 0xB5026F5AA96619E9ULL;
            g->mt[i] = v;
        }
        g->idx = 0;
    }
    uint64_t x = g->mt[g->idx++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= x >> 43;
    return x;
}

static double orc_u(orc_mt64 *g, double lo, double hi)
{
    double u = (double)(orc_mt64_next(g) >> 11) * (1.0 / 9007199254740992.0);
    return lo + (hi - lo) * u;
}

int orc_generate_system(uint64_t seed, int64_t n, double frac_outer, double frac_trojan, double *pos, double *vel,
                        double *mass, uint64_t *ids)
{
    static const double pm[8] = {3.301011e+23, 4.86732e+24, 5.972186e+24, 6.416928e+23,
                                 1.89813e+27, 5.683191e+26, 8.681013e+25, 1.024096e+26};
    static const double pa[8] = {0.3870982252718477, 0.723326849675607, 1.000371833994387, 1.52367818431121,
                                 5.205108585205607, 9.581451990534042, 19.22994588008584, 30.10071183142183};
    const double pi = 3.14159265358979323846, two_pi = 2.0 * pi, deg = pi / 180.0;
    const double sun = 1.989e30, mu = 1.48812e-34 * sun, j2000 = 2451544.5;
    if (n < 9 || frac_outer < 0 || frac_trojan < 0 || frac_outer + frac_trojan > 1) return 1;
    orc_mt64 *g = (orc_mt64 *)malloc(sizeof(orc_mt64));
    if (!g) return ORC_ERR_OOM;
    orc_mt64_seed(g, seed);
    const int64_t nast = n - 9;
    const int64_t n_outer = (int64_t)llround(frac_outer * (double)nast);
    const int64_t n_troj = (int64_t)llround(frac_trojan * (double)nast);
    const int64_t n_inner = nast - n_outer - n_troj;
    double q[8], st[6];
    for (int a = 0; a < 3; ++a) pos[a] = vel[a] = 0.0;
    mass[0] = sun;
    double lambda_j = 0.0;
    for (int k = 0; k < 8; ++k) {
        const double M = orc_u(g, 0.0, two_pi);
        if (k == 4) lambda_j = M;
        q[0] = 0.0; q[1] = pa[k]; q[2] = 0.0; q[3] = 0.0; q[4] = 0.0; q[5] = M; q[6] = j2000; q[7] = mu;
        orc_kepler_to_cartesian(q, 1, st);
        for (int a = 0; a < 3; ++a) { pos[3 * (1 + k) + a] = st[a]; vel[3 * (1 + k) + a] = st[3 + a]; }
        mass[1 + k] = pm[k];
    }
    const double lmin = log(1e12), lmax = log(1e20);
    for (int64_t k = 0; k < nast; ++k) {
        const int64_t b = 9 + k;
        double a, e, inc, Om, w, M;
        if (k < n_inner) {
            a = orc_u(g, 2.1, 3.3); e = orc_u(g, 0.0, 0.3); inc = orc_u(g, 0.0, 20.0) * deg;
            Om = orc_u(g, 0.0, two_pi); w = orc_u(g, 0.0, two_pi); M = orc_u(g, 0.0, two_pi);
        } else if (k < n_inner + n_outer) {
            a = orc_u(g, 30.0, 50.0); e = orc_u(g, 0.0, 0.2); inc = orc_u(g, 0.0, 30.0) * deg;
            Om = orc_u(g, 0.0, two_pi); w = orc_u(g, 0.0, two_pi); M = orc_u(g, 0.0, two_pi);
        } else {
            a = 5.2; e = orc_u(g, 0.0, 0.1); inc = orc_u(g, 0.0, 20.0) * deg;
            Om = orc_u(g, 0.0, two_pi); w = orc_u(g, 0.0, two_pi);
            const double side = ((k - n_inner - n_outer) & 1) ? -60.0 : 60.0;
            const double lam = lambda_j + (side + orc_u(g, -30.0, 30.0)) * deg;
            M = fmod(lam - Om - w, two_pi);
            if (M < 0) M += two_pi;
        }
        mass[b] = exp(orc_u(g, lmin, lmax));
        q[0] = e; q[1] = a; q[2] = inc; q[3] = w; q[4] = Om; q[5] = M; q[6] = j2000; q[7] = mu;
        orc_kepler_to_cartesian(q, 1, st);
        for (int c = 0; c < 3; ++c) { pos[3 * b + c] = st[c]; vel[3 * b + c] = st[3 + c]; }
    }
    for (int64_t i = 0; i < n; ++i) ids[i] = (uint64_t)i;
    free(g);
    return ORC_OK;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
