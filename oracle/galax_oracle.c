/*
 * galax_oracle.c -- CPU restatement of galax-core's FMM force path (test
 * infrastructure; see galax_oracle.h for the rules this file follows).
 *
 * Reference: knekvasil/galax, galax-core/src/lib.rs (cited as lib.rs:LINE),
 * galax-integrate/src/lib.rs and galax-cli/src/main.rs.
 *
 * Build: cc -O2 -fPIC -shared -fopenmp -ffp-contract=off (oracle/Makefile).
 */
#include "galax_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LIST_EMPTY 0xFFFFFFFFu

/* ------------------------------------------------------------------ utils */

static int g_threads = 0;
void gxo_set_threads(int n) { g_threads = n; }
int gxo_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* Rust `f64 as i64`: truncate toward zero, saturate, NaN -> 0. */
static int64_t f64_as_i64(double v) {
    if (v != v) return 0;
    if (v >= 9223372036854775808.0) return INT64_MAX;
    if (v < -9223372036854775808.0) return INT64_MIN;
    return (int64_t)v;
}

/* Rust `f64 as u64`: truncate, saturate at 0 and 2^64-1, NaN -> 0. */
static uint64_t f64_as_u64(double v) {
    if (!(v > 0.0)) return 0; /* NaN, negatives, -0 */
    if (v >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)v;
}

/* f64::min / f64::max: NaN operands are ignored. */
static double fmin_rs(double a, double b) { return (a != a) ? b : ((b != b) ? a : (b < a ? b : a)); }
static double fmax_rs(double a, double b) { return (a != a) ? b : ((b != b) ? a : (b > a ? b : a)); }

/* powi by binary exponentiation, the expansion LLVM uses for `f64::powi`. */
static double powi_rs(double a, int b) {
    int recip = b < 0;
    if (recip) b = -b;
    double r = 1.0;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return recip ? 1.0 / r : r;
}

static double g_fact[GXO_MAX_P];
static double g_binom[GXO_MAX_P][GXO_MAX_P];
static int g_tables_ready = 0;

/* cached_fact / cached_binom (lib.rs:15-39) */
static void init_tables(void) {
    if (g_tables_ready) return;
    g_fact[0] = 1.0;
    for (int i = 1; i < GXO_MAX_P; i++) g_fact[i] = g_fact[i - 1] * (double)i;
    memset(g_binom, 0, sizeof(g_binom));
    for (int n = 0; n < GXO_MAX_P; n++) {
        g_binom[n][0] = 1.0;
        g_binom[n][n] = 1.0;
        for (int k = 1; k < n; k++) g_binom[n][k] = g_binom[n - 1][k - 1] + g_binom[n - 1][k];
    }
    g_tables_ready = 1;
}

/* fill_powers (lib.rs:8-13) */
static void fill_powers(double *arr, double base, int64_t p) {
    arr[0] = 1.0;
    for (int64_t k = 1; k <= p; k++) arr[k] = arr[k - 1] * base;
}

int64_t gxo_num_moments(int64_t p) { return (p + 1) * (p + 2) / 2; }
int64_t gxo_moment_index(int64_t i, int64_t j) {
    int64_t n = i + j;
    return n * (n + 1) / 2 + j;
}
#define MI(i, j) gxo_moment_index((i), (j))

/* ---------------------------------------------------------------- Morton */

/* normalize (lib.rs:75-78) */
static uint64_t normalize(double x, double lo, double hi) {
    double t = (x - lo) / (hi - lo);
    /* f64::clamp(0.0, 1.0 - 1e-15): NaN passes through */
    if (t < 0.0) t = 0.0;
    if (t > 1.0 - 1e-15) t = 1.0 - 1e-15;
    return f64_as_u64(t * 2097152.0);
}

/* spread_bits (lib.rs:85-93) */
static uint64_t spread_bits(uint64_t v) {
    uint64_t x = v & ((1ull << 21) - 1);
    x = (x | (x << 16)) & 0x0000ffff0000ffffull;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

/* compact_bits (lib.rs:95-103) */
static uint64_t compact_bits(uint64_t x) {
    x &= 0x5555555555555555ull;
    x = (x | (x >> 1)) & 0x3333333333333333ull;
    x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
    x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
    x = (x | (x >> 16)) & 0x00000000ffffffffull;
    return x;
}

/* morton_encode (lib.rs:105-109) */
uint64_t gxo_morton_encode(double x, double y, double xmin, double xmax, double ymin, double ymax) {
    return spread_bits(normalize(x, xmin, xmax)) | (spread_bits(normalize(y, ymin, ymax)) << 1);
}

/* morton_decode / denormalize (lib.rs:80-83, 111-115) */
void gxo_morton_decode(uint64_t key, double xmin, double xmax, double ymin, double ymax, double *x, double *y) {
    uint64_t xi = compact_bits(key), yi = compact_bits(key >> 1);
    double csx = (xmax - xmin) / 2097152.0, csy = (ymax - ymin) / 2097152.0;
    *x = xmin + ((double)xi + 0.5) * csx;
    *y = ymin + ((double)yi + 0.5) * csy;
}

void gxo_morton_encode_many(const double *x, const double *y, int64_t n, double xmin, double xmax, double ymin,
                            double ymax, uint64_t *keys) {
    for (int64_t i = 0; i < n; i++) keys[i] = gxo_morton_encode(x[i], y[i], xmin, xmax, ymin, ymax);
}

/* ------------------------------------------------------------------ tree */

static gxo_tree *tree_alloc(int64_t cap) {
    gxo_tree *t = (gxo_tree *)calloc(1, sizeof(gxo_tree));
    t->cap = cap > 0 ? cap : 1;
    t->cx = (double *)malloc(sizeof(double) * t->cap);
    t->cy = (double *)malloc(sizeof(double) * t->cap);
    t->hw = (double *)malloc(sizeof(double) * t->cap);
    t->mass = (double *)malloc(sizeof(double) * t->cap);
    t->comx = (double *)malloc(sizeof(double) * t->cap);
    t->comy = (double *)malloc(sizeof(double) * t->cap);
    t->body_start = (int64_t *)malloc(sizeof(int64_t) * t->cap);
    t->body_end = (int64_t *)malloc(sizeof(int64_t) * t->cap);
    t->child = (int32_t *)malloc(sizeof(int32_t) * 4 * t->cap);
    t->parent = (int32_t *)malloc(sizeof(int32_t) * t->cap);
    t->is_leaf = (uint8_t *)malloc(t->cap);
    t->level_start = (int64_t *)malloc(sizeof(int64_t) * 80);
    return t;
}

static void tree_grow(gxo_tree *t, int64_t need) {
    if (need <= t->cap) return;
    int64_t c = t->cap;
    while (c < need) c *= 2;
    t->cx = (double *)realloc(t->cx, sizeof(double) * c);
    t->cy = (double *)realloc(t->cy, sizeof(double) * c);
    t->hw = (double *)realloc(t->hw, sizeof(double) * c);
    t->mass = (double *)realloc(t->mass, sizeof(double) * c);
    t->comx = (double *)realloc(t->comx, sizeof(double) * c);
    t->comy = (double *)realloc(t->comy, sizeof(double) * c);
    t->body_start = (int64_t *)realloc(t->body_start, sizeof(int64_t) * c);
    t->body_end = (int64_t *)realloc(t->body_end, sizeof(int64_t) * c);
    t->child = (int32_t *)realloc(t->child, sizeof(int32_t) * 4 * c);
    t->parent = (int32_t *)realloc(t->parent, sizeof(int32_t) * c);
    t->is_leaf = (uint8_t *)realloc(t->is_leaf, c);
    t->cap = c;
}

void gxo_tree_free(gxo_tree *t) {
    if (!t) return;
    free(t->cx); free(t->cy); free(t->hw); free(t->mass); free(t->comx); free(t->comy);
    free(t->body_start); free(t->body_end); free(t->child); free(t->parent); free(t->is_leaf);
    free(t->level_start);
    free(t);
}

/* Leaf nodes + bottom-up parent rounds, shared by Tree::build (lib.rs:219-354)
 * and build_with_constraints (lib.rs:615-692). */
static gxo_tree *tree_from_ranges(const double *x, const double *y, const double *m, const uint64_t *keys,
                                  const int64_t *rs, const int64_t *re, int64_t n_leaves, int64_t n_max,
                                  double xmin, double xmax, double ymin, double ymax) {
    gxo_tree *t = tree_alloc(n_leaves * 4 + 16);
    t->n_max = n_max;
    t->xmin = xmin; t->xmax = xmax; t->ymin = ymin; t->ymax = ymax;
    for (int64_t L = 0; L < n_leaves; L++) {
        double ms = 0.0, cxs = 0.0, cys = 0.0;
        double bx0 = 1.7976931348623157e308, bx1 = -1.7976931348623157e308;
        double by0 = 1.7976931348623157e308, by1 = -1.7976931348623157e308;
        for (int64_t i = rs[L]; i < re[L]; i++) {
            double mm = m[i];
            ms += mm;
            cxs += x[i] * mm;
            cys += y[i] * mm;
            bx0 = fmin_rs(bx0, x[i]); bx1 = fmax_rs(bx1, x[i]);
            by0 = fmin_rs(by0, y[i]); by1 = fmax_rs(by1, y[i]);
        }
        double cx = (bx0 + bx1) * 0.5, cy = (by0 + by1) * 0.5;
        double hw = fmax_rs(bx1 - bx0, by1 - by0) * 0.5 + 1e-15;
        t->cx[L] = cx; t->cy[L] = cy; t->hw[L] = hw; t->mass[L] = ms;
        t->comx[L] = ms > 0.0 ? cxs / ms : cx;
        t->comy[L] = ms > 0.0 ? cys / ms : cy;
        t->body_start[L] = rs[L]; t->body_end[L] = re[L];
        for (int k = 0; k < 4; k++) t->child[4 * L + k] = -1;
        t->parent[L] = -1;
        t->is_leaf[L] = 1;
    }
    int64_t nn = n_leaves;
    int32_t lev = 0;
    t->level_start[0] = 0;
    int64_t cur_s = 0, cur_e = nn;
    uint32_t shift = 2;
    while (cur_e - cur_s > 1) {
        int64_t i = cur_s;
        while (i < cur_e) {
            uint32_t sh = shift & 63u; /* release-mode Rust masks the shift amount */
            uint64_t gid = keys[t->body_start[i]] >> sh;
            int64_t j = i + 1;
            while (j < cur_e && j - i < 4) {
                if ((keys[t->body_start[j]] >> sh) != gid) break;
                j++;
            }
            double ms = 0.0, cxs = 0.0, cys = 0.0, mh = 0.0;
            double bx0 = 1.7976931348623157e308, bx1 = -1.7976931348623157e308;
            double by0 = 1.7976931348623157e308, by1 = -1.7976931348623157e308;
            for (int64_t s = i; s < j; s++) {
                ms += t->mass[s];
                cxs += t->comx[s] * t->mass[s];
                cys += t->comy[s] * t->mass[s];
                if (t->hw[s] > mh) mh = t->hw[s];
                double cl = t->cx[s] - t->hw[s], cr = t->cx[s] + t->hw[s];
                if (cl < bx0) bx0 = cl;
                if (cr > bx1) bx1 = cr;
                double cb = t->cy[s] - t->hw[s], ct = t->cy[s] + t->hw[s];
                if (cb < by0) by0 = cb;
                if (ct > by1) by1 = ct;
            }
            double cx = (bx0 + bx1) * 0.5, cy = (by0 + by1) * 0.5;
            tree_grow(t, nn + 1);
            int64_t pid = nn;
            for (int64_t s = i; s < j; s++) t->parent[s] = (int32_t)pid;
            t->cx[pid] = cx; t->cy[pid] = cy; t->hw[pid] = mh * 2.0; t->mass[pid] = ms;
            t->comx[pid] = ms > 0.0 ? cxs / ms : cx;
            t->comy[pid] = ms > 0.0 ? cys / ms : cy;
            t->body_start[pid] = t->body_start[i];
            t->body_end[pid] = t->body_end[j - 1];
            for (int k = 0; k < 4; k++) t->child[4 * pid + k] = (i + k < j) ? (int32_t)(i + k) : -1;
            t->parent[pid] = -1;
            t->is_leaf[pid] = 0;
            nn++;
            i = j;
        }
        lev++;
        t->level_start[lev] = cur_e;
        cur_s = cur_e;
        cur_e = nn;
        shift += 2;
    }
    t->n_levels = lev + 1;
    t->level_start[lev + 1] = nn;
    t->n_nodes = nn;
    return t;
}

typedef struct { uint64_t key; int64_t idx; } keyidx;
static int cmp_keyidx(const void *a, const void *b) {
    const keyidx *p = (const keyidx *)a, *q = (const keyidx *)b;
    if (p->key != q->key) return p->key < q->key ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

static void apply_perm(double *arr, const int64_t *perm, int64_t n, double *tmp) {
    for (int64_t i = 0; i < n; i++) tmp[i] = arr[perm[i]];
    memcpy(arr, tmp, sizeof(double) * n);
}

/* Tree::build (lib.rs:163-361) */
gxo_tree *gxo_tree_build(double *x, double *y, double *vx, double *vy, double *m, double *ax, double *ay,
                         int64_t n, int64_t n_max, double xmin, double xmax, double ymin, double ymax) {
    if (n <= 0) {
        gxo_tree *t = tree_alloc(1);
        t->n_nodes = 0; t->n_levels = 0; t->level_start[0] = 0;
        t->n_max = n_max; t->xmin = xmin; t->xmax = xmax; t->ymin = ymin; t->ymax = ymax;
        return t;
    }
    keyidx *ki = (keyidx *)malloc(sizeof(keyidx) * n);
    for (int64_t i = 0; i < n; i++) {
        ki[i].key = gxo_morton_encode(x[i], y[i], xmin, xmax, ymin, ymax);
        ki[i].idx = i;
    }
    /* stable sort_by_key == sort by (key, original index) */
    qsort(ki, (size_t)n, sizeof(keyidx), cmp_keyidx);
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * n);
    for (int64_t i = 0; i < n; i++) perm[i] = ki[i].idx;
    free(ki);
    double *tmp = (double *)malloc(sizeof(double) * n);
    apply_perm(x, perm, n, tmp); apply_perm(y, perm, n, tmp); apply_perm(vx, perm, n, tmp);
    apply_perm(vy, perm, n, tmp); apply_perm(m, perm, n, tmp); apply_perm(ax, perm, n, tmp);
    apply_perm(ay, perm, n, tmp);
    free(tmp); free(perm);
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * n);
    gxo_morton_encode_many(x, y, n, xmin, xmax, ymin, ymax, keys);
    int64_t nl = (n + n_max - 1) / n_max;
    int64_t *rs = (int64_t *)malloc(sizeof(int64_t) * nl), *re = (int64_t *)malloc(sizeof(int64_t) * nl);
    int64_t L = 0;
    for (int64_t s = 0; s < n; s += n_max) {
        rs[L] = s; re[L] = (s + n_max < n) ? s + n_max : n; L++;
    }
    gxo_tree *t = tree_from_ranges(x, y, m, keys, rs, re, L, n_max, xmin, xmax, ymin, ymax);
    free(keys); free(rs); free(re);
    return t;
}

/* build_with_constraints (lib.rs:592-694); `splits` must be sorted ascending. */
gxo_tree *gxo_tree_build_with_constraints(const double *x, const double *y, const double *m, int64_t n,
                                          int64_t n_max, double xmin, double xmax, double ymin, double ymax,
                                          const int64_t *splits, int64_t n_splits) {
    if (n <= 0) {
        gxo_tree *t = tree_alloc(1);
        t->n_nodes = 0; t->n_levels = 0; t->level_start[0] = 0;
        t->n_max = n_max; t->xmin = xmin; t->xmax = xmax; t->ymin = ymin; t->ymax = ymax;
        return t;
    }
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * n);
    gxo_morton_encode_many(x, y, n, xmin, xmax, ymin, ymax, keys);
    int64_t cap = n + 1;
    int64_t *rs = (int64_t *)malloc(sizeof(int64_t) * cap), *re = (int64_t *)malloc(sizeof(int64_t) * cap);
    int64_t L = 0, s = 0, k = 0;
    while (s < n) {
        int64_t bound = (s + n_max < n) ? s + n_max : n;
        while (k < n_splits && splits[k] <= s) k++;
        int64_t e = (k < n_splits && splits[k] < bound) ? splits[k] : bound;
        rs[L] = s; re[L] = e; L++;
        s = e;
    }
    gxo_tree *t = tree_from_ranges(x, y, m, keys, rs, re, L, n_max, xmin, xmax, ymin, ymax);
    free(keys); free(rs); free(re);
    return t;
}

/* compute_levels (lib.rs:426-438) */
void gxo_compute_levels(const gxo_tree *t, uint32_t *levels) {
    for (int64_t id = 0; id < t->n_nodes; id++) {
        uint32_t mx = 0;
        for (int k = 0; k < 4; k++) {
            int32_t c = t->child[4 * id + k];
            if (c >= 0 && levels[c] + 1 > mx) mx = levels[c] + 1;
        }
        levels[id] = mx;
    }
}

/* ------------------------------------------- bounding-volume candidate search
 * Output-identical acceleration of the reference's O(n^2) scans: candidates are
 * gathered conservatively (boxes widened by a margin that covers every rounding
 * in the exact test), always in ascending id order, and the reference's exact
 * floating-point test is then applied to each candidate. */

typedef struct {
    int64_t s, e, nb, p2;
    double *lx, *hx, *ly, *hy; /* heap-ordered boxes, 2*p2 entries */
    int64_t *always;           /* ids whose box is not finite */
    int64_t n_always;
    double maxabs;
} bvh_t;

#define BVH_B 8

static int node_box_finite(const gxo_tree *t, int64_t id) {
    return isfinite(t->cx[id]) && isfinite(t->cy[id]) && isfinite(t->hw[id]);
}

static void bvh_build(bvh_t *b, const gxo_tree *t, int64_t s, int64_t e) {
    b->s = s; b->e = e;
    b->nb = (e - s + BVH_B - 1) / BVH_B;
    if (b->nb < 1) b->nb = 1;
    b->p2 = 1;
    while (b->p2 < b->nb) b->p2 *= 2;
    int64_t nh = 2 * b->p2;
    b->lx = (double *)malloc(sizeof(double) * nh); b->hx = (double *)malloc(sizeof(double) * nh);
    b->ly = (double *)malloc(sizeof(double) * nh); b->hy = (double *)malloc(sizeof(double) * nh);
    b->always = (int64_t *)malloc(sizeof(int64_t) * (e - s + 1));
    b->n_always = 0;
    b->maxabs = 0.0;
    for (int64_t h = 0; h < nh; h++) { b->lx[h] = INFINITY; b->hx[h] = -INFINITY; b->ly[h] = INFINITY; b->hy[h] = -INFINITY; }
    for (int64_t id = s; id < e; id++) {
        int64_t h = b->p2 + (id - s) / BVH_B;
        if (!node_box_finite(t, id)) { b->always[b->n_always++] = id; continue; }
        double cx = t->cx[id], cy = t->cy[id], hw = t->hw[id];
        double a = fabs(cx) + fabs(cy) + fabs(hw);
        if (a > b->maxabs) b->maxabs = a;
        if (cx - hw < b->lx[h]) b->lx[h] = cx - hw;
        if (cx + hw > b->hx[h]) b->hx[h] = cx + hw;
        if (cy - hw < b->ly[h]) b->ly[h] = cy - hw;
        if (cy + hw > b->hy[h]) b->hy[h] = cy + hw;
    }
    for (int64_t h = b->p2 - 1; h >= 1; h--) {
        b->lx[h] = fmin(b->lx[2 * h], b->lx[2 * h + 1]); b->hx[h] = fmax(b->hx[2 * h], b->hx[2 * h + 1]);
        b->ly[h] = fmin(b->ly[2 * h], b->ly[2 * h + 1]); b->hy[h] = fmax(b->hy[2 * h], b->hy[2 * h + 1]);
    }
}

static void bvh_free(bvh_t *b) { free(b->lx); free(b->hx); free(b->ly); free(b->hy); free(b->always); }

static int cmp_i64(const void *a, const void *b) {
    int64_t p = *(const int64_t *)a, q = *(const int64_t *)b;
    return p < q ? -1 : (p > q);
}

/* All ids whose box may overlap [qx0,qx1]x[qy0,qy1], ascending.  Returns count;
 * *out grows as needed. */
static int64_t bvh_query(const bvh_t *b, const gxo_tree *t, double qx0, double qx1, double qy0, double qy1,
                         int64_t **out, int64_t *out_cap) {
    int64_t cnt = 0;
    int64_t stack[128];
    int sp = 0;
    stack[sp++] = 1;
    while (sp > 0) {
        int64_t h = stack[--sp];
        if (b->lx[h] > qx1 || b->hx[h] < qx0 || b->ly[h] > qy1 || b->hy[h] < qy0) continue;
        if (h >= b->p2) {
            int64_t bk = h - b->p2;
            int64_t i0 = b->s + bk * BVH_B, i1 = i0 + BVH_B;
            if (i1 > b->e) i1 = b->e;
            for (int64_t id = i0; id < i1; id++) {
                if (!node_box_finite(t, id)) continue;
                double cx = t->cx[id], cy = t->cy[id], hw = t->hw[id];
                if (cx - hw > qx1 || cx + hw < qx0 || cy - hw > qy1 || cy + hw < qy0) continue;
                if (cnt + 1 > *out_cap) { *out_cap = *out_cap * 2 + 64; *out = (int64_t *)realloc(*out, sizeof(int64_t) * *out_cap); }
                (*out)[cnt++] = id;
            }
        } else {
            stack[sp++] = 2 * h + 1; /* right pushed first: left visited first */
            stack[sp++] = 2 * h;
        }
    }
    if (b->n_always > 0) {
        if (cnt + b->n_always > *out_cap) { *out_cap = cnt + b->n_always + 64; *out = (int64_t *)realloc(*out, sizeof(int64_t) * *out_cap); }
        for (int64_t k = 0; k < b->n_always; k++) (*out)[cnt++] = b->always[k];
        qsort(*out, (size_t)cnt, sizeof(int64_t), cmp_i64);
    }
    return cnt;
}

static double bvh_margin(const bvh_t *b, double qabs) { return 1e-15 + 1e-12 * (b->maxabs + qabs + 1.0); }

/* ------------------------------------------------------ 2:1 constrained tree */

/* cells_adjacent (lib.rs:369-376) */
static int cells_adjacent(const gxo_tree *t, int64_t a, int64_t b) {
    double ratio = fmax_rs(t->hw[a], t->hw[b]) / fmin_rs(t->hw[a], t->hw[b]);
    if (ratio > 8.0) return 0;
    double dx = fabs(t->cx[a] - t->cx[b]), dy = fabs(t->cy[a] - t->cy[b]);
    return dx <= t->hw[a] + t->hw[b] + 1e-15 && dy <= t->hw[a] + t->hw[b] + 1e-15;
}

static void test_points(const gxo_tree *t, int64_t id, double *px, double *py) {
    double cx = t->cx[id], cy = t->cy[id], hw = t->hw[id];
    double d = hw * 2.0;
    px[0] = cx + d; py[0] = cy;
    px[1] = cx + d; py[1] = cy + d;
    px[2] = cx;     py[2] = cy + d;
    px[3] = cx - d; py[3] = cy + d;
    px[4] = cx - d; py[4] = cy;
    px[5] = cx - d; py[5] = cy - d;
    px[6] = cx;     py[6] = cy - d;
    px[7] = cx + d; py[7] = cy - d;
}

static int nb_candidate(const gxo_tree *t, int64_t node, int64_t other, double px, double py, double *dist) {
    if (other == node) return 0;
    double dx = fabs(px - t->cx[other]), dy = fabs(py - t->cy[other]);
    if (!(dx <= t->hw[other] + 1e-15 && dy <= t->hw[other] + 1e-15)) return 0;
    if (!cells_adjacent(t, node, other)) return 0;
    double ex = px - t->cx[other], ey = py - t->cy[other];
    *dist = ex * ex + ey * ey; /* powi(2) == x*x */
    return 1;
}

/* neighbors_geometric (lib.rs:382-423), literal scan over all nodes */
void gxo_neighbors_geometric(const gxo_tree *t, int32_t node, int32_t *out) {
    double px[8], py[8];
    test_points(t, node, px, py);
    for (int k = 0; k < 8; k++) {
        int32_t best = -1;
        double bd = 1.7976931348623157e308;
        for (int64_t o = 0; o < t->n_nodes; o++) {
            double d;
            if (nb_candidate(t, node, o, px[k], py[k], &d) && d < bd) { bd = d; best = (int32_t)o; }
        }
        out[k] = best;
    }
}

/* Same result through per-level bounding volumes. */
static void neighbors_geometric_accel(const gxo_tree *t, const bvh_t *lv, int nlv, int32_t node, int32_t *out,
                                      int64_t **buf, int64_t *cap) {
    double px[8], py[8];
    test_points(t, node, px, py);
    for (int k = 0; k < 8; k++) {
        int32_t best = -1;
        double bd = 1.7976931348623157e308;
        double qa = fabs(px[k]) + fabs(py[k]);
        for (int L = 0; L < nlv; L++) { /* levels are ascending id ranges */
            double mg = bvh_margin(&lv[L], qa);
            int64_t c = bvh_query(&lv[L], t, px[k] - mg, px[k] + mg, py[k] - mg, py[k] + mg, buf, cap);
            for (int64_t q = 0; q < c; q++) {
                double d;
                int64_t o = (*buf)[q];
                if (nb_candidate(t, node, o, px[k], py[k], &d) && d < bd) { bd = d; best = (int32_t)o; }
            }
        }
        out[k] = best;
    }
}

static int contains_i64(const int64_t *a, int64_t n, int64_t v) {
    for (int64_t i = 0; i < n; i++) if (a[i] == v) return 1;
    return 0;
}

/* build_constrained (lib.rs:541-588) */
gxo_tree *gxo_tree_build_constrained(const double *x, const double *y, const double *m, int64_t n, int64_t n_max,
                                     double xmin, double xmax, double ymin, double ymax, int accel) {
    int64_t *splits = NULL, ns = 0, scap = 0;
    int64_t *news = NULL, nn = 0, ncap = 0;
    int64_t *buf = NULL, bcap = 0;
    for (int iter = 0; iter < 10; iter++) {
        gxo_tree *t = gxo_tree_build_with_constraints(x, y, m, n, n_max, xmin, xmax, ymin, ymax, splits, ns);
        bvh_t *lv = NULL;
        if (accel && t->n_levels > 0) {
            lv = (bvh_t *)malloc(sizeof(bvh_t) * t->n_levels);
            for (int L = 0; L < t->n_levels; L++) bvh_build(&lv[L], t, t->level_start[L], t->level_start[L + 1]);
        }
        nn = 0;
        for (int64_t lid = 0; lid < t->n_nodes; lid++) {
            if (!t->is_leaf[lid]) continue;
            double hw = t->hw[lid];
            int32_t nb[8];
            if (accel) neighbors_geometric_accel(t, lv, t->n_levels, (int32_t)lid, nb, &buf, &bcap);
            else gxo_neighbors_geometric(t, (int32_t)lid, nb);
            for (int k = 0; k < 8; k++) {
                if (nb[k] < 0) continue;
                double nhw = t->hw[nb[k]];
                if (hw > nhw * 2.1) {
                    int64_t s = t->body_start[lid], e = t->body_end[lid];
                    if (e - s > 2) {
                        int64_t mid = (s + e) / 2;
                        if (!contains_i64(splits, ns, mid) && !contains_i64(news, nn, mid)) {
                            if (nn + 1 > ncap) { ncap = ncap * 2 + 16; news = (int64_t *)realloc(news, sizeof(int64_t) * ncap); }
                            news[nn++] = mid;
                        }
                    }
                    break;
                }
            }
        }
        if (lv) { for (int L = 0; L < t->n_levels; L++) bvh_free(&lv[L]); free(lv); }
        if (nn == 0) { free(splits); free(news); free(buf); return t; }
        gxo_tree_free(t);
        if (ns + nn > scap) { scap = ns + nn + 16; splits = (int64_t *)realloc(splits, sizeof(int64_t) * scap); }
        memcpy(splits + ns, news, sizeof(int64_t) * nn);
        ns += nn;
        qsort(splits, (size_t)ns, sizeof(int64_t), cmp_i64);
        int64_t w = 0;
        for (int64_t i = 0; i < ns; i++) if (w == 0 || splits[i] != splits[w - 1]) splits[w++] = splits[i];
        ns = w;
    }
    gxo_tree *t = gxo_tree_build_with_constraints(x, y, m, n, n_max, xmin, xmax, ymin, ymax, splits, ns);
    free(splits); free(news); free(buf);
    return t;
}

/* ----------------------------------------------------------------- lists */

static gxo_lists *lists_alloc(int64_t n_nodes) {
    gxo_lists *l = (gxo_lists *)calloc(1, sizeof(gxo_lists));
    l->n_nodes = n_nodes;
    int64_t nn = n_nodes > 0 ? n_nodes : 1;
    l->data = (uint32_t *)malloc(sizeof(uint32_t) * GXO_LIST_CAP * nn);
    for (int64_t i = 0; i < GXO_LIST_CAP * nn; i++) l->data[i] = LIST_EMPTY;
    l->lengths = (uint8_t *)calloc((size_t)nn, 1);
    return l;
}

void gxo_lists_free(gxo_lists *l) {
    if (!l) return;
    free(l->data); free(l->lengths); free(l);
}

static void list_push(gxo_lists *l, int64_t node, int64_t v) {
    uint8_t len = l->lengths[node];
    if (len < GXO_LIST_CAP) {
        l->data[(int64_t)GXO_LIST_CAP * node + len] = (uint32_t)v;
        l->lengths[node] = (uint8_t)(len + 1);
    }
}

/* V-list parent test (lib.rs:990-995): skipped iff dx > h_sum+1e-15 || dy > ... */
static int vlist_parent_near(const gxo_tree *t, int64_t P, int64_t pn) {
    double dx = fabs(t->cx[pn] - t->cx[P]), dy = fabs(t->cy[pn] - t->cy[P]);
    double hs = t->hw[P] + t->hw[pn];
    return !(dx > hs + 1e-15 || dy > hs + 1e-15);
}

/* V-list child adjacency (lib.rs:1000-1006) */
static int vlist_child_adjacent(const gxo_tree *t, int64_t n, int64_t c) {
    double cdx = fabs(t->cx[c] - t->cx[n]), cdy = fabs(t->cy[c] - t->cy[n]);
    int ax = cdx <= t->hw[n] + t->hw[c] + 1e-15;
    int ay = cdy <= t->hw[n] + t->hw[c] + 1e-15;
    return ax && ay;
}

/* InteractionLists::build (lib.rs:947-1025) */
gxo_lists *gxo_vlist_build(const gxo_tree *t, int accel) {
    gxo_lists *l = lists_alloc(t->n_nodes);
    for (int lv = 0; lv + 1 < t->n_levels; lv++) {
        int64_t s0 = t->level_start[lv], e0 = t->level_start[lv + 1];
        int64_t s1 = t->level_start[lv + 1], e1 = t->level_start[lv + 2];
        if (!accel) {
            for (int64_t nid = s0; nid < e0; nid++) {
                int64_t P = t->parent[nid];
                if (P < 0) continue;
                for (int64_t pn = s1; pn < e1; pn++) {
                    if (pn == P) continue;
                    if (!vlist_parent_near(t, P, pn)) continue;
                    for (int k = 0; k < 4; k++) {
                        int32_t c = t->child[4 * pn + k];
                        if (c < 0) continue;
                        if (vlist_child_adjacent(t, nid, c)) continue;
                        list_push(l, nid, c);
                    }
                }
            }
            continue;
        }
        /* Per-node query of the parent level (ascending id, early exit at the cap).
         * A subtree is pruned when no parent in it can be near P, or when every child
         * of every parent in it is certainly adjacent to the node (and so rejected). */
        bvh_t b;
        bvh_build(&b, t, s1, e1);
        if (b.n_always > 0) { /* non-finite boxes: literal scan for this level */
            bvh_free(&b);
            for (int64_t nid = s0; nid < e0; nid++) {
                int64_t P = t->parent[nid];
                if (P < 0) continue;
                for (int64_t pn = s1; pn < e1; pn++) {
                    if (pn == P || !vlist_parent_near(t, P, pn)) continue;
                    for (int k = 0; k < 4; k++) {
                        int32_t c = t->child[4 * pn + k];
                        if (c < 0 || vlist_child_adjacent(t, nid, c)) continue;
                        list_push(l, nid, c);
                    }
                }
            }
            continue;
        }
        int64_t nh = 2 * b.p2;
        double *cb = (double *)malloc(sizeof(double) * 5 * nh); /* child-centre box + min child hw */
        double cmax = 0.0;
        for (int64_t h = 0; h < nh; h++) {
            cb[5 * h] = INFINITY; cb[5 * h + 1] = -INFINITY; cb[5 * h + 2] = INFINITY; cb[5 * h + 3] = -INFINITY;
            cb[5 * h + 4] = INFINITY;
        }
        for (int64_t pn = s1; pn < e1; pn++) {
            int64_t h = b.p2 + (pn - s1) / BVH_B;
            for (int k = 0; k < 4; k++) {
                int32_t c = t->child[4 * pn + k];
                if (c < 0) continue;
                if (!node_box_finite(t, c)) { cb[5 * h + 4] = -INFINITY; continue; }
                cb[5 * h] = fmin(cb[5 * h], t->cx[c]); cb[5 * h + 1] = fmax(cb[5 * h + 1], t->cx[c]);
                cb[5 * h + 2] = fmin(cb[5 * h + 2], t->cy[c]); cb[5 * h + 3] = fmax(cb[5 * h + 3], t->cy[c]);
                cb[5 * h + 4] = fmin(cb[5 * h + 4], t->hw[c]);
                double a = fabs(t->cx[c]) + fabs(t->cy[c]) + t->hw[c];
                if (a > cmax) cmax = a;
            }
        }
        for (int64_t h = b.p2 - 1; h >= 1; h--)
            for (int q = 0; q < 5; q++)
                cb[5 * h + q] = (q == 1 || q == 3) ? fmax(cb[10 * h + q], cb[10 * h + 5 + q])
                                                   : fmin(cb[10 * h + q], cb[10 * h + 5 + q]);
#pragma omp parallel for schedule(dynamic, 64) num_threads(gxo_get_threads())
        for (int64_t nid = s0; nid < e0; nid++) {
            int64_t P = t->parent[nid];
            if (P < 0) continue;
            double qa = fabs(t->cx[P]) + fabs(t->cy[P]) + t->hw[P];
            double mg = bvh_margin(&b, qa);
            double qx0 = t->cx[P] - t->hw[P] - mg, qx1 = t->cx[P] + t->hw[P] + mg;
            double qy0 = t->cy[P] - t->hw[P] - mg, qy1 = t->cy[P] + t->hw[P] + mg;
            double ncx = t->cx[nid], ncy = t->cy[nid], nhw = t->hw[nid];
            double dl = 1e-12 * (fabs(ncx) + fabs(ncy) + nhw + cmax + 1.0);
            int pfin = node_box_finite(t, P);
            int64_t stack[128];
            int sp = 0;
            stack[sp++] = 1;
            while (sp > 0 && l->lengths[nid] < GXO_LIST_CAP) {
                int64_t h = stack[--sp];
                if (pfin && (b.lx[h] > qx1 || b.hx[h] < qx0 || b.ly[h] > qy1 || b.hy[h] < qy0)) continue;
                double wx = fmax(fabs(cb[5 * h] - ncx), fabs(cb[5 * h + 1] - ncx));
                double wy = fmax(fabs(cb[5 * h + 2] - ncy), fabs(cb[5 * h + 3] - ncy));
                double lim = nhw + cb[5 * h + 4] - dl;
                if (wx <= lim && wy <= lim) continue; /* every child adjacent to nid */
                if (h >= b.p2) {
                    int64_t i0 = s1 + (h - b.p2) * BVH_B, i1 = i0 + BVH_B;
                    if (i1 > e1) i1 = e1;
                    for (int64_t pn = i0; pn < i1 && l->lengths[nid] < GXO_LIST_CAP; pn++) {
                        if (pn == P || !vlist_parent_near(t, P, pn)) continue;
                        for (int k = 0; k < 4; k++) {
                            int32_t c = t->child[4 * pn + k];
                            if (c < 0 || vlist_child_adjacent(t, nid, c)) continue;
                            list_push(l, nid, c);
                        }
                    }
                } else {
                    stack[sp++] = 2 * h + 1;
                    stack[sp++] = 2 * h;
                }
            }
        }
        free(cb);
        bvh_free(&b);
    }
    return l;
}

/* U-list touch test (lib.rs:1380-1384) */
static int ulist_touch(const gxo_tree *t, int64_t a, int64_t b) {
    double dx = fabs(t->cx[a] - t->cx[b]), dy = fabs(t->cy[a] - t->cy[b]);
    return dx <= t->hw[a] + t->hw[b] + 1e-15 && dy <= t->hw[a] + t->hw[b] + 1e-15;
}

/* build_p2p_lists (lib.rs:1358-1392); leaves are ids [0, level_start[1]) */
gxo_lists *gxo_ulist_build(const gxo_tree *t, int accel) {
    gxo_lists *l = lists_alloc(t->n_nodes);
    if (t->n_nodes == 0) return l;
    int64_t nl = t->level_start[1];
    for (int64_t a = 0; a < nl; a++) if (!t->is_leaf[a]) return l; /* invariant of Tree::build */
    if (!accel) {
        for (int64_t a = 0; a < nl; a++) {
            list_push(l, a, a);
            for (int64_t b = 0; b < nl; b++) {
                if (a == b) continue;
                if (ulist_touch(t, a, b)) list_push(l, a, b);
            }
        }
        return l;
    }
    bvh_t b;
    bvh_build(&b, t, 0, nl);
    int64_t *buf = NULL, bcap = 0;
    for (int64_t a = 0; a < nl; a++) {
        list_push(l, a, a);
        double mg = bvh_margin(&b, fabs(t->cx[a]) + fabs(t->cy[a]) + t->hw[a]);
        int64_t c;
        if (node_box_finite(t, a)) {
            c = bvh_query(&b, t, t->cx[a] - t->hw[a] - mg, t->cx[a] + t->hw[a] + mg, t->cy[a] - t->hw[a] - mg,
                          t->cy[a] + t->hw[a] + mg, &buf, &bcap);
        } else {
            c = nl;
            if (c > bcap) { bcap = c; buf = (int64_t *)realloc(buf, sizeof(int64_t) * bcap); }
            for (int64_t q = 0; q < c; q++) buf[q] = q;
        }
        for (int64_t q = 0; q < c && l->lengths[a] < GXO_LIST_CAP; q++) {
            int64_t bb = buf[q];
            if (bb == a) continue;
            if (ulist_touch(t, a, bb)) list_push(l, a, bb);
        }
    }
    free(buf);
    bvh_free(&b);
    return l;
}

/* ---------------------------------------------------------------- passes */

/* p2m (lib.rs:848-887) */
void gxo_p2m(const double *x, const double *y, const double *m, const gxo_tree *t, int64_t p, double *mult) {
    init_tables();
    int64_t st = gxo_num_moments(p);
    memset(mult, 0, sizeof(double) * st * (t->n_nodes > 0 ? t->n_nodes : 0));
    for (int64_t id = 0; id < t->n_nodes; id++) {
        if (!t->is_leaf[id]) continue;
        double cx = t->comx[id], cy = t->comy[id];
        double *M = mult + id * st;
        for (int64_t b = t->body_start[id]; b < t->body_end[id]; b++) {
            double dx = x[b] - cx, dy = y[b] - cy, mass = m[b];
            double dxp[GXO_MAX_P], dyp[GXO_MAX_P];
            fill_powers(dxp, dx, p);
            fill_powers(dyp, dy, p);
            for (int64_t i = 0; i <= p; i++)
                for (int64_t j = 0; j <= p - i; j++)
                    M[MI(i, j)] += mass * dxp[i] * dyp[j] / (g_fact[i] * g_fact[j]);
        }
    }
    for (int64_t k = 0; k < st * t->n_nodes; k++) if (!isfinite(mult[k])) mult[k] = 0.0;
}

/* m2m (lib.rs:890-938) */
void gxo_m2m(double *mult, const gxo_tree *t, int64_t p) {
    init_tables();
    int64_t st = gxo_num_moments(p);
    for (int64_t id = 0; id < t->n_nodes; id++) {
        if (t->is_leaf[id]) continue;
        double *MP = mult + id * st;
        for (int k = 0; k < 4; k++) {
            int32_t c = t->child[4 * id + k];
            if (c < 0) continue;
            double dx = t->comx[c] - t->comx[id], dy = t->comy[c] - t->comy[id];
            const double *MC = mult + (int64_t)c * st;
            double dxp[GXO_MAX_P], dyp[GXO_MAX_P];
            fill_powers(dxp, dx, p);
            fill_powers(dyp, dy, p);
            for (int64_t oi = 0; oi <= p; oi++)
                for (int64_t oj = 0; oj <= p - oi; oj++) {
                    double sum = 0.0;
                    for (int64_t i = 0; i <= oi; i++)
                        for (int64_t j = 0; j <= oj; j++) {
                            if (i + j > p) continue;
                            sum += MC[MI(i, j)] * dxp[oi - i] * dyp[oj - j] / (g_fact[oi - i] * g_fact[oj - j]);
                        }
                    MP[MI(oi, oj)] += sum;
                }
        }
    }
    for (int64_t k = 0; k < st * t->n_nodes; k++) if (!isfinite(mult[k])) mult[k] = 0.0;
}

static int64_t kdi(int64_t k, int64_t l, int64_t p) { return (k + l) * (2 * p + 1) + l; }

/* compute_kernel_derivs (lib.rs:1040-1151): derivative polynomials N_{k,l} built by
 * the reference's recurrence, then evaluated term by term. */
void gxo_kernel_derivs(double dx, double dy, double eps, int64_t p, double *deriv) {
    int64_t order = 2 * p, S = order + 1;
    memset(deriv, 0, sizeof(double) * S * S);
    double x = dx, y = dy, eps2 = eps * eps;
    double r2 = x * x + y * y + eps2;
    double r = sqrt(r2);
    double *inv_r = (double *)calloc((size_t)(2 + 2 * order), sizeof(double));
    inv_r[1] = 1.0 / r;
    for (int64_t n = 3; n <= 1 + 2 * order; n += 2) inv_r[n] = inv_r[n - 2] / r2;
    /* poly[(k*S + l)][a*S + b] */
    double *poly = (double *)calloc((size_t)(S * S * S * S), sizeof(double));
#define PL(k, l) (poly + ((k) * S + (l)) * S * S)
    PL(0, 0)[0] = -1.0;
    for (int64_t n = 1; n <= order; n++) {
        for (int64_t k = 0; k <= n; k++) {
            int64_t l = n - k;
            double *coeff = PL(k, l);
            if (k > 0) {
                const double *prev = PL(k - 1, l);
                int64_t mm = 1 + 2 * (k - 1) + 2 * l;
                for (int64_t a = 0; a < S; a++)
                    for (int64_t b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (a > 0) {
                            double dc = c * (double)a;
                            if (a + 1 < S) coeff[(a + 1) * S + b] += dc;
                            if (b + 2 < S) coeff[(a - 1) * S + b + 2] += dc;
                            coeff[(a - 1) * S + b] += dc * eps2;
                        }
                    }
                for (int64_t a = 0; a < S; a++)
                    for (int64_t b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (a + 1 < S) coeff[(a + 1) * S + b] -= (double)mm * c;
                    }
            } else if (l > 0) {
                const double *prev = PL(k, l - 1);
                int64_t mm = 1 + 2 * k + 2 * (l - 1);
                for (int64_t a = 0; a < S; a++)
                    for (int64_t b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (b > 0) {
                            double dc = c * (double)b;
                            if (a + 2 < S) coeff[(a + 2) * S + b - 1] += dc;
                            if (b + 1 < S) coeff[a * S + b + 1] += dc;
                            coeff[a * S + b - 1] += dc * eps2;
                        }
                    }
                for (int64_t a = 0; a < S; a++)
                    for (int64_t b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (b + 1 < S) coeff[a * S + b + 1] -= (double)mm * c;
                    }
            }
        }
    }
    for (int64_t k = 0; k <= order; k++)
        for (int64_t l = 0; l <= order - k; l++) {
            double val = 0.0;
            const double *pl = PL(k, l);
            for (int64_t a = 0; a < S; a++)
                for (int64_t b = 0; b < S - a; b++) {
                    double c = pl[a * S + b];
                    if (c != 0.0) val += c * powi_rs(x, (int)a) * powi_rs(y, (int)b);
                }
            deriv[kdi(k, l, p)] = val * inv_r[1 + 2 * k + 2 * l];
        }
#undef PL
    free(poly);
    free(inv_r);
}

/* Cartesian Taylor coefficients of 1/R, R^2 = x^2+y^2+eps^2, from the three-term
 * recurrence  |k| R^2 a_k = -(2|k|-1)(x a_{k-ex} + y a_{k-ey}) - (|k|-1)(a_{k-2ex} + a_{k-2ey}),
 * a_0 = 1/R (the 3D Coulomb recurrence restricted to k_z = 0); G-derivatives are
 * -k! a_k.  Not part of the reference: a cross-check and the form the GPU uses. */
void gxo_kernel_derivs_recurrence(double dx, double dy, double eps, int64_t p, double *deriv) {
    init_tables();
    int64_t order = 2 * p, S = order + 1;
    memset(deriv, 0, sizeof(double) * S * S);
    double r2 = dx * dx + dy * dy + eps * eps;
    double ir2 = 1.0 / r2;
    double a[33][33];
    memset(a, 0, sizeof(a));
    a[0][0] = 1.0 / sqrt(r2);
    for (int64_t n = 1; n <= order; n++)
        for (int64_t k = 0; k <= n; k++) {
            int64_t l = n - k;
            double s1 = 0.0, s2 = 0.0;
            if (k >= 1) s1 += dx * a[k - 1][l];
            if (l >= 1) s1 += dy * a[k][l - 1];
            if (k >= 2) s2 += a[k - 2][l];
            if (l >= 2) s2 += a[k][l - 2];
            a[k][l] = (-(double)(2 * n - 1) * s1 - (double)(n - 1) * s2) * ir2 / (double)n;
        }
    double f[33];
    f[0] = 1.0;
    for (int i = 1; i < 33; i++) f[i] = f[i - 1] * (double)i;
    for (int64_t k = 0; k <= order; k++)
        for (int64_t l = 0; l <= order - k; l++) deriv[kdi(k, l, p)] = -f[k] * f[l] * a[k][l];
}

typedef struct { int32_t src, tgt, di; double w; } m2l_term;

/* m2l_plan (lib.rs:1160-1196) */
static int64_t m2l_plan(int64_t p, m2l_term *plan) {
    init_tables();
    int64_t n = 0;
    for (int64_t i = 0; i <= p; i++)
        for (int64_t j = 0; j <= p - i; j++) {
            double sign = ((i + j) % 2 == 0) ? 1.0 : -1.0;
            int64_t src = MI(i, j);
            for (int64_t oi = 0; oi <= p; oi++)
                for (int64_t oj = 0; oj <= p - oi; oj++) {
                    int64_t tgt = MI(oi, oj);
                    double lf = 1.0 / (g_fact[oi] * g_fact[oj]);
                    int64_t dk = i + oi, dl = j + oj;
                    if (dk + dl <= 2 * p) {
                        plan[n].src = (int32_t)src; plan[n].tgt = (int32_t)tgt;
                        plan[n].w = sign * lf; plan[n].di = (int32_t)kdi(dk, dl, p);
                        n++;
                    }
                }
        }
    return n;
}

/* Open-addressing map (i64,i64) -> int */
typedef struct { int64_t *kx, *ky; int32_t *val; int64_t cap, n; } kmap;
static uint64_t hash2(int64_t a, int64_t b) {
    uint64_t h = (uint64_t)a * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)b + 0x632BE59BD9B4E019ull + (h << 6) + (h >> 2);
    h ^= h >> 29; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 32;
    return h;
}
static void kmap_init(kmap *m, int64_t cap) {
    m->cap = 64; while (m->cap < cap * 2) m->cap *= 2;
    m->kx = (int64_t *)malloc(sizeof(int64_t) * m->cap); m->ky = (int64_t *)malloc(sizeof(int64_t) * m->cap);
    m->val = (int32_t *)malloc(sizeof(int32_t) * m->cap);
    for (int64_t i = 0; i < m->cap; i++) m->val[i] = -1;
    m->n = 0;
}
static void kmap_free(kmap *m) { free(m->kx); free(m->ky); free(m->val); }
static int32_t kmap_get_or_insert(kmap *m, int64_t a, int64_t b, int32_t newval, int *inserted) {
    if ((m->n + 1) * 2 > m->cap) {
        kmap o = *m;
        kmap_init(m, o.cap);
        for (int64_t i = 0; i < o.cap; i++) if (o.val[i] >= 0) { int d; kmap_get_or_insert(m, o.kx[i], o.ky[i], o.val[i], &d); }
        kmap_free(&o);
    }
    uint64_t h = hash2(a, b) & (uint64_t)(m->cap - 1);
    while (m->val[h] >= 0) {
        if (m->kx[h] == a && m->ky[h] == b) { *inserted = 0; return m->val[h]; }
        h = (h + 1) & (uint64_t)(m->cap - 1);
    }
    m->kx[h] = a; m->ky[h] = b; m->val[h] = newval; m->n++;
    *inserted = 1;
    return newval;
}

int64_t gxo_m2l_ref_keys(const gxo_lists *v, const gxo_tree *t, int32_t *pair_key, double *key_dxdy,
                         int64_t max_keys) {
    kmap km;
    kmap_init(&km, 1024);
    int64_t nk = 0, pair = 0;
    for (int64_t id = 0; id < t->n_nodes; id++) {
        int64_t len = v->lengths[id];
        for (int64_t s = 0; s < len; s++) {
            int64_t src = v->data[GXO_LIST_CAP * id + s];
            double dx = t->comx[id] - t->comx[src], dy = t->comy[id] - t->comy[src];
            int ins;
            int32_t k = kmap_get_or_insert(&km, f64_as_i64(dx), f64_as_i64(dy), (int32_t)nk, &ins);
            if (ins) {
                if (nk < max_keys && key_dxdy) { key_dxdy[2 * nk] = dx; key_dxdy[2 * nk + 1] = dy; }
                nk++;
            }
            if (pair_key) pair_key[pair] = k;
            pair++;
        }
    }
    kmap_free(&km);
    return nk;
}

/* m2l (lib.rs:1199-1259). REF mode reproduces the single-threaded cache: the first
 * pair (target id ascending, list slot ascending) to reach a key decides the
 * derivatives every later pair with that key uses. */
void gxo_m2l(double *locals, const double *mult, const gxo_lists *v, const gxo_tree *t, int64_t p, double eps,
             int deriv_mode) {
    int64_t st = gxo_num_moments(p), DS = (2 * p + 1) * (2 * p + 1);
    m2l_term plan[GXO_MAX_P * GXO_MAX_P * GXO_MAX_P * GXO_MAX_P / 4 + 64];
    int64_t np = m2l_plan(p, plan);
    int64_t n_pairs = 0;
    int64_t *poff = (int64_t *)malloc(sizeof(int64_t) * (t->n_nodes + 1));
    for (int64_t id = 0; id < t->n_nodes; id++) { poff[id] = n_pairs; n_pairs += v->lengths[id]; }
    poff[t->n_nodes] = n_pairs;
    int32_t *pk = NULL;
    double *table = NULL;
    if (deriv_mode == 0) {
        pk = (int32_t *)malloc(sizeof(int32_t) * (n_pairs + 1));
        int64_t nk = gxo_m2l_ref_keys(v, t, pk, NULL, 0);
        double *kd = (double *)malloc(sizeof(double) * 2 * (nk + 1));
        gxo_m2l_ref_keys(v, t, pk, kd, nk);
        table = (double *)malloc(sizeof(double) * DS * (nk + 1));
#pragma omp parallel for schedule(dynamic, 16) num_threads(gxo_get_threads())
        for (int64_t k = 0; k < nk; k++) gxo_kernel_derivs(kd[2 * k], kd[2 * k + 1], eps, p, table + k * DS);
        free(kd);
    }
#pragma omp parallel num_threads(gxo_get_threads())
    {
        double *dbuf = (double *)malloc(sizeof(double) * DS);
#pragma omp for schedule(dynamic, 64)
        for (int64_t id = 0; id < t->n_nodes; id++) {
            int64_t len = v->lengths[id];
            if (len == 0) continue;
            double *L = locals + id * st;
            for (int64_t s = 0; s < len; s++) {
                int64_t src = v->data[GXO_LIST_CAP * id + s];
                const double *M = mult + src * st;
                const double *G;
                if (deriv_mode == 0) {
                    G = table + (int64_t)pk[poff[id] + s] * DS;
                } else {
                    double dx = t->comx[id] - t->comx[src], dy = t->comy[id] - t->comy[src];
                    gxo_kernel_derivs(dx, dy, eps, p, dbuf);
                    G = dbuf;
                }
                for (int64_t q = 0; q < np; q++) {
                    double mv = M[plan[q].src];
                    if (mv == 0.0) continue;
                    L[plan[q].tgt] += mv * plan[q].w * G[plan[q].di];
                }
            }
        }
        free(dbuf);
    }
    free(pk); free(table); free(poff);
}

static void l2l_node(double *locals, const gxo_tree *t, int64_t id, int64_t p, int64_t st) {
    const double *LP = locals + id * st;
    for (int k = 0; k < 4; k++) {
        int32_t c = t->child[4 * id + k];
        if (c < 0) continue;
        double dx = t->comx[c] - t->comx[id], dy = t->comy[c] - t->comy[id];
        double *LC = locals + (int64_t)c * st;
        double dxp[GXO_MAX_P], dyp[GXO_MAX_P];
        fill_powers(dxp, dx, p);
        fill_powers(dyp, dy, p);
        for (int64_t oi = 0; oi <= p; oi++)
            for (int64_t oj = 0; oj <= p - oi; oj++) {
                double sum = 0.0;
                for (int64_t i = oi; i <= p; i++)
                    for (int64_t j = oj; j <= p - i; j++)
                        sum += LP[MI(i, j)] * g_binom[i][oi] * g_binom[j][oj] * dxp[i - oi] * dyp[j - oj];
                LC[MI(oi, oj)] += sum;
            }
    }
}

/* l2l (lib.rs:1262-1302).  order 0 walks node ids ascending exactly like the
 * reference (children before parents, so only one level of shift reaches each
 * node); order 1 walks ids descending, i.e. top-down. */
void gxo_l2l(double *locals, const gxo_tree *t, int64_t p, int order) {
    init_tables();
    int64_t st = gxo_num_moments(p);
    if (order == 0) {
        for (int64_t id = 0; id < t->n_nodes; id++) if (!t->is_leaf[id]) l2l_node(locals, t, id, p, st);
    } else {
        for (int64_t id = t->n_nodes - 1; id >= 0; id--) if (!t->is_leaf[id]) l2l_node(locals, t, id, p, st);
    }
}

/* l2p (lib.rs:1308-1355) */
void gxo_l2p(const double *x, const double *y, double *ax, double *ay, const double *locals, const gxo_tree *t,
             int64_t p) {
    int64_t st = gxo_num_moments(p);
#pragma omp parallel for schedule(dynamic, 64) num_threads(gxo_get_threads())
    for (int64_t id = 0; id < t->n_nodes; id++) {
        if (!t->is_leaf[id]) continue;
        const double *L = locals + id * st;
        for (int64_t b = t->body_start[id]; b < t->body_end[id]; b++) {
            double dux = x[b] - t->comx[id], duy = y[b] - t->comy[id];
            double xp[GXO_MAX_P], yp[GXO_MAX_P];
            fill_powers(xp, dux, p);
            fill_powers(yp, duy, p);
            double fx = 0.0, fy = 0.0;
            for (int64_t i = 0; i <= p; i++)
                for (int64_t j = 0; j <= p - i; j++) {
                    double c = L[MI(i, j)];
                    if (i >= 1) fx += c * (double)i * xp[i - 1] * yp[j];
                    if (j >= 1) fy += c * (double)j * xp[i] * yp[j - 1];
                }
            ax[b] -= fx;
            ay[b] -= fy;
        }
    }
}

/* p2p (lib.rs:1395-1462): sequential symmetric updates; a partner with a lower id
 * than the node is skipped. */
void gxo_p2p(const double *x, const double *y, const double *m, double *ax, double *ay, const gxo_tree *t,
             const gxo_lists *u, double eps) {
    double s2 = eps * eps;
    for (int64_t id = 0; id < t->n_nodes; id++) {
        if (!t->is_leaf[id]) continue;
        int64_t len = u->lengths[id];
        for (int64_t s = 0; s < len; s++) {
            int64_t pid = u->data[GXO_LIST_CAP * id + s];
            int64_t a0, a1, b0, b1;
            if (pid == id) {
                a0 = t->body_start[id]; a1 = t->body_end[id];
                for (int64_t i = a0; i < a1; i++) {
                    double axi = 0.0, ayi = 0.0;
                    for (int64_t j = i + 1; j < a1; j++) {
                        double dx = x[j] - x[i], dy = y[j] - y[i];
                        double r2 = dx * dx + dy * dy + s2;
                        double ir = 1.0 / sqrt(r2);
                        double ir3 = powi_rs(ir, 3);
                        double f = m[j] * ir3;
                        axi += f * dx;
                        ayi += f * dy;
                        ax[j] -= f * dx * m[i] / m[j];
                        ay[j] -= f * dy * m[i] / m[j];
                    }
                    ax[i] += axi;
                    ay[i] += ayi;
                }
            } else if (pid < id) {
                continue;
            } else {
                b0 = t->body_start[pid]; b1 = t->body_end[pid];
                a0 = t->body_start[id]; a1 = t->body_end[id];
                for (int64_t i = a0; i < a1; i++) {
                    double axi = 0.0, ayi = 0.0;
                    for (int64_t j = b0; j < b1; j++) {
                        double dx = x[j] - x[i], dy = y[j] - y[i];
                        double r2 = dx * dx + dy * dy + s2;
                        double ir = 1.0 / sqrt(r2);
                        double ir3 = powi_rs(ir, 3);
                        double f = m[j] * ir3;
                        axi += f * dx;
                        ayi += f * dy;
                        ax[j] -= f * dx * m[i] / m[j];
                        ay[j] -= f * dy * m[i] / m[j];
                    }
                    ax[i] += axi;
                    ay[i] += ayi;
                }
            }
        }
    }
}

/* compute_fmm_force (lib.rs:1466-1499) */
void gxo_compute_fmm_force(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                           const gxo_lists *v, const gxo_lists *u, int64_t p, double eps, int mode) {
    int64_t n = t->n_nodes > 0 ? t->body_end[t->n_nodes - 1] : 0;
    for (int64_t i = 0; i < n; i++) {
        if (fabs(x[i]) > 1e100 || fabs(y[i]) > 1e100 || !isfinite(x[i]) || !isfinite(y[i])) { x[i] = 0.0; y[i] = 0.0; }
        if (!isfinite(m[i]) || m[i] <= 0.0) m[i] = 1.0;
    }
    for (int64_t i = 0; i < n; i++) { ax[i] = 0.0; ay[i] = 0.0; }
    if (t->n_nodes == 0) return;
    int64_t st = gxo_num_moments(p);
    double *mult = (double *)malloc(sizeof(double) * st * t->n_nodes);
    double *loc = (double *)calloc((size_t)(st * t->n_nodes), sizeof(double));
    gxo_p2m(x, y, m, t, p, mult);
    gxo_m2m(mult, t, p);
    gxo_m2l(loc, mult, v, t, p, eps, mode == 0 ? 0 : 1);
    gxo_l2l(loc, t, p, mode == 0 ? 0 : 1);
    gxo_l2p(x, y, ax, ay, loc, t, p);
    gxo_p2p(x, y, m, ax, ay, t, u, eps);
    free(mult); free(loc);
}

/* ----------------------------------------------- N^2, diagnostics, integrator */

/* compute_n2_force (lib.rs:1685-1721) */
void gxo_n2_force(const double *x, const double *y, const double *m, int64_t n, double eps, double *ax,
                  double *ay) {
    double s2 = eps * eps;
#pragma omp parallel for schedule(static) num_threads(gxo_get_threads())
    for (int64_t i = 0; i < n; i++) {
        double fx = 0.0, fy = 0.0, xi = x[i], yi = y[i];
        for (int64_t j = 0; j < n; j++) {
            if (i == j) continue;
            double dx = x[j] - xi, dy = y[j] - yi;
            double r2 = dx * dx + dy * dy + s2;
            double ir = 1.0 / sqrt(r2);
            double ir3 = ir * ir * ir;
            double f = m[j] * ir3;
            fx += f * dx;
            fy += f * dy;
        }
        ax[i] = fx;
        ay[i] = fy;
    }
}

/* validate_fmm's exact sum (lib.rs:1537-1553) for the sampled targets */
void gxo_n2_sampled(const double *x, const double *y, const double *m, int64_t n, double eps, const int64_t *idx,
                    int64_t n_idx, double *ax, double *ay) {
    double s2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 4) num_threads(gxo_get_threads())
    for (int64_t q = 0; q < n_idx; q++) {
        int64_t i = idx[q];
        double fx = 0.0, fy = 0.0;
        for (int64_t j = 0; j < n; j++) {
            if (j == i) continue;
            double dx = x[j] - x[i], dy = y[j] - y[i];
            double r2 = dx * dx + dy * dy + s2;
            double ir3 = powi_rs(1.0 / sqrt(r2), 3);
            double f = m[j] * ir3;
            fx += f * dx;
            fy += f * dy;
        }
        ax[q] = fx;
        ay[q] = fy;
    }
}

/* compute_kinetic_energy (lib.rs:1638-1645) */
double gxo_kinetic_energy(const double *m, const double *vx, const double *vy, int64_t n) {
    double ke = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double v2 = vx[i] * vx[i] + vy[i] * vy[i];
        ke += 0.5 * m[i] * v2;
    }
    return ke;
}

/* compute_momentum (lib.rs:1648-1656) */
void gxo_momentum(const double *m, const double *vx, const double *vy, int64_t n, double *px, double *py) {
    double a = 0.0, b = 0.0;
    for (int64_t i = 0; i < n; i++) { a += m[i] * vx[i]; b += m[i] * vy[i]; }
    *px = a; *py = b;
}

/* compute_angular_momentum (lib.rs:1659-1665) */
double gxo_angular_momentum(const double *m, const double *x, const double *y, const double *vx, const double *vy,
                            int64_t n) {
    double l = 0.0;
    for (int64_t i = 0; i < n; i++) l += m[i] * (x[i] * vy[i] - y[i] * vx[i]);
    return l;
}

/* compute_fmm_potential_energy (lib.rs:1671-1683) */
double gxo_fmm_potential_energy(const double *m, const double *x, const double *y, const double *ax,
                                const double *ay, int64_t n) {
    double pe = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double am = sqrt(ax[i] * ax[i] + ay[i] * ay[i]);
        double r = fmax_rs(sqrt(x[i] * x[i] + y[i] * y[i]), 1.0);
        pe += m[i] * am * r;
    }
    return -0.5 * pe;
}

/* leapfrog_kdk + simulate (galax-integrate/src/lib.rs:158-237) */
int64_t gxo_simulate(double *x, double *y, double *vx, double *vy, double *m, double *ax, double *ay,
                     const gxo_tree *t, const gxo_lists *v, const gxo_lists *u, int64_t p, double eps, double dt,
                     int64_t n_steps, int64_t energy_every, int mode, double *diag) {
    int64_t n = t->n_nodes > 0 ? t->body_end[t->n_nodes - 1] : 0;
    double h = 0.5 * dt;
    int64_t nd = 0;
    for (int64_t step = 0; step < n_steps; step++) {
        for (int64_t i = 0; i < n; i++) { vx[i] += ax[i] * h; vy[i] += ay[i] * h; }
        for (int64_t i = 0; i < n; i++) { x[i] += vx[i] * dt; y[i] += vy[i] * dt; }
        gxo_compute_fmm_force(x, y, m, ax, ay, t, v, u, p, eps, mode);
        for (int64_t i = 0; i < n; i++) { vx[i] += ax[i] * h; vy[i] += ay[i] * h; }
        if (energy_every > 0 && (step + 1) % energy_every == 0) {
            double *d = diag + 6 * nd;
            d[0] = (double)(step + 1);
            d[1] = gxo_kinetic_energy(m, vx, vy, n);
            d[2] = gxo_fmm_potential_energy(m, x, y, ax, ay, n);
            gxo_momentum(m, vx, vy, n, &d[3], &d[4]);
            d[5] = gxo_angular_momentum(m, x, y, vx, vy, n);
            nd++;
        }
    }
    return nd;
}

/* softening default (galax-cli/src/main.rs:182-190) */
double gxo_cli_softening(const double *x, const double *y, int64_t n) {
    if (n <= 0) return 0.0;
    int64_t k = n < 1000 ? n : 1000;
    double sum = 0.0;
    for (int64_t i = 0; i < k; i++) {
        double dx = x[i] - x[(i + 1) % n], dy = y[i] - y[(i + 1) % n];
        sum += sqrt(dx * dx + dy * dy);
    }
    return sum / (double)k * 0.1;
}

/* ------------------------------------------------------------ accurate mode */

void gxo_csr_free(gxo_csr *c) {
    if (!c) return;
    free(c->off); free(c->idx); free(c);
}

/* R_leaf = max |x_i - com|; R_parent = max over children (|com_c - com_P| + R_c).
 * Distances are sqrt(dx*dx + dy*dy) with separately rounded operations so that
 * the GPU computes the same bits. */
void gxo_node_radii(const double *x, const double *y, const gxo_tree *t, double *radius) {
    for (int64_t id = 0; id < t->n_nodes; id++) {
        double r = 0.0;
        if (t->is_leaf[id]) {
            for (int64_t b = t->body_start[id]; b < t->body_end[id]; b++) {
                double ex = x[b] - t->comx[id], ey = y[b] - t->comy[id];
                double d = sqrt(ex * ex + ey * ey);
                if (d > r) r = d;
            }
        } else {
            for (int k = 0; k < 4; k++) {
                int32_t c = t->child[4 * id + k];
                if (c < 0) continue;
                double ex = t->comx[c] - t->comx[id], ey = t->comy[c] - t->comy[id];
                double d = sqrt(ex * ex + ey * ey) + radius[c];
                if (d > r) r = d;
            }
        }
        radius[id] = r;
    }
}

typedef struct { int64_t n, cap; int32_t *v; } ivec;
static void iv_push(ivec *a, int32_t x) {
    if (a->n + 1 > a->cap) { a->cap = a->cap * 2 + 64; a->v = (int32_t *)realloc(a->v, sizeof(int32_t) * a->cap); }
    a->v[a->n++] = x;
}

/* far when |com_a - com_b| theta > R_a + R_b, decided in float and compared squared:
 * the COM offset from the float (hi, lo) split of each COM (hi = (float)c,
 * lo = (float)(c - hi)), the radii rounded to float once -- the device plan does the
 * same separately rounded float operations (-ffp-contract=off here) */
typedef struct { float xh, xl, yh, yl; } hl4;
static int mac_far(const hl4 *hl, const float *R32, int64_t a, int64_t b, float theta2) {
    float ex = (hl[a].xh - hl[b].xh) + (hl[a].xl - hl[b].xl);
    float ey = (hl[a].yh - hl[b].yh) + (hl[a].yl - hl[b].yl);
    float d2 = ex * ex + ey * ey;
    float s = R32[a] + R32[b];
    return d2 * theta2 > s * s;
}

void gxo_mac_lists_build(const gxo_tree *t, const double *R, double theta, gxo_csr **far_out, gxo_csr **near_out) {
    int64_t nn = t->n_nodes;
    gxo_csr *far = (gxo_csr *)calloc(1, sizeof(gxo_csr)), *near = (gxo_csr *)calloc(1, sizeof(gxo_csr));
    far->n = near->n = nn;
    far->off = (int64_t *)calloc((size_t)(nn + 1), sizeof(int64_t));
    near->off = (int64_t *)calloc((size_t)(nn + 1), sizeof(int64_t));
    /* per-node vectors, filled top-down (descending id = parents first) */
    ivec *fv = (ivec *)calloc((size_t)(nn > 0 ? nn : 1), sizeof(ivec));
    ivec *nv = (ivec *)calloc((size_t)(nn > 0 ? nn : 1), sizeof(ivec));
    if (nn > 0) iv_push(&nv[nn - 1], (int32_t)(nn - 1)); /* the root is near itself */
    const float thf = (float)theta;
    const float theta2 = thf * thf;
    hl4 *hl = (hl4 *)malloc(sizeof(hl4) * (size_t)(nn > 0 ? nn : 1));
    float *R32 = (float *)malloc(sizeof(float) * (size_t)(nn > 0 ? nn : 1));
    for (int64_t i = 0; i < nn; i++) {
        float xh = (float)t->comx[i], yh = (float)t->comy[i];
        hl[i].xh = xh;
        hl[i].xl = (float)(t->comx[i] - (double)xh);
        hl[i].yh = yh;
        hl[i].yl = (float)(t->comy[i] - (double)yh);
        R32[i] = (float)R[i];
    }
    /* A node that is its parent's only child, against a candidate that is the only child
     * of its parent, holds the same bodies as the parent pair (y, P), which was near:
     * the pair stays near without a test (its COMs and radii differ from the parents'
     * only by rounding).  Morton rounds leave whole levels of such single-child chains
     * over the leaves; the device plan skips them with this rule. */
    for (int64_t id = nn - 1; id >= 0; id--) {
        int32_t P = t->parent[id];
        if (P < 0) continue;
        const int only_child = t->child[4 * P + 1] < 0;
        for (int64_t q = 0; q < nv[P].n; q++) {
            int32_t y = nv[P].v[q];
            const int y_single = t->child[4 * y + 1] < 0;
            for (int k = 0; k < 4; k++) {
                int32_t c = t->child[4 * y + k];
                if (c < 0) continue;
                if (!(only_child && y_single) && mac_far(hl, R32, id, c, theta2)) iv_push(&fv[id], c);
                else iv_push(&nv[id], c);
            }
        }
    }
    int64_t tf = 0, tn = 0;
    for (int64_t id = 0; id < nn; id++) {
        far->off[id] = tf; tf += fv[id].n;
        near->off[id] = tn; tn += t->is_leaf[id] ? nv[id].n : 0;
    }
    far->off[nn] = tf; near->off[nn] = tn;
    far->idx = (int32_t *)malloc(sizeof(int32_t) * (tf + 1));
    near->idx = (int32_t *)malloc(sizeof(int32_t) * (tn + 1));
    for (int64_t id = 0; id < nn; id++) {
        if (fv[id].n) memcpy(far->idx + far->off[id], fv[id].v, sizeof(int32_t) * fv[id].n);
        if (t->is_leaf[id] && nv[id].n) memcpy(near->idx + near->off[id], nv[id].v, sizeof(int32_t) * nv[id].n);
        free(fv[id].v); free(nv[id].v);
    }
    free(fv); free(nv);
    *far_out = far;
    *near_out = near;
    free(hl);
    free(R32);
}

/* The leaf-level split of the near lists (not in the reference).  A near pair
 * (a <- s), s != a, whose target bodies all see the source leaf from at least
 * d - R_a, with (d - R_a) theta_w > R_s, takes the source leaf's multipole evaluated at
 * each target body (M2P); failing that, one whose source bodies all lie at least d - R_s
 * from com_a, with (d - R_s) theta_w > R_a, adds them to the target leaf's local
 * expansion (P2L); the rest, and the leaf itself, stay P2P.  Both tests bound the
 * truncation by theta_w^(p+1), as the far test bounds M2L's.  Decided in float and
 * squared like mac_far, with the same COM offsets and float radii:
 *   M2P: d2 theta_w^2 > (R_s + theta_w R_a)^2,  P2L: d2 theta_w^2 > (R_a + theta_w R_s)^2.
 * List order is kept within each output list. */
void gxo_near_split(const gxo_tree *t, const double *R, double theta_w, const gxo_csr *near, gxo_csr **p2p_out,
                    gxo_csr **m2p_out, gxo_csr **p2l_out) {
    int64_t nn = t->n_nodes;
    gxo_csr *o[3];
    for (int k = 0; k < 3; k++) {
        o[k] = (gxo_csr *)calloc(1, sizeof(gxo_csr));
        o[k]->n = nn;
        o[k]->off = (int64_t *)calloc((size_t)(nn + 1), sizeof(int64_t));
        o[k]->idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(near->off[nn] + 1));
    }
    hl4 *hl = (hl4 *)malloc(sizeof(hl4) * (size_t)(nn > 0 ? nn : 1));
    float *R32 = (float *)malloc(sizeof(float) * (size_t)(nn > 0 ? nn : 1));
    for (int64_t i = 0; i < nn; i++) {
        float xh = (float)t->comx[i], yh = (float)t->comy[i];
        hl[i].xh = xh;
        hl[i].xl = (float)(t->comx[i] - (double)xh);
        hl[i].yh = yh;
        hl[i].yl = (float)(t->comy[i] - (double)yh);
        R32[i] = (float)R[i];
    }
    const float tw = (float)theta_w, tw2 = tw * tw;
    int64_t cnt[3] = {0, 0, 0};
    for (int64_t a = 0; a < nn; a++) {
        for (int k = 0; k < 3; k++) o[k]->off[a] = cnt[k];
        for (int64_t q = near->off[a]; q < near->off[a + 1]; q++) {
            int32_t s = near->idx[q];
            int kind = 0;
            if (s != a && theta_w > 0.0) {
                float ex = (hl[a].xh - hl[s].xh) + (hl[a].xl - hl[s].xl);
                float ey = (hl[a].yh - hl[s].yh) + (hl[a].yl - hl[s].yl);
                float d2 = ex * ex + ey * ey;
                float lhs = d2 * tw2;
                float sm = R32[s] + tw * R32[a];
                float sl = R32[a] + tw * R32[s];
                if (lhs > sm * sm) kind = 1;
                else if (lhs > sl * sl) kind = 2;
            }
            o[kind]->idx[cnt[kind]++] = s;
        }
    }
    for (int k = 0; k < 3; k++) o[k]->off[nn] = cnt[k];
    *p2p_out = o[0];
    *m2p_out = o[1];
    *p2l_out = o[2];
    free(hl);
    free(R32);
}

void gxo_compute_fmm_force_mac(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                               const gxo_csr *far, const gxo_csr *near, int64_t p, double eps) {
    gxo_compute_fmm_force_wx(x, y, m, ax, ay, t, far, near, NULL, NULL, p, eps);
}

/* gxo_compute_fmm_force_mac with the split near lists: P2L into the leaf locals after
 * the top-down L2L, L2P, M2P onto the bodies, then P2P over `near` (the remaining
 * pairs).  m2p / p2l may be NULL.
 *   M2P: a(x) = -sum_S (-1)^|S| M_s[S] G^(S+e)(x - com_s)   (e = e_x, e_y; G the
 *        reference's derivatives of -1/R, lib.rs:1040-1151)
 *   P2L: L_a[T] += m_j G^(T)(com_a - x_j) / T!   (M2L of a point mass, lib.rs:1199-1259) */
void gxo_compute_fmm_force_wx(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                              const gxo_csr *far, const gxo_csr *near, const gxo_csr *m2p, const gxo_csr *p2l,
                              int64_t p, double eps) {
    gxo_compute_fmm_force_wxb(x, y, m, ax, ay, t, far, near, m2p, p2l, p, eps, NULL, 0.0);
}

/* Body-level P2L of a P2P pair (a <- s), s != a (not in the reference): a source body j
 * of s with |x_j - com_a| theta_b > R_a goes into a's local expansion instead of P2P, the
 * truncation bounded by theta_b^(p+1) as the leaf-level P2L's.  Decided in float,
 * squared, with separately rounded operations: the offset is (x_j - com_s) + (com_s -
 * com_a), each difference formed in double and rounded once, as the device forms it. */
int gxo_body_p2l(const double *x, const double *y, const gxo_tree *t, const double *R, int64_t a, int64_t s,
                 int64_t j, double theta_b) {
    const float ox = (float)(x[j] - t->comx[s]), oy = (float)(y[j] - t->comy[s]);
    const float hx = (float)(t->comx[s] - t->comx[a]), hy = (float)(t->comy[s] - t->comy[a]);
    const float ex = ox + hx, ey = oy + hy;
    const float d2 = ex * ex + ey * ey;
    const float tb = (float)theta_b, tb2 = tb * tb, ra = (float)R[a];
    return d2 * tb2 > ra * ra;
}

/* gxo_compute_fmm_force_wx, and with theta_b > 0 (R the node radii) the body-level P2L
 * of the P2P pairs: those source bodies join the P2L sums and leave P2P. */
void gxo_compute_fmm_force_wxb(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                               const gxo_csr *far, const gxo_csr *near, const gxo_csr *m2p, const gxo_csr *p2l,
                               int64_t p, double eps, const double *R, double theta_b) {
    init_tables();
    const int body_split = R != NULL && theta_b > 0.0;
    int64_t n = t->n_nodes > 0 ? t->body_end[t->n_nodes - 1] : 0;
    for (int64_t i = 0; i < n; i++) {
        if (fabs(x[i]) > 1e100 || fabs(y[i]) > 1e100 || !isfinite(x[i]) || !isfinite(y[i])) { x[i] = 0.0; y[i] = 0.0; }
        if (!isfinite(m[i]) || m[i] <= 0.0) m[i] = 1.0;
    }
    for (int64_t i = 0; i < n; i++) { ax[i] = 0.0; ay[i] = 0.0; }
    if (t->n_nodes == 0) return;
    int64_t st = gxo_num_moments(p), DS = (2 * p + 1) * (2 * p + 1);
    double *mult = (double *)malloc(sizeof(double) * st * t->n_nodes);
    double *loc = (double *)calloc((size_t)(st * t->n_nodes), sizeof(double));
    gxo_p2m(x, y, m, t, p, mult);
    gxo_m2m(mult, t, p);
    m2l_term plan[GXO_MAX_P * GXO_MAX_P * GXO_MAX_P * GXO_MAX_P / 4 + 64];
    int64_t np = m2l_plan(p, plan);
#pragma omp parallel num_threads(gxo_get_threads())
    {
        double *G = (double *)malloc(sizeof(double) * DS);
#pragma omp for schedule(dynamic, 64)
        for (int64_t id = 0; id < t->n_nodes; id++) {
            double *L = loc + id * st;
            for (int64_t q = far->off[id]; q < far->off[id + 1]; q++) {
                int64_t src = far->idx[q];
                const double *M = mult + src * st;
                gxo_kernel_derivs_recurrence(t->comx[id] - t->comx[src], t->comy[id] - t->comy[src], eps, p, G);
                for (int64_t k = 0; k < np; k++) L[plan[k].tgt] += M[plan[k].src] * plan[k].w * G[plan[k].di];
            }
        }
        free(G);
    }
    gxo_l2l(loc, t, p, 1);
    if (body_split) {
        /* sanitising happened above, so the tests here and in P2P see the same positions */
#pragma omp parallel num_threads(gxo_get_threads())
        {
            double *G = (double *)malloc(sizeof(double) * DS);
#pragma omp for schedule(dynamic, 16)
            for (int64_t id = 0; id < t->n_nodes; id++) {
                double *L = loc + id * st;
                for (int64_t q = near->off[id]; q < near->off[id + 1]; q++) {
                    int64_t s = near->idx[q];
                    if (s == id) continue;
                    for (int64_t j = t->body_start[s]; j < t->body_end[s]; j++) {
                        if (!gxo_body_p2l(x, y, t, R, id, s, j, theta_b)) continue;
                        gxo_kernel_derivs_recurrence(t->comx[id] - x[j], t->comy[id] - y[j], eps, p, G);
                        for (int64_t oi = 0; oi <= p; oi++)
                            for (int64_t oj = 0; oj <= p - oi; oj++)
                                L[MI(oi, oj)] += m[j] * G[kdi(oi, oj, p)] / (g_fact[oi] * g_fact[oj]);
                    }
                }
            }
            free(G);
        }
    }
    if (p2l) {
#pragma omp parallel num_threads(gxo_get_threads())
        {
            double *G = (double *)malloc(sizeof(double) * DS);
#pragma omp for schedule(dynamic, 16)
            for (int64_t id = 0; id < t->n_nodes; id++) {
                double *L = loc + id * st;
                for (int64_t q = p2l->off[id]; q < p2l->off[id + 1]; q++) {
                    int64_t s = p2l->idx[q];
                    for (int64_t j = t->body_start[s]; j < t->body_end[s]; j++) {
                        gxo_kernel_derivs_recurrence(t->comx[id] - x[j], t->comy[id] - y[j], eps, p, G);
                        for (int64_t oi = 0; oi <= p; oi++)
                            for (int64_t oj = 0; oj <= p - oi; oj++)
                                L[MI(oi, oj)] += m[j] * G[kdi(oi, oj, p)] / (g_fact[oi] * g_fact[oj]);
                    }
                }
            }
            free(G);
        }
    }
    gxo_l2p(x, y, ax, ay, loc, t, p);
    if (m2p) {
        const int64_t pp = (p + 2) / 2; /* derivative orders up to 2 pp >= p + 1 */
        const int64_t DSp = (2 * pp + 1) * (2 * pp + 1);
#pragma omp parallel num_threads(gxo_get_threads())
        {
            double *G = (double *)malloc(sizeof(double) * DSp);
#pragma omp for schedule(dynamic, 16)
            for (int64_t id = 0; id < t->n_nodes; id++) {
                if (!t->is_leaf[id]) continue;
                for (int64_t i = t->body_start[id]; i < t->body_end[id]; i++) {
                    double fx = 0.0, fy = 0.0;
                    for (int64_t q = m2p->off[id]; q < m2p->off[id + 1]; q++) {
                        int64_t s = m2p->idx[q];
                        const double *M = mult + s * st;
                        gxo_kernel_derivs_recurrence(x[i] - t->comx[s], y[i] - t->comy[s], eps, pp, G);
                        for (int64_t si = 0; si <= p; si++)
                            for (int64_t sj = 0; sj <= p - si; sj++) {
                                double mv = ((si + sj) & 1) ? -M[MI(si, sj)] : M[MI(si, sj)];
                                fx += mv * G[kdi(si + 1, sj, pp)];
                                fy += mv * G[kdi(si, sj + 1, pp)];
                            }
                    }
                    ax[i] -= fx;
                    ay[i] -= fy;
                }
            }
            free(G);
        }
    }
    double s2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(gxo_get_threads())
    for (int64_t id = 0; id < t->n_nodes; id++) {
        if (!t->is_leaf[id]) continue;
        for (int64_t i = t->body_start[id]; i < t->body_end[id]; i++) {
            double fx = 0.0, fy = 0.0;
            for (int64_t q = near->off[id]; q < near->off[id + 1]; q++) {
                int64_t s = near->idx[q];
                const int split_s = body_split && s != id;
                for (int64_t j = t->body_start[s]; j < t->body_end[s]; j++) {
                    if (j == i) continue;
                    if (split_s && gxo_body_p2l(x, y, t, R, id, s, j, theta_b)) continue;
                    double dx = x[j] - x[i], dy = y[j] - y[i];
                    double r2 = dx * dx + dy * dy + s2;
                    double ir = 1.0 / sqrt(r2);
                    fx += m[j] * ir * ir * ir * dx;
                    fy += m[j] * ir * ir * ir * dy;
                }
            }
            ax[i] += fx;
            ay[i] += fy;
        }
    }
    free(mult); free(loc);
}

/* ------------------------------------------------------------ N^2 adjoint
 * Not in the reference (it has no gradients): the exact FP64 vector-Jacobian product
 * of the softened N^2 accelerations (compute_n2_force, lib.rs:1685-1721) and the
 * reverse leapfrog over it, used as the reference gradient of the GPU adjoint.
 *   a_i = sum_{k != i} m_k K(x_k - x_i),  K(d) = d (|d|^2+eps^2)^(-3/2)
 *   g_x,i = sum_k J(x_k - x_i) (m_i lam_k - m_k lam_i),  J = I/r^3 - 3 d d^T/r^5
 *   g_m,i = -sum_k lam_k . (x_k - x_i)/r^3 */
void gxo_n2_vjp(const double *x, const double *y, const double *m, int64_t n, double eps, const double *lx,
                const double *ly, double *gx, double *gy, double *gm) {
    double s2 = eps * eps;
#pragma omp parallel for schedule(static) num_threads(gxo_get_threads())
    for (int64_t i = 0; i < n; i++) {
        double ax = 0.0, ay = 0.0, am = 0.0;
        for (int64_t k = 0; k < n; k++) {
            if (k == i) continue;
            double dx = x[k] - x[i], dy = y[k] - y[i];
            double r2 = dx * dx + dy * dy + s2;
            double ir = 1.0 / sqrt(r2);
            double ir3 = ir * ir * ir, ir5 = ir3 * ir * ir;
            double wx = m[i] * lx[k] - m[k] * lx[i], wy = m[i] * ly[k] - m[k] * ly[i];
            double dw = dx * wx + dy * wy;
            ax += ir3 * wx - 3.0 * ir5 * dx * dw;
            ay += ir3 * wy - 3.0 * ir5 * dy * dw;
            am -= (lx[k] * dx + ly[k] * dy) * ir3;
        }
        gx[i] = ax;
        gy[i] = ay;
        gm[i] = am;
    }
}

/* Gradient at step 0 of a scalar loss of the final state for the N^2 leapfrog
 * (leapfrog_kdk_n2, galax-integrate/src/lib.rs:241-255) from the final-state
 * cotangents; all states are kept (small n). */
void gxo_n2_rollout_grad(const double *x0, const double *y0, const double *vx0, const double *vy0, const double *m,
                         int64_t n, double eps, double dt, int64_t T, const double *lxT, const double *lyT,
                         const double *lvxT, const double *lvyT, double *gx, double *gy, double *gvx, double *gvy,
                         double *gm) {
    double h = 0.5 * dt;
    double *X = (double *)malloc(sizeof(double) * n * (T + 1)), *Y = (double *)malloc(sizeof(double) * n * (T + 1));
    double *vx = (double *)malloc(sizeof(double) * n), *vy = (double *)malloc(sizeof(double) * n);
    double *ax = (double *)malloc(sizeof(double) * n), *ay = (double *)malloc(sizeof(double) * n);
    memcpy(X, x0, sizeof(double) * n);
    memcpy(Y, y0, sizeof(double) * n);
    memcpy(vx, vx0, sizeof(double) * n);
    memcpy(vy, vy0, sizeof(double) * n);
    gxo_n2_force(X, Y, m, n, eps, ax, ay);
    for (int64_t s = 0; s < T; s++) {
        double *xp = X + s * n, *yp = Y + s * n, *xn = X + (s + 1) * n, *yn = Y + (s + 1) * n;
        for (int64_t i = 0; i < n; i++) {
            vx[i] += ax[i] * h;
            vy[i] += ay[i] * h;
            xn[i] = xp[i] + vx[i] * dt;
            yn[i] = yp[i] + vy[i] * dt;
        }
        gxo_n2_force(xn, yn, m, n, eps, ax, ay);
        for (int64_t i = 0; i < n; i++) {
            vx[i] += ax[i] * h;
            vy[i] += ay[i] * h;
        }
    }
    double *lax = (double *)malloc(sizeof(double) * n), *lay = (double *)malloc(sizeof(double) * n);
    double *tx = (double *)malloc(sizeof(double) * n), *ty = (double *)malloc(sizeof(double) * n);
    double *tm = (double *)malloc(sizeof(double) * n);
    memcpy(gx, lxT, sizeof(double) * n);
    memcpy(gy, lyT, sizeof(double) * n);
    memcpy(gvx, lvxT, sizeof(double) * n);
    memcpy(gvy, lvyT, sizeof(double) * n);
    memset(gm, 0, sizeof(double) * n);
    for (int64_t s = T - 1; s >= -1; s--) {
        double c = (s == T - 1) ? h : dt;
        if (s == -1) c = h;
        for (int64_t i = 0; i < n; i++) { lax[i] = c * gvx[i]; lay[i] = c * gvy[i]; }
        gxo_n2_vjp(X + (s + 1) * n, Y + (s + 1) * n, m, n, eps, lax, lay, tx, ty, tm);
        for (int64_t i = 0; i < n; i++) { gx[i] += tx[i]; gy[i] += ty[i]; gm[i] += tm[i]; }
        if (s >= 0)
            for (int64_t i = 0; i < n; i++) { gvx[i] += dt * gx[i]; gvy[i] += dt * gy[i]; }
    }
    free(X); free(Y); free(vx); free(vy); free(ax); free(ay); free(lax); free(lay); free(tx); free(ty); free(tm);
}
