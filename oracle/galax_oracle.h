/*
 * galax_oracle.h -- CPU restatement of galax-core's FMM force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * galax_gb300/: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference leg may load it.  The product never links it.
 *
 * Every function restates an item of the reference (knekvasil/galax, Rust) and
 * cites the file:line it follows.  The reference itself cannot be compiled in
 * this environment (no Rust toolchain), so parity of this restatement is pinned
 * by the reference's own known-answer tests (restated in tests/test_oracle_*.py)
 * and is otherwise "parity unpinned" against the reference binary.
 *
 * Arithmetic rules followed throughout (they matter for bit-exact topology):
 *   - compiled with -ffp-contract=off: no FMA contraction, like rustc;
 *   - every sum is taken in the reference's order;
 *   - f64 -> integer casts saturate and map NaN to 0, like Rust `as`.
 */
#ifndef GALAX_ORACLE_H
#define GALAX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GXO_MAX_P 17
#define GXO_LIST_CAP 64

/* Tree as built by Tree::build (galax-core/src/lib.rs:163-361). */
typedef struct gxo_tree {
    int64_t n_nodes;
    int64_t cap;
    double *cx, *cy, *hw, *mass, *comx, *comy;
    int64_t *body_start, *body_end;
    int32_t *child;      /* 4 per node, -1 = None, slot order as in Node::children */
    int32_t *parent;     /* -1 = None */
    uint8_t *is_leaf;
    int32_t n_levels;    /* number of rounds + 1; level == round index */
    int64_t *level_start;/* n_levels + 1 entries; level L = ids [level_start[L], level_start[L+1]) */
    int64_t n_max;
    double xmin, xmax, ymin, ymax;
} gxo_tree;

/* Fixed-capacity interaction lists, the reference layout
 * (InteractionLists{data:[[u32;64]], lengths:[u8]}, lib.rs:941-944). */
typedef struct gxo_lists {
    int64_t n_nodes;
    uint32_t *data;      /* n_nodes * 64, unused slots = 0xFFFFFFFF */
    uint8_t *lengths;
} gxo_lists;

/* ---- Morton (lib.rs:73-115) ---- */
uint64_t gxo_morton_encode(double x, double y, double xmin, double xmax, double ymin, double ymax);
void gxo_morton_decode(uint64_t key, double xmin, double xmax, double ymin, double ymax, double *x, double *y);
void gxo_morton_encode_many(const double *x, const double *y, int64_t n, double xmin, double xmax,
                            double ymin, double ymax, uint64_t *keys);

/* ---- Tree (lib.rs:163-361, 541-694) ---- */
/* Tree::build: permutes the 7 arrays in place (stable sort by Morton key). */
gxo_tree *gxo_tree_build(double *x, double *y, double *vx, double *vy, double *m, double *ax, double *ay,
                         int64_t n, int64_t n_max, double xmin, double xmax, double ymin, double ymax);
/* build_with_constraints: no sort; extra leaf boundaries at sorted `splits`. */
gxo_tree *gxo_tree_build_with_constraints(const double *x, const double *y, const double *m, int64_t n,
                                          int64_t n_max, double xmin, double xmax, double ymin,
                                          double ymax, const int64_t *splits, int64_t n_splits);
/* build_constrained: 2:1 iterative rebuild.  accel=0: literal O(nodes) neighbour
 * scans; accel=1: output-identical bounding-volume search. */
gxo_tree *gxo_tree_build_constrained(const double *x, const double *y, const double *m, int64_t n,
                                     int64_t n_max, double xmin, double xmax, double ymin, double ymax,
                                     int accel);
void gxo_tree_free(gxo_tree *t);
/* neighbors_geometric (lib.rs:382-423); out[8], -1 = None */
void gxo_neighbors_geometric(const gxo_tree *t, int32_t node, int32_t *out);
/* compute_levels (lib.rs:426-438) */
void gxo_compute_levels(const gxo_tree *t, uint32_t *levels);

/* ---- Lists (lib.rs:947-1025, 1358-1392) ---- */
gxo_lists *gxo_vlist_build(const gxo_tree *t, int accel);
gxo_lists *gxo_ulist_build(const gxo_tree *t, int accel);
void gxo_lists_free(gxo_lists *l);

/* ---- Passes (lib.rs:825-1462) ---- */
int64_t gxo_num_moments(int64_t p);
int64_t gxo_moment_index(int64_t i, int64_t j);
void gxo_p2m(const double *x, const double *y, const double *m, const gxo_tree *t, int64_t p, double *mult);
void gxo_m2m(double *mult, const gxo_tree *t, int64_t p);
/* compute_kernel_derivs (lib.rs:1040-1151): out has (2p+1)^2 entries */
void gxo_kernel_derivs(double dx, double dy, double eps, int64_t p, double *out);
/* Recurrence-based derivatives of G = -1/sqrt(r^2+eps^2) (not in the reference;
 * used to cross-check the polynomial form).  Same (2p+1)^2 layout. */
void gxo_kernel_derivs_recurrence(double dx, double dy, double eps, int64_t p, double *out);
/* m2l (lib.rs:1199-1259). deriv_mode 0 = REF (single-threaded first-inserter
 * cache keyed on (dx as i64, dy as i64)); 1 = EXACT (derivatives per pair). */
void gxo_m2l(double *locals, const double *mult, const gxo_lists *v, const gxo_tree *t, int64_t p,
             double eps, int deriv_mode);
/* REF cache analysis: per pair in global (target asc, slot) order, the index of the
 * unique key it maps to; per unique key, the (dx,dy) of its first pair. Returns n_keys. */
int64_t gxo_m2l_ref_keys(const gxo_lists *v, const gxo_tree *t, int32_t *pair_key, double *key_dxdy,
                         int64_t max_keys);
/* l2l (lib.rs:1262-1302). order 0 = REF (node id ascending), 1 = top-down. */
void gxo_l2l(double *locals, const gxo_tree *t, int64_t p, int order);
void gxo_l2p(const double *x, const double *y, double *ax, double *ay, const double *locals,
             const gxo_tree *t, int64_t p);
void gxo_p2p(const double *x, const double *y, const double *m, double *ax, double *ay, const gxo_tree *t,
             const gxo_lists *u, double eps);
/* compute_fmm_force (lib.rs:1466-1499).  Sanitises x, y, m in place like the reference.
 * mode: 0 = REF, 1 = EXACT derivatives + top-down L2L. */
void gxo_compute_fmm_force(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                           const gxo_lists *v, const gxo_lists *u, int64_t p, double eps, int mode);

/* ---- Oracle, diagnostics, integrator ---- */
void gxo_n2_force(const double *x, const double *y, const double *m, int64_t n, double eps, double *ax,
                  double *ay);
/* Exact force for selected targets with validate_fmm's inner loop (lib.rs:1537-1553). */
void gxo_n2_sampled(const double *x, const double *y, const double *m, int64_t n, double eps,
                    const int64_t *idx, int64_t n_idx, double *ax, double *ay);
double gxo_kinetic_energy(const double *m, const double *vx, const double *vy, int64_t n);
void gxo_momentum(const double *m, const double *vx, const double *vy, int64_t n, double *px, double *py);
double gxo_angular_momentum(const double *m, const double *x, const double *y, const double *vx,
                            const double *vy, int64_t n);
double gxo_fmm_potential_energy(const double *m, const double *x, const double *y, const double *ax,
                                const double *ay, int64_t n);
/* simulate (galax-integrate/src/lib.rs:158-237): n_steps KDK steps with a static
 * tree; diag (n_steps/energy_every rows x 6: step, KE, PE, px, py, Lz). */
int64_t gxo_simulate(double *x, double *y, double *vx, double *vy, double *m, double *ax, double *ay,
                     const gxo_tree *t, const gxo_lists *v, const gxo_lists *u, int64_t p, double eps,
                     double dt, int64_t n_steps, int64_t energy_every, int mode, double *diag);
/* softening rule of galax-cli/src/main.rs:182-190 */
double gxo_cli_softening(const double *x, const double *y, int64_t n);

/* ---- Accurate mode (not in the reference) ----
 * Near/far classification on the same tree: top-down, a child pair (x, c) whose
 * parents are near is far (M2L) when |com_x - com_c| > (R_x + R_c)/theta, else near;
 * near leaf pairs are P2P.  R = bound on the distance from the COM to any body of
 * the subtree, from the positions at build time.  Every body pair is counted once. */
typedef struct gxo_csr { int64_t n; int64_t *off; int32_t *idx; } gxo_csr;
void gxo_node_radii(const double *x, const double *y, const gxo_tree *t, double *radius);
void gxo_mac_lists_build(const gxo_tree *t, const double *radius, double theta, gxo_csr **far_out,
                         gxo_csr **near_out);
void gxo_csr_free(gxo_csr *c);
/* p2m, m2m, m2l (exact derivatives over `far`), top-down l2l, l2p, gather P2P over
 * `near`.  Sanitises like compute_fmm_force. */
void gxo_compute_fmm_force_mac(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                               const gxo_csr *far, const gxo_csr *near, int64_t p, double eps);

/* Leaf-level split of the near lists into P2P, M2P and P2L (criterion theta_w, see the
 * source), and the evaluation with them; m2p / p2l may be NULL. */
void gxo_near_split(const gxo_tree *t, const double *R, double theta_w, const gxo_csr *near, gxo_csr **p2p_out,
                    gxo_csr **m2p_out, gxo_csr **p2l_out);
void gxo_compute_fmm_force_wx(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                              const gxo_csr *far, const gxo_csr *near, const gxo_csr *m2p, const gxo_csr *p2l,
                              int64_t p, double eps);
int gxo_body_p2l(const double *x, const double *y, const gxo_tree *t, const double *R, int64_t a, int64_t s,
                 int64_t j, double theta_b);
void gxo_compute_fmm_force_wxb(double *x, double *y, double *m, double *ax, double *ay, const gxo_tree *t,
                               const gxo_csr *far, const gxo_csr *near, const gxo_csr *m2p, const gxo_csr *p2l,
                               int64_t p, double eps, const double *R, double theta_b);

/* ---- N^2 adjoint (not in the reference; the reference gradient of the GPU adjoint) ---- */
void gxo_n2_vjp(const double *x, const double *y, const double *m, int64_t n, double eps, const double *lx,
                const double *ly, double *gx, double *gy, double *gm);
void gxo_n2_rollout_grad(const double *x0, const double *y0, const double *vx0, const double *vy0, const double *m,
                         int64_t n, double eps, double dt, int64_t T, const double *lxT, const double *lyT,
                         const double *lvxT, const double *lvyT, double *gx, double *gy, double *gvx, double *gvy,
                         double *gm);

void gxo_set_threads(int n);
int gxo_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
