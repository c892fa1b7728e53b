/*
 * galax_gb300.h -- C ABI of libgalaxcu.so, the GB300 (sm_103a) FMM force backend.
 *
 * This is the drop-in boundary for knekvasil/galax's GPU force backend
 * (galax-gpu/src/lib.rs, `GpuContext`).  Each entry point names the reference
 * interface it replaces.  Plain pointers and sizes only; all host arrays are
 * caller-owned FP64 structure-of-arrays and are touched only during the call;
 * device buffers are owned by the context.  One CUDA stream per context; a
 * context is not thread-safe (callers serialise calls on it), distinct contexts
 * are independent.  Nothing in the library traps or aborts on the device:
 * every call returns a gx_status and gx_last_error() gives the message.
 */
#ifndef GALAX_GB300_H
#define GALAX_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GX_ABI_VERSION 1

/* Status codes.  Mirrors GpuError (galax-gpu/src/lib.rs:42-59: InitFailed,
 * ShaderCompilation -> KERNEL_LOAD, BufferAllocation -> ALLOC) plus the
 * conditions the reference reports by panicking. */
typedef enum gx_status {
    GX_OK = 0,
    GX_ERR_INIT = 1,          /* no CUDA device / context creation failed */
    GX_ERR_KERNEL_LOAD = 2,   /* the sm_103a image does not load on this device */
    GX_ERR_ALLOC = 3,         /* device or pinned-host allocation failed */
    GX_ERR_INVALID_ARG = 4,   /* bad pointer, size, order p, mode ... */
    GX_ERR_NONFINITE = 5,     /* non-finite values were met (not fatal; see gx_last_status) */
    GX_ERR_CAP_EXCEEDED = 6,  /* a size is beyond the configured maximum */
    GX_ERR_TIMEOUT = 7,       /* a bounded device wait gave up */
    GX_ERR_STATE = 8,         /* call out of order (e.g. forces before a tree) */
    GX_ERR_CUDA = 9           /* a CUDA runtime error; see gx_last_error */
} gx_status;

/* Evaluation modes. */
enum {
    GX_MODE_REF = 0,      /* galax-core semantics: capped V/U lists, first-inserter
                             derivative cache, node-id-ascending L2L (lib.rs:1466-1499) */
    GX_MODE_EXACT = 1,    /* REF lists, per-pair derivatives, top-down L2L */
    GX_MODE_ACCURATE = 2  /* MAC near/far lists on the same tree (theta), per-pair
                             derivatives, top-down L2L; not in the reference */
};
enum {
    GX_PREC_FP64 = 0,     /* FP64 end to end */
    GX_PREC_MIXED = 1     /* FP32 P2M/L2P/P2P, FP32 M2L; FP64 state and reductions */
};
/* gx_build_tree flags */
enum {
    GX_BUILD_BALANCED = 1 /* build_constrained (lib.rs:541-588) instead of Tree::build */
};
/* list selectors for gx_export_lists */
enum { GX_LIST_V = 0, GX_LIST_U = 1 };

/* GpuConfig (galax-gpu/src/lib.rs:22-40).  eps64 > 0 overrides the f32 eps. */
typedef struct gx_config {
    uint32_t max_n;             /* default 262144 */
    uint32_t max_nodes;         /* default 524288 */
    uint32_t max_interactions;  /* default 1<<24 */
    uint32_t p;                 /* expansion order, 0..16; default 4 */
    float eps;                  /* softening, f32 as in the reference; default 0.1 */
    double eps64;               /* FP64 softening; used when > 0 */
    int32_t device;             /* CUDA device ordinal; default 0 */
} gx_config;

typedef struct gx_ctx gx_ctx;

/* GpuConfig::default (galax-gpu/src/lib.rs:32-40). */
int gx_config_default(gx_config *cfg);

/* GpuContext::new (galax-gpu/src/lib.rs:268-390): creates the stream and checks
 * the kernel image; buffers grow on demand up to the configured maxima. */
int gx_create(const gx_config *cfg, gx_ctx **out);
int gx_destroy(gx_ctx *ctx);
const char *gx_last_error(const gx_ctx *ctx);
int gx_abi_version(void);

/* Evaluation mode, precision and MAC opening angle (theta, ACCURATE only). */
int gx_set_mode(gx_ctx *ctx, int mode, int precision, double theta);
/* The leaf-level split of the ACCURATE near lists (no counterpart in the reference,
 * whose U-list pairs are all P2P, galax-core/src/lib.rs:1395-1462).  With theta_w > 0 a
 * near leaf pair (target a, source s, s != a) whose target bodies all see s from
 * (d - R_a) with (d - R_a) theta_w > R_s evaluates s's multipole at each target body
 * (M2P); else one whose source bodies all lie (d - R_s) from a's centre of mass with
 * (d - R_s) theta_w > R_a adds them to a's local expansion (P2L); the rest stay P2P.
 * Both bound the truncation by theta_w^(p+1).  theta_w = 0 (the default) turns it off.
 * The adjoint entry points need it off. */
int gx_set_near_split(gx_ctx *ctx, double theta_w);
/* Leaf pairs of the current ACCURATE plan taken by M2P and by P2L (0 with the split off). */
int gx_plan_split_info(gx_ctx *ctx, int64_t *n_m2p_pairs, int64_t *n_p2l_pairs);
/* The body-level P2L of the P2P pairs left by the near-list split (no counterpart in the
 * reference).  With theta_b > 0, theta_w > 0 and leaves of at most 32 bodies, a source
 * body j of a P2P leaf pair (target a, source s, s != a) with |x_j - com_a| theta_b > R_a
 * goes into a's local expansion (truncation bounded by theta_b^(p+1)) instead of P2P;
 * decided per body in FP32 from the plan's positions, like the leaf-level tests.
 * theta_b = 0 (the default) turns it off; the adjoint entry points need the near-list
 * split, and with it this, off. */
int gx_set_body_split(gx_ctx *ctx, double theta_b);
/* Of the current ACCURATE plan: body-body P2P interactions moved to body-level P2L, and
 * the body-level P2L evaluations (one per source body and target leaf); 0 when off. */
int gx_plan_body_split_info(gx_ctx *ctx, int64_t *n_p2p_moved, int64_t *n_body_p2l);
/* Changes p and the softening of an existing context. */
int gx_set_params(gx_ctx *ctx, uint32_t p, double eps);

/* GpuContext::upload_tree_data (galax-gpu/src/lib.rs:392-462): a host-built tree
 * (galax-core Tree::build, lib.rs:163-361) with its V-list and U-list in the
 * reference's fixed layout (InteractionLists, lib.rs:941-944: n_nodes*64 u32,
 * unused slots 0xFFFFFFFF, and u8 lengths).  Bodies are taken to be in tree
 * order (body ranges index them).  child: 4 per node, -1 = none.  parent: -1 = none. */
int gx_upload_tree(gx_ctx *ctx, int64_t n_nodes, int64_t n_bodies, const double *cx, const double *cy,
                   const double *hw, const double *mass, const double *comx, const double *comy,
                   const int64_t *body_start, const int64_t *body_end, const int32_t *child,
                   const int32_t *parent, const uint8_t *is_leaf, const uint32_t *vlist_data,
                   const uint8_t *vlist_len, const uint32_t *ulist_data, const uint8_t *ulist_len);

/* Device tree build: Tree::build (lib.rs:163-361) or, with GX_BUILD_BALANCED,
 * build_constrained (lib.rs:541-588), then InteractionLists::build
 * (lib.rs:947-1025) and build_p2p_lists (lib.rs:1358-1392), all on the GPU and
 * bit-exact with the reference.  Like Tree::build it permutes the seven host
 * arrays in place into Morton order (any of vx, vy, ax, ay may be NULL).
 * bounds = {x_min, x_max, y_min, y_max}. */
int gx_build_tree(gx_ctx *ctx, int64_t n, double *x, double *y, double *vx, double *vy, double *m,
                  double *ax, double *ay, int64_t n_max, const double bounds[4], int flags);
/* Tree::build (galax-core/src/lib.rs:163-361) over the RESIDENT bodies: Morton keys,
 * device radix sort, permutation of the seven resident arrays, leaves and parents, with
 * no host round trip -- for a run that rebuilds the tree every step instead of keeping
 * it static as the reference's CLI does (galax-cli/src/main.rs:159).  perm (optional,
 * host, n_bodies entries) receives for every body its index before the rebuild.  The
 * plans (and, in REF mode, the V/U lists) are rebuilt by the next evaluation.
 * GX_BUILD_BALANCED runs build_constrained (lib.rs:541-694), which does not reorder. */
int gx_rebuild_resident(gx_ctx *ctx, int64_t n_max, const double bounds[4], int flags, int64_t *perm);
/* Shape of the current tree (any output may be NULL). */
int gx_tree_info(gx_ctx *ctx, int64_t *n_nodes, int64_t *n_leaves, int32_t *n_levels, int64_t *n_bodies);
/* morton_encode (galax-core/src/lib.rs:95-109) of n bodies at once on the device, bit-exact:
 * host x, y in, host keys out; bounds = {x_min, x_max, y_min, y_max}. */
int gx_morton_encode(gx_ctx *ctx, int64_t n, const double *x, const double *y, const double bounds[4],
                     uint64_t *keys);
/* Copies the current tree to host arrays (any pointer may be NULL); the Tree the
 * CLI keeps on the host.  level_start has n_levels+1 entries. */
int gx_export_tree(gx_ctx *ctx, double *cx, double *cy, double *hw, double *mass, double *comx,
                   double *comy, int64_t *body_start, int64_t *body_end, int32_t *child, int32_t *parent,
                   uint8_t *is_leaf, int64_t *level_start);
/* Copies a REF list (GX_LIST_V / GX_LIST_U) in the reference layout. */
int gx_export_lists(gx_ctx *ctx, int which, uint32_t *data, uint8_t *lengths);
/* Sizes of the plan of the current mode (built if needed): far (M2L) pairs, near (P2P)
 * leaf pairs and P2P body-body interactions (any output may be NULL). */
int gx_plan_info(gx_ctx *ctx, int64_t *n_far_pairs, int64_t *n_near_pairs, int64_t *n_p2p_interactions);

/* GpuContext::step + read_accelerations (galax-gpu/src/lib.rs:464-566): uploads
 * x, y, m (tree order), runs the six passes, writes ax, ay.  Inputs are sanitised
 * on the device like compute_fmm_force (lib.rs:1474-1482).  Page-locked ax, ay
 * (gx_host_alloc, cudaHostAlloc, cudaHostRegister) are written by the device
 * directly, and page-locked x, y, m read directly once the plan exists; other
 * memory is copied before and after the evaluation. */
int gx_compute_forces(gx_ctx *ctx, const double *x, const double *y, const double *m, double *ax, double *ay);

/* Device-resident state (no per-step host traffic). */
int gx_upload_bodies(gx_ctx *ctx, int64_t n, const double *x, const double *y, const double *vx,
                     const double *vy, const double *m, const double *ax, const double *ay);
int gx_download_bodies(gx_ctx *ctx, double *x, double *y, double *vx, double *vy, double *m, double *ax,
                       double *ay);
/* One force evaluation on the resident bodies (fills the resident ax, ay). */
int gx_forces_resident(gx_ctx *ctx);
/* simulate / simulate_gpu (galax-integrate/src/lib.rs:204-237, 327-368) on the
 * resident bodies: n_steps KDK steps with the static tree; every energy_every
 * steps a row {step, KE, FMM PE, px, py, Lz} is written to diag (6 doubles per row).
 * *n_diag receives the row count. */
int gx_kdk_run(gx_ctx *ctx, int64_t n_steps, double dt, int64_t energy_every, double *diag, int64_t *n_diag);
/* gx_kdk_run with a rebuild policy (the reference keeps the tree static): every
 * rebuild_every steps (0 = never) the tree is rebuilt on the device from the drifted
 * positions, with the parameters of the last gx_build_tree / gx_rebuild_resident,
 * before that step's force evaluation.  Rebuilds reorder the resident bodies;
 * gx_body_ids gives the mapping. */
int gx_kdk_run_rebuild(gx_ctx *ctx, int64_t n_steps, double dt, int64_t energy_every, int64_t rebuild_every,
                       double *diag, int64_t *n_diag);
/* For every resident body, its index in the order of the last gx_upload_bodies or
 * gx_build_tree (device rebuilds reorder the bodies; this undoes it).  ids: n_bodies. */
int gx_body_ids(gx_ctx *ctx, int64_t *ids);
/* Diagnostics of the resident bodies (lib.rs:1638-1683): {KE, FMM PE, px, py, Lz}. */
int gx_diagnostics(gx_ctx *ctx, double out[5]);
/* GpuContext::n2_debug (galax-gpu/src/lib.rs:670-714) restricted to sampled
 * targets: exact FP64 softened sum (validate_fmm, lib.rs:1537-1553) over all
 * resident bodies for the targets idx[0..n_idx). */
int gx_n2_sampled(gx_ctx *ctx, const int64_t *idx, int64_t n_idx, double *ax, double *ay);

/* The same sampled exact sum without a context and without allocating: for
 * callers that cannot allocate device memory when they want the check, because
 * their device memory belongs to another runtime's caching allocator (which may
 * hold nearly all of HBM, so a cudaMalloc would fail or fragment its pool).  No
 * counterpart in the reference.
 * x, y, m are the caller's device arrays of n bodies; idx (host, n_idx entries,
 * each in [0, n)) and the host outputs ax, ay are staged through a file-scope
 * device array of GX_N2_STATIC_MAX_SAMPLES slots (96 KiB, held by every GPU that
 * loads the library until exit); more samples return GX_ERR_CAP_EXCEEDED.  The
 * first call on a device looks up that array's device address (once per device,
 * with the device current) and keeps it for the life of the process: the device's
 * primary context is assumed, and after a cudaDeviceReset the library must not be
 * called again in that process.  Calls share the array and it keeps the last
 * call's contents (each call overwrites all it reads); calls that overlap on the
 * GPU race.  stream is a cudaStream_t (NULL = the legacy default stream) that must
 * not be capturing: the call copies through pageable host memory and returns
 * after the stream has finished the work. */
#define GX_N2_STATIC_MAX_SAMPLES 4096
int gx_n2_sampled_static(const double *x, const double *y, const double *m, int64_t n, double eps,
                         const int64_t *idx, int64_t n_idx, double *ax, double *ay, void *stream);

/* Reverse mode (GX_MODE_ACCURATE); no counterpart in the reference, which has no
 * gradients: the backward() of the force operator.  gx_force_vjp returns, for
 * cotangents lam of the accelerations of the resident bodies, g_x = sum lam . da/dx
 * and g_m = sum lam . da/dm (host arrays, tree order), the exact transpose of the
 * frozen-tree evaluation (L2P^T with the Hessian of the local expansion, L2L^T,
 * M2L^T, M2M^T, P2M^T, Hessian-vector P2P), in the context's precision (FP64, or
 * FP32 passes with FP64 outputs in the mixed form).  p in 0..8. */
int gx_force_vjp(gx_ctx *ctx, const double *lam_x, const double *lam_y, double *gx, double *gy, double *gm);
/* Leapfrog rollout from the resident state (simulate, galax-integrate/src/lib.rs:204-237)
 * keeping a checkpoint (positions, velocities, accelerations, masses and the leaf
 * locals of that step) every checkpoint_every steps; the resident state ends at step
 * n_steps.  rebuild_every = 0 keeps the tree static (the reference's CLI); 1 rebuilds
 * it on the device from the drifted positions before every step's force evaluation
 * (bodies are reordered: gx_body_ids, read right after this call, maps the final
 * order to the order at the start). */
int gx_rollout_forward(gx_ctx *ctx, int64_t n_steps, double dt, int64_t checkpoint_every,
                       int64_t rebuild_every);
/* Reverse leapfrog of the last gx_rollout_forward: given dL/d(x, y, vx, vy) at the
 * final step (host arrays in the final body order), returns dL/d(x, y, vx, vy) at
 * step 0 and dL/dm, in the body order at the start of the rollout.  Segments between
 * checkpoints are recomputed (deterministically, so bit for bit); under the rebuild
 * policy every step's tree is rebuilt, bit-identically, and the cotangents are carried
 * back through each rebuild's permutation.  The resident bodies are left at an
 * intermediate state.  *peak_bytes (may be NULL) receives the device bytes of the
 * checkpoint, segment, permutation and adjoint buffers. */
int gx_rollout_backward(gx_ctx *ctx, const double *lx, const double *ly, const double *lvx, const double *lvy,
                        double *gx0, double *gy0, double *gvx0, double *gvy0, double *gm, int64_t *peak_bytes);

/* Device time of the last force evaluation per pass, in ms:
 * {total, prepare, p2m, m2m, m2l, l2l, l2p+p2p}; returns 7 entries.  The near field
 * (P2P) runs on a second, lower-priority stream beside m2m..l2l, so those passes
 * include the slots it takes, and the last entry is the wait for it plus L2P. */
int gx_last_timings(gx_ctx *ctx, double out[7]);
/* Number of kernels the last force evaluation launched. */
int gx_last_launch_count(gx_ctx *ctx, int64_t *count);
/* Device status bits of the last force evaluation: GX_STATUS_SANITIZED when
 * non-finite or out-of-range positions were zeroed and non-positive or non-finite
 * masses set to 1 before it, as compute_fmm_force does (galax-core/src/lib.rs:1474-1482:
 * the reference does it silently; the evaluation still returns GX_OK). */
#define GX_STATUS_SANITIZED 1u
int gx_last_status(gx_ctx *ctx, uint32_t *status);

/* Page-locked host memory for the host-buffer entry points (cudaMallocHost);
 * NULL on failure. */
void *gx_host_alloc(size_t bytes);
void gx_host_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
