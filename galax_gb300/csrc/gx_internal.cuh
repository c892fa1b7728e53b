// gx_internal.cuh -- shared declarations of libgalaxcu (GB300 / sm_103a FMM backend).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/galax_gb300.h"
#include "../../include/galax_gb300_bench.h"

#define GX_MAXP 16
#define GX_LIST_CAP 64
#define GX_WARP 32

// ---------------------------------------------------------------- device buffers
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// Host-side error helper: records the message in the context and returns the code.
// One tree with its ACCURATE plan, held outside the context: the node arrays, the
// Morton keys, the per-tree auxiliaries, the near/far lists, the P2P items and the M2L
// units, with their counts and validity flags.  gx_tree_plan_swap exchanges it with the
// context's own (pointer swaps, no copies): a reverse rollout keeps the trees it builds
// while recomputing a segment and takes them back instead of rebuilding.
struct gx_tree_plan {
    static constexpr int N_BUFS = 29;
    DevBuf b[N_BUFS];
    std::vector<int64_t> level_start;
    int64_t n_nodes = 0, n_leaves = 0, max_leaf = 0, n_far_pairs = 0, n_near_pairs = 0, n_p2p_inter = 0;
    int64_t items_n = 0, units_n = 0;
    int32_t n_levels = 0;
    int chain_levels = 0;
    bool have_tree = false, aux_valid = false, plan_acc_valid = false, plan_ref_valid = false,
         ref_lists_valid = false, items_valid = false;
    int plan_p = -1;
    double plan_eps = -1.0, plan_theta = -1.0;
};

struct gx_ctx;
void gx_tree_plan_swap(gx_ctx *ctx, gx_tree_plan &t);
size_t gx_tree_plan_bytes(const gx_tree_plan &t);
void gx_tree_plan_free(gx_tree_plan &t);
int gx_fail(gx_ctx *ctx, int code, const std::string &msg);
int gx_cuda_check(gx_ctx *ctx, cudaError_t e, const char *what);

#define GX_CUDA(ctx, call)                                             \
    do {                                                               \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return gx_cuda_check((ctx), _e, #call); \
    } while (0)
#define GX_TRY(call)                  \
    do {                              \
        int _s = (call);              \
        if (_s != GX_OK) return _s;   \
    } while (0)

// Grow-only device allocation; contents are not preserved on growth.
int gx_ensure(gx_ctx *ctx, DevBuf &b, size_t bytes);
template <class T>
inline T *dptr(const DevBuf &b) { return reinterpret_cast<T *>(b.p); }

// Device status word bits (read back at pass boundaries).
enum : unsigned {
    GX_DEV_NONFINITE_INPUT = 1u,
    GX_DEV_LIST_OVERFLOW = 2u,
    GX_DEV_STACK_OVERFLOW = 4u,
};

// ---------------------------------------------------------------- the context
struct gx_ctx {
    gx_config cfg{};
    int device = 0;
    int p = 4;
    double eps = 0.1;
    int mode = GX_MODE_REF;
    int prec = GX_PREC_FP64;
    double theta = 0.5;
    cudaStream_t stream = nullptr;
    // second stream: the near field (P2P) runs beside the far-field chain
    // (M2M, M2L, L2L) of the same evaluation; forked after P2M, joined before L2P
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string err;
    int sm_count = 0;

    // tree (device, SoA); node ids are int32, body indices int32
    int64_t n_nodes = 0, n_bodies = 0, n_leaves = 0;
    int32_t n_levels = 0;
    std::vector<int64_t> level_start;  // n_levels + 1
    bool have_tree = false;
    DevBuf cx, cy, hw, mass, comx, comy, bs, be, child, parent, is_leaf;
    DevBuf keys;  // Morton keys of the bodies in tree order (device build only)

    // bodies (device, tree order)
    DevBuf x, y, vx, vy, m, ax, ay;
    DevBuf body_alt[7];  // spare copies of x, y, vx, vy, m, ax, ay: the targets of a device sort's gather
    bool have_bodies = false;

    // REF lists, reference layout (built with the tree by gx_build_tree, lazily after
    // gx_rebuild_resident)
    DevBuf vdata, vlen, udata, ulen;
    bool ref_lists_valid = false;
    DevBuf perm;  // uint32: pre-sort index of each body after the last device sort
    // parameters of the last tree build (reused by device rebuilds)
    int64_t build_n_max = 0;
    double build_bounds[4] = {0, 0, 0, 0};
    int build_flags = 0;
    // int32: for each resident body, its index in the order of the last upload (or
    // build_tree); device rebuilds permute it with the bodies
    DevBuf ids;

    // plans (static per tree, mode, p, eps)
    bool plan_ref_valid = false, plan_acc_valid = false;
    double plan_eps = -1.0, plan_theta = -1.0;
    int plan_p = -1;
    DevBuf p2p_off, p2p_idx;         // REF gather lists: per leaf, the source leaves
    int64_t n_p2p_pairs = 0;
    DevBuf ref_voff;                 // per node: offset of its V pairs (REF pair order)
    DevBuf ref_did;                  // per V pair: derivative-set id
    DevBuf ref_G;                    // n_keys x (2p+1)^2 doubles
    int64_t n_ref_keys = 0, n_v_pairs = 0;
    DevBuf radius;                   // accurate mode node radii
    DevBuf radius32;                 // the radii rounded to FP32 (MAC operands)
    DevBuf anc;                      // per leaf, its ancestor at every level (level-major), -1 above the root
    DevBuf has_far_ref, has_far_acc; // per node: 1 if its M2L list is non-empty
    DevBuf comhl;                    // per node COM as FP32 (x_hi, x_lo, y_hi, y_lo)
    DevBuf far_off, far_idx, near_off, near_idx;
    int64_t n_far_pairs = 0, n_near_pairs = 0, n_p2p_inter = 0;
    // P2P work items (source lists cut into pieces of at most 32 leaves), per plan
    struct Items {
        DevBuf leaf, qb, nq, off;  // int32, int64, int32, int64[n_leaves+1]
        int64_t n = 0;
        bool valid = false;
    } items_ref, items_acc;
    // ACCURATE M2L work units (far lists cut into pieces of at most GX_M2L_UNIT
    // sources), per plan: unit -> node, first index, length; node_u[nn+1] = the
    // node's first unit
    struct M2LUnits {
        DevBuf node, start, len, node_u;  // int32, int64, int32, int64[n_nodes+1]
        int64_t n = 0;
    } m2l_units;
    DevBuf m2l_part;  // per-unit partial locals of nodes cut into several units
    // ACCURATE near-list split (theta_w > 0): every leaf's near list is partitioned in
    // place into [P2P | M2P | P2L] sources; the leaf's near count becomes its P2P count
    // and split_cnt holds (M2P count, P2L count) per leaf.  M2P sources become extra work
    // items of the leaf (item_nq < 0), P2L sources units of at most GX_P2L_UNIT leaves.
    double theta_w = 0.0, plan_theta_w = 0.0;
    DevBuf split_cnt;      // int32 [2 * n_leaves]
    DevBuf split_tot;      // int64 [4]: P2P, M2P, P2L pairs (device totals of the split)
    int64_t n_m2p_pairs = 0, n_p2l_pairs = 0, n_m2p_items = 0;
    DevBuf m2p_list;  // int32: the item indices of the M2P items, leaf by leaf
    DevBuf m2p_off;   // int64 [n_leaves + 1]: each leaf's first entry in m2p_list
    // [leaf-level units | body-level units]: leaf_u[a] is leaf a's first leaf-level unit,
    // n_leafu + body_u[a] its first body-level one
    struct P2LUnits {
        DevBuf leaf, start, len, leaf_u, body_u;  // int32, int64, int32, int64[n_leaves+1] x 2
        int64_t n = 0, n_leafu = 0, n_body = 0;
    } p2l_units;
    DevBuf p2l_part;  // per-unit partial locals of leaves with several P2L units
    // Body-level P2L of the P2P pairs (theta_b > 0, leaves of at most 32 bodies): a
    // source body j of a P2P row (a <- s), s != a, with |x_j - com_a| theta_b > R_a joins
    // a's local expansion instead of P2P.  p2p_mask holds, per P2P entry of near_idx, the
    // bit set of such bodies of s (0 for the self row); the P2P items then run over the
    // other bodies, and every GX_BODY_UNIT P2P rows of a leaf are a body-P2L unit (its
    // length stored negated in the P2L units) over the masked ones.
    double theta_b = 0.0, plan_theta_b = 0.0;
    bool plan_body_split = false;  // the current ACCURATE plan has the masks
    DevBuf p2p_mask;               // uint32 per near_idx entry
    DevBuf body_off32;             // plan scratch: float2 (x - com_leaf, y - com_leaf) per body
    int64_t n_body_p2l = 0, n_p2p_moved = 0;  // body-P2L evaluations, P2P interactions moved to them
    DevBuf m2l_cnt;   // plan scratch: units per node
    DevBuf plan_ctr;       // ACCURATE plan: device running totals and overflow flags
    // sizes of the last tree and plan: the first capacities of the next build and plan
    // (their arrays may be fresh ones swapped in from a gx_tree_plan)
    int64_t hint_nodes = 0, hint_far = 0, hint_near = 0;
    int hint_big_rounds = 0;  // tree build: rounds of the last build run by the multi-block kernels
    // ACCURATE plan: levels 1 .. chain_levels are single-child chains over the leaves
    // (level l holds node x + l nl above leaf x); with chain_levels >= 2 the plan and M2M
    // skip levels 1 .. chain_levels - 1 (no far lists there), else 0
    int chain_levels = 0;
    bool near_after_far = false;  // measurement only: the near field after the far-field chain
    // gx_compute_forces into page-locked host arrays: their device addresses, written by
    // the final sum of the evaluation being enqueued (null otherwise)
    double *out_ax = nullptr, *out_ay = nullptr;
    const double *in_x = nullptr, *in_y = nullptr, *in_m = nullptr;  // the same for the inputs, read by k_prepare
    unsigned last_status = 0;     // device status bits of the last force evaluation
    DevBuf tree_state;     // tree build: device round state and level starts
    int64_t mac_ucap = 0;  // ACCURATE plan: capacity of the per-level unit arrays
    DevBuf part;                   // per-item partial accelerations
    int64_t max_leaf = 0;          // largest leaf body count
    bool aux_valid = false;        // anc / comhl built for the current tree

    // expansions
    DevBuf M, L, Lf;
    DevBuf Mf32, Lf32, Lff32;
    DevBuf pos32;  // mixed form: bodies as FP32 (x - com_leaf, y - com_leaf, m, 0)
    DevBuf fl32;   // mixed form: the L2P (fx, fy) of every body, summed with the P2P partials after the join

    // adjoint: cotangents, VJP outputs, transposed expansions, checkpoints
    DevBuf adj_lx, adj_ly, adj_lvx, adj_lvy, adj_lm, adj_gx, adj_gy, adj_gm, adj_lax, adj_lay, adj_lf;
    DevBuf adj_dL, adj_dM, adj_dMleaf, adj_lam32;
    DevBuf ckpt, seg;
    int64_t roll_steps = 0, roll_k = 1;
    double roll_dt = 0.0;
    int roll_prec = GX_PREC_FP64;
    int64_t roll_rebuild = 0;
    DevBuf roll_perms;  // uint32 [T+1][n]: the permutation of every rebuild of a rollout
    bool roll_valid = false;
    std::vector<gx_tree_plan> tp_cache;  // reverse rollout: the trees of a segment's states

    // scratch
    DevBuf scratch_a, scratch_b, scratch_c, scratch_d, scratch_e, scratch_f, scratch_g;
    DevBuf status;     // unsigned, device status word
    DevBuf red;        // reduction scratch (doubles)
    DevBuf flush;      // L2 flush buffer for timing

    // timing
    cudaEvent_t ev[16] = {};
    double last_ms[7] = {0, 0, 0, 0, 0, 0, 0};
    double last_p2p_ms = 0;  // the P2P kernel alone (events on the near-field stream)
    int64_t last_launches = 0;
    int64_t launches = 0;
};

// ---------------------------------------------------------------- sub-modules
// gx_tree.cu
int gx_tree_build_device(gx_ctx *ctx, int64_t n, int64_t n_max, const double bounds[4], int flags);
// Morton keys of n bodies (device arrays) on the context stream; idx (optional) gets 0..n-1
void gx_launch_morton(gx_ctx *ctx, const double *x, const double *y, int64_t n, const double bounds[4], uint64_t *keys,
                      uint32_t *idx);
// gx_lists.cu
int gx_lists_build_ref(gx_ctx *ctx);
int gx_plan_ref(gx_ctx *ctx);
int gx_plan_accurate(gx_ctx *ctx);
int gx_plan_items(gx_ctx *ctx, bool accurate);
int gx_plan_tree_aux(gx_ctx *ctx);
int gx_plan_near_split(gx_ctx *ctx);
int gx_plan_body_masks(gx_ctx *ctx);
// gx_fmm.cu
int gx_forces_device(gx_ctx *ctx, bool timed);
// gx_api.cu: device rebuild with the last build's parameters (permutes the resident
// bodies and ids; invalidates the plans), plan check, ids reset
int gx_rebuild_internal(gx_ctx *ctx);
int gx_ensure_plan_public(gx_ctx *ctx);
int gx_ids_reset(gx_ctx *ctx);
int gx_poly_table_host(int p, double eps, std::vector<double> &out);
// gx_scan.cu
int gx_exclusive_scan_i64(gx_ctx *ctx, const int64_t *in, int64_t *out, int64_t n);
int gx_exclusive_scan_i32(gx_ctx *ctx, const int32_t *in, int32_t *out, int64_t n, int32_t *total_host);
// exclusive scan of min(*n_dev + n_add, n_cap) entries, the length read on the device;
// the grand total goes to *total_dev when given
int gx_exclusive_scan_i64_devn(gx_ctx *ctx, const int64_t *in, int64_t *out, const int64_t *n_dev, int64_t n_add,
                               int64_t n_cap, int64_t *total_dev = nullptr);
// m arrays at a common stride (in + k * stride -> out + k * stride), one set of launches;
// total_dev (if given) receives m totals
int gx_exclusive_scan_i64_devn_multi(gx_ctx *ctx, const int64_t *in, int64_t *out, int m, int64_t stride,
                                     const int64_t *n_dev, int64_t n_add, int64_t n_cap, int64_t *total_dev = nullptr);
int gx_radix_sort_u64(gx_ctx *ctx, uint64_t *keys, uint32_t *vals, int64_t n, int begin_bit, int end_bit,
                      uint64_t *keys_alt, uint32_t *vals_alt, bool *result_in_alt);
// gx_kdk.cu
int gx_kdk_device(gx_ctx *ctx, int64_t n_steps, double dt, int64_t energy_every, double *diag, int64_t *n_diag,
                  int64_t rebuild_every = 0);
int gx_diag_device(gx_ctx *ctx, double out[5]);
int gx_n2_device(gx_ctx *ctx, const int64_t *idx, int64_t n_idx, double *ax, double *ay);

// grid helpers
inline unsigned gx_blocks(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// The body-level P2L applies to the P2P pairs of the near-list split (ACCURATE, theta_w
// > 0) with theta_b > 0 over leaves of at most 32 bodies (one mask word per P2P row);
// otherwise every P2P row keeps all its bodies.
inline bool gx_body_split_on(const gx_ctx *ctx) {
    return ctx->mode == GX_MODE_ACCURATE && ctx->theta_w > 0.0 && ctx->theta_b > 0.0 && ctx->max_leaf <= 32;
}

// ---------------------------------------------------------------- device helpers
#ifdef __CUDACC__
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__host__ __device__ constexpr int gx_nc(int p) { return (p + 1) * (p + 2) / 2; }
constexpr int GX_M2L_UNIT = 256;  // far sources per M2L work unit (8 rounds of a warp)
constexpr int GX_P2L_UNIT = 32;   // source leaves per P2L work unit (one per lane)
constexpr int GX_BODY_UNIT = 96;  // P2P rows per body-level P2L unit (three per lane)
__host__ __device__ constexpr int gx_mi(int i, int j) { return (i + j) * (i + j + 1) / 2 + j; }
__host__ __device__ constexpr int gx_kdi(int k, int l, int p) { return (k + l) * (2 * p + 1) + l; }
#endif
