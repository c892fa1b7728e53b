// gx_api.cu -- the extern "C" boundary of libgalaxcu.so (declared in
// include/galax_gb300.h).  Host-side orchestration only; all compute is in the
// kernels of gx_tree.cu, gx_lists.cu, gx_fmm.cu and gx_kdk.cu.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gx_internal.cuh"

int gx_tree_balance(gx_ctx *ctx, int64_t n_max, const double bounds[4]);

int gx_fail(gx_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int gx_cuda_check(gx_ctx *ctx, cudaError_t e, const char *what) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    int code = GX_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation) code = GX_ERR_ALLOC;
    if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidKernelImage) code = GX_ERR_KERNEL_LOAD;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) code = GX_ERR_INIT;
    return gx_fail(ctx, code, buf);
}

int gx_ensure(gx_ctx *ctx, DevBuf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return GX_OK;
    if (b.p) {
        cudaStreamSynchronize(ctx->stream);  // nothing queued may still use the old block
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t nb = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&b.p, nb);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        char msg[128];
        snprintf(msg, sizeof msg, "device allocation of %zu bytes failed", nb);
        return gx_fail(ctx, GX_ERR_ALLOC, msg);
    }
    b.bytes = nb;
    return GX_OK;
}

static void free_buf(DevBuf &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

static int check_ctx(gx_ctx *ctx) { return ctx ? GX_OK : GX_ERR_INVALID_ARG; }

// the context's members that make up a gx_tree_plan, in a fixed order
static void tree_plan_members(gx_ctx *ctx, DevBuf *(&m)[gx_tree_plan::N_BUFS]) {
    DevBuf *l[gx_tree_plan::N_BUFS] = {
        &ctx->cx, &ctx->cy, &ctx->hw, &ctx->mass, &ctx->comx, &ctx->comy, &ctx->bs, &ctx->be, &ctx->child,
        &ctx->parent, &ctx->is_leaf, &ctx->keys, &ctx->radius, &ctx->radius32, &ctx->anc, &ctx->has_far_acc,
        &ctx->comhl, &ctx->far_off, &ctx->far_idx, &ctx->near_off, &ctx->near_idx, &ctx->items_acc.leaf,
        &ctx->items_acc.qb, &ctx->items_acc.nq, &ctx->items_acc.off, &ctx->m2l_units.node, &ctx->m2l_units.start,
        &ctx->m2l_units.len, &ctx->m2l_units.node_u};
    for (int k = 0; k < gx_tree_plan::N_BUFS; k++) m[k] = l[k];
}

void gx_tree_plan_swap(gx_ctx *ctx, gx_tree_plan &t) {
    DevBuf *m[gx_tree_plan::N_BUFS];
    tree_plan_members(ctx, m);
    for (int k = 0; k < gx_tree_plan::N_BUFS; k++) std::swap(*m[k], t.b[k]);
    std::swap(ctx->level_start, t.level_start);
    std::swap(ctx->n_nodes, t.n_nodes);
    std::swap(ctx->n_leaves, t.n_leaves);
    std::swap(ctx->max_leaf, t.max_leaf);
    std::swap(ctx->n_far_pairs, t.n_far_pairs);
    std::swap(ctx->n_near_pairs, t.n_near_pairs);
    std::swap(ctx->n_p2p_inter, t.n_p2p_inter);
    std::swap(ctx->items_acc.n, t.items_n);
    std::swap(ctx->m2l_units.n, t.units_n);
    std::swap(ctx->n_levels, t.n_levels);
    std::swap(ctx->chain_levels, t.chain_levels);
    std::swap(ctx->have_tree, t.have_tree);
    std::swap(ctx->aux_valid, t.aux_valid);
    std::swap(ctx->plan_acc_valid, t.plan_acc_valid);
    std::swap(ctx->plan_ref_valid, t.plan_ref_valid);
    std::swap(ctx->ref_lists_valid, t.ref_lists_valid);
    std::swap(ctx->items_acc.valid, t.items_valid);
    std::swap(ctx->plan_p, t.plan_p);
    std::swap(ctx->plan_eps, t.plan_eps);
    std::swap(ctx->plan_theta, t.plan_theta);
}

size_t gx_tree_plan_bytes(const gx_tree_plan &t) {
    size_t s = 0;
    for (const DevBuf &d : t.b) s += d.bytes;
    return s;
}

void gx_tree_plan_free(gx_tree_plan &t) {
    for (DevBuf &d : t.b) {
        if (d.p) cudaFree(d.p);
        d.p = nullptr;
        d.bytes = 0;
    }
}

static int sync_status(gx_ctx *ctx, unsigned *out) {
    GX_CUDA(ctx, cudaMemcpyAsync(out, ctx->status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

extern "C" {

int gx_abi_version(void) { return GX_ABI_VERSION; }

int gx_config_default(gx_config *cfg) {
    if (!cfg) return GX_ERR_INVALID_ARG;
    cfg->max_n = 262144;
    cfg->max_nodes = 524288;
    cfg->max_interactions = 1u << 24;
    cfg->p = 4;
    cfg->eps = 0.1f;
    cfg->eps64 = 0.0;
    cfg->device = 0;
    return GX_OK;
}

const char *gx_last_error(const gx_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gx_create(const gx_config *cfg, gx_ctx **out) {
    if (!cfg || !out) return GX_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->p > GX_MAXP) return GX_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GX_ERR_INIT;
    }
    if (cfg->device < 0 || cfg->device >= ndev) return GX_ERR_INVALID_ARG;
    if (cudaSetDevice(cfg->device) != cudaSuccess) return GX_ERR_INIT;
    gx_ctx *ctx = new gx_ctx();
    ctx->cfg = *cfg;
    ctx->device = cfg->device;
    ctx->p = (int)cfg->p;
    ctx->eps = cfg->eps64 > 0.0 ? cfg->eps64 : (double)cfg->eps;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, cfg->device);
    // the main stream at the highest priority, the near-field stream at the lowest:
    // the far-field chain (short M2M/L2L launches, then M2L) takes SMs first and P2P
    // fills whatever it leaves idle
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
        delete ctx;
        return GX_ERR_INIT;
    }
    for (auto &e : ctx->ev) cudaEventCreate(&e);
    if (cudaStreamCreateWithPriority(&ctx->stream2, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        gx_destroy(ctx);
        return GX_ERR_INIT;
    }
    // kernel-image check: the status allocation and a memset are the first device work
    int s = gx_ensure(ctx, ctx->status, 64);
    if (s != GX_OK) {
        gx_destroy(ctx);
        return s;
    }
    cudaMemsetAsync(ctx->status.p, 0, 64, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        gx_destroy(ctx);
        return GX_ERR_INIT;
    }
    *out = ctx;
    return GX_OK;
}

int gx_destroy(gx_ctx *ctx) {
    if (!ctx) return GX_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    DevBuf *bufs[] = {&ctx->cx, &ctx->cy, &ctx->hw, &ctx->mass, &ctx->comx, &ctx->comy, &ctx->bs, &ctx->be,
                      &ctx->child, &ctx->parent, &ctx->is_leaf, &ctx->keys, &ctx->x, &ctx->y, &ctx->vx, &ctx->vy,
                      &ctx->m, &ctx->ax, &ctx->ay, &ctx->vdata, &ctx->vlen, &ctx->udata, &ctx->ulen, &ctx->p2p_off,
                      &ctx->p2p_idx, &ctx->ref_voff, &ctx->ref_did, &ctx->ref_G, &ctx->radius, &ctx->anc, &ctx->has_far_ref, &ctx->has_far_acc, &ctx->comhl, &ctx->far_off, &ctx->far_idx,
                      &ctx->near_off, &ctx->near_idx, &ctx->M, &ctx->L, &ctx->Lf, &ctx->Mf32, &ctx->Lf32,
                      &ctx->Lff32, &ctx->pos32, &ctx->fl32, &ctx->part, &ctx->items_ref.leaf, &ctx->items_ref.qb, &ctx->items_ref.nq, &ctx->items_ref.off, &ctx->items_acc.leaf, &ctx->items_acc.qb, &ctx->items_acc.nq, &ctx->items_acc.off, &ctx->scratch_a, &ctx->scratch_b, &ctx->scratch_c, &ctx->scratch_d,
                      &ctx->scratch_e, &ctx->scratch_f, &ctx->scratch_g, &ctx->status, &ctx->red, &ctx->flush, &ctx->adj_lx, &ctx->adj_ly, &ctx->adj_lvx, &ctx->adj_lvy, &ctx->adj_lm, &ctx->adj_gx, &ctx->adj_gy, &ctx->adj_gm, &ctx->adj_lax, &ctx->adj_lay, &ctx->adj_lf, &ctx->adj_dL, &ctx->adj_dM, &ctx->adj_dMleaf, &ctx->adj_lam32, &ctx->ckpt, &ctx->seg, &ctx->ids, &ctx->perm, &ctx->roll_perms, &ctx->radius32,
                      &ctx->m2l_units.node, &ctx->m2l_units.start, &ctx->m2l_units.len, &ctx->m2l_units.node_u,
                      &ctx->m2l_part, &ctx->plan_ctr, &ctx->tree_state, &ctx->m2l_cnt, &ctx->split_cnt,
                      &ctx->split_tot, &ctx->p2l_units.leaf, &ctx->p2l_units.start, &ctx->p2l_units.len,
                      &ctx->p2l_units.leaf_u, &ctx->p2l_units.body_u, &ctx->p2l_part, &ctx->m2p_list,
                      &ctx->m2p_off, &ctx->p2p_mask, &ctx->body_off32};
    for (DevBuf *b : bufs) free_buf(*b);
    for (DevBuf &b : ctx->body_alt) free_buf(b);
    for (gx_tree_plan &t : ctx->tp_cache) gx_tree_plan_free(t);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream2) {
        cudaStreamSynchronize(ctx->stream2);
        cudaStreamDestroy(ctx->stream2);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GX_OK;
}

int gx_set_mode(gx_ctx *ctx, int mode, int precision, double theta) {
    GX_TRY(check_ctx(ctx));
    if (mode < GX_MODE_REF || mode > GX_MODE_ACCURATE) return gx_fail(ctx, GX_ERR_INVALID_ARG, "unknown mode");
    if (precision != GX_PREC_FP64 && precision != GX_PREC_MIXED) return gx_fail(ctx, GX_ERR_INVALID_ARG, "unknown precision");
    if (mode == GX_MODE_ACCURATE && !(theta > 0.0 && theta < 2.0))
        return gx_fail(ctx, GX_ERR_INVALID_ARG, "theta must be in (0, 2)");
    ctx->mode = mode;
    ctx->prec = precision;
    if (mode == GX_MODE_ACCURATE && theta != ctx->theta) ctx->plan_acc_valid = false;
    if (mode == GX_MODE_ACCURATE) ctx->theta = theta;
    return GX_OK;
}

int gx_set_near_split(gx_ctx *ctx, double theta_w) {
    GX_TRY(check_ctx(ctx));
    if (!(theta_w >= 0.0 && theta_w < 2.0)) return gx_fail(ctx, GX_ERR_INVALID_ARG, "theta_w must be in [0, 2)");
    if (theta_w != ctx->theta_w) ctx->plan_acc_valid = false;
    ctx->theta_w = theta_w;
    return GX_OK;
}

int gx_set_body_split(gx_ctx *ctx, double theta_b) {
    GX_TRY(check_ctx(ctx));
    if (!(theta_b >= 0.0 && theta_b < 2.0)) return gx_fail(ctx, GX_ERR_INVALID_ARG, "theta_b must be in [0, 2)");
    if (theta_b != ctx->theta_b) ctx->plan_acc_valid = false;
    ctx->theta_b = theta_b;
    return GX_OK;
}

int gx_set_params(gx_ctx *ctx, uint32_t p, double eps) {
    GX_TRY(check_ctx(ctx));
    if (p > GX_MAXP) return gx_fail(ctx, GX_ERR_INVALID_ARG, "p must be in 0..16");
    if (!(eps >= 0.0) || !isfinite(eps)) return gx_fail(ctx, GX_ERR_INVALID_ARG, "eps must be finite and >= 0");
    if ((int)p != ctx->p || eps != ctx->eps) ctx->plan_ref_valid = false;
    ctx->p = (int)p;
    ctx->eps = eps;
    return GX_OK;
}

// Copies the given host arrays to the resident bodies.  A NULL array is zeroed when
// zero_missing is set; otherwise its resident contents are kept (zeroed only if the
// buffer had to be allocated).
}  // extern "C"

namespace {
__global__ void k_iota_i32(int64_t n, int32_t *v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (int32_t)i;
}
__global__ void k_gather_i32(int64_t n, const uint32_t *perm, const int32_t *in, int32_t *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[perm[i]];
}
}  // namespace

// Device Tree::build over the resident bodies with the last build's parameters.
int gx_rebuild_internal(gx_ctx *ctx) {
    if (ctx->build_n_max <= 0) return gx_fail(ctx, GX_ERR_STATE, "no tree parameters: build a tree first");
    const int64_t n = ctx->n_bodies;
    ctx->have_tree = false;
    ctx->plan_ref_valid = ctx->plan_acc_valid = ctx->aux_valid = ctx->ref_lists_valid = false;
    if (ctx->ids.bytes < sizeof(int32_t) * (size_t)(n > 0 ? n : 1)) GX_TRY(gx_ids_reset(ctx));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
    if ((ctx->build_flags & GX_BUILD_BALANCED) && n > 0) {
        GX_TRY(gx_tree_balance(ctx, ctx->build_n_max, ctx->build_bounds));
    } else {
        GX_TRY(gx_tree_build_device(ctx, n, ctx->build_n_max, ctx->build_bounds, 0));
        if (n > 0) {  // ids follow the bodies
            GX_TRY(gx_ensure(ctx, ctx->scratch_g, sizeof(int32_t) * (size_t)n));
            k_gather_i32<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, dptr<uint32_t>(ctx->perm),
                                                                    dptr<int32_t>(ctx->ids), dptr<int32_t>(ctx->scratch_g));
            std::swap(ctx->ids.p, ctx->scratch_g.p);
            std::swap(ctx->ids.bytes, ctx->scratch_g.bytes);
            ctx->launches++;
        }
    }
    if (ctx->cfg.max_nodes && (uint64_t)ctx->n_nodes > ctx->cfg.max_nodes)
        return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "tree node count exceeds max_nodes");
    ctx->max_leaf = std::min<int64_t>(ctx->build_n_max, n);
    ctx->have_tree = true;
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

int gx_ids_reset(gx_ctx *ctx) {
    int64_t n = ctx->n_bodies;
    GX_TRY(gx_ensure(ctx, ctx->ids, sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));
    if (n > 0) k_iota_i32<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, dptr<int32_t>(ctx->ids));
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

extern "C" {

static int upload_bodies_impl(gx_ctx *ctx, int64_t n, const double *x, const double *y, const double *vx,
                              const double *vy, const double *m, const double *ax, const double *ay,
                              bool zero_missing = true) {
    if (n < 0) return gx_fail(ctx, GX_ERR_INVALID_ARG, "n < 0");
    if (ctx->cfg.max_n && (uint64_t)n > ctx->cfg.max_n) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "n exceeds max_n");
    size_t bytes = sizeof(double) * (size_t)(n > 0 ? n : 1);
    DevBuf *dst[7] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->m, &ctx->ax, &ctx->ay};
    const double *src[7] = {x, y, vx, vy, m, ax, ay};
    bool same_n = ctx->have_bodies && ctx->n_bodies == n;
    for (int k = 0; k < 7; k++) {
        void *before = dst[k]->p;
        GX_TRY(gx_ensure(ctx, *dst[k], bytes));
        if (n == 0) continue;
        if (!src[k] && !zero_missing && same_n && before == dst[k]->p) continue;
        if (src[k]) {
            GX_CUDA(ctx, cudaMemcpyAsync(dst[k]->p, src[k], sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        } else {
            GX_CUDA(ctx, cudaMemsetAsync(dst[k]->p, 0, sizeof(double) * n, ctx->stream));
        }
    }
    ctx->have_bodies = true;
    return GX_OK;
}

int gx_upload_bodies(gx_ctx *ctx, int64_t n, const double *x, const double *y, const double *vx, const double *vy,
                     const double *m, const double *ax, const double *ay) {
    GX_TRY(check_ctx(ctx));
    if (!x || !y || !m) return gx_fail(ctx, GX_ERR_INVALID_ARG, "x, y and m are required");
    if (ctx->have_tree && n != ctx->n_bodies) return gx_fail(ctx, GX_ERR_INVALID_ARG, "n differs from the tree's body count");
    GX_TRY(upload_bodies_impl(ctx, n, x, y, vx, vy, m, ax, ay));
    ctx->n_bodies = n;
    GX_TRY(gx_ids_reset(ctx));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

int gx_download_bodies(gx_ctx *ctx, double *x, double *y, double *vx, double *vy, double *m, double *ax, double *ay) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "no resident bodies");
    int64_t n = ctx->n_bodies;
    DevBuf *srcb[7] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->m, &ctx->ax, &ctx->ay};
    double *dst[7] = {x, y, vx, vy, m, ax, ay};
    for (int k = 0; k < 7; k++)
        if (dst[k] && n > 0)
            GX_CUDA(ctx, cudaMemcpyAsync(dst[k], srcb[k]->p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

int gx_build_tree(gx_ctx *ctx, int64_t n, double *x, double *y, double *vx, double *vy, double *m, double *ax,
                  double *ay, int64_t n_max, const double bounds[4], int flags) {
    GX_TRY(check_ctx(ctx));
    if (n < 0 || n_max <= 0 || !bounds) return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad n, n_max or bounds");
    if (n > 0 && (!x || !y || !m)) return gx_fail(ctx, GX_ERR_INVALID_ARG, "x, y and m are required");
    ctx->have_tree = false;
    ctx->plan_ref_valid = ctx->plan_acc_valid = ctx->aux_valid = ctx->roll_valid = false;
    GX_TRY(upload_bodies_impl(ctx, n, x, y, vx, vy, m, ax, ay));
    ctx->n_bodies = n;
    ctx->build_n_max = n_max;
    for (int k = 0; k < 4; k++) ctx->build_bounds[k] = bounds[k];
    ctx->build_flags = flags;
    GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
    if (flags & GX_BUILD_BALANCED) {
        if (n == 0) {
            GX_TRY(gx_tree_build_device(ctx, 0, n_max, bounds, 0));
        } else {
            GX_TRY(gx_tree_balance(ctx, n_max, bounds));
        }
    } else {
        GX_TRY(gx_tree_build_device(ctx, n, n_max, bounds, 0));
    }
    if (ctx->cfg.max_nodes && (uint64_t)ctx->n_nodes > ctx->cfg.max_nodes)
        return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "tree node count exceeds max_nodes");
    // the reference's V/U lists are built when first needed (REF mode, gx_export_lists)
    ctx->ref_lists_valid = false;
    ctx->max_leaf = std::min<int64_t>(n_max, n);
    // Tree::build permutes the caller's arrays (lib.rs:204); so do we.
    if (!(flags & GX_BUILD_BALANCED)) GX_TRY(gx_download_bodies(ctx, x, y, vx, vy, m, ax, ay));
    GX_TRY(gx_ids_reset(ctx));  // the caller's arrays are now in tree order
    ctx->have_tree = true;
    return GX_OK;
}

int gx_upload_tree(gx_ctx *ctx, int64_t n_nodes, int64_t n_bodies, const double *cx, const double *cy,
                   const double *hw, const double *mass, const double *comx, const double *comy,
                   const int64_t *body_start, const int64_t *body_end, const int32_t *child, const int32_t *parent,
                   const uint8_t *is_leaf, const uint32_t *vlist_data, const uint8_t *vlist_len,
                   const uint32_t *ulist_data, const uint8_t *ulist_len) {
    GX_TRY(check_ctx(ctx));
    if (n_nodes < 0 || n_bodies < 0 || n_bodies >= 0x7fffffffLL || n_nodes >= 0x7fffffffLL)
        return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad sizes");
    if (n_nodes > 0 && (!cx || !cy || !hw || !mass || !comx || !comy || !body_start || !body_end || !child || !parent ||
                        !is_leaf || !vlist_data || !vlist_len || !ulist_data || !ulist_len))
        return gx_fail(ctx, GX_ERR_INVALID_ARG, "null tree array");
    if (ctx->cfg.max_nodes && (uint64_t)n_nodes > ctx->cfg.max_nodes)
        return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "n_nodes exceeds max_nodes");
    ctx->have_tree = false;
    ctx->plan_ref_valid = ctx->plan_acc_valid = ctx->aux_valid = ctx->roll_valid = false;
    // levels = height (compute_levels, lib.rs:426-438); Tree::build appends each
    // round contiguously, which the device passes rely on.
    std::vector<int32_t> lev((size_t)n_nodes);
    std::vector<int32_t> bs32((size_t)n_nodes), be32((size_t)n_nodes);
    int32_t maxlev = 0;
    int64_t nl = 0;
    for (int64_t i = 0; i < n_nodes; i++) {
        int32_t l = 0;
        for (int k = 0; k < 4; k++) {
            int32_t c = child[4 * i + k];
            if (c >= 0) {
                if (c >= i) return gx_fail(ctx, GX_ERR_INVALID_ARG, "child id must precede its parent");
                l = std::max(l, lev[c] + 1);
            }
        }
        lev[i] = l;
        maxlev = std::max(maxlev, l);
        if (is_leaf[i]) {
            if (l != 0) return gx_fail(ctx, GX_ERR_INVALID_ARG, "leaf with children");
            nl++;
        }
        if (body_start[i] < 0 || body_end[i] > n_bodies || body_start[i] > body_end[i])
            return gx_fail(ctx, GX_ERR_INVALID_ARG, "body range out of bounds");
        bs32[i] = (int32_t)body_start[i];
        be32[i] = (int32_t)body_end[i];
    }
    std::vector<int64_t> ls;
    ls.push_back(0);
    for (int64_t i = 0; i < n_nodes; i++) {
        if (i > 0 && lev[i] < lev[i - 1]) return gx_fail(ctx, GX_ERR_INVALID_ARG, "levels are not contiguous");
        if (i > 0 && lev[i] != lev[i - 1]) ls.push_back(i);
    }
    ls.push_back(n_nodes);
    for (int64_t i = 0; i < nl; i++)
        if (!is_leaf[i]) return gx_fail(ctx, GX_ERR_INVALID_ARG, "leaves must come first");
    struct F { DevBuf *b; const void *src; size_t sz; };
    F f[] = {{&ctx->cx, cx, 8}, {&ctx->cy, cy, 8}, {&ctx->hw, hw, 8}, {&ctx->mass, mass, 8},
             {&ctx->comx, comx, 8}, {&ctx->comy, comy, 8}, {&ctx->bs, bs32.data(), 4}, {&ctx->be, be32.data(), 4},
             {&ctx->child, child, 16}, {&ctx->parent, parent, 4}, {&ctx->is_leaf, is_leaf, 1},
             {&ctx->vlen, vlist_len, 1}, {&ctx->ulen, ulist_len, 1},
             {&ctx->vdata, vlist_data, 4 * GX_LIST_CAP}, {&ctx->udata, ulist_data, 4 * GX_LIST_CAP}};
    for (auto &e : f) {
        GX_TRY(gx_ensure(ctx, *e.b, e.sz * (size_t)(n_nodes > 0 ? n_nodes : 1)));
        if (n_nodes > 0)
            GX_CUDA(ctx, cudaMemcpyAsync(e.b->p, e.src, e.sz * (size_t)n_nodes, cudaMemcpyHostToDevice, ctx->stream));
    }
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->n_nodes = n_nodes;
    ctx->n_leaves = nl;
    ctx->n_levels = n_nodes > 0 ? maxlev + 1 : 0;
    ctx->level_start = n_nodes > 0 ? ls : std::vector<int64_t>(1, 0);
    if (ctx->have_bodies && ctx->n_bodies != n_bodies) ctx->have_bodies = false;
    ctx->n_bodies = n_bodies;
    ctx->max_leaf = 0;
    for (int64_t i = 0; i < nl; i++) ctx->max_leaf = std::max(ctx->max_leaf, body_end[i] - body_start[i]);
    ctx->ref_lists_valid = true;  // the caller's lists
    ctx->have_tree = true;
    return GX_OK;
}

int gx_rebuild_resident(gx_ctx *ctx, int64_t n_max, const double bounds[4], int flags, int64_t *perm) {
    GX_TRY(check_ctx(ctx));
    if (n_max <= 0 || !bounds) return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad n_max or bounds");
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "no resident bodies: call gx_upload_bodies first");
    ctx->build_n_max = n_max;
    for (int k = 0; k < 4; k++) ctx->build_bounds[k] = bounds[k];
    ctx->build_flags = flags;
    ctx->roll_valid = false;
    GX_TRY(gx_rebuild_internal(ctx));
    const int64_t n = ctx->n_bodies;
    if (perm && n > 0) {
        if (flags & GX_BUILD_BALANCED) {
            for (int64_t i = 0; i < n; i++) perm[i] = i;  // build_constrained does not reorder
        } else {
            std::vector<uint32_t> p32((size_t)n);
            GX_CUDA(ctx, cudaMemcpyAsync(p32.data(), ctx->perm.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost,
                                         ctx->stream));
            GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int64_t i = 0; i < n; i++) perm[i] = p32[(size_t)i];
        }
    }
    return GX_OK;
}

int gx_body_ids(gx_ctx *ctx, int64_t *ids) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "no resident bodies");
    if (!ids) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null array");
    const int64_t n = ctx->n_bodies;
    if (n == 0) return GX_OK;
    if (ctx->ids.bytes < sizeof(int32_t) * (size_t)n) GX_TRY(gx_ids_reset(ctx));
    std::vector<int32_t> v((size_t)n);
    GX_CUDA(ctx, cudaMemcpyAsync(v.data(), ctx->ids.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t i = 0; i < n; i++) ids[i] = v[(size_t)i];
    return GX_OK;
}

int gx_morton_encode(gx_ctx *ctx, int64_t n, const double *x, const double *y, const double bounds[4],
                     uint64_t *keys) {
    GX_TRY(check_ctx(ctx));
    if (n < 0 || (n > 0 && (!x || !y || !keys)) || !bounds) return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad arguments");
    if (n == 0) return GX_OK;
    GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(double) * 2 * (size_t)n));
    GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(uint64_t) * (size_t)n));
    double *dx = dptr<double>(ctx->scratch_a), *dy = dx + n;
    GX_CUDA(ctx, cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(dy, y, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    gx_launch_morton(ctx, dx, dy, n, bounds, dptr<uint64_t>(ctx->scratch_b), nullptr);
    GX_CUDA(ctx, cudaGetLastError());
    GX_CUDA(ctx, cudaMemcpyAsync(keys, ctx->scratch_b.p, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

int gx_tree_info(gx_ctx *ctx, int64_t *n_nodes, int64_t *n_leaves, int32_t *n_levels, int64_t *n_bodies) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_tree) return gx_fail(ctx, GX_ERR_STATE, "no tree");
    if (n_nodes) *n_nodes = ctx->n_nodes;
    if (n_leaves) *n_leaves = ctx->n_leaves;
    if (n_levels) *n_levels = ctx->n_levels;
    if (n_bodies) *n_bodies = ctx->n_bodies;
    return GX_OK;
}

int gx_export_tree(gx_ctx *ctx, double *cx, double *cy, double *hw, double *mass, double *comx, double *comy,
                   int64_t *body_start, int64_t *body_end, int32_t *child, int32_t *parent, uint8_t *is_leaf,
                   int64_t *level_start) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_tree) return gx_fail(ctx, GX_ERR_STATE, "no tree");
    size_t nn = (size_t)ctx->n_nodes;
    if (nn > 0) {
        struct F { DevBuf *b; void *dst; size_t sz; };
        F f[] = {{&ctx->cx, cx, 8}, {&ctx->cy, cy, 8}, {&ctx->hw, hw, 8}, {&ctx->mass, mass, 8},
                 {&ctx->comx, comx, 8}, {&ctx->comy, comy, 8}, {&ctx->child, child, 16}, {&ctx->parent, parent, 4},
                 {&ctx->is_leaf, is_leaf, 1}};
        for (auto &e : f)
            if (e.dst) GX_CUDA(ctx, cudaMemcpyAsync(e.dst, e.b->p, e.sz * nn, cudaMemcpyDeviceToHost, ctx->stream));
        std::vector<int32_t> b32(nn), e32(nn);
        GX_CUDA(ctx, cudaMemcpyAsync(b32.data(), ctx->bs.p, 4 * nn, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(e32.data(), ctx->be.p, 4 * nn, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < nn; i++) {
            if (body_start) body_start[i] = b32[i];
            if (body_end) body_end[i] = e32[i];
        }
    }
    if (level_start)
        for (size_t i = 0; i < ctx->level_start.size(); i++) level_start[i] = ctx->level_start[i];
    return GX_OK;
}

int gx_export_lists(gx_ctx *ctx, int which, uint32_t *data, uint8_t *lengths) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_tree) return gx_fail(ctx, GX_ERR_STATE, "no tree");
    if (which != GX_LIST_V && which != GX_LIST_U) return gx_fail(ctx, GX_ERR_INVALID_ARG, "unknown list");
    if (!ctx->ref_lists_valid) GX_TRY(gx_lists_build_ref(ctx));
    DevBuf &d = which == GX_LIST_V ? ctx->vdata : ctx->udata;
    DevBuf &l = which == GX_LIST_V ? ctx->vlen : ctx->ulen;
    size_t nn = (size_t)ctx->n_nodes;
    if (nn == 0) return GX_OK;
    if (data) GX_CUDA(ctx, cudaMemcpyAsync(data, d.p, 4 * GX_LIST_CAP * nn, cudaMemcpyDeviceToHost, ctx->stream));
    if (lengths) GX_CUDA(ctx, cudaMemcpyAsync(lengths, l.p, nn, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

static int ensure_plan(gx_ctx *ctx) {
    if (!ctx->have_tree) return gx_fail(ctx, GX_ERR_STATE, "no tree: call gx_build_tree or gx_upload_tree first");
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "no bodies");
    if (!ctx->aux_valid) GX_TRY(gx_plan_tree_aux(ctx));
    if (ctx->mode == GX_MODE_ACCURATE) {
        if (!ctx->plan_acc_valid || ctx->plan_theta != ctx->theta || ctx->plan_theta_w != ctx->theta_w) {
            GX_TRY(gx_plan_accurate(ctx));
            if (ctx->theta_w > 0.0) GX_TRY(gx_plan_near_split(ctx));
            GX_TRY(gx_plan_items(ctx, true));
            GX_TRY(gx_plan_body_masks(ctx));
            ctx->plan_theta_w = ctx->theta_w;
        }
    } else {
        if (!ctx->ref_lists_valid) {
            GX_TRY(gx_lists_build_ref(ctx));
            ctx->plan_ref_valid = false;
        }
        if (!ctx->plan_ref_valid || ctx->plan_p != ctx->p || ctx->plan_eps != ctx->eps) {
            GX_TRY(gx_plan_ref(ctx));
            GX_TRY(gx_plan_items(ctx, false));
        }
    }
    return GX_OK;
}

}  // extern "C"
int gx_ensure_plan_public(gx_ctx *ctx) { return ensure_plan(ctx); }
extern "C" {

int gx_plan_split_info(gx_ctx *ctx, int64_t *n_m2p_pairs, int64_t *n_p2l_pairs) {
    GX_TRY(check_ctx(ctx));
    GX_TRY(ensure_plan(ctx));
    const bool on = ctx->mode == GX_MODE_ACCURATE && ctx->theta_w > 0.0;
    if (n_m2p_pairs) *n_m2p_pairs = on ? ctx->n_m2p_pairs : 0;
    if (n_p2l_pairs) *n_p2l_pairs = on ? ctx->n_p2l_pairs : 0;
    return GX_OK;
}

int gx_plan_body_split_info(gx_ctx *ctx, int64_t *n_p2p_moved, int64_t *n_body_p2l) {
    GX_TRY(check_ctx(ctx));
    GX_TRY(ensure_plan(ctx));
    int64_t moved = 0, evals = 0;
    if (ctx->plan_body_split && gx_body_split_on(ctx)) {
        // from host copies of the P2P items and their masks: a masked body of row (a <- s)
        // moves |a| interactions to one body-P2L evaluation
        const gx_ctx::Items &I = ctx->items_acc;
        const int64_t nn = ctx->n_nodes;
        std::vector<int32_t> leaf((size_t)I.n + 1), nq((size_t)I.n + 1), bs((size_t)nn), be((size_t)nn);
        std::vector<int64_t> qb((size_t)I.n + 1);
        if (I.n > 0) {
            GX_CUDA(ctx, cudaMemcpyAsync(leaf.data(), I.leaf.p, 4 * I.n, cudaMemcpyDeviceToHost, ctx->stream));
            GX_CUDA(ctx, cudaMemcpyAsync(nq.data(), I.nq.p, 4 * I.n, cudaMemcpyDeviceToHost, ctx->stream));
            GX_CUDA(ctx, cudaMemcpyAsync(qb.data(), I.qb.p, 8 * I.n, cudaMemcpyDeviceToHost, ctx->stream));
        }
        GX_CUDA(ctx, cudaMemcpyAsync(bs.data(), ctx->bs.p, 4 * nn, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(be.data(), ctx->be.p, 4 * nn, cudaMemcpyDeviceToHost, ctx->stream));
        const size_t nm = ctx->p2p_mask.bytes / 4;
        std::vector<uint32_t> mask(nm);
        GX_CUDA(ctx, cudaMemcpyAsync(mask.data(), ctx->p2p_mask.p, 4 * nm, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int64_t it = 0; it < I.n; it++) {
            if (nq[it] <= 0) continue;
            const int64_t nt = be[leaf[it]] - bs[leaf[it]];
            for (int k = 0; k < nq[it]; k++) {
                const int64_t c = __builtin_popcount(mask[qb[it] + k]);
                evals += c;
                moved += c * nt;
            }
        }
    }
    if (n_p2p_moved) *n_p2p_moved = moved;
    if (n_body_p2l) *n_body_p2l = evals;
    return GX_OK;
}

int gx_plan_info(gx_ctx *ctx, int64_t *n_far_pairs, int64_t *n_near_pairs, int64_t *n_p2p_interactions) {
    GX_TRY(check_ctx(ctx));
    GX_TRY(ensure_plan(ctx));
    if (ctx->mode == GX_MODE_ACCURATE) {
        if (n_far_pairs) *n_far_pairs = ctx->n_far_pairs;
        if (n_near_pairs) *n_near_pairs = ctx->n_near_pairs;
    } else {
        if (n_far_pairs) *n_far_pairs = ctx->n_v_pairs;
        if (n_near_pairs) *n_near_pairs = ctx->n_p2p_pairs;
    }
    if (n_p2p_interactions) {
        // sum over target leaves of (targets x sources), from the host copy of the lists
        int64_t nl = ctx->n_leaves, nn = ctx->n_nodes;
        std::vector<int32_t> bs((size_t)nn), be((size_t)nn);
        GX_CUDA(ctx, cudaMemcpyAsync(bs.data(), ctx->bs.p, 4 * nn, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(be.data(), ctx->be.p, 4 * nn, cudaMemcpyDeviceToHost, ctx->stream));
        std::vector<int64_t> st((size_t)nl + 1);
        std::vector<int32_t> cnt((size_t)nl);
        int64_t tot_idx;
        const int32_t *idxp;
        if (ctx->mode == GX_MODE_ACCURATE) {
            GX_CUDA(ctx, cudaMemcpyAsync(st.data(), ctx->near_off.p, 8 * nl, cudaMemcpyDeviceToHost, ctx->stream));
            GX_CUDA(ctx, cudaMemcpyAsync(cnt.data(), static_cast<char *>(ctx->near_off.p) + 8 * nn, 4 * nl,
                                         cudaMemcpyDeviceToHost, ctx->stream));
            idxp = dptr<int32_t>(ctx->near_idx);
            GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            tot_idx = 0;
            for (int64_t a = 0; a < nl; a++) tot_idx = std::max(tot_idx, st[a] + cnt[a]);
        } else {
            GX_CUDA(ctx, cudaMemcpyAsync(st.data(), ctx->p2p_off.p, 8 * (nl + 1), cudaMemcpyDeviceToHost, ctx->stream));
            GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int64_t a = 0; a < nl; a++) cnt[a] = (int32_t)(st[a + 1] - st[a]);
            idxp = dptr<int32_t>(ctx->p2p_idx);
            tot_idx = st[nl];
        }
        std::vector<int32_t> idx((size_t)tot_idx + 1);
        if (tot_idx > 0)
            GX_CUDA(ctx, cudaMemcpyAsync(idx.data(), idxp, 4 * tot_idx, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int64_t inter = 0;
        for (int64_t a = 0; a < nl; a++) {
            int64_t nt = be[a] - bs[a], ns = 0;
            for (int64_t q = st[a]; q < st[a] + cnt[a]; q++) ns += be[idx[q]] - bs[idx[q]];
            inter += nt * ns - nt;  // minus self pairs
        }
        *n_p2p_interactions = inter;
    }
    return GX_OK;
}

// The device address of a page-locked host array of n doubles (cudaHostAlloc or
// cudaHostRegister), or null for any other memory.
// The array counts as mapped only when its first and its last element resolve to the
// same page-locked allocation (a registered range shorter than the array would let a
// kernel run past it over the host link); otherwise it takes the staged copies.
static double *mapped_host(const double *p, int64_t n) {
    if (!p || n <= 0) return nullptr;
    cudaPointerAttributes at{}, at_last{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory on older runtimes: not an error of the call
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    if (cudaPointerGetAttributes(&at_last, p + (n - 1)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at_last.type != cudaMemoryTypeHost ||
        static_cast<const double *>(at_last.devicePointer) != static_cast<const double *>(at.devicePointer) + (n - 1))
        return nullptr;
    return static_cast<double *>(at.devicePointer);
}

// Whether ensure_plan has nothing to do (the plan of the current tree and mode exists).
static bool plan_current(const gx_ctx *ctx) {
    if (!ctx->have_tree || !ctx->have_bodies || !ctx->aux_valid) return false;
    if (ctx->mode == GX_MODE_ACCURATE)
        return ctx->plan_acc_valid && ctx->plan_theta == ctx->theta && ctx->plan_theta_w == ctx->theta_w;
    return ctx->ref_lists_valid && ctx->plan_ref_valid && ctx->plan_p == ctx->p && ctx->plan_eps == ctx->eps;
}

// Enqueue one evaluation (the plan first if it is stale).
static int forces_launch(gx_ctx *ctx, bool timed) {
    GX_TRY(ensure_plan(ctx));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
    return gx_forces_device(ctx, timed);
}

// Wait for the stream, check the device status word, record the pass timings.
static int forces_finish(gx_ctx *ctx, bool timed) {
    unsigned st = 0;
    GX_TRY(sync_status(ctx, &st));
    ctx->last_status = st;
    if (timed && ctx->n_nodes > 0) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[6]);
        ctx->last_ms[0] = ms;
        for (int k = 0; k < 6; k++) {
            cudaEventElapsedTime(&ms, ctx->ev[k], ctx->ev[k + 1]);
            ctx->last_ms[k + 1] = ms;
        }
        cudaEventElapsedTime(&ms, ctx->ev[14], ctx->ev[15]);
        ctx->last_p2p_ms = ms;
    }
    return GX_OK;
}

static int forces_and_check(gx_ctx *ctx, bool timed) {
    GX_TRY(forces_launch(ctx, timed));
    return forces_finish(ctx, timed);
}

int gx_compute_forces(gx_ctx *ctx, const double *x, const double *y, const double *m, double *ax, double *ay) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_tree) return gx_fail(ctx, GX_ERR_STATE, "no tree: call gx_build_tree or gx_upload_tree first");
    if (!x || !y || !m || !ax || !ay) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null array");
    int64_t n = ctx->n_bodies;
    // page-locked inputs are read by the evaluation's first kernel itself (no separate
    // copies), page-locked outputs written by its last one, so that the transfers over
    // the host link overlap those kernels instead of preceding or following them
    const double *hx = mapped_host(x, n), *hy = mapped_host(y, n), *hm = mapped_host(m, n);
    double *hax = mapped_host(ax, n), *hay = mapped_host(ay, n);
    const bool direct_in = hx && hy && hm && plan_current(ctx);  // a plan built now would read the old positions
    const bool direct = hax && hay && ctx->n_nodes > 0;
    if (direct_in) {
        GX_TRY(upload_bodies_impl(ctx, n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false));
        ctx->in_x = hx;
        ctx->in_y = hy;
        ctx->in_m = hm;
    } else {
        GX_TRY(upload_bodies_impl(ctx, n, x, y, nullptr, nullptr, m, nullptr, nullptr, false));
    }
    if (direct) {
        ctx->out_ax = hax;
        ctx->out_ay = hay;
    }
    const int rc = forces_launch(ctx, true);
    ctx->out_ax = ctx->out_ay = nullptr;
    ctx->in_x = ctx->in_y = ctx->in_m = nullptr;
    // kernels enqueued before a failure may still read or write the caller's arrays:
    // let them finish before the call returns
    if (rc != GX_OK && (direct || direct_in)) cudaStreamSynchronize(ctx->stream);
    GX_TRY(rc);
    // otherwise the read-back is queued behind the evaluation: one wait for both
    if (n > 0 && !direct) {
        GX_CUDA(ctx, cudaMemcpyAsync(ax, ctx->ax.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(ay, ctx->ay.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    return forces_finish(ctx, true);
}

int gx_forces_resident(gx_ctx *ctx) {
    GX_TRY(check_ctx(ctx));
    return forces_and_check(ctx, true);
}

int gx_kdk_run(gx_ctx *ctx, int64_t n_steps, double dt, int64_t energy_every, double *diag, int64_t *n_diag) {
    return gx_kdk_run_rebuild(ctx, n_steps, dt, energy_every, 0, diag, n_diag);
}

int gx_kdk_run_rebuild(gx_ctx *ctx, int64_t n_steps, double dt, int64_t energy_every, int64_t rebuild_every,
                       double *diag, int64_t *n_diag) {
    GX_TRY(check_ctx(ctx));
    if (n_steps < 0 || rebuild_every < 0) return gx_fail(ctx, GX_ERR_INVALID_ARG, "n_steps < 0 or rebuild_every < 0");
    if (rebuild_every > 0 && ctx->build_n_max <= 0)
        return gx_fail(ctx, GX_ERR_STATE, "rebuilds need the parameters of a device tree build");
    GX_TRY(ensure_plan(ctx));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
    GX_TRY(gx_kdk_device(ctx, n_steps, dt, energy_every, diag, n_diag, rebuild_every));
    return GX_OK;
}

int gx_diagnostics(gx_ctx *ctx, double out[5]) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "no resident bodies");
    if (!out) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null output");
    return gx_diag_device(ctx, out);
}

int gx_n2_sampled(gx_ctx *ctx, const int64_t *idx, int64_t n_idx, double *ax, double *ay) {
    GX_TRY(check_ctx(ctx));
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "no resident bodies");
    if (n_idx < 0 || (n_idx > 0 && (!idx || !ax || !ay))) return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad sample arrays");
    return gx_n2_device(ctx, idx, n_idx, ax, ay);
}

int gx_last_timings(gx_ctx *ctx, double out[7]) {
    GX_TRY(check_ctx(ctx));
    if (!out) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null output");
    for (int k = 0; k < 7; k++) out[k] = ctx->last_ms[k];
    return GX_OK;
}

int gx_last_status(gx_ctx *ctx, uint32_t *status) {
    GX_TRY(check_ctx(ctx));
    if (!status) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null output");
    *status = ctx->last_status & GX_STATUS_SANITIZED;
    return GX_OK;
}

int gx_last_launch_count(gx_ctx *ctx, int64_t *count) {
    GX_TRY(check_ctx(ctx));
    if (!count) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null output");
    *count = ctx->last_launches;
    return GX_OK;
}

int gx_bench_forces(gx_ctx *ctx, int32_t reps, int32_t flush_l2, double *ms_each, int32_t which,
                    double *kernel_ms_each) {
    GX_TRY(check_ctx(ctx));
    if (reps <= 0) return gx_fail(ctx, GX_ERR_INVALID_ARG, "reps <= 0");
    GX_TRY(ensure_plan(ctx));
    size_t flush_bytes = (size_t)256 << 20;  // twice the 129 MB L2
    if (flush_l2) GX_TRY(gx_ensure(ctx, ctx->flush, flush_bytes));
    ctx->near_after_far = which == 2;
    for (int r = 0; r < reps; r++) {
        if (flush_l2) GX_CUDA(ctx, cudaMemsetAsync(ctx->flush.p, r & 0xff, flush_bytes, ctx->stream));
        const int rc = forces_and_check(ctx, true);
        if (rc != GX_OK) {
            ctx->near_after_far = false;
            return rc;
        }
        if (ms_each) ms_each[r] = ctx->last_ms[0];
        if (kernel_ms_each) kernel_ms_each[r] = which == 1 ? ctx->last_ms[4] : ctx->last_p2p_ms;
    }
    ctx->near_after_far = false;
    return GX_OK;
}

void *gx_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void gx_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
