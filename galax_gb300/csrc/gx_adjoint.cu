// gx_adjoint.cu -- reverse-mode differentiation of the force evaluation and of the
// leapfrog rollout, with checkpoints.  Kernels in gx_adjoint_impl.cuh.
//
// Rollout (galax-integrate/src/lib.rs:158-189, static tree):
//   v' = v_n + h/2 a_n,  x_{n+1} = x_n + h v',  a_{n+1} = F(x_{n+1}, m),  v_{n+1} = v' + h/2 a_{n+1}
// Reverse step n, holding lx = dL/dx_{n+1}, lv = dL/dv_{n+1}:
//   la = c lv with c = h (each interior a_{n+1} feeds two half kicks) or h/2 at n+1 = T
//   (gx, gm) = VJP_F(x_{n+1}; la);  lx += gx;  lm += gm
//   lv += h lx;  (lx, lv) now hold dL/dx_n, dL/dv_n
// and finally VJP_F(x_0; h/2 lv_0).  The forward keeps a checkpoint every k steps
// (positions, velocities, accelerations and the leaf locals of that evaluation); the
// backward recomputes the k-1 interior states of each segment from its checkpoint
// (k = 1 stores every state and recomputes nothing).  The kernels are deterministic,
// so the recomputed states are the forward ones bit for bit.
#include "gx_internal.cuh"

#define GX_VJP_DECL(PP)                                                                                 \
    int gx_run_force_vjp_##PP(gx_ctx *, int, const double *, const double *, const void *, const double *, \
                              const double *, double *, double *, double *);
GX_VJP_DECL(0)
GX_VJP_DECL(1)
GX_VJP_DECL(2)
GX_VJP_DECL(3)
GX_VJP_DECL(4)
GX_VJP_DECL(5)
GX_VJP_DECL(6)
GX_VJP_DECL(7)
GX_VJP_DECL(8)

namespace {

// VJP at positions (X, Y) with the forward's leaf locals lf of those positions, in the
// context's precision (FP32 rows for the mixed form, FP64 rows otherwise).
int force_vjp(gx_ctx *ctx, const double *X, const double *Y, const void *lf, const double *lx, const double *ly,
              double *gx, double *gy, double *gm) {
    int f32 = ctx->prec == GX_PREC_MIXED;
    switch (ctx->p) {
        case 0: return gx_run_force_vjp_0(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 1: return gx_run_force_vjp_1(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 2: return gx_run_force_vjp_2(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 3: return gx_run_force_vjp_3(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 4: return gx_run_force_vjp_4(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 5: return gx_run_force_vjp_5(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 6: return gx_run_force_vjp_6(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 7: return gx_run_force_vjp_7(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        case 8: return gx_run_force_vjp_8(ctx, f32, X, Y, lf, lx, ly, gx, gy, gm);
        default: return gx_fail(ctx, GX_ERR_INVALID_ARG, "the adjoint supports p in 0..8");
    }
}

// bytes of one set of leaf locals in the context's precision, rounded up to 256
size_t lf_bytes(const gx_ctx *ctx) {
    int nc = (ctx->p + 1) * (ctx->p + 2) / 2;
    size_t row = ctx->prec == GX_PREC_MIXED ? sizeof(float) * (size_t)((nc + 3) / 4 * 4)
                                            : sizeof(double) * (size_t)((nc + 1) / 2 * 2);
    size_t b = row * (size_t)(ctx->n_leaves > 0 ? ctx->n_leaves : 1);
    return (b + 255) / 256 * 256;
}
// the leaf locals of the last forward evaluation
const void *current_lf(const gx_ctx *ctx) { return ctx->prec == GX_PREC_MIXED ? ctx->Lff32.p : ctx->Lf.p; }

__global__ void k_axpy(int64_t n, double a, const double *x, double *y) {  // y += a x
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __dadd_rn(y[i], __dmul_rn(a, x[i]));
}

// lx += gx; ly += gy; lm += gm; lvx += dt lx; lvy += dt ly (one reverse leapfrog step)
__global__ void k_adj_step(int64_t n, double dt, const double *gx, const double *gy, const double *gm, double *lx,
                           double *ly, double *lm, double *lvx, double *lvy) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = __dadd_rn(lx[i], gx[i]), b = __dadd_rn(ly[i], gy[i]);
    lx[i] = a;
    ly[i] = b;
    lm[i] = __dadd_rn(lm[i], gm[i]);
    lvx[i] = __dadd_rn(lvx[i], __dmul_rn(dt, a));
    lvy[i] = __dadd_rn(lvy[i], __dmul_rn(dt, b));
}

__global__ void k_scale2(int64_t n, double c, const double *x, const double *y, double *ox, double *oy) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ox[i] = __dmul_rn(c, x[i]);
    oy[i] = __dmul_rn(c, y[i]);
}

__global__ void k_kick_drift_a(int64_t n, double h, double dt, double *x, double *y, double *vx, double *vy,
                               const double *ax, const double *ay) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double u = __dadd_rn(vx[i], __dmul_rn(ax[i], h));
    double v = __dadd_rn(vy[i], __dmul_rn(ay[i], h));
    vx[i] = u;
    vy[i] = v;
    x[i] = __dadd_rn(x[i], __dmul_rn(u, dt));
    y[i] = __dadd_rn(y[i], __dmul_rn(v, dt));
}

__global__ void k_kick_a(int64_t n, double h, double *vx, double *vy, const double *ax, const double *ay) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vx[i] = __dadd_rn(vx[i], __dmul_rn(ax[i], h));
    vy[i] = __dadd_rn(vy[i], __dmul_rn(ay[i], h));
}

int check_mode(gx_ctx *ctx) {
    if (!ctx->have_tree || !ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "adjoint needs a tree and bodies");
    if (ctx->mode != GX_MODE_ACCURATE)
        return gx_fail(ctx, GX_ERR_STATE, "the adjoint is defined for GX_MODE_ACCURATE (set it with gx_set_mode)");
    if (ctx->theta_w > 0.0)
        return gx_fail(ctx, GX_ERR_STATE,
                       "the adjoint transposes P2P, not M2P/P2L: turn the near-list split off (gx_set_near_split 0)");
    return GX_OK;
}

// Checkpoint slot j holds the state after min(j K, T) steps: x, y, vx, vy, ax, ay, m
// (FP64, in that state's body order) and the leaf locals of its force evaluation.
constexpr int SLOT_ARRAYS = 7;
struct Slots {
    char *base;
    size_t stride, lfoff;
    int64_t n;
    double *x(int64_t j) const { return reinterpret_cast<double *>(base + (size_t)j * stride); }
    double *arr(int64_t j, int k) const { return x(j) + (size_t)k * (size_t)n; }
    void *lf(int64_t j) const { return base + (size_t)j * stride + lfoff; }
};
Slots ckpt_slots(gx_ctx *ctx) {
    int64_t n = ctx->n_bodies > 0 ? ctx->n_bodies : 1;
    size_t lfoff = (sizeof(double) * SLOT_ARRAYS * (size_t)n + 255) / 256 * 256;
    return Slots{reinterpret_cast<char *>(ctx->ckpt.p), lfoff + lf_bytes(ctx), lfoff, n};
}

// out[perm[i]] = in[i] for five arrays (cotangents back to the order before a rebuild)
__global__ void k_unpermute5(int64_t n, const uint32_t *perm, const double *a0, const double *a1, const double *a2,
                             const double *a3, const double *a4, double *b0, double *b1, double *b2, double *b3,
                             double *b4) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t j = perm[i];
    b0[j] = a0[i];
    b1[j] = a1[i];
    b2[j] = a2[i];
    b3[j] = a3[i];
    b4[j] = a4[i];
}

// Rebuild the tree at the resident positions and record (or check nothing of) its
// permutation in slot k of the rollout's permutation store.
int rollout_rebuild(gx_ctx *ctx, int64_t k) {
    GX_TRY(gx_rebuild_internal(ctx));
    GX_TRY(gx_ensure_plan_public(ctx));
    if (k >= 0) {
        const size_t pb = sizeof(uint32_t) * (size_t)ctx->n_bodies;
        GX_CUDA(ctx, cudaMemcpyAsync(reinterpret_cast<char *>(ctx->roll_perms.p) + (size_t)k * pb, ctx->perm.p, pb,
                                     cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return GX_OK;
}

}  // namespace

extern "C" {

int gx_force_vjp(gx_ctx *ctx, const double *lam_x, const double *lam_y, double *gx, double *gy, double *gm) {
    if (!ctx) return GX_ERR_INVALID_ARG;
    GX_TRY(check_mode(ctx));
    if (!lam_x || !lam_y || !gx || !gy || !gm) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null array");
    GX_TRY(gx_ensure_plan_public(ctx));
    int64_t n = ctx->n_bodies;
    size_t b = sizeof(double) * (size_t)(n > 0 ? n : 1);
    DevBuf *bufs[] = {&ctx->adj_lx, &ctx->adj_ly, &ctx->adj_gx, &ctx->adj_gy, &ctx->adj_gm};
    for (DevBuf *d : bufs) GX_TRY(gx_ensure(ctx, *d, b));
    if (n == 0) return GX_OK;
    GX_CUDA(ctx, cudaMemcpyAsync(ctx->adj_lx.p, lam_x, b, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(ctx->adj_ly.p, lam_y, b, cudaMemcpyHostToDevice, ctx->stream));
    GX_TRY(gx_forces_device(ctx, false));  // the locals of the resident positions
    GX_TRY(force_vjp(ctx, dptr<double>(ctx->x), dptr<double>(ctx->y), current_lf(ctx), dptr<double>(ctx->adj_lx),
                     dptr<double>(ctx->adj_ly), dptr<double>(ctx->adj_gx), dptr<double>(ctx->adj_gy),
                     dptr<double>(ctx->adj_gm)));
    GX_CUDA(ctx, cudaMemcpyAsync(gx, ctx->adj_gx.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(gy, ctx->adj_gy.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(gm, ctx->adj_gm.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

int gx_rollout_forward(gx_ctx *ctx, int64_t n_steps, double dt, int64_t checkpoint_every, int64_t rebuild_every) {
    if (!ctx) return GX_ERR_INVALID_ARG;
    GX_TRY(check_mode(ctx));
    if (n_steps < 0 || checkpoint_every <= 0) return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad n_steps or interval");
    if (rebuild_every != 0 && rebuild_every != 1)
        return gx_fail(ctx, GX_ERR_INVALID_ARG, "rebuild_every must be 0 (static tree) or 1 (every step)");
    if (rebuild_every && (ctx->build_n_max <= 0 || (ctx->build_flags & GX_BUILD_BALANCED)))
        return gx_fail(ctx, GX_ERR_STATE, "rebuilds need the parameters of a (non-balanced) device tree build");
    GX_TRY(gx_ensure_plan_public(ctx));
    ctx->roll_valid = false;
    const int64_t n = ctx->n_bodies, T = n_steps, K = checkpoint_every;
    const int64_t nseg = (T + K - 1) / K;
    const size_t lfb = lf_bytes(ctx);
    {
        int64_t nn = n > 0 ? n : 1;
        size_t stride = (sizeof(double) * SLOT_ARRAYS * (size_t)nn + 255) / 256 * 256 + lfb;
        GX_TRY(gx_ensure(ctx, ctx->ckpt, stride * (size_t)(nseg + 1)));
        if (rebuild_every) GX_TRY(gx_ensure(ctx, ctx->roll_perms, sizeof(uint32_t) * (size_t)nn * (size_t)(T + 1)));
    }
    Slots S = ckpt_slots(ctx);
    const double h = 0.5 * dt;
    const unsigned g = gx_blocks(n, 256);
    DevBuf *st[SLOT_ARRAYS] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->ax, &ctx->ay, &ctx->m};
    auto save = [&](int64_t j) -> int {
        for (int k = 0; k < SLOT_ARRAYS; k++)
            GX_CUDA(ctx, cudaMemcpyAsync(S.arr(j, k), st[k]->p, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                         ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(S.lf(j), current_lf(ctx), lfb, cudaMemcpyDeviceToDevice, ctx->stream));
        return GX_OK;
    };
    GX_TRY(gx_ids_reset(ctx));  // gradients come back in the order the bodies have now
    if (rebuild_every && n > 0) GX_TRY(rollout_rebuild(ctx, 0));
    GX_TRY(gx_forces_device(ctx, false));  // a_0
    GX_TRY(save(0));
    for (int64_t s = 0; s < T && n > 0; s++) {
        k_kick_drift_a<<<g, 256, 0, ctx->stream>>>(n, h, dt, dptr<double>(ctx->x), dptr<double>(ctx->y),
                                                   dptr<double>(ctx->vx), dptr<double>(ctx->vy), dptr<double>(ctx->ax),
                                                   dptr<double>(ctx->ay));
        if (rebuild_every) GX_TRY(rollout_rebuild(ctx, s + 1));
        GX_TRY(gx_forces_device(ctx, false));
        k_kick_a<<<g, 256, 0, ctx->stream>>>(n, h, dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                             dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        ctx->launches += 2;
        if ((s + 1) % K == 0 || s + 1 == T) GX_TRY(save((s + 1 + K - 1) / K));
    }
    GX_CUDA(ctx, cudaGetLastError());
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->roll_steps = T;
    ctx->roll_dt = dt;
    ctx->roll_k = K;
    ctx->roll_prec = ctx->prec;
    ctx->roll_rebuild = rebuild_every;
    ctx->roll_valid = true;
    return GX_OK;
}

int gx_rollout_backward(gx_ctx *ctx, const double *lx, const double *ly, const double *lvx, const double *lvy,
                        double *gx0, double *gy0, double *gvx0, double *gvy0, double *gm, int64_t *peak_bytes) {
    if (!ctx) return GX_ERR_INVALID_ARG;
    GX_TRY(check_mode(ctx));
    if (!ctx->roll_valid) return gx_fail(ctx, GX_ERR_STATE, "gx_rollout_backward needs gx_rollout_forward first");
    if (ctx->roll_prec != ctx->prec)
        return gx_fail(ctx, GX_ERR_STATE, "the precision changed between gx_rollout_forward and gx_rollout_backward");
    if (!lx || !ly || !lvx || !lvy || !gx0 || !gy0 || !gvx0 || !gvy0 || !gm)
        return gx_fail(ctx, GX_ERR_INVALID_ARG, "null array");
    const int64_t n = ctx->n_bodies, T = ctx->roll_steps, K = ctx->roll_k;
    const int64_t nseg = (T + K - 1) / K;
    const double dt = ctx->roll_dt, h = 0.5 * dt;
    const size_t b = sizeof(double) * (size_t)(n > 0 ? n : 1);
    const size_t lfb = lf_bytes(ctx);
    // adjoint state (lx, ly, lvx, lvy, lm), VJP outputs (gx, gy, gm), la
    DevBuf *bufs[] = {&ctx->adj_lx, &ctx->adj_ly, &ctx->adj_lvx, &ctx->adj_lvy, &ctx->adj_lm,
                      &ctx->adj_gx, &ctx->adj_gy, &ctx->adj_gm, &ctx->adj_lax, &ctx->adj_lay};
    for (DevBuf *d : bufs) GX_TRY(gx_ensure(ctx, *d, b));
    double *LX = dptr<double>(ctx->adj_lx), *LY = dptr<double>(ctx->adj_ly), *LVX = dptr<double>(ctx->adj_lvx),
           *LVY = dptr<double>(ctx->adj_lvy), *LM = dptr<double>(ctx->adj_lm), *GX = dptr<double>(ctx->adj_gx),
           *GY = dptr<double>(ctx->adj_gy), *GM = dptr<double>(ctx->adj_gm), *LAX = dptr<double>(ctx->adj_lax),
           *LAY = dptr<double>(ctx->adj_lay);
    // recomputed interior states of a segment: positions, masses (their order changes
    // with rebuilds) and leaf locals of up to K-1 states
    const size_t seg_arr = (3 * b + 255) / 256 * 256;
    const size_t seg_stride = seg_arr + lfb;
    GX_TRY(gx_ensure(ctx, ctx->seg, seg_stride * (size_t)(K > 1 ? K - 1 : 1)));
    Slots S = ckpt_slots(ctx);
    char *seg = reinterpret_cast<char *>(ctx->seg.p);
    auto seg_x = [&](int64_t j) { return reinterpret_cast<double *>(seg + (size_t)j * seg_stride); };
    auto seg_l = [&](int64_t j) { return static_cast<void *>(seg + (size_t)j * seg_stride + seg_arr); };
    const bool RB = ctx->roll_rebuild != 0;
    const uint32_t *perms = dptr<uint32_t>(ctx->roll_perms);
    // under the rebuild policy, the trees (and plans) built while a segment is
    // recomputed are kept and taken back by the reverse sweep instead of rebuilt
    const bool keep_trees = RB && K > 1;
    if (keep_trees && (int64_t)ctx->tp_cache.size() < K - 1) ctx->tp_cache.resize((size_t)(K - 1));
    // make (px, py, pm) the resident state and, under the rebuild policy, rebuild its
    // tree (the positions are already in that tree's order, so the bodies stay put)
    auto set_state = [&](const double *px, const double *py, const double *pm) -> int {
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->x.p, px, b, cudaMemcpyDeviceToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->y.p, py, b, cudaMemcpyDeviceToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->m.p, pm, b, cudaMemcpyDeviceToDevice, ctx->stream));
        if (RB) GX_TRY(rollout_rebuild(ctx, -1));
        return GX_OK;
    };
    // cotangents of the state after the rebuild of step k back to the order before it
    auto unpermute = [&](int64_t k) -> int {
        k_unpermute5<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, perms + (size_t)k * (size_t)n, LX, LY, LVX, LVY, LM,
                                                                 GX, GY, LAX, LAY, GM);
        ctx->launches++;
        std::swap(ctx->adj_lx.p, ctx->adj_gx.p);
        std::swap(ctx->adj_ly.p, ctx->adj_gy.p);
        std::swap(ctx->adj_lvx.p, ctx->adj_lax.p);
        std::swap(ctx->adj_lvy.p, ctx->adj_lay.p);
        std::swap(ctx->adj_lm.p, ctx->adj_gm.p);
        LX = dptr<double>(ctx->adj_lx);
        LY = dptr<double>(ctx->adj_ly);
        LVX = dptr<double>(ctx->adj_lvx);
        LVY = dptr<double>(ctx->adj_lvy);
        LM = dptr<double>(ctx->adj_lm);
        GX = dptr<double>(ctx->adj_gx);
        GY = dptr<double>(ctx->adj_gy);
        GM = dptr<double>(ctx->adj_gm);
        LAX = dptr<double>(ctx->adj_lax);
        LAY = dptr<double>(ctx->adj_lay);
        return GX_OK;
    };
    if (n > 0) {
        GX_CUDA(ctx, cudaMemcpyAsync(LX, lx, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(LY, ly, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(LVX, lvx, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(LVY, lvy, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemsetAsync(LM, 0, b, ctx->stream));
    }
    const unsigned g = gx_blocks(n, 256);
    DevBuf *st[SLOT_ARRAYS] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->ax, &ctx->ay, &ctx->m};
    for (int64_t sgi = nseg - 1; sgi >= 0 && n > 0; sgi--) {
        const int64_t s0 = sgi * K, s1 = std::min(T, s0 + K);
        // recompute the interior states s0+1 .. s1-1 from the checkpoint of s0
        if (s1 - s0 > 1) {
            for (int k = 0; k < SLOT_ARRAYS; k++)
                GX_CUDA(ctx, cudaMemcpyAsync(st[k]->p, S.arr(sgi, k), b, cudaMemcpyDeviceToDevice, ctx->stream));
            for (int64_t s = s0; s < s1 - 1; s++) {
                k_kick_drift_a<<<g, 256, 0, ctx->stream>>>(n, h, dt, dptr<double>(ctx->x), dptr<double>(ctx->y),
                                                           dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                           dptr<double>(ctx->ax), dptr<double>(ctx->ay));
                if (RB) GX_TRY(rollout_rebuild(ctx, -1));  // deterministic: the forward's permutation again
                GX_TRY(gx_forces_device(ctx, false));
                k_kick_a<<<g, 256, 0, ctx->stream>>>(n, h, dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                     dptr<double>(ctx->ax), dptr<double>(ctx->ay));
                ctx->launches += 2;
                int64_t j = s - s0;  // state s+1 -> seg slot s - s0
                GX_CUDA(ctx, cudaMemcpyAsync(seg_x(j), ctx->x.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
                GX_CUDA(ctx, cudaMemcpyAsync(seg_x(j) + n, ctx->y.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
                GX_CUDA(ctx, cudaMemcpyAsync(seg_x(j) + 2 * n, ctx->m.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
                GX_CUDA(ctx, cudaMemcpyAsync(seg_l(j), current_lf(ctx), lfb, cudaMemcpyDeviceToDevice, ctx->stream));
                if (keep_trees) gx_tree_plan_swap(ctx, ctx->tp_cache[(size_t)j]);  // keep state s+1's tree
            }
        }
        // reverse through the segment: state s+1 for s = s1-1 .. s0
        for (int64_t s = s1 - 1; s >= s0; s--) {
            const double *px, *py, *pm;
            const void *pl;
            if (s + 1 == s1) {
                px = S.arr(sgi + 1, 0);
                py = S.arr(sgi + 1, 1);
                pm = S.arr(sgi + 1, 6);
                pl = S.lf(sgi + 1);
            } else {
                px = seg_x(s - s0);
                py = seg_x(s - s0) + n;
                pm = seg_x(s - s0) + 2 * n;
                pl = seg_l(s - s0);
            }
            if (keep_trees && s + 1 != s1) {
                // state s+1 with the tree kept when it was recomputed: its bodies are in that
                // tree's order, so a rebuild would reproduce the same tree and plan
                GX_CUDA(ctx, cudaMemcpyAsync(ctx->x.p, px, b, cudaMemcpyDeviceToDevice, ctx->stream));
                GX_CUDA(ctx, cudaMemcpyAsync(ctx->y.p, py, b, cudaMemcpyDeviceToDevice, ctx->stream));
                GX_CUDA(ctx, cudaMemcpyAsync(ctx->m.p, pm, b, cudaMemcpyDeviceToDevice, ctx->stream));
                gx_tree_plan_swap(ctx, ctx->tp_cache[(size_t)(s - s0)]);
            } else {
                GX_TRY(set_state(px, py, pm));
            }
            const double c = (s + 1 == T) ? h : dt;  // a_{s+1} feeds one half kick at T, two elsewhere
            if (RB) {
                // cotangents of state s+1 are in its (rebuilt) order until the force VJP is done
                k_scale2<<<g, 256, 0, ctx->stream>>>(n, c, LVX, LVY, LAX, LAY);
                GX_TRY(force_vjp(ctx, px, py, pl, LAX, LAY, GX, GY, GM));
                k_adj_step<<<g, 256, 0, ctx->stream>>>(n, 0.0, GX, GY, GM, LX, LY, LM, LVX, LVY);
                GX_TRY(unpermute(s + 1));
                k_axpy<<<g, 256, 0, ctx->stream>>>(n, dt, LX, LVX);
                k_axpy<<<g, 256, 0, ctx->stream>>>(n, dt, LY, LVY);
                ctx->launches += 4;
            } else {
                k_scale2<<<g, 256, 0, ctx->stream>>>(n, c, LVX, LVY, LAX, LAY);
                GX_TRY(force_vjp(ctx, px, py, pl, LAX, LAY, GX, GY, GM));
                k_adj_step<<<g, 256, 0, ctx->stream>>>(n, dt, GX, GY, GM, LX, LY, LM, LVX, LVY);
                ctx->launches += 2;
            }
        }
        GX_CUDA(ctx, cudaGetLastError());
    }
    if (n > 0) {
        // a_0 feeds the first half kick only
        GX_TRY(set_state(S.arr(0, 0), S.arr(0, 1), S.arr(0, 6)));
        k_scale2<<<g, 256, 0, ctx->stream>>>(n, h, LVX, LVY, LAX, LAY);
        GX_TRY(force_vjp(ctx, S.arr(0, 0), S.arr(0, 1), S.lf(0), LAX, LAY, GX, GY, GM));
        k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GX, LX);
        k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GY, LY);
        k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GM, LM);
        ctx->launches += 4;
        if (RB) GX_TRY(unpermute(0));  // back to the order the bodies had when the rollout began
        GX_CUDA(ctx, cudaMemcpyAsync(gx0, LX, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gy0, LY, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gvx0, LVX, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gvy0, LVY, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gm, LM, b, cudaMemcpyDeviceToHost, ctx->stream));
    }
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (peak_bytes) {
        size_t tot = ctx->ckpt.bytes + ctx->seg.bytes + ctx->adj_dL.bytes + ctx->adj_dM.bytes + ctx->adj_dMleaf.bytes +
                     ctx->adj_lam32.bytes + (ctx->roll_rebuild ? ctx->roll_perms.bytes : 0);
        for (DevBuf *d : bufs) tot += d->bytes;
        if (keep_trees)
            for (const gx_tree_plan &t : ctx->tp_cache) tot += gx_tree_plan_bytes(t);
        *peak_bytes = (int64_t)tot;
    }
    return GX_OK;
}

}  // extern "C"
