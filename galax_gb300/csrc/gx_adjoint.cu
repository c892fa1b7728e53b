// gx_adjoint.cu -- reverse-mode differentiation of the force evaluation and of the
// leapfrog rollout, with checkpoints.  Kernels in gx_adjoint_impl.cuh.
//
// Rollout (galax-integrate/src/lib.rs:158-189, static tree):
//   v' = v_n + h/2 a_n,  x_{n+1} = x_n + h v',  a_{n+1} = F(x_{n+1}, m),  v_{n+1} = v' + h/2 a_{n+1}
// Reverse step n, holding lx = dL/dx_{n+1}, lv = dL/dv_{n+1}:
//   la = c lv with c = h (each interior a_{n+1} feeds two half kicks) or h/2 at n+1 = T
//   (gx, gm) = VJP_F(x_{n+1}; la);  lx += gx;  lm += gm
//   lv += h lx;  (lx, lv) now hold dL/dx_n, dL/dv_n
// and finally VJP_F(x_0; h/2 lv_0).  States are recomputed from checkpoints taken
// every k steps; the kernels are deterministic, so the recomputed states are the
// forward ones bit for bit.
#include "gx_internal.cuh"

int gx_run_force_vjp_1(gx_ctx *, const double *, const double *, double *, double *, double *);
int gx_run_force_vjp_2(gx_ctx *, const double *, const double *, double *, double *, double *);
int gx_run_force_vjp_3(gx_ctx *, const double *, const double *, double *, double *, double *);
int gx_run_force_vjp_4(gx_ctx *, const double *, const double *, double *, double *, double *);
int gx_run_force_vjp_5(gx_ctx *, const double *, const double *, double *, double *, double *);
int gx_run_force_vjp_6(gx_ctx *, const double *, const double *, double *, double *, double *);
int gx_run_force_vjp_8(gx_ctx *, const double *, const double *, double *, double *, double *);

namespace {

int force_vjp(gx_ctx *ctx, const double *lx, const double *ly, double *gx, double *gy, double *gm) {
    switch (ctx->p) {
        case 1: return gx_run_force_vjp_1(ctx, lx, ly, gx, gy, gm);
        case 2: return gx_run_force_vjp_2(ctx, lx, ly, gx, gy, gm);
        case 3: return gx_run_force_vjp_3(ctx, lx, ly, gx, gy, gm);
        case 4: return gx_run_force_vjp_4(ctx, lx, ly, gx, gy, gm);
        case 5: return gx_run_force_vjp_5(ctx, lx, ly, gx, gy, gm);
        case 6: return gx_run_force_vjp_6(ctx, lx, ly, gx, gy, gm);
        case 8: return gx_run_force_vjp_8(ctx, lx, ly, gx, gy, gm);
        default: return gx_fail(ctx, GX_ERR_INVALID_ARG, "the adjoint supports p in {1,2,3,4,5,6,8}");
    }
}

int row_stride_f64(int p) {
    int nc = (p + 1) * (p + 2) / 2;
    return (nc + 1) / 2 * 2;
}
int row_stride_f32(int p) {
    int nc = (p + 1) * (p + 2) / 2;
    return (nc + 3) / 4 * 4;
}

// FP32 leaf locals (mixed forward) -> FP64 rows for the VJP
__global__ void k_widen_rows(int64_t nl, int nc, int ns32, int ns64, const float *in, double *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nl * nc) return;
    int64_t leaf = i / nc;
    int k = (int)(i % nc);
    out[leaf * ns64 + k] = (double)in[leaf * ns32 + k];
}

__global__ void k_axpy(int64_t n, double a, const double *x, double *y) {  // y += a x
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __dadd_rn(y[i], __dmul_rn(a, x[i]));
}

__global__ void k_scale(int64_t n, double a, const double *x, double *y) {  // y = a x
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i];
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
    return GX_OK;
}

// Forward evaluation at the resident positions, then its FP64 leaf locals into dst
// (stride row_stride_f64) for the VJP.
int forward_with_locals(gx_ctx *ctx, double *dst_lf) {
    GX_TRY(gx_forces_device(ctx, false));
    int64_t nl = ctx->n_leaves;
    int nc = (ctx->p + 1) * (ctx->p + 2) / 2, ns64 = row_stride_f64(ctx->p);
    if (ctx->prec == GX_PREC_MIXED) {
        k_widen_rows<<<gx_blocks(nl * nc, 256), 256, 0, ctx->stream>>>(nl, nc, row_stride_f32(ctx->p), ns64,
                                                                       dptr<float>(ctx->Lff32), dst_lf);
        ctx->launches++;
    } else {
        GX_CUDA(ctx, cudaMemcpyAsync(dst_lf, ctx->Lf.p, sizeof(double) * ns64 * (size_t)nl, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
    }
    return GX_OK;
}

// VJP at stored positions (px, py) with stored leaf locals lf.
int vjp_at(gx_ctx *ctx, const double *px, const double *py, const double *lf, const double *lx, const double *ly,
           double *gx, double *gy, double *gm) {
    int64_t n = ctx->n_bodies, nl = ctx->n_leaves;
    int ns64 = row_stride_f64(ctx->p);
    if (px != dptr<double>(ctx->x))
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->x.p, px, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    if (py != dptr<double>(ctx->y))
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->y.p, py, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    GX_TRY(gx_ensure(ctx, ctx->Lf, sizeof(double) * ns64 * (size_t)(nl > 0 ? nl : 1)));
    if (lf != dptr<double>(ctx->Lf))
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->Lf.p, lf, sizeof(double) * ns64 * (size_t)nl, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
    return force_vjp(ctx, lx, ly, gx, gy, gm);
}

}  // namespace

extern "C" {

int gx_force_vjp(gx_ctx *ctx, const double *lam_x, const double *lam_y, double *gx, double *gy, double *gm) {
    if (!ctx) return GX_ERR_INVALID_ARG;
    GX_TRY(check_mode(ctx));
    if (!lam_x || !lam_y || !gx || !gy || !gm) return gx_fail(ctx, GX_ERR_INVALID_ARG, "null array");
    extern int gx_ensure_plan_public(gx_ctx *);
    GX_TRY(gx_ensure_plan_public(ctx));
    int64_t n = ctx->n_bodies, nl = ctx->n_leaves;
    size_t b = sizeof(double) * (size_t)(n > 0 ? n : 1);
    DevBuf *bufs[] = {&ctx->adj_lx, &ctx->adj_ly, &ctx->adj_gx, &ctx->adj_gy, &ctx->adj_gm};
    for (DevBuf *d : bufs) GX_TRY(gx_ensure(ctx, *d, b));
    GX_TRY(gx_ensure(ctx, ctx->adj_lf, sizeof(double) * row_stride_f64(ctx->p) * (size_t)(nl > 0 ? nl : 1)));
    if (n == 0) return GX_OK;
    GX_CUDA(ctx, cudaMemcpyAsync(ctx->adj_lx.p, lam_x, b, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(ctx->adj_ly.p, lam_y, b, cudaMemcpyHostToDevice, ctx->stream));
    GX_TRY(forward_with_locals(ctx, dptr<double>(ctx->adj_lf)));
    GX_TRY(vjp_at(ctx, dptr<double>(ctx->x), dptr<double>(ctx->y), dptr<double>(ctx->adj_lf), dptr<double>(ctx->adj_lx),
                  dptr<double>(ctx->adj_ly), dptr<double>(ctx->adj_gx), dptr<double>(ctx->adj_gy),
                  dptr<double>(ctx->adj_gm)));
    GX_CUDA(ctx, cudaMemcpyAsync(gx, ctx->adj_gx.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(gy, ctx->adj_gy.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(gm, ctx->adj_gm.p, b, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

int gx_rollout_forward(gx_ctx *ctx, int64_t n_steps, double dt, int64_t checkpoint_every) {
    if (!ctx) return GX_ERR_INVALID_ARG;
    GX_TRY(check_mode(ctx));
    if (n_steps < 0 || checkpoint_every <= 0) return gx_fail(ctx, GX_ERR_INVALID_ARG, "bad n_steps or interval");
    extern int gx_ensure_plan_public(gx_ctx *);
    GX_TRY(gx_ensure_plan_public(ctx));
    int64_t n = ctx->n_bodies;
    int64_t nck = n_steps / checkpoint_every + 1;
    GX_TRY(gx_ensure(ctx, ctx->ckpt, sizeof(double) * 4 * (size_t)(n > 0 ? n : 1) * (size_t)nck));
    double *ck = dptr<double>(ctx->ckpt);
    double h = 0.5 * dt;
    auto save = [&](int64_t slot) -> int {
        DevBuf *src[4] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy};
        for (int k = 0; k < 4; k++)
            GX_CUDA(ctx, cudaMemcpyAsync(ck + ((size_t)slot * 4 + k) * (size_t)n, src[k]->p, sizeof(double) * n,
                                         cudaMemcpyDeviceToDevice, ctx->stream));
        return GX_OK;
    };
    GX_TRY(gx_forces_device(ctx, false));  // a_0
    GX_TRY(save(0));
    for (int64_t s = 0; s < n_steps; s++) {
        k_kick_drift_a<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, h, dt, dptr<double>(ctx->x), dptr<double>(ctx->y),
                                                                   dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                                   dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        GX_TRY(gx_forces_device(ctx, false));
        k_kick_a<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, h, dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                             dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        ctx->launches += 2;
        if ((s + 1) % checkpoint_every == 0) GX_TRY(save((s + 1) / checkpoint_every));
    }
    GX_CUDA(ctx, cudaGetLastError());
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->roll_steps = n_steps;
    ctx->roll_dt = dt;
    ctx->roll_k = checkpoint_every;
    ctx->roll_valid = true;
    return GX_OK;
}

int gx_rollout_backward(gx_ctx *ctx, const double *lx, const double *ly, const double *lvx, const double *lvy,
                        double *gx0, double *gy0, double *gvx0, double *gvy0, double *gm, int64_t *peak_bytes) {
    if (!ctx) return GX_ERR_INVALID_ARG;
    GX_TRY(check_mode(ctx));
    if (!ctx->roll_valid) return gx_fail(ctx, GX_ERR_STATE, "gx_rollout_backward needs gx_rollout_forward first");
    if (!lx || !ly || !lvx || !lvy || !gx0 || !gy0 || !gvx0 || !gvy0 || !gm)
        return gx_fail(ctx, GX_ERR_INVALID_ARG, "null array");
    int64_t n = ctx->n_bodies, nl = ctx->n_leaves, T = ctx->roll_steps, K = ctx->roll_k;
    double dt = ctx->roll_dt, h = 0.5 * dt;
    int ns64 = row_stride_f64(ctx->p);
    size_t b = sizeof(double) * (size_t)(n > 0 ? n : 1);
    // adjoint state (lx, ly, lvx, lvy, lm), VJP outputs (gx, gy, gm), la
    DevBuf *bufs[] = {&ctx->adj_lx, &ctx->adj_ly, &ctx->adj_lvx, &ctx->adj_lvy, &ctx->adj_lm,
                      &ctx->adj_gx, &ctx->adj_gy, &ctx->adj_gm, &ctx->adj_lax, &ctx->adj_lay};
    for (DevBuf *d : bufs) GX_TRY(gx_ensure(ctx, *d, b));
    // segment storage: positions and FP64 leaf locals of up to K+1 states
    size_t seg_pos = 2 * (size_t)(n > 0 ? n : 1), seg_lf = (size_t)ns64 * (size_t)(nl > 0 ? nl : 1);
    GX_TRY(gx_ensure(ctx, ctx->seg, sizeof(double) * (seg_pos + seg_lf) * (size_t)(K + 1)));
    if (peak_bytes)
        *peak_bytes = (int64_t)(ctx->ckpt.bytes + ctx->seg.bytes + 10 * b + ctx->adj_dL.bytes + ctx->adj_dM.bytes +
                                ctx->adj_dMleaf.bytes);
    double *LX = dptr<double>(ctx->adj_lx), *LY = dptr<double>(ctx->adj_ly), *LVX = dptr<double>(ctx->adj_lvx),
           *LVY = dptr<double>(ctx->adj_lvy), *LM = dptr<double>(ctx->adj_lm), *GX = dptr<double>(ctx->adj_gx),
           *GY = dptr<double>(ctx->adj_gy), *GM = dptr<double>(ctx->adj_gm), *LAX = dptr<double>(ctx->adj_lax),
           *LAY = dptr<double>(ctx->adj_lay);
    double *seg = dptr<double>(ctx->seg), *ck = dptr<double>(ctx->ckpt);
    auto seg_x = [&](int64_t j) { return seg + (size_t)j * (seg_pos + seg_lf); };
    auto seg_y = [&](int64_t j) { return seg_x(j) + n; };
    auto seg_l = [&](int64_t j) { return seg_x(j) + seg_pos; };
    if (n > 0) {
        GX_CUDA(ctx, cudaMemcpyAsync(LX, lx, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(LY, ly, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(LVX, lvx, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(LVY, lvy, b, cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemsetAsync(LM, 0, b, ctx->stream));
    }
    const unsigned g = gx_blocks(n, 256);
    int64_t nseg = (T + K - 1) / K;
    for (int64_t sgi = nseg - 1; sgi >= 0; sgi--) {
        int64_t s0 = sgi * K, s1 = std::min(T, s0 + K);
        // restore the checkpoint of step s0 and recompute the states s0 .. s1
        DevBuf *dst[4] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy};
        for (int k = 0; k < 4; k++)
            GX_CUDA(ctx, cudaMemcpyAsync(dst[k]->p, ck + ((size_t)sgi * 4 + k) * (size_t)n, b, cudaMemcpyDeviceToDevice,
                                         ctx->stream));
        GX_TRY(forward_with_locals(ctx, seg_l(0)));  // a_{s0} and its locals
        GX_CUDA(ctx, cudaMemcpyAsync(seg_x(0), ctx->x.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(seg_y(0), ctx->y.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
        for (int64_t s = s0; s < s1; s++) {
            k_kick_drift_a<<<g, 256, 0, ctx->stream>>>(n, h, dt, dptr<double>(ctx->x), dptr<double>(ctx->y),
                                                       dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                       dptr<double>(ctx->ax), dptr<double>(ctx->ay));
            int64_t j = s + 1 - s0;
            GX_TRY(forward_with_locals(ctx, seg_l(j)));
            k_kick_a<<<g, 256, 0, ctx->stream>>>(n, h, dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                 dptr<double>(ctx->ax), dptr<double>(ctx->ay));
            ctx->launches += 2;
            GX_CUDA(ctx, cudaMemcpyAsync(seg_x(j), ctx->x.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
            GX_CUDA(ctx, cudaMemcpyAsync(seg_y(j), ctx->y.p, b, cudaMemcpyDeviceToDevice, ctx->stream));
        }
        // reverse through the segment
        for (int64_t s = s1 - 1; s >= s0; s--) {
            int64_t j = s + 1 - s0;
            double c = (s + 1 == T) ? h : dt;
            k_scale<<<g, 256, 0, ctx->stream>>>(n, c, LVX, LAX);
            k_scale<<<g, 256, 0, ctx->stream>>>(n, c, LVY, LAY);
            GX_TRY(vjp_at(ctx, seg_x(j), seg_y(j), seg_l(j), LAX, LAY, GX, GY, GM));
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GX, LX);
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GY, LY);
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GM, LM);
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, dt, LX, LVX);
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, dt, LY, LVY);
            ctx->launches += 7;
        }
        if (sgi == 0) {  // a_0 feeds the first half kick only
            k_scale<<<g, 256, 0, ctx->stream>>>(n, h, LVX, LAX);
            k_scale<<<g, 256, 0, ctx->stream>>>(n, h, LVY, LAY);
            GX_TRY(vjp_at(ctx, seg_x(0), seg_y(0), seg_l(0), LAX, LAY, GX, GY, GM));
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GX, LX);
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GY, LY);
            k_axpy<<<g, 256, 0, ctx->stream>>>(n, 1.0, GM, LM);
            ctx->launches += 5;
        }
        GX_CUDA(ctx, cudaGetLastError());
    }
    if (n > 0) {
        GX_CUDA(ctx, cudaMemcpyAsync(gx0, LX, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gy0, LY, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gvx0, LVX, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gvy0, LVY, b, cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(gm, LM, b, cudaMemcpyDeviceToHost, ctx->stream));
    }
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

}  // extern "C"
