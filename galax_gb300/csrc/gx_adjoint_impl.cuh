// gx_adjoint_impl.cuh -- vector-Jacobian product of the ACCURATE-mode force evaluation.
//
// Forward (frozen tree: node COMs, lists and radii are constants):
//   M_leaf[S] = sum_j m_j u_j^S / S!                    (P2M, u_j = x_j - com_leaf)
//   M_P       = sum_c SM(c->P) M_c                      (M2M)
//   L_t[T]    = -(1/T!) sum_s sum_S (-1)^|S| M_s[S] A(com_t - com_s)[S+T]   (M2L)
//   Lf_leaf   = sum_{a in ancestors} SL(a->leaf) L_a    (L2L)
//   a_j       = -grad Phi(u_j) + sum_k m_k K(x_k - x_j) (L2P + P2P), Phi(u) = sum_T Lf[T] u^T,
//               K(d) = d (|d|^2 + eps^2)^(-3/2)
// Given the cotangent lam_j of every a_j, the adjoint returns g_x = sum lam . da/dx and
// g_m = sum lam . da/dm by running the transposed operators in reverse:
//   L2P^T (plus the Hessian term of the local polynomial), L2L^T as an upward pass,
//   M2L^T as a gather over the (symmetric) far lists, M2M^T straight from every
//   ancestor to the leaf, P2M^T, and the Hessian-vector product of P2P over the
//   (symmetric) near lists.  Every operator is the exact transpose of the forward
//   one, so the result agrees with finite differences of the forward evaluation.
#pragma once
#include "gx_fmm_impl.cuh"

namespace {

// monomial powers with factorials folded in: pf[k] = u^k / k!
template <int P, class T>
__device__ __forceinline__ void pow_fact(T u, T *pf) {
    const int PP = gx_rt_order(P);
    pf[0] = T(1);
#pragma unroll
    for (int k = 1; k <= PP; k++) pf[k] = pf[k - 1] * u * (T)(1.0 / k);
}

// ---- A1: L2P^T and the Hessian term.  Warp per leaf, lane per body.
//   g_x,j   = -H_Phi(u_j) lam_j
//   dLf[T]  = -sum_j (lam_x T1 u^(T-e1) + lam_y T2 u^(T-e2))
template <int P>
__global__ void __launch_bounds__(128) k_adj_l2p(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                 const double *__restrict__ comx, const double *__restrict__ comy,
                                                 const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                 const double *__restrict__ Lf, const double *__restrict__ lx,
                                                 const double *__restrict__ ly, double *__restrict__ gx,
                                                 double *__restrict__ gy, double *__restrict__ dL) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    double lf[NC];
    load_row<NC>(Lf + leaf * NS, lf);
    double acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = 0.0;
    for (int32_t i = bs[leaf] + lane; i < be[leaf]; i += 32) {
        double u = x[i] - comx[leaf], v = y[i] - comy[leaf];
        double pu[P + 1], pv[P + 1];
        pu[0] = 1.0;
        pv[0] = 1.0;
#pragma unroll
        for (int q = 1; q <= PP; q++) {
            pu[q] = pu[q - 1] * u;
            pv[q] = pv[q - 1] * v;
        }
        double lam_x = lx[i], lam_y = ly[i];
        double hxx = 0.0, hxy = 0.0, hyy = 0.0;
#pragma unroll
        for (int a = 0; a <= PP; a++)
#pragma unroll
            for (int b = 0; b <= PP - a; b++) {
                double c = lf[gx_mi(a, b)];
                if (a >= 2) hxx += c * (double)(a * (a - 1)) * pu[a - 2] * pv[b];
                if (b >= 2) hyy += c * (double)(b * (b - 1)) * pu[a] * pv[b - 2];
                if (a >= 1 && b >= 1) hxy += c * (double)(a * b) * pu[a - 1] * pv[b - 1];
                double t = 0.0;
                if (a >= 1) t += lam_x * (double)a * pu[a - 1] * pv[b];
                if (b >= 1) t += lam_y * (double)b * pu[a] * pv[b - 1];
                acc[gx_mi(a, b)] -= t;
            }
        gx[i] = -(hxx * lam_x + hxy * lam_y);
        gy[i] = -(hxy * lam_x + hyy * lam_y);
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) {
        double s = warp_sum_t<double>(acc[k]);
        if (lane == (k & 31)) dL[leaf * NS + k] = s;
    }
}

// ---- A2: L2L^T, one level of the upward pass: dL[P][U] = sum_c sum_{T<=U} dL[c][T] C(U,T) e^(U-T),
// e = com_c - com_P.  The leaves' rows are already in place; internal rows are written here.
template <int P>
__global__ void __launch_bounds__(128) k_adj_l2l_up(int64_t s, int64_t e, const int4 *__restrict__ child,
                                                    const double *__restrict__ comx, const double *__restrict__ comy,
                                                    double *__restrict__ dL) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t node = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= e) return;
    int4 c4 = child[node];
    int cc[4] = {c4.x, c4.y, c4.z, c4.w};
    double out[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = 0.0;
    for (int q = 0; q < 4; q++) {
        int c = cc[q];
        if (c < 0) continue;
        double ex = comx[c] - comx[node], ey = comy[c] - comy[node];
        double px[P + 1], py[P + 1];
        px[0] = 1.0;
        py[0] = 1.0;
#pragma unroll
        for (int k = 1; k <= PP; k++) {
            px[k] = px[k - 1] * ex;
            py[k] = py[k - 1] * ey;
        }
        double dc[NC];
        load_row<NC>(dL + (int64_t)c * NS, dc);
#pragma unroll
        for (int ui = 0; ui <= PP; ui++)
#pragma unroll
            for (int uj = 0; uj <= PP - ui; uj++)
#pragma unroll
                for (int ti = 0; ti <= ui; ti++)
#pragma unroll
                    for (int tj = 0; tj <= uj; tj++)
                        out[gx_mi(ui, uj)] += dc[gx_mi(ti, tj)] * (cbinom(ui, ti) * cbinom(uj, tj)) * px[ui - ti] *
                                              py[uj - tj];
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) dL[node * NS + k] = out[k];
}

// ---- A3: M2L^T as a gather over far(s) (far lists are symmetric):
//   dM[s][S] = -(-1)^|S| sum_{t in far(s)} sum_T A(com_t - com_s)[S+T] dL[t][T] / T!
template <int P>
__global__ void __launch_bounds__(128) k_adj_m2l(int64_t nn, const int32_t *__restrict__ idx,
                                                 const int64_t *__restrict__ start, const int32_t *__restrict__ cnt,
                                                 const double *__restrict__ comx, const double *__restrict__ comy,
                                                 double eps2, const double *__restrict__ dL, double *__restrict__ dM) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    constexpr int ND = nc2(2 * P);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (node >= nn) return;
    int64_t st = start[node];
    int len = cnt[node];
    double scx = comx[node], scy = comy[node];
    double acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = 0.0;
    for (int q = lane; q < len; q += 32) {
        int64_t t = idx[st + q];
        double A[ND];
        derivs_scaled<P, double>(comx[t] - scx, comy[t] - scy, eps2, A);
        double lt[NC];
        load_row<NC>(dL + t * NS, lt);
#pragma unroll
        for (int ti = 0; ti <= PP; ti++)
#pragma unroll
            for (int tj = 0; tj <= PP - ti; tj++) {
                double w = lt[gx_mi(ti, tj)] * (cinvfact(ti) * cinvfact(tj));
#pragma unroll
                for (int si = 0; si <= PP; si++)
#pragma unroll
                    for (int sj = 0; sj <= PP - si; sj++) acc[gx_mi(si, sj)] += w * A[gx_mi(si + ti, sj + tj)];
            }
    }
#pragma unroll
    for (int si = 0; si <= PP; si++)
#pragma unroll
        for (int sj = 0; sj <= PP - si; sj++) {
            int k = gx_mi(si, sj);
            double v = warp_sum_t<double>(acc[k]);
            if (lane == (k & 31)) dM[node * NS + k] = ((si + sj) & 1) ? v : -v;
        }
}

// ---- A4: M2M^T straight to the leaves: the moments of an ancestor a are the leaf's
// moments shifted by d = com_leaf - com_a (SM(leaf->a), composed exactly along the
// chain), so dM_leaf[S] = sum_a sum_{T>=S} dM_a[T] d^(T-S)/(T-S)!.  Warp per leaf,
// lane per ancestor, warp reduction.
template <int P>
__global__ void __launch_bounds__(128) k_adj_m2m_direct(int64_t nl, int n_levels, const int32_t *__restrict__ anc,
                                                        const uint8_t *__restrict__ has_far,
                                                        const double *__restrict__ comx, const double *__restrict__ comy,
                                                        const double *__restrict__ dM, double *__restrict__ dMleaf) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    double out[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = 0.0;
    for (int j = lane; j < n_levels; j += 32) {
        int32_t a = anc[(int64_t)j * nl + leaf];
        if (a < 0 || !has_far[a]) continue;
        double da[NC];
        load_row<NC>(dM + (int64_t)a * NS, da);
        double px[P + 1], py[P + 1];
        pow_fact<P, double>(comx[leaf] - comx[a], px);
        pow_fact<P, double>(comy[leaf] - comy[a], py);
#pragma unroll
        for (int si = 0; si <= PP; si++)
#pragma unroll
            for (int sj = 0; sj <= PP - si; sj++)
#pragma unroll
                for (int ti = si; ti <= PP; ti++)
#pragma unroll
                    for (int tj = sj; tj <= PP - ti; tj++)
                        out[gx_mi(si, sj)] += da[gx_mi(ti, tj)] * px[ti - si] * py[tj - sj];
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) {
        double v = warp_sum_t<double>(out[k]);
        if (lane == (k & 31)) dMleaf[leaf * NS + k] = v;
    }
}

// ---- A5: P2M^T: g_m,j += sum_S dM[S] u^S/S!,  g_x,j += m_j sum_S dM[S] grad(u^S/S!).
// Thread per body (the leaf id comes from the body -> leaf map).
template <int P>
__global__ void __launch_bounds__(128) k_adj_p2m(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                 const double *__restrict__ m, const double *__restrict__ comx,
                                                 const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                 const int32_t *__restrict__ be, const double *__restrict__ dMleaf,
                                                 double *__restrict__ gx, double *__restrict__ gy,
                                                 double *__restrict__ gm) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    const int PP = gx_rt_order(P);
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    double dm[NC];
    load_row<NC>(dMleaf + leaf * NS, dm);
    for (int32_t i = bs[leaf] + lane; i < be[leaf]; i += 32) {
        double px[P + 1], py[P + 1];
        pow_fact<P, double>(x[i] - comx[leaf], px);
        pow_fact<P, double>(y[i] - comy[leaf], py);
        double sm = 0.0, sx = 0.0, sy = 0.0;
#pragma unroll
        for (int a = 0; a <= PP; a++)
#pragma unroll
            for (int b = 0; b <= PP - a; b++) {
                double c = dm[gx_mi(a, b)];
                sm += c * px[a] * py[b];
                if (a >= 1) sx += c * px[a - 1] * py[b];
                if (b >= 1) sy += c * px[a] * py[b - 1];
            }
        gm[i] += sm;
        gx[i] += m[i] * sx;
        gy[i] += m[i] * sy;
    }
}

// ---- A6: Hessian-vector P2P over the near lists (symmetric at leaf level):
//   g_x,i += sum_k J(x_k - x_i) (m_i lam_k - m_k lam_i),  J(d) = I/r^3 - 3 d d^T / r^5
//   g_m,i -= sum_k lam_k . (x_k - x_i) / r^3           (r^2 = |d|^2 + eps^2, k != i)
// Work items as in the forward P2P: one warp per (target leaf, <= 32 source leaves),
// partial sums per item, summed in item order afterwards.
__global__ void __launch_bounds__(128) k_adj_p2p_items(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                       const int64_t *__restrict__ item_qb,
                                                       const int32_t *__restrict__ item_nq, const double *__restrict__ x,
                                                       const double *__restrict__ y, const double *__restrict__ m,
                                                       const double *__restrict__ lx, const double *__restrict__ ly,
                                                       const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                       const int32_t *__restrict__ src_idx, double eps2, int tchunks,
                                                       double4 *__restrict__ part) {
    __shared__ double4 sb[4][32];
    __shared__ double sm_[4][32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (it >= n_items) return;
    int32_t leaf = item_leaf[it];
    int64_t qb = item_qb[it];
    int nq = item_nq[it];
    int32_t t0 = bs[leaf], t1 = be[leaf];
    int sl = lane < nq ? src_idx[qb + lane] : -1;
    int sbeg = sl >= 0 ? bs[sl] : 0, send = sl >= 0 ? be[sl] : 0;
    for (int tc = 0; tc < tchunks; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        bool valid = i < t1;
        double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0, mi = valid ? m[i] : 0.0;
        double lxi = valid ? lx[i] : 0.0, lyi = valid ? ly[i] : 0.0;
        double gxa = 0.0, gya = 0.0, gma = 0.0;
        if (t0 + tc * 32 < t1) {
            for (int k = 0; k < nq; k++) {
                int s0 = __shfl_sync(0xffffffffu, sbeg, k), s1 = __shfl_sync(0xffffffffu, send, k);
                for (int sc = s0; sc < s1; sc += 32) {
                    int j = sc + lane;
                    __syncwarp();
                    if (j < s1) {
                        sb[w][lane] = make_double4(x[j], y[j], lx[j], ly[j]);
                        sm_[w][lane] = m[j];
                    }
                    __syncwarp();
                    int ns = min(32, s1 - sc);
                    for (int kk = 0; kk < ns; kk++) {
                        if (sc + kk == i) continue;
                        double4 bj = sb[w][kk];
                        double mj = sm_[w][kk];
                        double dx = bj.x - xi, dy = bj.y - yi;
                        double r2 = dx * dx + dy * dy + eps2;
                        double ir = rsqrt(r2);
                        double ir3 = ir * ir * ir, ir5 = ir3 * ir * ir;
                        double wx = mi * bj.z - mj * lxi, wy = mi * bj.w - mj * lyi;
                        double dw = dx * wx + dy * wy;
                        gxa += ir3 * wx - 3.0 * ir5 * dx * dw;
                        gya += ir3 * wy - 3.0 * ir5 * dy * dw;
                        gma -= (bj.z * dx + bj.w * dy) * ir3;
                    }
                }
            }
        }
        part[(it * tchunks + tc) * 32 + lane] = make_double4(gxa, gya, gma, 0.0);
    }
}

__global__ void __launch_bounds__(128) k_adj_p2p_reduce(int64_t nl, const int32_t *__restrict__ bs,
                                                        const int32_t *__restrict__ be, const int64_t *__restrict__ item_off,
                                                        int tchunks, const double4 *__restrict__ part,
                                                        double *__restrict__ gx, double *__restrict__ gy,
                                                        double *__restrict__ gm) {
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    for (int tc = 0; tc < tchunks && t0 + tc * 32 < t1; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        if (i >= t1) continue;
        double sx = 0.0, sy = 0.0, smm = 0.0;
        for (int64_t it = item_off[leaf]; it < item_off[leaf + 1]; it++) {
            double4 v = part[(it * tchunks + tc) * 32 + lane];
            sx += v.x;
            sy += v.y;
            smm += v.z;
        }
        gx[i] += sx;
        gy[i] += sy;
        gm[i] += smm;
    }
}

// Full VJP on the resident bodies.  Needs the forward local expansions of the same
// positions (ctx->Lf after a forward evaluation in ACCURATE FP64).
template <int P>
int run_force_vjp(gx_ctx *ctx, const double *lx, const double *ly, double *gx, double *gy, double *gm) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    const int64_t nn = ctx->n_nodes, nl = ctx->n_leaves;
    cudaStream_t st = ctx->stream;
    if (nn == 0) return GX_OK;
    const double *X = dptr<double>(ctx->x), *Y = dptr<double>(ctx->y), *Mb = dptr<double>(ctx->m);
    const double *comx = dptr<double>(ctx->comx), *comy = dptr<double>(ctx->comy);
    const int32_t *bs = dptr<int32_t>(ctx->bs), *be = dptr<int32_t>(ctx->be);
    const int4 *child = dptr<int4>(ctx->child);
    const double eps2 = ctx->eps * ctx->eps;
    const unsigned gw = (unsigned)((nl * 32 + 127) / 128);
    GX_TRY(gx_ensure(ctx, ctx->adj_dL, sizeof(double) * NS * (size_t)nn));
    GX_TRY(gx_ensure(ctx, ctx->adj_dM, sizeof(double) * NS * (size_t)nn));
    GX_TRY(gx_ensure(ctx, ctx->adj_dMleaf, sizeof(double) * NS * (size_t)nl));
    double *dL = dptr<double>(ctx->adj_dL), *dM = dptr<double>(ctx->adj_dM), *dMl = dptr<double>(ctx->adj_dMleaf);
    // A1: L2P^T and the Hessian term (writes gx, gy)
    k_adj_l2p<P><<<gw, 128, 0, st>>>(nl, X, Y, comx, comy, bs, be, dptr<double>(ctx->Lf), lx, ly, gx, gy, dL);
    // A2: L2L^T upward, level by level (leaves are level 0)
    for (int lv = 1; lv < ctx->n_levels; lv++) {
        int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
        k_adj_l2l_up<P><<<gx_blocks(e - s, 128), 128, 0, st>>>(s, e, child, comx, comy, dL);
    }
    // A3: M2L^T
    const int64_t *fs = dptr<int64_t>(ctx->far_off);
    k_adj_m2l<P><<<(unsigned)((nn * 32 + 127) / 128), 128, 0, st>>>(nn, dptr<int32_t>(ctx->far_idx), fs,
                                                                    reinterpret_cast<const int32_t *>(fs + nn), comx,
                                                                    comy, eps2, dL, dM);
    // A4: M2M^T to the leaves
    k_adj_m2m_direct<P><<<gw, 128, 0, st>>>(nl, ctx->n_levels, dptr<int32_t>(ctx->anc), dptr<uint8_t>(ctx->has_far_acc),
                                            comx, comy, dM, dMl);
    // A5: P2M^T (adds to gx, gy; writes gm)
    GX_CUDA(ctx, cudaMemsetAsync(gm, 0, sizeof(double) * (size_t)ctx->n_bodies, st));
    k_adj_p2m<P><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, dMl, gx, gy, gm);
    // A6: Hessian-vector P2P
    const gx_ctx::Items &I = ctx->items_acc;
    const int tchunks = (int)std::max<int64_t>(1, (ctx->max_leaf + 31) / 32);
    GX_TRY(gx_ensure(ctx, ctx->part, sizeof(double4) * 32 * (size_t)tchunks * (size_t)(I.n + 1)));
    double4 *part = dptr<double4>(ctx->part);
    if (I.n > 0)
        k_adj_p2p_items<<<(unsigned)((I.n * 32 + 127) / 128), 128, 0, st>>>(
            I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb), dptr<int32_t>(I.nq), X, Y, Mb, lx, ly, bs, be,
            dptr<int32_t>(ctx->near_idx), eps2, tchunks, part);
    k_adj_p2p_reduce<<<gw, 128, 0, st>>>(nl, bs, be, dptr<int64_t>(I.off), tchunks, part, gx, gy, gm);
    ctx->launches += 6 + (ctx->n_levels - 1);
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

}  // namespace

#define GX_ADJ_INSTANTIATE(PP)                                                                              \
    int gx_run_force_vjp_##PP(gx_ctx *ctx, const double *lx, const double *ly, double *gx, double *gy, \
                              double *gm) {                                                              \
        return run_force_vjp<PP>(ctx, lx, ly, gx, gy, gm);                                              \
    }
