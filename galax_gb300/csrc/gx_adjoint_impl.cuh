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
//   one, so in FP64 the result agrees with finite differences of the forward
//   evaluation.  T = float is the mixed form: the same operators in FP32 on the
//   forward's FP32 leaf locals, FP32 body offsets from the leaf COM and per-leaf-pair
//   FP32 shifts (as the mixed forward), with the outputs accumulated in FP64.
#pragma once
#include "gx_fmm_impl.cuh"

namespace {

// monomial powers with factorials folded in: pf[k] = u^k / k!
template <int P, class T>
__device__ __forceinline__ void pow_fact(T u, T *pf) {
    const int PP = gx_rt_order(P);
    pf[0] = T(1);
#pragma unroll
    for (int k = 1; k <= PP; k++) pf[k] = pf[k - 1] * u * tab_inv<T>(k);
}

// ---- A1: L2P^T and the Hessian term.  Warp per leaf, lane per body.
//   g_x,j   = -H_Phi(u_j) lam_j
//   dLf[T]  = -sum_j (lam_x T1 u^(T-e1) + lam_y T2 u^(T-e2))
// The FP32 form also packs the bodies (u, v, m) and cotangents for its P2P pass.
template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_l2p(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                 const double *__restrict__ m, const double *__restrict__ comx,
                                                 const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                 const int32_t *__restrict__ be, const T *__restrict__ Lf,
                                                 const double *__restrict__ lx, const double *__restrict__ ly,
                                                 double *__restrict__ gx, double *__restrict__ gy, T *__restrict__ dL,
                                                 float4 *__restrict__ pos32, float2 *__restrict__ lam32) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    T lf[NC];
    load_row<NC>(Lf + leaf * NS, lf);
    T acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = T(0);
    const double cxl = comx[leaf], cyl = comy[leaf];
    for (int32_t i = bs[leaf] + lane; i < be[leaf]; i += 32) {
        T u = (T)(x[i] - cxl), v = (T)(y[i] - cyl);
        T pu[P + 1], pv[P + 1];
        pu[0] = T(1);
        pv[0] = T(1);
#pragma unroll
        for (int q = 1; q <= PP; q++) {
            pu[q] = pu[q - 1] * u;
            pv[q] = pv[q - 1] * v;
        }
        T lam_x = (T)lx[i], lam_y = (T)ly[i];
        if constexpr (sizeof(T) == 4) {
            pos32[i] = make_float4(u, v, (float)m[i], 0.f);
            lam32[i] = make_float2(lam_x, lam_y);
        }
        T hxx = T(0), hxy = T(0), hyy = T(0);
#pragma unroll
        for (int a = 0; a <= PP; a++)
#pragma unroll
            for (int b = 0; b <= PP - a; b++) {
                T c = lf[gx_mi(a, b)];
                if (a >= 2) hxx += c * (T)(a * (a - 1)) * pu[a - 2] * pv[b];
                if (b >= 2) hyy += c * (T)(b * (b - 1)) * pu[a] * pv[b - 2];
                if (a >= 1 && b >= 1) hxy += c * (T)(a * b) * pu[a - 1] * pv[b - 1];
                T t = T(0);
                if (a >= 1) t += lam_x * (T)a * pu[a - 1] * pv[b];
                if (b >= 1) t += lam_y * (T)b * pu[a] * pv[b - 1];
                acc[gx_mi(a, b)] -= t;
            }
        gx[i] = -(double)(hxx * lam_x + hxy * lam_y);
        gy[i] = -(double)(hxy * lam_x + hyy * lam_y);
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) {
        T s = warp_sum_t<T>(acc[k]);
        if (lane == (k & 31)) dL[leaf * NS + k] = s;
    }
}

// ---- A2: L2L^T, one level of the upward pass: dL[P][U] = sum_c sum_{T<=U} dL[c][T] C(U,T) e^(U-T),
// e = com_c - com_P.  The leaves' rows are already in place; internal rows are written here.
template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_l2l_up(int64_t s, int64_t e, const int4 *__restrict__ child,
                                                    const double *__restrict__ comx, const double *__restrict__ comy,
                                                    T *__restrict__ dL) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t node = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= e) return;
    int4 c4 = child[node];
    int cc[4] = {c4.x, c4.y, c4.z, c4.w};
    T out[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = T(0);
    for (int q = 0; q < 4; q++) {
        int c = cc[q];
        if (c < 0) continue;
        T ex = (T)(comx[c] - comx[node]), ey = (T)(comy[c] - comy[node]);
        T px[P + 1], py[P + 1];
        px[0] = T(1);
        py[0] = T(1);
#pragma unroll
        for (int k = 1; k <= PP; k++) {
            px[k] = px[k - 1] * ex;
            py[k] = py[k - 1] * ey;
        }
        T dc[NC];
        load_row<NC>(dL + (int64_t)c * NS, dc);
#pragma unroll
        for (int ui = 0; ui <= PP; ui++)
#pragma unroll
            for (int uj = 0; uj <= PP - ui; uj++)
#pragma unroll
                for (int ti = 0; ti <= ui; ti++)
#pragma unroll
                    for (int tj = 0; tj <= uj; tj++)
                        out[gx_mi(ui, uj)] += dc[gx_mi(ti, tj)] * (tab_binom<T>(ui, ti) * tab_binom<T>(uj, tj)) *
                                              px[ui - ti] * py[uj - tj];
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) dL[node * NS + k] = out[k];
}

// ---- A3: M2L^T as a gather over far(s) (far lists are symmetric):
//   dM[s][S] = -(-1)^|S| sum_{t in far(s)} sum_T A(com_t - com_s)[S+T] dL[t][T] / T!
// The FP32 form forms com_t - com_s from the FP32 (hi, lo) COMs exactly as the
// forward M2L forms it for the pair (t, s).  Work units as in the forward M2L (far
// lists cut into pieces of at most GX_M2L_UNIT entries, one warp each); a node with
// one unit writes dM directly, otherwise k_adj_m2l_combine sums the units' partials
// in unit order.  Nodes without far entries are not written: has_far = 0 keeps A4
// from reading them.
template <int P, class T>
__global__ void __launch_bounds__(128, (sizeof(T) == 4 && P <= 4) ? 8 : 1)
    k_adj_m2l(int64_t n_units, const int32_t *__restrict__ unode, const int64_t *__restrict__ ustart,
              const int32_t *__restrict__ ulen, const int64_t *__restrict__ node_u, const int32_t *__restrict__ idx,
              const double *__restrict__ comx, const double *__restrict__ comy, const float4 *__restrict__ comhl,
              double eps2d, const T *__restrict__ dL, T *__restrict__ dM, T *__restrict__ part) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (u >= n_units) return;
    const int64_t node = unode[u];
    const bool single = node_u[node + 1] - node_u[node] == 1;
    const int64_t st = ustart[u];
    const int len = ulen[u];
    double scx = comx[node], scy = comy[node];
    float4 shl = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (sizeof(T) == 4) shl = comhl[node];
    const T eps2 = (T)eps2d;
    T acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = T(0);
    int64_t t = lane < len ? (int64_t)idx[st + lane] : 0;
    for (int q = lane; q < len; q += 32) {
        int64_t nt = q + 32 < len ? (int64_t)idx[st + q + 32] : 0;
        T lt[NC];
        load_row<NC>(dL + t * NS, lt);
        T dx, dy;
        if constexpr (sizeof(T) == 4) {
            float4 thl = comhl[t];
            dx = (thl.x - shl.x) + (thl.y - shl.y);
            dy = (thl.z - shl.z) + (thl.w - shl.w);
        } else {
            dx = comx[t] - scx;
            dy = comy[t] - scy;
        }
#pragma unroll
        for (int ti = 0; ti <= PP; ti++)
#pragma unroll
            for (int tj = 0; tj <= PP - ti; tj++) lt[gx_mi(ti, tj)] *= tab_ifp<T>(ti, tj);
        m2l_fused<P, T>(dx, dy, eps2, lt, acc);
        t = nt;
    }
#pragma unroll
    for (int si = 0; si <= PP; si++)
#pragma unroll
        for (int sj = 0; sj <= PP - si; sj++) {
            int k = gx_mi(si, sj);
            T v = warp_sum_t<T>(acc[k]);
            if (lane == (k & 31)) {
                if (single) dM[node * NS + k] = ((si + sj) & 1) ? v : -v;
                else part[u * NS + k] = v;
            }
        }
}

template <int P, class T>
__global__ void k_adj_m2l_combine(int64_t nn, const int64_t *__restrict__ node_u, const T *__restrict__ part,
                                  T *__restrict__ dM) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t node = t / NC;
    int k = (int)(t - node * NC);
    if (node >= nn || k >= NCr) return;
    int64_t u0 = node_u[node], u1 = node_u[node + 1];
    if (u1 - u0 < 2) return;
    T s = T(0);
    for (int64_t u = u0; u < u1; u++) s += part[u * NS + k];
    int n = 0;  // coefficient k = gx_mi(si, sj) with si + sj = n
    while ((n + 1) * (n + 2) / 2 <= k) n++;
    dM[node * NS + k] = (n & 1) ? s : -s;
}

// ---- A4: M2M^T straight to the leaves: the moments of an ancestor a are the leaf's
// moments shifted by d = com_leaf - com_a (SM(leaf->a), composed exactly along the
// chain), so dM_leaf[S] = sum_a sum_{T>=S} dM_a[T] d^(T-S)/(T-S)!.  Warp per leaf,
// lane per ancestor, warp reduction.
template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_m2m_direct(int64_t nl, int n_levels, const int32_t *__restrict__ anc,
                                                        const uint8_t *__restrict__ has_far,
                                                        const double *__restrict__ comx, const double *__restrict__ comy,
                                                        const T *__restrict__ dM, T *__restrict__ dMleaf) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    T out[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = T(0);
    for (int j = lane; j < n_levels; j += 32) {
        int32_t a = anc[(int64_t)j * nl + leaf];
        if (a < 0 || !has_far[a]) continue;
        T da[NC];
        load_row<NC>(dM + (int64_t)a * NS, da);
        T px[P + 1], py[P + 1];
        pow_fact<P, T>((T)(comx[leaf] - comx[a]), px);
        pow_fact<P, T>((T)(comy[leaf] - comy[a]), py);
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
        T v = warp_sum_t<T>(out[k]);
        if (lane == (k & 31)) dMleaf[leaf * NS + k] = v;
    }
}

// ---- A5: P2M^T: g_m,j += sum_S dM[S] u^S/S!,  g_x,j += m_j sum_S dM[S] grad(u^S/S!).
// Warp per leaf, lane per body.
template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_p2m(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                 const double *__restrict__ m, const double *__restrict__ comx,
                                                 const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                 const int32_t *__restrict__ be, const T *__restrict__ dMleaf,
                                                 double *__restrict__ gx, double *__restrict__ gy,
                                                 double *__restrict__ gm) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    T dm[NC];
    load_row<NC>(dMleaf + leaf * NS, dm);
    const double cxl = comx[leaf], cyl = comy[leaf];
    for (int32_t i = bs[leaf] + lane; i < be[leaf]; i += 32) {
        T px[P + 1], py[P + 1];
        pow_fact<P, T>((T)(x[i] - cxl), px);
        pow_fact<P, T>((T)(y[i] - cyl), py);
        T sm = T(0), sx = T(0), sy = T(0);
#pragma unroll
        for (int a = 0; a <= PP; a++)
#pragma unroll
            for (int b = 0; b <= PP - a; b++) {
                T c = dm[gx_mi(a, b)];
                sm += c * px[a] * py[b];
                if (a >= 1) sx += c * px[a - 1] * py[b];
                if (b >= 1) sy += c * px[a] * py[b - 1];
            }
        T mi = (T)m[i];
        gm[i] += (double)sm;
        gx[i] += (double)(mi * sx);
        gy[i] += (double)(mi * sy);
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

// FP32 form of A6 on the packed bodies (u, v, m) and cotangents of k_adj_l2p<float>;
// a source leaf is moved into the target leaf's frame by one FP32 shift per leaf
// pair formed in FP64 (as in the mixed forward P2P).  Full 32-source rows of other
// leaves run on packed .f32x2 arithmetic, two sources per instruction (the lo half
// of every accumulator takes the even sources, the hi half the odd ones); the own
// leaf and partial rows run the scalar loop, which also skips the body itself.
__global__ void __launch_bounds__(128, 6) k_adj_p2p32_items(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                         const int64_t *__restrict__ item_qb,
                                                         const int32_t *__restrict__ item_nq,
                                                         const float4 *__restrict__ pos, const float2 *__restrict__ lam,
                                                         const double *__restrict__ comx, const double *__restrict__ comy,
                                                         const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                         const int32_t *__restrict__ src_idx, float eps2, int tchunks,
                                                         float4 *__restrict__ part) {
    __shared__ __align__(16) float sx[4][32], sy[4][32], sm[4][32], slx[4][32], sly[4][32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (it >= n_items) return;
    int32_t leaf = item_leaf[it];
    int64_t qb = item_qb[it];
    int nq = item_nq[it];
    int32_t t0 = bs[leaf], t1 = be[leaf];
    double tcx = comx[leaf], tcy = comy[leaf];
    int sl = lane < nq ? src_idx[qb + lane] : -1;
    int sbeg = 0, send = 0;
    float shx = 0.f, shy = 0.f;
    if (sl >= 0) {
        sbeg = bs[sl];
        send = be[sl];
        shx = (float)(comx[sl] - tcx);
        shy = (float)(comy[sl] - tcy);
    }
    for (int tc = 0; tc < tchunks; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        bool valid = i < t1;
        float4 me = valid ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float2 li = valid ? lam[i] : make_float2(0.f, 0.f);
        const float xi = me.x, yi = me.y, mi = me.z, lxi = li.x, lyi = li.y;
        const uint64_t XI = pk2(xi, xi), YI = pk2(yi, yi), E2 = pk2(eps2, eps2), MI = pk2(mi, mi);
        const uint64_t NLXI = pk2(-lxi, -lxi), NLYI = pk2(-lyi, -lyi), N3 = pk2(-3.f, -3.f);
        uint64_t GX = 0, GY = 0, GMN = 0;  // packed sums; GMN accumulates +lam.d/r^3
        float gxa = 0.f, gya = 0.f, gma = 0.f;
        if (t0 + tc * 32 < t1) {
            for (int k = 0; k < nq; k++) {
                int s0 = __shfl_sync(0xffffffffu, sbeg, k), s1 = __shfl_sync(0xffffffffu, send, k);
                float gxs = __shfl_sync(0xffffffffu, shx, k), gys = __shfl_sync(0xffffffffu, shy, k);
                int srcl = __shfl_sync(0xffffffffu, sl, k);
                for (int sc = s0; sc < s1; sc += 32) {
                    int j = sc + lane;
                    __syncwarp();
                    if (j < s1) {
                        float4 b = pos[j];
                        float2 l = lam[j];
                        sx[w][lane] = b.x + gxs;
                        sy[w][lane] = b.y + gys;
                        sm[w][lane] = b.z;
                        slx[w][lane] = l.x;
                        sly[w][lane] = l.y;
                    }
                    __syncwarp();
                    int ns = min(32, s1 - sc);
                    if (ns == 32 && srcl != leaf) {
#pragma unroll 4
                        for (int kk = 0; kk < 32; kk += 2) {
                            const uint64_t X = *reinterpret_cast<const uint64_t *>(&sx[w][kk]);
                            const uint64_t Y = *reinterpret_cast<const uint64_t *>(&sy[w][kk]);
                            const uint64_t Mj = *reinterpret_cast<const uint64_t *>(&sm[w][kk]);
                            const uint64_t LXj = *reinterpret_cast<const uint64_t *>(&slx[w][kk]);
                            const uint64_t LYj = *reinterpret_cast<const uint64_t *>(&sly[w][kk]);
                            const uint64_t dx = sub2(X, XI), dy = sub2(Y, YI);
                            const uint64_t r2 = fma2(dx, dx, fma2(dy, dy, E2));
                            float ra, rb;
                            upk2(r2, ra, rb);
                            const uint64_t ir = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                            const uint64_t ir2 = mul2(ir, ir);
                            const uint64_t ir3 = mul2(ir2, ir);
                            const uint64_t ir5 = mul2(ir3, ir2);
                            const uint64_t wx = fma2(Mj, NLXI, mul2(MI, LXj));  // mi lx_j - m_j lx_i
                            const uint64_t wy = fma2(Mj, NLYI, mul2(MI, LYj));
                            const uint64_t nc = mul2(mul2(N3, ir5), fma2(dx, wx, mul2(dy, wy)));  // -3 dw / r^5
                            GX = fma2(ir3, wx, fma2(nc, dx, GX));
                            GY = fma2(ir3, wy, fma2(nc, dy, GY));
                            GMN = fma2(fma2(LXj, dx, mul2(LYj, dy)), ir3, GMN);
                        }
                    } else {
                        const bool own = srcl == leaf;
                        for (int kk = 0; kk < ns; kk++) {
                            float dx = sx[w][kk] - xi, dy = sy[w][kk] - yi;
                            float mj = sm[w][kk], lxj = slx[w][kk], lyj = sly[w][kk];
                            float ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                            float ir2 = ir * ir;
                            float ir3 = ir2 * ir;
                            float ir5 = ir3 * ir2;
                            float wx = fmaf(mi, lxj, -mj * lxi), wy = fmaf(mi, lyj, -mj * lyi);
                            float c = 3.f * ir5 * fmaf(dx, wx, dy * wy);
                            float dl = fmaf(lxj, dx, lyj * dy);
                            bool self = own && sc + kk == i;
                            ir3 = self ? 0.f : ir3;
                            c = self ? 0.f : c;
                            gxa = fmaf(ir3, wx, fmaf(-c, dx, gxa));
                            gya = fmaf(ir3, wy, fmaf(-c, dy, gya));
                            gma = fmaf(-dl, ir3, gma);
                        }
                    }
                }
            }
        }
        float a0, a1, b0, b1, c0, c1;
        upk2(GX, a0, a1);
        upk2(GY, b0, b1);
        upk2(GMN, c0, c1);
        part[(it * tchunks + tc) * 32 + lane] = make_float4((a0 + a1) + gxa, (b0 + b1) + gya, gma - (c0 + c1), 0.f);
    }
}

// The same A6 when every leaf holds at most 32 bodies (n_max <= 32): each source leaf
// is one row, the item's source-leaf table is written to shared memory once per item,
// and the next row's bodies and cotangents are fetched while the current row computes.
// Same arithmetic and accumulation order as k_adj_p2p32_items with one target chunk.
__global__ void __launch_bounds__(128, 6) k_adj_p2p32_rows(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                        const int64_t *__restrict__ item_qb,
                                                        const int32_t *__restrict__ item_nq,
                                                        const float4 *__restrict__ pos, const float2 *__restrict__ lam,
                                                        const double *__restrict__ comx, const double *__restrict__ comy,
                                                        const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                        const int32_t *__restrict__ src_idx, float eps2,
                                                        float4 *__restrict__ part) {
    __shared__ __align__(16) float sx[4][32], sy[4][32], sm[4][32], slx[4][32], sly[4][32];
    __shared__ __align__(16) int4 meta[4][32];  // per source leaf: begin, end, shift x, shift y (FP32 bits)
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (it >= n_items) return;
    const int32_t leaf = item_leaf[it];
    const int nq = item_nq[it];
    const int32_t t0 = bs[leaf], t1 = be[leaf];
    bool own_lane = false;
    if (lane < nq) {
        int32_t sl = src_idx[item_qb[it] + lane];
        double tcx = comx[leaf], tcy = comy[leaf];
        meta[w][lane] = make_int4(bs[sl], be[sl], __float_as_int((float)(comx[sl] - tcx)),
                                  __float_as_int((float)(comy[sl] - tcy)));
        own_lane = sl == leaf;
    }
    const unsigned ownm = __ballot_sync(0xffffffffu, own_lane);
    const int kown = ownm ? __ffs(ownm) - 1 : -1;
    __syncwarp();
    const int32_t i = t0 + lane;
    const bool valid = i < t1;
    const float4 me = valid ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 li = valid ? lam[i] : make_float2(0.f, 0.f);
    const float xi = me.x, yi = me.y, mi = me.z, lxi = li.x, lyi = li.y;
    const uint64_t XI = pk2(xi, xi), YI = pk2(yi, yi), E2 = pk2(eps2, eps2), MI = pk2(mi, mi);
    const uint64_t NLXI = pk2(-lxi, -lxi), NLYI = pk2(-lyi, -lyi), N3 = pk2(-3.f, -3.f);
    uint64_t GX = 0, GY = 0, GMN = 0;  // packed sums; GMN accumulates +lam.d/r^3
    float gxa = 0.f, gya = 0.f, gma = 0.f;
    auto fetch = [&](int4 m, float4 &b, float2 &l) {
        int j = m.x + lane;
        b = j < m.y ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        l = j < m.y ? lam[j] : make_float2(0.f, 0.f);
        b.x += __int_as_float(m.z);
        b.y += __int_as_float(m.w);
    };
    float4 cb = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 cl = make_float2(0.f, 0.f);
    if (nq > 0) fetch(meta[w][0], cb, cl);
    for (int k = 0; k < nq; k++) {
        float4 nb = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 nl2 = make_float2(0.f, 0.f);
        if (k + 1 < nq) fetch(meta[w][k + 1], nb, nl2);
        __syncwarp();
        sx[w][lane] = cb.x;
        sy[w][lane] = cb.y;
        sm[w][lane] = cb.z;
        slx[w][lane] = cl.x;
        sly[w][lane] = cl.y;
        __syncwarp();
        const int2 se = *reinterpret_cast<const int2 *>(&meta[w][k]);  // this row's begin, end
        const int ns = se.y - se.x;
        if (ns == 32 && k != kown) {
#pragma unroll 4
            for (int kk = 0; kk < 32; kk += 2) {
                const uint64_t X = *reinterpret_cast<const uint64_t *>(&sx[w][kk]);
                const uint64_t Y = *reinterpret_cast<const uint64_t *>(&sy[w][kk]);
                const uint64_t Mj = *reinterpret_cast<const uint64_t *>(&sm[w][kk]);
                const uint64_t LXj = *reinterpret_cast<const uint64_t *>(&slx[w][kk]);
                const uint64_t LYj = *reinterpret_cast<const uint64_t *>(&sly[w][kk]);
                const uint64_t dx = sub2(X, XI), dy = sub2(Y, YI);
                const uint64_t r2 = fma2(dx, dx, fma2(dy, dy, E2));
                float ra, rb;
                upk2(r2, ra, rb);
                const uint64_t ir = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                const uint64_t ir2 = mul2(ir, ir);
                const uint64_t ir3 = mul2(ir2, ir);
                const uint64_t ir5 = mul2(ir3, ir2);
                const uint64_t wx = fma2(Mj, NLXI, mul2(MI, LXj));  // mi lx_j - m_j lx_i
                const uint64_t wy = fma2(Mj, NLYI, mul2(MI, LYj));
                const uint64_t nc = mul2(mul2(N3, ir5), fma2(dx, wx, mul2(dy, wy)));  // -3 dw / r^5
                GX = fma2(ir3, wx, fma2(nc, dx, GX));
                GY = fma2(ir3, wy, fma2(nc, dy, GY));
                GMN = fma2(fma2(LXj, dx, mul2(LYj, dy)), ir3, GMN);
            }
        } else {
            const bool own = k == kown;
            for (int kk = 0; kk < ns; kk++) {
                float dx = sx[w][kk] - xi, dy = sy[w][kk] - yi;
                float mj = sm[w][kk], lxj = slx[w][kk], lyj = sly[w][kk];
                float ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                float ir2 = ir * ir;
                float ir3 = ir2 * ir;
                float ir5 = ir3 * ir2;
                float wx = fmaf(mi, lxj, -mj * lxi), wy = fmaf(mi, lyj, -mj * lyi);
                float c = 3.f * ir5 * fmaf(dx, wx, dy * wy);
                float dl = fmaf(lxj, dx, lyj * dy);
                bool self = own && se.x + kk == i;
                ir3 = self ? 0.f : ir3;
                c = self ? 0.f : c;
                gxa = fmaf(ir3, wx, fmaf(-c, dx, gxa));
                gya = fmaf(ir3, wy, fmaf(-c, dy, gya));
                gma = fmaf(-dl, ir3, gma);
            }
        }
        cb = nb;
        cl = nl2;
    }
    float a0, a1, b0, b1, c0, c1;
    upk2(GX, a0, a1);
    upk2(GY, b0, b1);
    upk2(GMN, c0, c1);
    part[it * 32 + lane] = make_float4((a0 + a1) + gxa, (b0 + b1) + gya, gma - (c0 + c1), 0.f);
}

template <class V, class S>
__global__ void __launch_bounds__(128) k_adj_p2p_reduce(int64_t nl, const int32_t *__restrict__ bs,
                                                        const int32_t *__restrict__ be, const int64_t *__restrict__ item_off,
                                                        int tchunks, const V *__restrict__ part, double *__restrict__ gx,
                                                        double *__restrict__ gy, double *__restrict__ gm) {
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    for (int tc = 0; tc < tchunks && t0 + tc * 32 < t1; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        if (i >= t1) continue;
        // four independent accumulators keep the loads of long slot ranges in flight;
        // the slots of a long item range are mostly group sums (k_fold_items)
        S ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, am[4] = {0, 0, 0, 0};
        const ItemSlots sl(item_off[leaf], item_off[leaf + 1]);
        int j = 0;
        for (; j + 4 <= sl.n; j += 4) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                V v = part[((int64_t)sl[j + u] * tchunks + tc) * 32 + lane];
                ax[u] += v.x;
                ay[u] += v.y;
                am[u] += v.z;
            }
        }
        if (j < sl.n) {  // the last round predicated: its loads in flight together
            V v[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (j + u < sl.n) v[u] = part[((int64_t)sl[j + u] * tchunks + tc) * 32 + lane];
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (j + u < sl.n) {
                    ax[u] += v[u].x;
                    ay[u] += v[u].y;
                    am[u] += v[u].z;
                }
        }
        const S sx = (ax[0] + ax[1]) + (ax[2] + ax[3]), sy = (ay[0] + ay[1]) + (ay[2] + ay[3]),
                smm = (am[0] + am[1]) + (am[2] + am[3]);
        gx[i] += (double)sx;
        gy[i] += (double)sy;
        gm[i] += (double)smm;
    }
}

// Full VJP at positions (X, Y) with the forward's leaf locals lf (rows of T) of those
// positions; masses and the frozen tree/plan come from the context.
template <int P, class T>
int run_force_vjp(gx_ctx *ctx, const double *X, const double *Y, const void *lf_rows, const double *lx,
                  const double *ly, double *gx, double *gy, double *gm) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int64_t nn = ctx->n_nodes, nl = ctx->n_leaves, n = ctx->n_bodies;
    cudaStream_t st = ctx->stream;
    if (nn == 0 || n == 0) return GX_OK;
    const double *Mb = dptr<double>(ctx->m);
    const double *comx = dptr<double>(ctx->comx), *comy = dptr<double>(ctx->comy);
    const int32_t *bs = dptr<int32_t>(ctx->bs), *be = dptr<int32_t>(ctx->be);
    const int4 *child = dptr<int4>(ctx->child);
    const double eps2 = ctx->eps * ctx->eps;
    const unsigned gw = (unsigned)((nl * 32 + 127) / 128);
    const T *Lf = reinterpret_cast<const T *>(lf_rows);
    GX_TRY(gx_ensure(ctx, ctx->adj_dL, sizeof(T) * NS * (size_t)nn));
    GX_TRY(gx_ensure(ctx, ctx->adj_dM, sizeof(T) * NS * (size_t)nn));
    GX_TRY(gx_ensure(ctx, ctx->adj_dMleaf, sizeof(T) * NS * (size_t)nl));
    T *dL = dptr<T>(ctx->adj_dL), *dM = dptr<T>(ctx->adj_dM), *dMl = dptr<T>(ctx->adj_dMleaf);
    constexpr bool F32 = sizeof(T) == 4;
    float4 *pos32 = nullptr;
    float2 *lam32 = nullptr;
    if (F32) {
        GX_TRY(gx_ensure(ctx, ctx->pos32, sizeof(float4) * (size_t)n));
        GX_TRY(gx_ensure(ctx, ctx->adj_lam32, sizeof(float2) * (size_t)n));
        pos32 = dptr<float4>(ctx->pos32);
        lam32 = dptr<float2>(ctx->adj_lam32);
    }
    // A1: L2P^T and the Hessian term (writes gx, gy; the FP32 form also packs bodies)
    k_adj_l2p<P, T><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, Lf, lx, ly, gx, gy, dL, pos32, lam32);
    // A6 (items) on the second, lower-priority stream beside A2..A5: it needs only the
    // bodies packed by A1 and writes per-item partials, summed in order after the join
    const gx_ctx::Items &I = ctx->items_acc;
    const int tchunks = (int)std::max<int64_t>(1, (ctx->max_leaf + 31) / 32);
    const unsigned gi = (unsigned)((I.n * 32 + 127) / 128);
    GX_TRY(gx_ensure(ctx, ctx->part, (F32 ? sizeof(float4) : sizeof(double4)) * 32 * (size_t)tchunks * (size_t)(I.n + 1)));
    GX_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
    GX_CUDA(ctx, cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0));
    if (I.n > 0) {
        if (F32 && tchunks == 1)
            k_adj_p2p32_rows<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                           dptr<int32_t>(I.nq), pos32, lam32, comx, comy, bs, be,
                                                           dptr<int32_t>(ctx->near_idx), (float)eps2,
                                                           dptr<float4>(ctx->part));
        else if (F32)
            k_adj_p2p32_items<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                            dptr<int32_t>(I.nq), pos32, lam32, comx, comy, bs, be,
                                                            dptr<int32_t>(ctx->near_idx), (float)eps2, tchunks,
                                                            dptr<float4>(ctx->part));
        else
            k_adj_p2p_items<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                          dptr<int32_t>(I.nq), X, Y, Mb, lx, ly, bs, be,
                                                          dptr<int32_t>(ctx->near_idx), eps2, tchunks,
                                                          dptr<double4>(ctx->part));
        if (I.n > GX_FOLD_MIN) {
            const unsigned gf = (unsigned)(((I.n + GX_FOLD - 1) / GX_FOLD * 32 + 127) / 128);
            if (F32)
                k_fold_items<float4><<<gf, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.off),
                                                                   tchunks, dptr<float4>(ctx->part));
            else
                k_fold_items<double4><<<gf, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.off),
                                                                    tchunks, dptr<double4>(ctx->part));
        }
    }
    GX_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->stream2));
    // A2: L2L^T upward, level by level (leaves are level 0)
    for (int lv = 1; lv < ctx->n_levels; lv++) {
        int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
        k_adj_l2l_up<P, T><<<gx_blocks(e - s, 128), 128, 0, st>>>(s, e, child, comx, comy, dL);
    }
    // A3: M2L^T
    const gx_ctx::M2LUnits &U = ctx->m2l_units;
    if (U.n > 0) {
        const int64_t *node_u = dptr<int64_t>(U.node_u);
        GX_TRY(gx_ensure(ctx, ctx->m2l_part, sizeof(T) * NS * (size_t)(U.n + 1)));
        k_adj_m2l<P, T><<<(unsigned)((U.n * 32 + 127) / 128), 128, 0, st>>>(
            U.n, dptr<int32_t>(U.node), dptr<int64_t>(U.start), dptr<int32_t>(U.len), node_u,
            dptr<int32_t>(ctx->far_idx), comx, comy, F32 ? dptr<float4>(ctx->comhl) : nullptr, eps2, dL, dM,
            dptr<T>(ctx->m2l_part));
        k_adj_m2l_combine<P, T><<<gx_blocks(nn * NC, 256), 256, 0, st>>>(nn, node_u, dptr<T>(ctx->m2l_part), dM);
    }
    // A4: M2M^T to the leaves
    k_adj_m2m_direct<P, T><<<gw, 128, 0, st>>>(nl, ctx->n_levels, dptr<int32_t>(ctx->anc),
                                               dptr<uint8_t>(ctx->has_far_acc), comx, comy, dM, dMl);
    // A5: P2M^T (adds to gx, gy; writes gm)
    GX_CUDA(ctx, cudaMemsetAsync(gm, 0, sizeof(double) * (size_t)n, st));
    k_adj_p2m<P, T><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, dMl, gx, gy, gm);
    // A6: join, then the ordered sums of the partials (add to gx, gy, gm)
    GX_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0));
    if (F32)
        k_adj_p2p_reduce<float4, float><<<gw, 128, 0, st>>>(nl, bs, be, dptr<int64_t>(I.off), tchunks,
                                                            dptr<float4>(ctx->part), gx, gy, gm);
    else
        k_adj_p2p_reduce<double4, double><<<gw, 128, 0, st>>>(nl, bs, be, dptr<int64_t>(I.off), tchunks,
                                                              dptr<double4>(ctx->part), gx, gy, gm);
    ctx->launches += 6 + (ctx->n_levels - 1) + (I.n > GX_FOLD_MIN ? 1 : 0);
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

}  // namespace

#define GX_ADJ_INSTANTIATE(PP)                                                                             \
    int gx_run_force_vjp_##PP(gx_ctx *ctx, int f32, const double *X, const double *Y, const void *lf,     \
                              const double *lx, const double *ly, double *gx, double *gy, double *gm) {  \
        return f32 ? run_force_vjp<PP, float>(ctx, X, Y, lf, lx, ly, gx, gy, gm)                         \
                   : run_force_vjp<PP, double>(ctx, X, Y, lf, lx, ly, gx, gy, gm);                       \
    }
