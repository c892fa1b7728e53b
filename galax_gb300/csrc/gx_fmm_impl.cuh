// gx_fmm_impl.cuh -- the six FMM passes of compute_fmm_force (galax-core/src/lib.rs:1466-1499)
// as sm_103a kernels, templated on the expansion order P (0..16).
//
// Layout in HBM: bodies are FP64 SoA in tree (Morton) order; expansions are one
// contiguous row of C(P) = (P+1)(P+2)/2 coefficients per node (120 B at P=4 in FP64),
// so a warp reading one node's row reads one contiguous segment.
//
//   P2M   (lib.rs:848-887)   warp per leaf, lane per body, warp-shuffle reduction
//   M2M   (lib.rs:890-938)   warp per parent, lane per output coefficient, per level
//   M2L   (lib.rs:1199-1259) warp per target node, lane per list entry, warp reduction
//   L2L   (lib.rs:1262-1302) REF: node-id-ascending order means every leaf receives
//                            its own M2L local plus one shift of its parent's M2L local;
//                            other modes: top-down per level
//   L2P   (lib.rs:1308-1355) + P2P (lib.rs:1395-1462) fused: warp per target leaf,
//                            lane per body, source leaves staged in shared memory
//
// M2L contraction.  With M'[S] = (-1)^|S| M[S] and the kernel derivatives G, the
// reference's plan (lib.rs:1160-1196) is L[T] = (1/T!) sum_S M'[S] G[S+T]; the 1/T!
// factor is applied once per target after the sum over its sources.
#pragma once
#include "gx_internal.cuh"

namespace {

__host__ __device__ constexpr double cfact(int n) { return n <= 1 ? 1.0 : (double)n * cfact(n - 1); }
__host__ __device__ constexpr double cinvfact(int n) { return 1.0 / cfact(n); }
__host__ __device__ constexpr double cbinom(int n, int k) {
    return (k < 0 || k > n) ? 0.0 : ((k == 0 || k == n) ? 1.0 : cbinom(n - 1, k - 1) + cbinom(n - 1, k));
}
__host__ __device__ constexpr int nc2(int q) { return (q + 1) * (q + 2) / 2; }  // entries with k+l <= q

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class T>
__device__ __forceinline__ T rsqrt_t(T v);
template <>
__device__ __forceinline__ double rsqrt_t<double>(double v) { return rsqrt(v); }
template <>
__device__ __forceinline__ float rsqrt_t<float>(float v) { return rsqrtf(v); }

// ---------------------------------------------------------------- prepare
// compute_fmm_force's input sanitising (lib.rs:1474-1482) and the zeroing of a.
__global__ void k_prepare(int64_t n, double *x, double *y, double *m, double *ax, double *ay, unsigned *status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double xi = x[i], yi = y[i], mi = m[i];
    bool bad = false;
    if (fabs(xi) > 1e100 || fabs(yi) > 1e100 || !isfinite(xi) || !isfinite(yi)) {
        x[i] = 0.0;
        y[i] = 0.0;
        bad = true;
    }
    if (!isfinite(mi) || mi <= 0.0) {
        m[i] = 1.0;
        bad = true;
    }
    if (bad) atomicOr(status, GX_DEV_NONFINITE_INPUT);
    ax[i] = 0.0;
    ay[i] = 0.0;
}

// ---------------------------------------------------------------- P2M
template <int P, class T>
__global__ void __launch_bounds__(128) k_p2m(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                             const double *__restrict__ m, const double *__restrict__ comx,
                                             const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                             const int32_t *__restrict__ be, T *__restrict__ M) {
    constexpr int NC = nc2(P);
    constexpr int UF = P <= 5 ? 64 : 1;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (leaf >= nl) return;
    int32_t b0 = bs[leaf], b1 = be[leaf];
    double cxl = comx[leaf], cyl = comy[leaf];
    T acc[NC];
#pragma unroll UF
    for (int k = 0; k < NC; k++) acc[k] = T(0);
    for (int32_t b = b0 + lane; b < b1; b += 32) {
        T dx = (T)(x[b] - cxl), dy = (T)(y[b] - cyl), mm = (T)m[b];
        T px[P + 1], py[P + 1];
        px[0] = T(1);
        py[0] = T(1);
#pragma unroll UF
        for (int k = 1; k <= P; k++) {
            px[k] = px[k - 1] * dx;
            py[k] = py[k - 1] * dy;
        }
#pragma unroll UF
        for (int i = 0; i <= P; i++)
#pragma unroll UF
            for (int j = 0; j <= P - i; j++)
                acc[gx_mi(i, j)] += mm * px[i] * py[j] * (T)(cinvfact(i) * cinvfact(j));
    }
#pragma unroll UF
    for (int k = 0; k < NC; k++) {
        T v = warp_sum_t<T>(acc[k]);
        if (lane == (k & 31)) M[leaf * NC + k] = isfinite(v) ? v : T(0);
    }
}

// ---------------------------------------------------------------- M2M
template <int P, class T>
__global__ void __launch_bounds__(128) k_m2m(int64_t s, int64_t e, const int4 *__restrict__ child,
                                             const double *__restrict__ comx, const double *__restrict__ comy,
                                             T *__restrict__ M) {
    constexpr int NC = nc2(P);
    constexpr int UF = P <= 5 ? 64 : 1;
    int64_t node = s + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (node >= e) return;
    int4 c4 = child[node];
    int cc[4] = {c4.x, c4.y, c4.z, c4.w};
    double pcx = comx[node], pcy = comy[node];
    for (int o = lane; o < NC; o += 32) {
        // decode o -> (oi, oj): o = n(n+1)/2 + oj with n = oi + oj
        int nn = 0;
        while ((nn + 1) * (nn + 2) / 2 <= o) nn++;
        int oj = o - nn * (nn + 1) / 2, oi = nn - oj;
        T sum = T(0);
        for (int k = 0; k < 4; k++) {
            int c = cc[k];
            if (c < 0) continue;
            T dx = (T)(comx[c] - pcx), dy = (T)(comy[c] - pcy);
            T px[P + 1], py[P + 1];
            px[0] = T(1);
            py[0] = T(1);
#pragma unroll UF
            for (int q = 1; q <= P; q++) {
                px[q] = px[q - 1] * dx;
                py[q] = py[q - 1] * dy;
            }
            const T *Mc = M + (int64_t)c * NC;
            T part = T(0);
            for (int i = 0; i <= oi; i++)
                for (int j = 0; j <= oj; j++)
                    part += Mc[gx_mi(i, j)] * px[oi - i] * py[oj - j] * (T)(cinvfact(oi - i) * cinvfact(oj - j));
            sum += part;
        }
        M[node * NC + o] = sum;
    }
}

template <class T>
__global__ void k_scrub(int64_t n, T *v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !isfinite(v[i])) v[i] = T(0);
}

// ---------------------------------------------------------------- M2L
// Derivatives of 1/R (R^2 = dx^2+dy^2+eps^2) scaled by k! l!:  A[k,l] = k! l! a_kl with
// |k| R^2 a_k = -(2|k|-1)(dx a_{k-ex} + dy a_{k-ey}) - (|k|-1)(a_{k-2ex} + a_{k-2ey}), a_0 = 1/R.
// The kernel of the reference is G = -1/R, so G^(k,l) = -A[k,l].
template <int P, class T>
__device__ __forceinline__ void derivs_scaled(T dx, T dy, T eps2, T *A) {
    constexpr int Q = 2 * P;
    constexpr int UF = P <= 5 ? 64 : 1;
    T r2 = dx * dx + dy * dy + eps2;
    T ir = rsqrt_t<T>(r2);
    T ir2 = ir * ir;
    A[0] = ir;
#pragma unroll UF
    for (int n = 1; n <= Q; n++) {
#pragma unroll UF
        for (int k = 0; k <= n; k++) {
            int l = n - k;
            T s1 = T(0), s2 = T(0);
            // a_{k-1,l} = A[k-1,l]/((k-1)! l!)  ->  in A units: A[k,l] = k!l! a_kl
            if (k >= 1) s1 += dx * A[gx_mi(k - 1, l)] * (T)k;
            if (l >= 1) s1 += dy * A[gx_mi(k, l - 1)] * (T)l;
            if (k >= 2) s2 += A[gx_mi(k - 2, l)] * (T)(k * (k - 1));
            if (l >= 2) s2 += A[gx_mi(k, l - 2)] * (T)(l * (l - 1));
            A[gx_mi(k, l)] = (-(T)(2 * n - 1) * s1 - (T)(n - 1) * s2) * ir2 * (T)(1.0 / n);
        }
    }
}

// REF mode: derivative sets from the first-inserter table (FP64).
template <int P>
__global__ void __launch_bounds__(128) k_m2l_ref(int64_t nn, const uint32_t *__restrict__ vdata,
                                                 const uint8_t *__restrict__ vlen, const int64_t *__restrict__ voff,
                                                 const int32_t *__restrict__ did, const double *__restrict__ G,
                                                 const double *__restrict__ M, double *__restrict__ L) {
    constexpr int NC = nc2(P);
    constexpr int UF = P <= 5 ? 64 : 1;
    constexpr int S = 2 * P + 1;
    int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (node >= nn) return;
    int len = vlen[node];
    double acc[NC];
#pragma unroll UF
    for (int k = 0; k < NC; k++) acc[k] = 0.0;
    for (int s = lane; s < len; s += 32) {
        uint32_t src = vdata[node * GX_LIST_CAP + s];
        const double *g = G + (int64_t)did[voff[node] + s] * (S * S);
        const double *Ms = M + (int64_t)src * NC;
        double ms[NC];
#pragma unroll UF
        for (int k = 0; k < NC; k++) ms[k] = Ms[k];
#pragma unroll UF
        for (int i = 0; i <= P; i++)
#pragma unroll UF
            for (int j = 0; j <= P - i; j++) {
                double mv = ms[gx_mi(i, j)];
                if (mv == 0.0) continue;  // lib.rs:1252: zero source terms are skipped
                double sm = ((i + j) & 1) ? -mv : mv;
#pragma unroll UF
                for (int oi = 0; oi <= P; oi++)
#pragma unroll UF
                    for (int oj = 0; oj <= P - oi; oj++)
                        acc[gx_mi(oi, oj)] += sm * g[gx_kdi(i + oi, j + oj, P)];
            }
    }
#pragma unroll UF
    for (int oi = 0; oi <= P; oi++)
#pragma unroll UF
        for (int oj = 0; oj <= P - oi; oj++) {
            int k = gx_mi(oi, oj);
            double v = warp_sum_t<double>(acc[k]);
            if (lane == (k & 31)) L[node * NC + k] = v * (cinvfact(oi) * cinvfact(oj));
        }
}

// EXACT / ACCURATE: per-pair derivatives.  Lists given as start/count per node.
template <int P, class T, class IDX>
__global__ void __launch_bounds__(128) k_m2l_exact(int64_t nn, const IDX *__restrict__ idx,
                                                   const int64_t *__restrict__ start, const int32_t *__restrict__ cnt,
                                                   const uint8_t *__restrict__ cnt8, int64_t fixed_stride,
                                                   const double *__restrict__ comx, const double *__restrict__ comy,
                                                   double eps2d, const T *__restrict__ M, T *__restrict__ L) {
    constexpr int NC = nc2(P);
    constexpr int UF = P <= 5 ? 64 : 1;
    constexpr int ND = nc2(2 * P);
    int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (node >= nn) return;
    int64_t st = start ? start[node] : node * fixed_stride;
    int len = cnt ? cnt[node] : (int)cnt8[node];
    double tcx = comx[node], tcy = comy[node];
    T eps2 = (T)eps2d;
    T acc[NC];
#pragma unroll UF
    for (int k = 0; k < NC; k++) acc[k] = T(0);
    for (int s = lane; s < len; s += 32) {
        int64_t src = (int64_t)idx[st + s];
        T dx = (T)(tcx - comx[src]), dy = (T)(tcy - comy[src]);
        T A[ND];
        derivs_scaled<P, T>(dx, dy, eps2, A);
        const T *Ms = M + src * NC;
        T ms[NC];
#pragma unroll UF
        for (int k = 0; k < NC; k++) ms[k] = Ms[k];
#pragma unroll UF
        for (int i = 0; i <= P; i++)
#pragma unroll UF
            for (int j = 0; j <= P - i; j++) {
                T sm = ((i + j) & 1) ? -ms[gx_mi(i, j)] : ms[gx_mi(i, j)];
#pragma unroll UF
                for (int oi = 0; oi <= P; oi++)
#pragma unroll UF
                    for (int oj = 0; oj <= P - oi; oj++) acc[gx_mi(oi, oj)] += sm * A[gx_mi(i + oi, j + oj)];
            }
    }
    // G = -A: L[T] = -(1/T!) sum_S M'[S] A[S+T]
#pragma unroll UF
    for (int oi = 0; oi <= P; oi++)
#pragma unroll UF
        for (int oj = 0; oj <= P - oi; oj++) {
            int k = gx_mi(oi, oj);
            T v = warp_sum_t<T>(acc[k]);
            if (lane == (k & 31)) L[node * NC + k] = v * (T)(-cinvfact(oi) * cinvfact(oj));
        }
}

// ---------------------------------------------------------------- L2L
template <int P, class T>
__device__ __forceinline__ T l2l_term(const T *LP, int oi, int oj, const T *px, const T *py) {
    T sum = T(0);
    for (int i = oi; i <= P; i++)
        for (int j = oj; j <= P - i; j++)
            sum += LP[gx_mi(i, j)] * (T)(cbinom(i, oi) * cbinom(j, oj)) * px[i - oi] * py[j - oj];
    return sum;
}

// REF: Lout[leaf] = L[leaf] + shift(L[parent(leaf)])
template <int P, class T>
__global__ void __launch_bounds__(128) k_l2l_ref_leaves(int64_t nl, const int32_t *__restrict__ parent,
                                                        const double *__restrict__ comx, const double *__restrict__ comy,
                                                        const T *__restrict__ L, T *__restrict__ Lout) {
    constexpr int NC = nc2(P);
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (leaf >= nl) return;
    int32_t par = parent[leaf];
    T px[P + 1], py[P + 1];
    px[0] = T(1);
    py[0] = T(1);
    if (par >= 0) {
        T dx = (T)(comx[leaf] - comx[par]), dy = (T)(comy[leaf] - comy[par]);
        for (int q = 1; q <= P; q++) {
            px[q] = px[q - 1] * dx;
            py[q] = py[q - 1] * dy;
        }
    }
    for (int o = lane; o < NC; o += 32) {
        int nn = 0;
        while ((nn + 1) * (nn + 2) / 2 <= o) nn++;
        int oj = o - nn * (nn + 1) / 2, oi = nn - oj;
        T v = L[leaf * NC + o];
        if (par >= 0) v += l2l_term<P, T>(L + (int64_t)par * NC, oi, oj, px, py);
        Lout[leaf * NC + o] = v;
    }
}

// top-down: L[x] += shift(L[parent(x)]) for the nodes of one level
template <int P, class T>
__global__ void __launch_bounds__(128) k_l2l_level(int64_t s, int64_t e, const int32_t *__restrict__ parent,
                                                   const double *__restrict__ comx, const double *__restrict__ comy,
                                                   T *__restrict__ L) {
    constexpr int NC = nc2(P);
    int64_t x = s + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (x >= e) return;
    int32_t par = parent[x];
    if (par < 0) return;
    T px[P + 1], py[P + 1];
    px[0] = T(1);
    py[0] = T(1);
    T dx = (T)(comx[x] - comx[par]), dy = (T)(comy[x] - comy[par]);
    for (int q = 1; q <= P; q++) {
        px[q] = px[q - 1] * dx;
        py[q] = py[q - 1] * dy;
    }
    for (int o = lane; o < NC; o += 32) {
        int nn = 0;
        while ((nn + 1) * (nn + 2) / 2 <= o) nn++;
        int oj = o - nn * (nn + 1) / 2, oi = nn - oj;
        L[x * NC + o] += l2l_term<P, T>(L + (int64_t)par * NC, oi, oj, px, py);
    }
}

// ---------------------------------------------------------------- L2P + P2P
// FP64: a_i = -grad(local) + sum_j m_j (x_j - x_i) / (r^2+eps^2)^(3/2)
template <int P>
__global__ void __launch_bounds__(128) k_l2p_p2p64(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                   const double *__restrict__ m, const double *__restrict__ comx,
                                                   const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                   const int32_t *__restrict__ be, const double *__restrict__ Lf,
                                                   const int64_t *__restrict__ off, const int32_t *__restrict__ cnt,
                                                   const int32_t *__restrict__ src_idx, double eps2,
                                                   double *__restrict__ ax, double *__restrict__ ay) {
    constexpr int NC = nc2(P);
    constexpr int UF = P <= 5 ? 64 : 1;
    __shared__ double sx[4][32], sy[4][32], sm[4][32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    double lcx = comx[leaf], lcy = comy[leaf];
    const double *Ll = Lf + leaf * NC;
    int64_t q0 = off[leaf];
    int64_t q1 = cnt ? q0 + cnt[leaf] : off[leaf + 1];
    for (int32_t tc = t0; tc < t1; tc += 32) {
        int32_t i = tc + lane;
        bool valid = i < t1;
        double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0;
        // L2P (lib.rs:1321-1345)
        double fx = 0.0, fy = 0.0;
        {
            double du = xi - lcx, dv = yi - lcy;
            double px[P + 1], py[P + 1];
            px[0] = 1.0;
            py[0] = 1.0;
#pragma unroll UF
            for (int q = 1; q <= P; q++) {
                px[q] = px[q - 1] * du;
                py[q] = py[q - 1] * dv;
            }
#pragma unroll UF
            for (int a = 0; a <= P; a++)
#pragma unroll UF
                for (int b = 0; b <= P - a; b++) {
                    double c = Ll[gx_mi(a, b)];
                    if (a >= 1) fx += c * (double)a * px[a - 1] * py[b];
                    if (b >= 1) fy += c * (double)b * px[a] * py[b - 1];
                }
        }
        double accx = -fx, accy = -fy;
        for (int64_t q = q0; q < q1; q++) {
            int32_t sl = src_idx[q];
            int32_t s0 = bs[sl], s1 = be[sl];
            for (int32_t sc = s0; sc < s1; sc += 32) {
                int32_t j = sc + lane;
                __syncwarp();
                if (j < s1) {
                    sx[w][lane] = x[j];
                    sy[w][lane] = y[j];
                    sm[w][lane] = m[j];
                }
                __syncwarp();
                int nsrc = min(32, s1 - sc);
                for (int k = 0; k < nsrc; k++) {
                    double dx = sx[w][k] - xi, dy = sy[w][k] - yi;
                    double r2 = dx * dx + dy * dy + eps2;
                    double ir = rsqrt(r2);
                    double f = sm[w][k] * (ir * ir * ir);
                    if (sc + k == i) f = 0.0;
                    accx += f * dx;
                    accy += f * dy;
                }
            }
        }
        if (valid) {
            ax[i] = accx;
            ay[i] = accy;
        }
    }
}

// MIXED: FP32 arithmetic on coordinates relative to the target leaf's COM
// (offsets formed in FP64, rounded once), FP32 accumulation, FP64 result.
template <int P>
__global__ void __launch_bounds__(128) k_l2p_p2p32(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                   const double *__restrict__ m, const double *__restrict__ comx,
                                                   const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                   const int32_t *__restrict__ be, const float *__restrict__ Lf,
                                                   const int64_t *__restrict__ off, const int32_t *__restrict__ cnt,
                                                   const int32_t *__restrict__ src_idx, float eps2,
                                                   double *__restrict__ ax, double *__restrict__ ay) {
    constexpr int NC = nc2(P);
    constexpr int UF = P <= 5 ? 64 : 1;
    __shared__ float4 sb[4][32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    double lcx = comx[leaf], lcy = comy[leaf];
    const float *Ll = Lf + leaf * NC;
    int64_t q0 = off[leaf];
    int64_t q1 = cnt ? q0 + cnt[leaf] : off[leaf + 1];
    for (int32_t tc = t0; tc < t1; tc += 32) {
        int32_t i = tc + lane;
        bool valid = i < t1;
        float xi = valid ? (float)(x[i] - lcx) : 0.f, yi = valid ? (float)(y[i] - lcy) : 0.f;
        float fx = 0.f, fy = 0.f;
        {
            float px[P + 1], py[P + 1];
            px[0] = 1.f;
            py[0] = 1.f;
#pragma unroll UF
            for (int q = 1; q <= P; q++) {
                px[q] = px[q - 1] * xi;
                py[q] = py[q - 1] * yi;
            }
#pragma unroll UF
            for (int a = 0; a <= P; a++)
#pragma unroll UF
                for (int b = 0; b <= P - a; b++) {
                    float c = Ll[gx_mi(a, b)];
                    if (a >= 1) fx += c * (float)a * px[a - 1] * py[b];
                    if (b >= 1) fy += c * (float)b * px[a] * py[b - 1];
                }
        }
        float accx = 0.f, accy = 0.f;
        for (int64_t q = q0; q < q1; q++) {
            int32_t sl = src_idx[q];
            int32_t s0 = bs[sl], s1 = be[sl];
            for (int32_t sc = s0; sc < s1; sc += 32) {
                int32_t j = sc + lane;
                __syncwarp();
                if (j < s1) sb[w][lane] = make_float4((float)(x[j] - lcx), (float)(y[j] - lcy), (float)m[j], 0.f);
                __syncwarp();
                int nsrc = min(32, s1 - sc);
                for (int k = 0; k < nsrc; k++) {
                    float4 b = sb[w][k];
                    float dx = b.x - xi, dy = b.y - yi;
                    float r2 = fmaf(dx, dx, fmaf(dy, dy, eps2));
                    float ir = rsqrtf(r2);
                    float f = b.z * (ir * ir * ir);
                    f = (sc + k == i) ? 0.f : f;
                    accx = fmaf(f, dx, accx);
                    accy = fmaf(f, dy, accy);
                }
            }
        }
        if (valid) {
            ax[i] = (double)accx - (double)fx;
            ay[i] = (double)accy - (double)fy;
        }
    }
}

// ---------------------------------------------------------------- orchestration
struct Timer {
    gx_ctx *ctx;
    bool on;
    int k = 0;
    void mark() {
        if (on) cudaEventRecord(ctx->ev[k++], ctx->stream);
    }
};

template <int P>
int run_forces(gx_ctx *ctx, bool timed) {
    constexpr int NC = nc2(P);
    const int64_t n = ctx->n_bodies, nn = ctx->n_nodes, nl = ctx->n_leaves;
    const bool mixed = ctx->prec == GX_PREC_MIXED;
    const int mode = ctx->mode;
    cudaStream_t st = ctx->stream;
    Timer tm{ctx, timed};
    int64_t launches0 = ctx->launches;
    tm.mark();  // 0
    k_prepare<<<gx_blocks(n, 256), 256, 0, st>>>(n, dptr<double>(ctx->x), dptr<double>(ctx->y), dptr<double>(ctx->m),
                                                 dptr<double>(ctx->ax), dptr<double>(ctx->ay), dptr<unsigned>(ctx->status));
    ctx->launches++;
    tm.mark();  // 1
    if (nn == 0) {
        GX_CUDA(ctx, cudaGetLastError());
        return GX_OK;
    }
    const double *X = dptr<double>(ctx->x), *Y = dptr<double>(ctx->y), *Mb = dptr<double>(ctx->m);
    const double *comx = dptr<double>(ctx->comx), *comy = dptr<double>(ctx->comy);
    const int32_t *bs = dptr<int32_t>(ctx->bs), *be = dptr<int32_t>(ctx->be), *parent = dptr<int32_t>(ctx->parent);
    const int4 *child = dptr<int4>(ctx->child);
    const unsigned gw = (unsigned)((nl * 32 + 127) / 128);
    const double eps2 = ctx->eps * ctx->eps;

    if (!mixed) {
        GX_TRY(gx_ensure(ctx, ctx->M, sizeof(double) * NC * (size_t)nn));
        GX_TRY(gx_ensure(ctx, ctx->L, sizeof(double) * NC * (size_t)nn));
        GX_TRY(gx_ensure(ctx, ctx->Lf, sizeof(double) * NC * (size_t)nl));
        double *M = dptr<double>(ctx->M), *L = dptr<double>(ctx->L), *Lf = dptr<double>(ctx->Lf);
        k_p2m<P, double><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, M);
        ctx->launches++;
        tm.mark();  // 2
        for (int lv = 1; lv < ctx->n_levels; lv++) {
            int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
            k_m2m<P, double><<<(unsigned)(((e - s) * 32 + 127) / 128), 128, 0, st>>>(s, e, child, comx, comy, M);
            ctx->launches++;
        }
        if (ctx->n_levels > 1) {
            k_scrub<double><<<gx_blocks(NC * nn, 256), 256, 0, st>>>(NC * nn, M);
            ctx->launches++;
        }
        tm.mark();  // 3
        const unsigned gn = (unsigned)((nn * 32 + 127) / 128);
        if (mode == GX_MODE_REF) {
            k_m2l_ref<P><<<gn, 128, 0, st>>>(nn, dptr<uint32_t>(ctx->vdata), dptr<uint8_t>(ctx->vlen),
                                             dptr<int64_t>(ctx->ref_voff), dptr<int32_t>(ctx->ref_did),
                                             dptr<double>(ctx->ref_G), M, L);
        } else if (mode == GX_MODE_EXACT) {
            k_m2l_exact<P, double, uint32_t><<<gn, 128, 0, st>>>(nn, dptr<uint32_t>(ctx->vdata), nullptr, nullptr,
                                                                 dptr<uint8_t>(ctx->vlen), GX_LIST_CAP, comx, comy,
                                                                 eps2, M, L);
        } else {
            const int64_t *fs = dptr<int64_t>(ctx->far_off);
            k_m2l_exact<P, double, int32_t><<<gn, 128, 0, st>>>(nn, dptr<int32_t>(ctx->far_idx), fs,
                                                                reinterpret_cast<const int32_t *>(fs + nn), nullptr, 0,
                                                                comx, comy, eps2, M, L);
        }
        ctx->launches++;
        tm.mark();  // 4
        const double *Lleaf = L;
        if (mode == GX_MODE_REF) {
            k_l2l_ref_leaves<P, double><<<gw, 128, 0, st>>>(nl, parent, comx, comy, L, Lf);
            ctx->launches++;
            Lleaf = Lf;
        } else {
            for (int lv = ctx->n_levels - 2; lv >= 0; lv--) {
                int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
                k_l2l_level<P, double><<<(unsigned)(((e - s) * 32 + 127) / 128), 128, 0, st>>>(s, e, parent, comx, comy, L);
                ctx->launches++;
            }
        }
        tm.mark();  // 5
        if (mode == GX_MODE_ACCURATE) {
            const int64_t *ns = dptr<int64_t>(ctx->near_off);
            k_l2p_p2p64<P><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, Lleaf, ns,
                                               reinterpret_cast<const int32_t *>(ns + nn), dptr<int32_t>(ctx->near_idx),
                                               eps2, dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        } else {
            k_l2p_p2p64<P><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, Lleaf, dptr<int64_t>(ctx->p2p_off),
                                               nullptr, dptr<int32_t>(ctx->p2p_idx), eps2, dptr<double>(ctx->ax),
                                               dptr<double>(ctx->ay));
        }
        ctx->launches++;
        tm.mark();  // 6
    } else {
        GX_TRY(gx_ensure(ctx, ctx->Mf32, sizeof(float) * NC * (size_t)nn));
        GX_TRY(gx_ensure(ctx, ctx->Lf32, sizeof(float) * NC * (size_t)nn));
        GX_TRY(gx_ensure(ctx, ctx->Lff32, sizeof(float) * NC * (size_t)nl));
        float *M = dptr<float>(ctx->Mf32), *L = dptr<float>(ctx->Lf32), *Lf = dptr<float>(ctx->Lff32);
        k_p2m<P, float><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, M);
        ctx->launches++;
        tm.mark();
        for (int lv = 1; lv < ctx->n_levels; lv++) {
            int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
            k_m2m<P, float><<<(unsigned)(((e - s) * 32 + 127) / 128), 128, 0, st>>>(s, e, child, comx, comy, M);
            ctx->launches++;
        }
        if (ctx->n_levels > 1) {
            k_scrub<float><<<gx_blocks(NC * nn, 256), 256, 0, st>>>(NC * nn, M);
            ctx->launches++;
        }
        tm.mark();
        const unsigned gn = (unsigned)((nn * 32 + 127) / 128);
        if (mode == GX_MODE_ACCURATE) {
            const int64_t *fs = dptr<int64_t>(ctx->far_off);
            k_m2l_exact<P, float, int32_t><<<gn, 128, 0, st>>>(nn, dptr<int32_t>(ctx->far_idx), fs,
                                                               reinterpret_cast<const int32_t *>(fs + nn), nullptr, 0,
                                                               comx, comy, eps2, M, L);
        } else {
            k_m2l_exact<P, float, uint32_t><<<gn, 128, 0, st>>>(nn, dptr<uint32_t>(ctx->vdata), nullptr, nullptr,
                                                                dptr<uint8_t>(ctx->vlen), GX_LIST_CAP, comx, comy, eps2,
                                                                M, L);
        }
        ctx->launches++;
        tm.mark();
        const float *Lleaf = L;
        if (mode == GX_MODE_REF) {
            k_l2l_ref_leaves<P, float><<<gw, 128, 0, st>>>(nl, parent, comx, comy, L, Lf);
            ctx->launches++;
            Lleaf = Lf;
        } else {
            for (int lv = ctx->n_levels - 2; lv >= 0; lv--) {
                int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
                k_l2l_level<P, float><<<(unsigned)(((e - s) * 32 + 127) / 128), 128, 0, st>>>(s, e, parent, comx, comy, L);
                ctx->launches++;
            }
        }
        tm.mark();
        if (mode == GX_MODE_ACCURATE) {
            const int64_t *ns = dptr<int64_t>(ctx->near_off);
            k_l2p_p2p32<P><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, Lleaf, ns,
                                               reinterpret_cast<const int32_t *>(ns + nn), dptr<int32_t>(ctx->near_idx),
                                               (float)eps2, dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        } else {
            k_l2p_p2p32<P><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, Lleaf, dptr<int64_t>(ctx->p2p_off),
                                               nullptr, dptr<int32_t>(ctx->p2p_idx), (float)eps2,
                                               dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        }
        ctx->launches++;
        tm.mark();
    }
    GX_CUDA(ctx, cudaGetLastError());
    ctx->last_launches = ctx->launches - launches0;
    return GX_OK;
}

}  // namespace

#define GX_FMM_INSTANTIATE(PP) \
    int gx_run_forces_##PP(gx_ctx *ctx, bool timed) { return run_forces<PP>(ctx, timed); }
